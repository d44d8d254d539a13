"""The seeded synthetic channels that stand in for a dataset
(tpls_gb300/channel.py): deterministic, phi = z - h(x, y) on every point,
the base profile plus bounded noise, periodic rows, the time-step bound."""
import numpy as np
import pytest

from tpls_gb300.channel import WORKLOADS, interface_height, make_case


@pytest.mark.parametrize("name,size", [("A", (16, 8, 12)), ("B", (24, 12, 16))])
def test_make_case_layout_and_determinism(name, size):
    nx, ny, nz = size
    p, uin, st = make_case(name, nx=nx, ny=ny, nz=nz)
    p2, uin2, st2 = make_case(name, nx=nx, ny=ny, nz=nz)
    assert p == p2 and np.array_equal(uin, uin2)
    for k in st:
        assert np.array_equal(st[k], st2[k]), k
    assert st["PHI2"].shape == (nx + 2, ny + 2, nz + 2)
    assert st["U2"].shape == st["V2"].shape == (nx + 2, ny + 2, nz)
    assert st["W2"].shape == (nx + 2, ny + 2, nz + 1)
    assert all(a.flags.f_contiguous for a in st.values())
    # cubic cells, smoothing width 1.5 dx
    assert p.dx == p.dy == p.dz == 1.0 / nz and p.smooth_width == 1.5 * p.dx
    # phi = z - h(x, y) at every point including ghosts
    w = WORKLOADS[name]
    xi = (np.arange(nx + 2) - 0.5) * p.dx
    yj = (np.arange(ny + 2) - 0.5) * p.dy
    zk = (np.arange(nz + 2) - 0.5) * p.dz
    h = interface_height(w, xi[:, None], yj[None, :], nx * p.dx, ny * p.dy)
    assert np.array_equal(st["PHI2"], zk[None, None, :] - h[:, :, None])
    # u = base profile (the inlet) plus noise of at most 1e-3; v, w noise only
    assert np.max(np.abs(st["U2"] - uin[None, None, :])) <= 1e-3
    assert np.max(np.abs(st["V2"])) <= 1e-3 and np.max(np.abs(st["W2"])) <= 1e-3
    assert np.max(np.abs(st["V2"])) > 0
    # periodic y rows, walls of w, p = -x
    for k in ("U2", "V2", "W2"):
        a = st[k]
        assert np.array_equal(a[:, 0, :], a[:, ny, :]) and np.array_equal(a[:, ny + 1, :], a[:, 1, :])
    assert not np.any(st["W2"][:, :, 0]) and not np.any(st["W2"][:, :, nz])
    assert np.allclose(st["PRES"], np.broadcast_to(-xi[:, None, None], st["PRES"].shape), rtol=0, atol=1e-15)
    # CFL 0.2 on the base flow, or half the capillary limit if smaller
    dt = min(0.2 * p.dx / np.max(np.abs(uin)), 0.5 * np.sqrt(p.dx ** 3 / (2.0 * np.pi)))
    assert p.dt == dt


def test_seeds_differ_between_workloads():
    a = make_case("A", nx=16, ny=8, nz=12)[2]["V2"]
    b = make_case("B", nx=16, ny=8, nz=12)[2]["V2"]
    assert not np.array_equal(a, b)


def test_diffuse_interface_case_adds_its_state():
    p, _, st = make_case("A", nx=16, ny=8, nz=12, idm="dim")
    assert p.idm == 1 and p.epn == 1.5 * p.dz
    assert np.array_equal(st["PHI3"], st["PHI2"]) and not np.any(st["CONVPREV_PHI"])
