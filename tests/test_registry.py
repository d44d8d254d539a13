"""Host-array registry (tpls_register_host): a driver that keeps calling the
per-routine entries with the same host arrays gets the same results as with
plain host arrays, while those arrays stay device-resident (the host copies
change only on tpls_download_host).  Runs a short momentum/pressure sequence
of the reference's time loop (main_ns_hybrid.F90:646-913: viscosity, SOR
sweeps of u, source term, pressure solve, projection) both ways on a ragged
box-geometry grid and requires bit-identical results."""
import numpy as np
import pytest

from tpls_gb300.api import TplsError, TplsGpu
from tpls_gb300.channel import make_case

NX, NY, NZ = 37, 19, 23


def _inputs(g, st, seed):
    rng = np.random.default_rng(seed)
    u3, v3, w3 = (np.array(st[k], order="F") for k in ("U2", "V2", "W2"))
    rhs_u = np.asfortranarray(rng.normal(scale=1e-3, size=g.shape("uv")))
    va = np.zeros(g.shape("va"), order="F")
    return {"u3": u3, "v3": v3, "w3": w3, "rhs_u": rhs_u, "va": va,
            "phi": np.array(st["PHI2"], order="F"), "pres_old": np.array(st["PRES_OLD"], order="F")}


def _sequence(g, p, uin, a, register):
    if register:
        for x in a.values():
            g.register_host(x)
    start = {k: v.copy() for k, v in a.items()}
    g.get_viscosity(a["phi"], p.smooth_width, p.re, p.mu_minus, p.mu_plus, viscosity_aug=a["va"])
    for it in range(4):
        g.do_sor_u(a["u3"], a["rhs_u"], a["va"], p.dx, p.dy, p.dz, p.dt, it % 2, (it // 2) % 2)
    rhs_p = g.get_source_pres(a["u3"], a["v3"], a["w3"], p.dx, p.dy, p.dz, p.dt)
    pres, its, _, reason = g.pressure_solve(a["pres_old"], rhs_p, a["u3"], uin, p.dx, p.dy, p.dz, p.dt,
                                            rtol=1e-10, maxits=200)
    g.get_uvw_pres(a["u3"], a["v3"], a["w3"], pres, p.dx, p.dy, p.dz, p.dt, uin)
    if register:
        for k, x in a.items():  # the host copies are untouched until downloaded
            assert np.array_equal(x, start[k], equal_nan=True), k
        g.download_host()
        for x in a.values():
            g.unregister_host(x)
    return rhs_p, pres, reason


@pytest.mark.gpu
def test_registered_arrays_match_host_arrays_and_stay_on_device():
    p, uin, st = make_case("A", nx=NX, ny=NY, nz=NZ, geometry="box")
    g = TplsGpu(NX, NY, NZ, p, uin)
    try:
        a_host = _inputs(g, st, 3)
        a_reg = {k: v.copy(order="F") for k, v in a_host.items()}
        r_host = _sequence(g, p, uin, a_host, False)
        r_reg = _sequence(g, p, uin, a_reg, True)
        assert r_host[2] == 2 and r_reg[2] == 2
        for x, y in zip(r_host[:2], r_reg[:2]):
            assert np.array_equal(x, y)
        for k in a_host:
            assert np.array_equal(a_host[k], a_reg[k], equal_nan=True), k
    finally:
        g.close()


@pytest.mark.gpu
def test_registry_upload_download_and_overlap():
    p, uin, st = make_case("A", nx=NX, ny=NY, nz=NZ)
    g = TplsGpu(NX, NY, NZ, p, uin)
    try:
        u = np.array(st["U2"], order="F")
        g.register_host(u)
        with pytest.raises(TplsError):
            g.register_host(u)  # overlaps the registered range
        ref = u.copy()
        u[:] = 0.0  # host change not yet uploaded: the mirror keeps the old values
        g.download_host(u)
        assert np.array_equal(u, ref)
        u *= 2.0
        g.upload_host(u)
        u[:] = 0.0
        g.download_host(u)
        assert np.array_equal(u, 2.0 * ref)
        # a set_field through the registered address loads the mirror
        g.set_field("U3", u)
        assert np.array_equal(g.get_field("U3")[:, 1:NY + 1], 2.0 * ref[:, 1:NY + 1])
        g.unregister_host(u)
        with pytest.raises(TplsError):
            g.download_host(u)
    finally:
        g.close()
