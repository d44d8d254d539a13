"""The diffuse-interface (Cahn-Hilliard) path, idm = dim
(cahn_hilliard_solver.f90:41-382 and main_ns_hybrid.F90:595-612, 646-724),
against the CPU oracle: the `dim` routine through its per-routine entry,
and whole FP64 steps per step (tolerance 1e-11 relative max-norm, pressure
solved to 1e-14, as the level-set parity tests)."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from tpls_gb300.api import TplsGpu
from tpls_gb300.channel import make_case

from _util import relmax

pytestmark = pytest.mark.gpu

TOL = 1e-11
SIZES = {"A": (64, 32, 48), "odd": (37, 19, 23)}


@pytest.mark.parametrize("size", list(SIZES))
def test_dim_routine_matches_oracle(size):
    nx, ny, nz = SIZES[size]
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz, idm="dim")
    rng = np.random.default_rng(11)
    C = np.asfortranarray(st["PHI2"] + 0.5)
    Cold = np.asfortranarray(np.clip(C + 1e-3 * rng.standard_normal(C.shape), 0.0, 1.0))
    conv2 = np.asfortranarray(1e-2 * rng.standard_normal(C.shape))
    cprev = np.asfortranarray(1e-2 * rng.standard_normal(C.shape))
    guess = np.asfortranarray(C + 1e-3 * rng.standard_normal(C.shape))
    o = Oracle(nx, ny, nz, params, uin)
    g = TplsGpu(nx, ny, nz, params, uin)
    args = (C, Cold, conv2, cprev, guess, params.max_iteration_dim, params.epn, params.pe, params.height,
            params.dx, params.dy, params.dz, params.dt)
    no, co = o.dim(*args)
    ng, cg = g.dim(*args)
    assert relmax(ng, no) < TOL
    assert relmax(cg, co) < TOL
    g.close()


@pytest.mark.parametrize("size", list(SIZES))
def test_dim_steps_match_oracle(size):
    """Per step: the GPU context is loaded with the oracle's state (its
    ConvPrevPhi and phi3 included), both take one step."""
    nx, ny, nz = SIZES[size]
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz, idm="dim", p_rtol=1e-14, p_maxits=400)
    o = Oracle(nx, ny, nz, params, uin)
    o.set_state(st)
    g = TplsGpu(nx, ny, nz, params, uin)
    rows = (slice(None), slice(1, ny + 1), slice(None))
    for step in range(3):
        g.set_state(o.get_state())
        o.step(1)
        g.step(1)
        for k in ("PHI2", "PHI3", "CONVPREV_PHI", "U2", "V2", "W2"):
            e = relmax(g.get_field(k), o.get_field(k), rows)
            assert e < TOL, (step, k, e)
        dp = (g.get_field("PRES") - o.get_field("PRES"))[1:nx + 1, 1:ny + 1, 1:nz + 1]
        assert np.max(np.abs(dp)) <= 1e-11 * np.max(np.abs(o.get_field("PRES"))), step
        assert g.stats()["p_reason"] == 2
    g.close()


def test_dim_graph_and_eager_steps_are_identical():
    nx, ny, nz = SIZES["A"]
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz, idm="dim")
    a, b = TplsGpu(nx, ny, nz, params, uin), TplsGpu(nx, ny, nz, params, uin)
    b.graphs_enable(False)
    for g in (a, b):
        g.set_state(st)
        assert g.step(4) == 0
    sa, sb = a.get_state(), b.get_state()
    assert all(np.array_equal(sa[k], sb[k]) for k in sa)
    a.close()
    b.close()
