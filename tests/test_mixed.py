"""FP32-mixed form (TPLS_PREC_FP32_MIXED) against the FP64 GPU form.

The mixed form runs WENO5, redistancing, CSF, the momentum stencils and
sweeps and the multigrid smoothing in FP32 (WENO5 on rounded copies of the
FP64 state, the momentum stencils on the state split into exact FP32
pairs); the state, the AB3 updates, the CG recurrences
and dot products, the coarsest solve, the projection and the volume
integral stay FP64.  Tolerances (relative max-norm over the field):
phi and u 1e-5 after one step and after 20 steps; v and w (whose scale is
the +-1e-3 noise and the interface-driven secondary flow) 1e-4 after one
step; p 1e-3 after one step: u3 is the FP32 iterate, so its rounding
(~6e-8 |u|) enters RHS_p = div(u3)/dt and moves p by ~1e-4 of its scale,
while the projection removes that divergent noise from the velocity;
liquid volume equal to 1e-8 relative after 20 steps."""
import numpy as np
import pytest

from tpls_gb300.api import STATE_FIELDS, TPLS_FLAG_NO_TMA, TplsGpu
from tpls_gb300.channel import make_case

from _util import relmax

pytestmark = pytest.mark.gpu

NX, NY, NZ = 64, 32, 48
ROWS = (slice(None), slice(1, NY + 1), slice(None))


def _ctx(precision, size=(NX, NY, NZ), **kw):
    nx, ny, nz = size
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz, precision=precision, **kw)
    g = TplsGpu(nx, ny, nz, params, uin)
    g.set_state(st)
    return g


# the FP32 sweeps own four x points per thread: 37 and 33 leave ragged last
# groups (one point for v and w at 33), odd ny takes the unfused ghost-row
# path, and 8x6x160 is a tall column for the odd half-sweep's column march
@pytest.mark.parametrize("size", [(NX, NY, NZ), (37, 19, 23), (33, 17, 31), (8, 6, 160)])
def test_mixed_one_step_from_fp64_state(size):
    ref = _ctx(0, size, p_rtol=1e-12, p_maxits=400)
    ref.step(5)
    s5 = ref.get_state()
    mix = _ctx(1, size, p_rtol=1e-12, p_maxits=400)
    mix.set_state(s5)
    ref2 = _ctx(0, size, p_rtol=1e-12, p_maxits=400)
    ref2.set_state(s5)
    assert ref2.step(1) == 0 and mix.step(1) == 0
    rows = (slice(None), slice(1, size[1] + 1), slice(None))
    e = {k: relmax(mix.get_field(k), ref2.get_field(k), rows) for k in ("PHI2", "U2", "V2", "W2", "PRES")}
    assert e["PHI2"] < 1e-5 and e["U2"] < 1e-5, e
    assert e["V2"] < 1e-4 and e["W2"] < 1e-4, e
    assert e["PRES"] < 1e-3, e
    for g in (ref, ref2, mix):
        g.close()


def test_mixed_twenty_steps_and_volume():
    ref, mix = _ctx(0), _ctx(1)
    assert ref.step(20) == 0 and mix.step(20) == 0
    assert relmax(mix.get_field("PHI2"), ref.get_field("PHI2"), ROWS) < 1e-5
    assert relmax(mix.get_field("U2"), ref.get_field("U2"), ROWS) < 1e-5
    vr, vm = ref.stats()["liquid_volume"], mix.stats()["liquid_volume"]
    assert abs(vm - vr) <= 1e-8 * abs(vr)
    ref.close()
    mix.close()


def test_mixed_deterministic_and_u3():
    """Deterministic; u3 is the FP64 state plus the FP32 defect, close to
    the FP64 form's u3 (not an FP32-rounded field)."""
    a, b, r = _ctx(1), _ctx(1), _ctx(0)
    a.step(4)
    b.step(4)
    r.step(4)
    sa, sb = a.get_state(), b.get_state()
    assert all(np.array_equal(sa[k], sb[k]) for k in STATE_FIELDS)
    u3 = a.get_field("U3")
    assert not np.array_equal(u3, u3.astype(np.float32).astype(np.float64))
    assert relmax(u3, r.get_field("U3"), ROWS) < 1e-6
    for g in (a, b, r):
        g.close()


def test_mixed_with_every_part_fp64_equals_fp64_form():
    """fp64_parts = all four parts: the FP32-mixed driver then launches the
    FP64 form's kernels in the same order, so the state is bit-identical."""
    ref = _ctx(0)
    params, uin, st = make_case("A", nx=NX, ny=NY, nz=NZ, precision=1, fp64_parts=15)
    mix = TplsGpu(NX, NY, NZ, params, uin)
    mix.set_state(st)
    assert ref.step(3) == 0 and mix.step(3) == 0
    a, b = ref.get_state(), mix.get_state()
    assert all(np.array_equal(a[k], b[k]) for k in STATE_FIELDS)
    assert np.array_equal(ref.get_field("U3"), mix.get_field("U3"))
    ref.close()
    mix.close()


@pytest.mark.parametrize("parts", [0, 2, 16, 18])
def test_mixed_hundred_steps_fp32_and_fp64_stencils(parts):
    """100 steps with the momentum stencils in FP32 (parts 0: velocity
    values split into exact FP32 pairs, the sweeps' coefficients recomputed
    from the FP32 viscosity) and in FP64 (parts 16): phi and u stay within
    1e-5 of the FP64 form, v and w within 1e-4, the liquid volume within
    1e-8.  Parts 2 keeps the redistancing iterations in FP64 (the default
    setting), parts 18 both."""
    ref = _ctx(0)
    mix = _ctx(1, fp64_parts=parts)
    assert ref.step(100) == 0 and mix.step(100) == 0
    e = {k: relmax(mix.get_field(k), ref.get_field(k), ROWS) for k in ("PHI2", "U2", "V2", "W2")}
    assert e["PHI2"] < 1e-5 and e["U2"] < 1e-5, e
    assert e["V2"] < 1e-4 and e["W2"] < 1e-4, e
    vr, vm = ref.stats()["liquid_volume"], mix.stats()["liquid_volume"]
    assert abs(vm - vr) <= 1e-8 * abs(vr)
    ref.close()
    mix.close()


def test_tma_staged_advection_is_bit_identical():
    """The FP32 advection with its phi tiles staged by TMA (the default)
    against the same kernel reading phi through the caches
    (TPLS_FLAG_NO_TMA): same arithmetic, so the states are bit-identical,
    on the 64x32x48 channel, on ragged grids (partial tiles at the x, y and
    z ends, ny below the tile height) and on a wide one (12 tiles in x, the
    row pitch of the largest served grids); no block's wait ran out."""
    for size in ((NX, NY, NZ), (37, 5, 23), (70, 19, 9), (384, 16, 24)):
        a = _ctx(1, size, fp64_parts=2)
        b = _ctx(1, size, fp64_parts=2, flags=TPLS_FLAG_NO_TMA)
        assert a.step(3) == 0 and b.step(3) == 0
        sa, sb = a.get_state(), b.get_state()
        for k in STATE_FIELDS:
            assert np.array_equal(sa[k], sb[k]), (size, k)
        assert np.array_equal(a.get_field("CONV2_PHI"), b.get_field("CONV2_PHI"))
        assert a.stats()["kernel_timeouts"] == 0
        a.close()
        b.close()


def test_tma_wait_limit_reports_and_returns():
    """The staged advection's wait for its tile is bounded: a block launched
    with no load issued (nothing completes its barrier) gives up after the
    limit, reports it and writes NaN instead of leaving garbage; the context
    stays usable."""
    import ctypes as C
    g = _ctx(1, fp64_parts=2)
    t, nan = C.c_int(-1), C.c_int(-1)
    assert g.lib.tpls_selftest_wait_limit(g.ctx, C.byref(t), C.byref(nan)) == 0
    assert t.value == 1 and nan.value == 1
    assert g.step(2) == 0 and g.stats()["kernel_timeouts"] == 0
    f = _ctx(0)
    assert f.lib.tpls_selftest_wait_limit(f.ctx, C.byref(t), C.byref(nan)) == 3  # no TMA path
    g.close()
    f.close()
