"""The no-allocation entry point against the allocating one.

tpls_get_difference_noalloc serves callers that cannot allocate device
memory (a latency-bound step loop, or a program whose device memory belongs
to another pool or to a fixed HBM budget).  It must give the same sum as
tpls_get_difference on two calls in a row (the second call proves the
shared scratch array carries nothing over), and refuse inputs larger than
its fixed scratch.  Collected last so a failure here leaves every other
test already run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, as for tpls_get_difference in the parity tests


def _noalloc(lib):
    f = lib.tpls_get_difference_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def test_no_alloc_difference_matches_allocating_entry_twice():
    """Two calls in a row, the second on a smaller grid (fewer rows than the
    first call left in the shared scratch): each must equal the NumPy sum of
    (ua - ub)^2 over i 1..nx, j 1..ny and every plane, and the allocating
    entry's result."""
    torch = pytest.importorskip("torch")
    from tpls_gb300.api import TplsGpu, load_library
    from tpls_gb300.channel import make_case

    lib = load_library()
    fn = _noalloc(lib)
    rng = np.random.default_rng(2026)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call, (nx, ny, nz) in enumerate(((37, 19, 23), (20, 11, 9))):
        params, uin, _ = make_case("A", nx=nx, ny=ny, nz=nz)
        g = TplsGpu(nx, ny, nz, params, uin)
        ua = np.asfortranarray(rng.normal(size=(nx + 2, ny + 2, nz)) * (call + 1))
        ub = np.asfortranarray(rng.normal(size=(nx + 2, ny + 2, nz)))
        d = (ua - ub)[1:nx + 1, 1:ny + 1, :]
        expect = float(np.sum(d * d))
        assert abs(g.get_difference(ua, ub) - expect) <= TOL * expect
        g.close()
        da = torch.from_numpy(ua.ravel(order="F")).cuda()
        db = torch.from_numpy(ub.ravel(order="F")).cuda()
        s = fn(da.data_ptr(), db.data_ptr(), nx, ny, nz, out.data_ptr(), stream)
        assert s == 0, lib.tpls_status_string(s)
        torch.cuda.synchronize()
        got = float(out.item())
        assert abs(got - expect) <= TOL * expect, (call, got, expect)


def test_no_alloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from tpls_gb300.api import load_library

    lib = load_library()
    fn = _noalloc(lib)
    a = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    # 300 rows x 300 planes > 65536 rows: refused before any launch
    s = fn(a.data_ptr(), a.data_ptr(), 4, 300, 300, out.data_ptr(), None)
    assert s == 5  # TPLS_ERR_NOALLOC_LIMIT
