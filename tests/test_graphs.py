"""CUDA-graph steps: every step as one graph launch whose pressure
iterations run under a device-side WHILE node.  The graph path must give
bit-identical state to the kernel-by-kernel path (same kernels, same
order, deterministic reductions), count the same kernels, and report the
pressure outcome through the stats."""
import numpy as np
import pytest

from tpls_gb300.api import STATE_FIELDS, TplsGpu
from tpls_gb300.channel import make_case

pytestmark = pytest.mark.gpu

SIZES = [(64, 32, 48), (37, 19, 23)]


def _pair(nx, ny, nz, precision=0, **kw):
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz, precision=precision, **kw)
    out = []
    for graphs in (False, True):
        g = TplsGpu(nx, ny, nz, params, uin)
        g.set_state(st)
        g.graphs_enable(graphs)
        out.append(g)
    return out


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("dims", SIZES)
def test_graph_steps_bit_identical(dims, precision):
    eager, graph = _pair(*dims, precision=precision)
    # 7 steps: every history phase captured, two graph launches per phase
    assert eager.step(7) == 0
    assert graph.step(7) == 0
    for k in STATE_FIELDS + ["U3", "V3", "W3", "RHS_P"]:
        a, b = graph.get_field(k), eager.get_field(k)
        assert np.array_equal(a, b), k
    se, sg = eager.stats(), graph.stats()
    for k in ("p_its", "p_reason", "p_rnorm", "p_bnorm", "steps_done", "err_u", "err_phi"):
        assert se[k] == sg[k], k
    assert eager.kernel_launches() == graph.kernel_launches()
    eager.close()
    graph.close()


def test_async_steps_and_reason():
    """step_async enqueues without waiting; a pressure cap of one iteration
    at a tight tolerance is reported as KSP_DIVERGED_ITS through p_worst,
    and the run continues (the state still advances every step)."""
    nx, ny, nz = 32, 16, 24
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz, p_rtol=1e-14, p_maxits=1)
    g = TplsGpu(nx, ny, nz, params, uin)
    g.set_state(st)
    g.step_async(4)
    s = g.stats()
    assert s["steps_done"] == 4
    assert s["p_worst"] == -3 and s["p_reason"] == -3 and s["p_its"] == 1
    assert g.stats()["p_worst"] == 0  # reset by the read
    assert g.step(2) == -3
    g.close()


def test_graph_mode_survives_field_upload():
    """Uploading state between graph launches (pointers unchanged) gives the
    same result as a fresh context started from that state (3 steps bring
    the history phase back to that of a fresh context)."""
    nx, ny, nz = 32, 16, 24
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz)
    g = TplsGpu(nx, ny, nz, params, uin)
    g.set_state(st)
    g.step(3)
    mid = g.get_state()
    g.set_state(mid)
    g.step(2)
    h = TplsGpu(nx, ny, nz, params, uin)
    h.set_state(mid)
    h.step(2)
    a, b = g.get_state(), h.get_state()
    assert all(np.array_equal(a[k], b[k]) for k in STATE_FIELDS)
    g.close()
    h.close()


def test_batched_transfers_match_single_field_path():
    """tpls_set_fields / tpls_get_fields: a download of the whole state
    followed, without a host wait, by an upload of the same arrays leaves
    the state as it was (the upload waits for the download on the device);
    a context loaded with set_fields steps bit-identically to one loaded
    field by field; get_fields returns what get_field does."""
    nx, ny, nz = 37, 19, 23
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz)
    a = TplsGpu(nx, ny, nz, params, uin)
    b = TplsGpu(nx, ny, nz, params, uin)
    a.set_state(st)
    a.step(2)
    ref = a.get_state()
    bufs = {k: np.zeros_like(v, order="F") for k, v in ref.items()}
    for _ in range(3):  # round trips through the same host arrays
        a.get_fields_into(bufs)
        a.set_fields(bufs)
    a.sync()
    for k, v in a.get_state().items():
        assert np.array_equal(v, ref[k]), k
    b.set_fields(bufs)
    assert a.step(2) == 0 and b.step(2) == 0
    out = {k: np.zeros_like(v, order="F") for k, v in ref.items()}
    b.get_fields_into(out)
    b.sync()
    sa = a.get_state()
    for k in sa:
        assert np.array_equal(out[k], sa[k]), k
    a.close()
    b.close()


@pytest.mark.gpu
def test_download_is_not_overwritten_by_the_next_steps():
    """tpls_get_fields returns before its copies finish; steps enqueued right
    after it (graph-launched and async) wait for them, so the host arrays
    hold the state of the call, not of a later step."""
    nx, ny, nz = 64, 32, 48
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz)
    g = TplsGpu(nx, ny, nz, params, uin)
    g.set_state(st)
    g.step(1)
    ref = g.get_state()
    bufs = {k: np.zeros_like(v, order="F") for k, v in ref.items()}
    g.get_fields_into(bufs)
    g.step_async(3)  # no host wait between the download and the steps
    g.sync()
    for k in ref:
        assert np.array_equal(bufs[k], ref[k]), k
    assert not np.array_equal(g.get_field("PHI2"), ref["PHI2"])
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("size", [(64, 32, 200), (37, 19, 150), (8, 6, 400)])
def test_segment_chained_odd_sweep_is_bit_identical(size):
    """The odd half-sweep with one block per 64-level segment, each segment
    taking the value entering it from the segment below (the default for
    columns of 3 or more segments), and with one block walking each whole
    column (TPLS_FLAG_ODD_COLUMNS): the same operations, so the states are
    bit-identical; 4, 3 and 7 segments per column; no wait ran out."""
    from tpls_gb300.api import TPLS_FLAG_ODD_COLUMNS
    nx, ny, nz = size
    out = []
    for flags in (0, TPLS_FLAG_ODD_COLUMNS):
        params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz, flags=flags)
        g = TplsGpu(nx, ny, nz, params, uin)
        g.set_state(st)
        assert g.step(3) == 0
        out.append(g.get_state())
        assert g.stats()["kernel_timeouts"] == 0
        g.close()
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), (size, k)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_download_after_async_step_reads_that_step(precision):
    """tpls_get_fields enqueued right after tpls_step_async: the fields final
    after the step's front are copied while its back still runs, the others
    after it; all equal the state after that step, although two more steps
    are enqueued before the host waits."""
    nx, ny, nz = 64, 32, 48
    kw = {"precision": precision, "fp64_parts": 2 if precision else 0}
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz, **kw)
    ref = TplsGpu(nx, ny, nz, params, uin)
    ref.set_state(st)
    assert ref.step(2) == 0
    want = ref.get_state()
    ref.close()
    g = TplsGpu(nx, ny, nz, params, uin)
    g.set_state(st)
    assert g.step(1) == 0
    bufs = {k: np.zeros_like(v, order="F") for k, v in want.items()}
    g.step_async(1)
    g.get_fields_into(bufs)
    g.step_async(2)
    g.sync()
    for k in want:
        assert np.array_equal(bufs[k], want[k]), k
    assert g.stats()["p_worst"] == 0
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_upload_during_the_back_of_a_step(precision):
    """tpls_set_fields enqueued right after tpls_step_async: the fields final
    after the step's front are written while its back still runs (that back
    reads none of them), the others after it; the next steps start from the
    uploaded state exactly as when it is loaded after a wait."""
    nx, ny, nz = 37, 19, 23
    kw = {"precision": precision, "fp64_parts": 2 if precision else 0}
    params, uin, st = make_case("A", nx=nx, ny=ny, nz=nz, **kw)
    out = []
    for early in (True, False):
        g = TplsGpu(nx, ny, nz, params, uin)
        g.set_state(st)
        assert g.step(1) == 0
        if early:
            g.step_async(1)
            g.set_fields(st)
        else:
            assert g.step(1) == 0
            g.sync()
            g.set_state(st)  # field by field after a wait
        assert g.step(2) == 0
        out.append(g.get_state())
        g.close()
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k
