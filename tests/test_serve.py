"""Job server: scheduling on the CPU mock backend (admission by footprint,
memory budget, slot limit, continuous admission as jobs finish, snapshot
cadence, latency accounting), the footprint function of the C ABI (host
only), and on the GPU that every job's result is the same alone and in a
mix of concurrently running jobs."""
import numpy as np
import pytest

from tpls_gb300.serve import GpuBackend, JobSpec, MockBackend, Server, draw_jobs, summarize


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += dt


def _jobs(n, rate=50.0, seed=5, budget=(50, 200)):
    return draw_jobs(n, rate=rate, seed=seed, max_dims=(128, 64, 64), budget_range=budget)


def test_draw_jobs_seeded_and_in_range():
    a, b = draw_jobs(200), draw_jobs(200)
    assert [x.__dict__ for x in a] == [x.__dict__ for x in b]
    arr = [x.arrival for x in a]
    assert all(t2 > t1 for t1, t2 in zip(arr, arr[1:]))
    for x in a:
        assert x.nx in range(64, 385, 32) and x.ny in range(32, 193, 32) and x.nz in range(32, 193, 16)
        assert 50 <= x.steps <= 1000 and 1.0 <= x.m <= 20.0


def test_mock_server_completes_every_job_with_snapshots():
    clk = FakeClock()
    be = MockBackend(clk, rate=5e8)
    jobs = _jobs(40)
    srv = Server(be, budget_bytes=2e9, max_active=8, clock=clk, sleep=clk.sleep, idle_sleep=1e-3)
    res = srv.run(jobs)
    assert [r.spec.id for r in res] == [j.id for j in jobs]
    for r in res:
        assert r.steps_done == r.spec.steps
        want = list(range(50, r.spec.steps, 50)) + [r.spec.steps]
        assert [s.step for s in r.snapshots] == want
        assert r.admitted >= r.arrival and r.finished > r.admitted
    assert srv.peak_bytes <= 2e9 and srv.peak_active <= 8
    s = summarize(res)
    assert s["jobs"] == 40 and s["p99_latency_s"] >= s["p50_latency_s"] > 0


def test_mock_server_budget_limits_concurrency():
    """With a budget that fits two jobs, at most two run at once, and a job
    that arrives while two run waits for a finish (continuous admission)."""
    clk = FakeClock()
    be = MockBackend(clk, rate=1e8, bytes_per_cell=100.0)
    jobs = [JobSpec(q, 64, 32, 32, 2.0, 1.0, 100.0, 0.05, 100, 1, 0.01 * q, 7 + q) for q in range(5)]
    fp = be.footprint(jobs[0])
    srv = Server(be, budget_bytes=2 * fp + 1, max_active=16, clock=clk, sleep=clk.sleep, idle_sleep=1e-3)
    res = srv.run(jobs)
    assert srv.peak_active == 2
    # jobs 2..4 could only start once an earlier one had finished
    fin = sorted(r.finished for r in res[:2])
    assert all(r.admitted >= fin[0] - 1e-9 for r in res[2:])


def test_mock_server_fails_a_diverged_job_at_once_and_frees_its_slot():
    """A job whose pressure solve reports DIVERGED_NAN (injected on the host
    from step 100) is failed at the first chunk that shows it, closed, and
    its slot goes to the queue; every other job runs to its budget."""
    clk = FakeClock()
    jobs = [JobSpec(q, 64, 32, 32, 2.0, 1.0, 100.0, 0.05, 400, 1, 0.01 * q, 7 + q) for q in range(4)]
    be = MockBackend(clk, rate=1e8, bytes_per_cell=100.0, fail_at={1: 100})
    fp = be.footprint(jobs[0])
    srv = Server(be, budget_bytes=2 * fp + 1, max_active=16, clock=clk, sleep=clk.sleep, idle_sleep=1e-3)
    res = srv.run(jobs)
    bad = res[1]
    assert bad.failed and bad.worst_reason == -9 and bad.steps_done == 100
    assert [s.step for s in bad.snapshots] == [50]  # no snapshot of the diverged state
    for r in res[:1] + res[2:]:
        assert not r.failed and r.steps_done == 400
    # job 2 arrived while 0 and 1 ran: it got job 1's slot before job 0 finished
    assert res[2].admitted < res[0].finished
    assert sorted(be.closed) == [0, 1, 2, 3]
    assert summarize(res)["failed_jobs"] == 1


def test_mock_server_creates_and_destroys_contexts_off_the_issue_thread():
    """Context creation and teardown run on the server's worker thread; the
    steps are issued from the scheduler's thread."""
    import threading
    clk = FakeClock()
    seen = {"open": set(), "close": set(), "enqueue": set()}

    class Recording(MockBackend):
        def open(self, spec):
            seen["open"].add(threading.current_thread().name)
            return super().open(spec)

        def close(self, h):
            seen["close"].add(threading.current_thread().name)
            return super().close(h)

        def enqueue(self, h, n):
            seen["enqueue"].add(threading.current_thread().name)
            return super().enqueue(h, n)

    res = Server(Recording(clk, rate=5e8), budget_bytes=2e9, max_active=4, clock=clk, sleep=clk.sleep,
                 idle_sleep=1e-3).run(_jobs(6))
    assert all(r.steps_done == r.spec.steps for r in res)
    main = threading.current_thread().name
    assert seen["enqueue"] == {main}
    assert main not in seen["open"] and main not in seen["close"]


def test_mock_server_rejects_job_over_budget():
    clk = FakeClock()
    be = MockBackend(clk)
    big = JobSpec(0, 384, 192, 192, 2.0, 1.0, 100.0, 0.05, 50, 1, 0.0, 1)
    with pytest.raises(ValueError):
        Server(be, budget_bytes=1e6, clock=clk, sleep=clk.sleep).run([big])


def test_footprint_bytes_host_only():
    be = GpuBackend()
    small = JobSpec(0, 64, 32, 32, 2.0, 1.0, 100.0, 0.05, 50, 1, 0.0, 1)
    big = JobSpec(1, 384, 192, 192, 2.0, 1.0, 100.0, 0.05, 50, 1, 0.0, 1)
    f_mixed, f_64 = be.footprint(big), be.footprint(JobSpec(**{**big.__dict__, "precision": 0}))
    assert 0 < be.footprint(small) < f_mixed < f_64
    cells = 384 * 192 * 192
    assert 150 * cells < f_mixed < 600 * cells  # FP32 work arrays + FP64 state
    assert be.lib.tpls_footprint_bytes(2, 32, 32, 0) == -1


@pytest.mark.gpu
def test_footprint_covers_actual_allocation():
    import torch
    from tpls_gb300.batch import open_instance
    be = GpuBackend()
    for prec in (0, 1):
        spec = JobSpec(0, 160, 96, 80, 2.0, 1.0, 100.0, 0.05, 50, prec, 0.0, 3)
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        g = open_instance(spec.instance(), prec)
        g.step(1)
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        used = free0 - free1
        fp = be.footprint(spec)
        assert used <= fp + (64 << 20), (prec, used, fp)  # graphs/driver slack
        assert fp <= 1.5 * used + (64 << 20), (prec, used, fp)
        g.close()


@pytest.mark.gpu
def test_gpu_server_result_same_alone_and_in_mix():
    """Six jobs of uneven grids (both precisions) served concurrently; each
    job's snapshots and final phi equal those of the same job served alone."""
    jobs = draw_jobs(6, rate=200.0, seed=11, max_dims=(128, 64, 64), budget_range=(50, 120))
    for q, j in enumerate(jobs):
        j.precision = q % 2
    mix = Server(GpuBackend(keep_phi=True), budget_bytes=40e9, max_active=6).run(jobs)
    for j, rm in zip(jobs, mix):
        alone = Server(GpuBackend(keep_phi=True), budget_bytes=40e9).run([JobSpec(**{**j.__dict__, "arrival": 0.0})])[0]
        assert [s.step for s in rm.snapshots] == [s.step for s in alone.snapshots]
        for a, b in zip(rm.snapshots, alone.snapshots):
            assert a.phi_digest == b.phi_digest
            assert np.array_equal(a.height, b.height)
        assert rm.worst_reason == 0
        h = rm.snapshots[-1].height
        assert np.all((h > 0.2) & (h < 0.8))  # the interface stays near mid-channel


@pytest.mark.gpu
def test_contexts_created_on_a_thread_while_steps_are_captured():
    """Contexts created and destroyed on a worker thread while the main
    thread captures other contexts' step graphs (each context's first three
    steps capture one graph each), as the server does: every capture and
    every step succeeds."""
    import threading
    from tpls_gb300.batch import Instance, open_instance
    stop, first = threading.Event(), threading.Event()
    errors, churned = [], []

    def churn():
        try:
            q = 0
            while not stop.is_set():
                g = open_instance(Instance(100 + q, 96, 64, 48, 2.0, 1.0, 100.0, 0.05, 50 + q), q % 2)
                g.close()
                q += 1
                first.set()
            churned.append(q)
        except Exception as e:  # reported on the main thread
            errors.append(e)
            first.set()

    t = threading.Thread(target=churn)
    t.start()
    first.wait(timeout=120)  # the churn is under way before the captures start
    try:
        for q in range(12):
            g = open_instance(Instance(q, 64, 32, 32, 2.0, 1.0, 100.0, 0.05, 7 + q), q % 2)
            assert g.step(3) == 0
            assert g.stats()["p_worst"] == 0
            g.close()
    finally:
        stop.set()
        t.join()
    assert not errors, errors
    assert churned and churned[0] > 0
