"""Serving: a request loop that runs simulation jobs for many clients on
one GPU.

A job is (grid, fluid ratios, step budget, precision).  Jobs arrive over
time; the server

* admits them in arrival order, first fit among the first `lookahead`
  queued jobs, while the sum of the admitted jobs' device footprints
  (tpls_footprint_bytes, exact to the allocator's 2 MiB unit) stays under
  the memory budget and fewer than `max_active` jobs run;
* keeps every admitted job's state on the device (one context each);
* advances all admitted jobs at once: each job's steps are CUDA-graph
  launches on its own stream, enqueued in chunks that end at the job's
  next snapshot, so the jobs' kernels overlap on the GPU, and new jobs join
  as soon as memory and a slot free up (continuous batching, not a queue
  of whole runs);
* every `snapshot_every` steps (and at the end) reads phi and the
  interface height h(x, y) into the job's result, and the job's pressure
  solve outcome: a job whose solve returned DIVERGED_NAN (the reference's
  KSP reason -9, pressure_solver.F90:88-145) is failed at once and its
  memory and slot are freed for the queue;
* frees a job's device memory when its budget is done;
* creates and destroys the jobs' contexts on a worker thread, so device
  allocation and release (which can wait for the device) never hold up the
  issue of running jobs' steps.

The backend interface (footprint / open / enqueue / done / snapshot / stats
/ close) has a GPU implementation over the C ABI and a CPU mock with a
modelled device, which the scheduler tests use.

The served workload: 2000 jobs with Poisson arrivals; grids and fluid
parameters drawn as in the batched workload with grids up to 384x192x192
(nx in {64..384 step 32}, ny in {32..192 step 32}, nz in {32..192 step
16}); step budgets uniform in 50..1000; 160 GB admission budget.
"""
from __future__ import annotations

import hashlib
import time
from dataclasses import dataclass, field

import numpy as np

from .batch import Instance
from .channel import SEED0

SERVE_SEED = SEED0 + 4
GB = 1e9


@dataclass
class JobSpec:
    id: int
    nx: int
    ny: int
    nz: int
    m: float
    r: float
    re: float
    amp: float
    steps: int
    precision: int
    arrival: float  # seconds after the stream starts
    seed: int

    @property
    def cells(self) -> int:
        return self.nx * self.ny * self.nz

    def instance(self) -> Instance:
        return Instance(self.id, self.nx, self.ny, self.nz, self.m, self.r, self.re, self.amp, self.seed)


@dataclass
class Snapshot:
    step: int
    height: np.ndarray          # (nx, ny) interface height, -1 where none
    phi_digest: str             # sha1 of the phi array
    phi: np.ndarray | None = None


@dataclass
class JobResult:
    spec: JobSpec
    arrival: float = 0.0        # arrival on the server clock (scaled)
    admitted: float = -1.0
    finished: float = -1.0
    steps_done: int = 0
    snapshots: list = field(default_factory=list)
    worst_reason: int = 0
    final: dict | None = None
    failed: bool = False        # stopped early: its pressure solve diverged to NaN

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def draw_jobs(n: int = 2000, rate: float = 1.0, seed: int = SERVE_SEED, precision: int = 1,
              max_dims: tuple = (384, 192, 192), budget_range: tuple = (50, 1000)) -> list[JobSpec]:
    """Seeded job stream: Poisson arrivals at `rate` jobs/s, grids and fluid
    parameters as the batched workload with the grid bounds of max_dims."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for q in range(n):
        t += float(rng.exponential(1.0 / rate))
        nx = int(rng.choice(np.arange(64, max_dims[0] + 1, 32)))
        ny = int(rng.choice(np.arange(32, max_dims[1] + 1, 32)))
        nz = int(rng.choice(np.arange(32, max_dims[2] + 1, 16)))
        m = float(np.exp(rng.uniform(0.0, np.log(20.0))))
        r = float(rng.uniform(1.0, 10.0))
        re = float(rng.uniform(50.0, 500.0))
        amp = float(rng.uniform(0.01, 0.1))
        steps = int(rng.integers(budget_range[0], budget_range[1] + 1))
        out.append(JobSpec(q, nx, ny, nz, m, r, re, amp, steps, precision, t, seed + 10000 + q))
    return out


class GpuBackend:
    """Jobs as contexts of the C ABI, graph-launched steps on their own
    streams."""

    def __init__(self, keep_phi: bool = False):
        import ctypes as C
        from .api import load_library
        self.C = C
        self.lib = load_library()
        self.device = self._current_device()
        self.lib.tpls_footprint_bytes.restype = C.c_longlong
        self.lib.tpls_footprint_bytes.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
        self.lib.tpls_query.argtypes = [C.c_void_p]
        self.lib.tpls_interface_height.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        self.keep_phi = keep_phi

    @staticmethod
    def _current_device() -> int:
        try:
            import torch
            return int(torch.cuda.current_device()) if torch.cuda.is_available() else 0
        except Exception:
            return 0

    def thread_init(self) -> None:
        """Make the server's device current in a worker thread (a new host
        thread starts on device 0)."""
        try:
            import torch
            if torch.cuda.is_available():
                torch.cuda.set_device(self.device)
        except Exception:
            pass

    def footprint(self, spec: JobSpec) -> int:
        return int(self.lib.tpls_footprint_bytes(spec.nx, spec.ny, spec.nz, spec.precision))

    def open(self, spec: JobSpec):
        from .batch import open_instance
        return open_instance(spec.instance(), spec.precision)

    def enqueue(self, h, nsteps: int) -> None:
        h.step_async(nsteps)

    def done(self, h) -> bool:
        s = self.lib.tpls_query(h.ctx)
        if s < 0 or s > 1:
            raise RuntimeError(f"tpls_query: status {s}")
        return s == 1

    def snapshot(self, h, step: int) -> Snapshot:
        phi = h.get_field("PHI2")
        hh = np.empty((h.nx, h.ny), order="F")
        s = self.lib.tpls_interface_height(h.ctx, hh.ctypes.data_as(self.C.POINTER(self.C.c_double)))
        if s:
            raise RuntimeError(f"tpls_interface_height: status {s}")
        return Snapshot(step, hh, hashlib.sha1(phi.tobytes()).hexdigest(), phi if self.keep_phi else None)

    def stats(self, h) -> dict:
        return h.stats()

    def close(self, h) -> None:
        h.close()


class MockBackend:
    """CPU stand-in with a modelled device: enqueued steps of all jobs share
    a device that processes `rate` cell-steps per second in total; a job's
    chunk completes when its share of that throughput has covered it.
    Footprint: `bytes_per_cell` per cell.  Snapshots are seeded arrays."""

    def __init__(self, clock, rate: float = 2e8, bytes_per_cell: float = 400.0, fail_at: dict | None = None):
        import threading
        self.clock = clock
        self.rate = rate
        self.bpc = bytes_per_cell
        self.jobs = {}
        self.next_h = 0
        self.t_last = None
        # job id -> step count from which its pressure solve reports
        # DIVERGED_NAN (a host-side injected failure)
        self.fail_at = dict(fail_at or {})
        self.lock = threading.RLock()  # open/close run on the server's worker thread
        self.closed = []

    def thread_init(self) -> None:
        pass

    def _advance(self):
        now = self.clock()
        if self.t_last is None:
            self.t_last = now
        dt = now - self.t_last
        self.t_last = now
        busy = [j for j in self.jobs.values() if j["pending"] > 0]
        while dt > 0 and busy:
            share = self.rate / len(busy)  # cell-steps/s per busy job
            # time until the first busy job finishes its chunk
            tmin = min(j["pending"] / share for j in busy)
            step = min(dt, tmin)
            for j in busy:
                j["pending"] = max(0.0, j["pending"] - share * step)
            dt -= step
            busy = [j for j in busy if j["pending"] > 1e-9]

    def footprint(self, spec: JobSpec) -> int:
        return int(spec.cells * self.bpc)

    def open(self, spec: JobSpec):
        with self.lock:
            self._advance()
            h = self.next_h
            self.next_h += 1
            self.jobs[h] = {"spec": spec, "pending": 0.0, "steps": 0}
            return h

    def enqueue(self, h, nsteps: int) -> None:
        with self.lock:
            self._advance()
            j = self.jobs[h]
            j["pending"] += j["spec"].cells * nsteps
            j["steps"] += nsteps

    def done(self, h) -> bool:
        with self.lock:
            self._advance()
            return self.jobs[h]["pending"] <= 1e-9

    def snapshot(self, h, step: int) -> Snapshot:
        with self.lock:
            sp = self.jobs[h]["spec"]
        rng = np.random.default_rng(sp.seed + step)
        hh = 0.5 + 0.01 * rng.standard_normal((sp.nx, sp.ny))
        return Snapshot(step, hh, hashlib.sha1(hh.tobytes()).hexdigest())

    def stats(self, h) -> dict:
        with self.lock:
            j = self.jobs[h]
            f = self.fail_at.get(j["spec"].id)
            worst = -9 if (f is not None and j["steps"] >= f) else 0
            return {"steps_done": j["steps"], "p_worst": worst}

    def close(self, h) -> None:
        with self.lock:
            self.closed.append(self.jobs[h]["spec"].id)
            del self.jobs[h]


DIVERGED_NAN = -9  # KSP reason of a pressure solve whose residual became NaN


class Server:
    def __init__(self, backend, budget_bytes: float = 160 * GB, max_active: int = 64, snapshot_every: int = 50,
                 lookahead: int = 8, clock=time.perf_counter, sleep=time.sleep, idle_sleep: float = 2e-4,
                 io_threads: int = 1):
        self.be = backend
        self.budget = budget_bytes
        self.max_active = max_active
        self.snap = snapshot_every
        self.lookahead = lookahead
        self.clock = clock
        self.sleep = sleep
        self.idle_sleep = idle_sleep
        self.peak_bytes = 0
        self.peak_active = 0
        # 0: contexts are created and destroyed on the scheduler's own thread
        self.io_threads = io_threads

    def run(self, jobs: list[JobSpec], time_scale: float = 1.0) -> list[JobResult]:
        """Serve the stream; arrival times are scaled by time_scale.  Returns
        one result per job in id order."""
        from concurrent.futures import ThreadPoolExecutor
        for j in jobs:
            fp = self.be.footprint(j)
            if fp > self.budget:
                raise ValueError(f"job {j.id} needs {fp / GB:.1f} GB, above the {self.budget / GB:.0f} GB budget")
        pool = (ThreadPoolExecutor(max_workers=self.io_threads, initializer=self.be.thread_init)
                if self.io_threads > 0 else None)
        try:
            return self._run(jobs, time_scale, pool)
        finally:
            if pool is not None:
                pool.shutdown(wait=True)

    def _run(self, jobs, time_scale, pool) -> list[JobResult]:
        pending = sorted(jobs, key=lambda j: j.arrival)
        queue: list[JobSpec] = []
        opening = {}  # id -> dict(fut, res, fp): contexts being created
        active = {}   # id -> dict(h, res, fp, inflight)
        closing = []  # (future, fp): contexts being destroyed, memory still held
        results = {}
        used = 0
        t0 = self.clock()
        nxt = 0

        def call(fn, *a):  # on the worker thread, or inline without one
            if pool is None:
                class Done:
                    def __init__(self, v):
                        self.v = v

                    def done(self):
                        return True

                    def result(self):
                        return self.v
                return Done(fn(*a))
            return pool.submit(fn, *a)

        def retire(jid, a, failed=False):
            r = a["res"]
            r.failed = failed
            r.finished = self.clock() - t0
            closing.append((call(self.be.close, a["h"]), a["fp"]))
            results[jid] = r
            del active[jid]

        while nxt < len(pending) or queue or active or opening or closing:
            now = self.clock() - t0
            progressed = False
            # memory of destroyed contexts returns to the budget
            for c in [c for c in closing if c[0].done()]:
                c[0].result()
                used -= c[1]
                closing.remove(c)
                progressed = True
            while nxt < len(pending) and pending[nxt].arrival * time_scale <= now:
                queue.append(pending[nxt])
                nxt += 1
            # admission: first fit among the head of the queue
            q = 0
            while q < min(len(queue), self.lookahead) and len(active) + len(opening) < self.max_active:
                spec = queue[q]
                fp = self.be.footprint(spec)
                if used + fp <= self.budget:
                    queue.pop(q)
                    res = JobResult(spec, arrival=spec.arrival * time_scale, admitted=self.clock() - t0)
                    opening[spec.id] = {"fut": call(self.be.open, spec), "res": res, "fp": fp}
                    used += fp
                    self.peak_bytes = max(self.peak_bytes, used)
                    progressed = True
                else:
                    q += 1
            for jid in [j for j, o in opening.items() if o["fut"].done()]:
                o = opening.pop(jid)
                active[jid] = {"h": o["fut"].result(), "res": o["res"], "fp": o["fp"], "inflight": 0}
                progressed = True
            self.peak_active = max(self.peak_active, len(active))
            # issue: every idle job gets the chunk up to its next snapshot
            for a in active.values():
                if a["inflight"] == 0:
                    r = a["res"]
                    left = r.spec.steps - r.steps_done
                    n = min(self.snap - r.steps_done % self.snap, left)
                    self.be.enqueue(a["h"], n)
                    a["inflight"] = n
                    progressed = True
            # completion
            for jid in list(active):
                a = active[jid]
                if a["inflight"] and self.be.done(a["h"]):
                    r = a["res"]
                    r.steps_done += a["inflight"]
                    a["inflight"] = 0
                    st = self.be.stats(a["h"])
                    worst = int(st.get("p_worst", 0))
                    r.worst_reason = min(r.worst_reason, worst)
                    progressed = True
                    if worst == DIVERGED_NAN:  # no further step of this job means anything
                        r.final = st
                        retire(jid, a, failed=True)
                        continue
                    r.snapshots.append(self.be.snapshot(a["h"], r.steps_done))
                    if r.steps_done >= r.spec.steps:
                        r.final = st
                        retire(jid, a)
            if not progressed:
                self.sleep(self.idle_sleep)
        return [results[j.id] for j in sorted(jobs, key=lambda j: j.id)]


def summarize(results: list[JobResult]) -> dict:
    lat = np.array([r.latency for r in results])
    t_end = max(r.finished for r in results)
    t_start = min(r.arrival for r in results)
    cell_steps = sum(r.spec.cells * r.spec.steps for r in results)
    span = max(t_end - t_start, 1e-9)
    return {"jobs": len(results), "seconds": span, "jobs_per_s": len(results) / span,
            "cell_steps_per_s": cell_steps / span, "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "mean_latency_s": float(lat.mean()),
            "diverged_jobs": int(sum(1 for r in results if r.worst_reason < 0)),
            "failed_jobs": int(sum(1 for r in results if r.failed))}
