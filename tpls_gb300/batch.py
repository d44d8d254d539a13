"""Batched channels: many independent TPLS channels of uneven grid sizes
advanced together on one GPU.

Each member is an ordinary context (tpls_gpu_create) holding its own
device-resident state; a batch (tpls_batch_create) advances all members by
one CUDA-graph launch per step, the graph holding every member's step as a
parallel branch with its pressure iterations under a device-side WHILE
node.  The members' kernels therefore share the GPU's SMs concurrently,
which small channels (64x32x32 = 65k cells cannot fill 152 SMs) need.

The batched workload: 48 instances with seeded draws nx in {64..256 step
32}, ny in {32..128 step 32}, nz in {32..128 step 16}, viscosity ratio m
log-uniform in [1, 20], density ratio r uniform in [1, 10] (recorded only:
the reference has no density ratio), Re uniform in [50, 500], interface
amplitude uniform in [0.01, 0.1] (the bound of the 4 seeded modes, whose
wavelengths are kept >= 1, the channel height: with cubic cells a box can
be as narrow as Ly = 32/128, where 4 spanwise modes of amplitude 0.1 would
fold the interface), 200 steps each in the FP32-mixed form.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np

from .api import TplsError, TplsGpu, load_library
from .channel import SEED0, Workload, make_case

BATCH_SEED = SEED0 + 3


@dataclass
class Instance:
    idx: int
    nx: int
    ny: int
    nz: int
    m: float
    r: float
    re: float
    amp: float
    seed: int

    @property
    def cells(self) -> int:
        return self.nx * self.ny * self.nz

    def workload(self) -> Workload:
        return Workload(f"instance {self.idx}: {self.nx}x{self.ny}x{self.nz}, m={self.m:.3g}, Re={self.re:.3g}",
                        self.nx, self.ny, self.nz, self.m, self.re, self.r, self.amp, 4, 200, self.seed,
                        min_wavelength=1.0)


def draw_instances(n: int = 48, seed: int = BATCH_SEED, max_dims: tuple | None = None) -> list[Instance]:
    """The seeded instance list of the batched workload (max_dims clips the
    grid draws, e.g. for small test batches)."""
    rng = np.random.default_rng(seed)
    out = []
    for q in range(n):
        nx = int(rng.choice(np.arange(64, 257, 32)))
        ny = int(rng.choice(np.arange(32, 129, 32)))
        nz = int(rng.choice(np.arange(32, 129, 16)))
        m = float(np.exp(rng.uniform(0.0, np.log(20.0))))
        r = float(rng.uniform(1.0, 10.0))
        re = float(rng.uniform(50.0, 500.0))
        amp = float(rng.uniform(0.01, 0.1))
        if max_dims:
            nx, ny, nz = min(nx, max_dims[0]), min(ny, max_dims[1]), min(nz, max_dims[2])
        out.append(Instance(q, nx, ny, nz, m, r, re, amp, seed + 1000 + q))
    return out


# FP32-mixed instances keep the redistancing iterations in FP64
# (TPLS_PART_LEVELSET): phi and u stay within 1e-7 of the FP64 form over 500
# steps of the 512x256x256 channel, at 2.3x its speed
MIXED_PARTS = 2


def open_instance(inst: Instance, precision: int = 1, tune: bool = False, **kw) -> TplsGpu:
    kw.setdefault("fp64_parts", MIXED_PARTS if precision == 1 else 0)
    params, uin, st = make_case(inst.workload(), precision=precision, **kw)
    g = TplsGpu(inst.nx, inst.ny, inst.nz, params, uin)
    g.set_state(st)
    if tune:
        g.autotune()
        g.set_state(st)
    return g


class Batch:
    """tpls_batch over existing contexts (which stay owned by the caller)."""

    def __init__(self, members: list[TplsGpu], multi_sweeps: bool = False):
        """multi_sweeps: the members' FP32 momentum sweeps as multi-instance
        launches (tpls_batch_multi_sweeps; FP32-mixed members with FP32
        sweeps, even ny, equal sweep counts)."""
        self.lib = load_library()
        self.lib.tpls_batch_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)]
        self.lib.tpls_batch_multi_sweeps.argtypes = [C.c_void_p, C.c_int]
        self.lib.tpls_batch_destroy.argtypes = [C.c_void_p]
        self.lib.tpls_batch_step.argtypes = [C.c_void_p, C.c_int]
        self.lib.tpls_batch_step_async.argtypes = [C.c_void_p, C.c_int]
        self.members = members
        arr = (C.c_void_p * len(members))(*[m.ctx for m in members])
        h = C.c_void_p()
        s = self.lib.tpls_batch_create(arr, len(members), C.byref(h))
        if s:
            raise TplsError(f"tpls_batch_create: {self.lib.tpls_status_string(s).decode()}")
        self.h = h
        if multi_sweeps:
            s = self.lib.tpls_batch_multi_sweeps(self.h, 1)
            if s:
                self.close()
                raise TplsError(f"tpls_batch_multi_sweeps: {self.lib.tpls_status_string(s).decode()}")

    def step(self, nsteps: int = 1) -> int:
        s = self.lib.tpls_batch_step(self.h, nsteps)
        if s > 0:
            raise TplsError(f"tpls_batch_step: {self.lib.tpls_status_string(s).decode()}")
        return s

    def step_async(self, nsteps: int = 1) -> None:
        s = self.lib.tpls_batch_step_async(self.h, nsteps)
        if s:
            raise TplsError(f"tpls_batch_step_async: {self.lib.tpls_status_string(s).decode()}")

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.tpls_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_batched(instances: list[Instance], steps: int, precision: int = 1, warmup: int = 0) -> dict:
    """All instances in one batch; returns wall time of the timed steps and
    the members' final status."""
    import torch
    members = [open_instance(i, precision) for i in instances]
    b = Batch(members)
    if warmup:
        b.step(warmup)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rc = b.step(steps)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    stats = [m.stats() for m in members]
    b.close()
    for m in members:
        m.close()
    return {"seconds": dt, "rc": rc, "stats": stats}


def run_one_by_one(instances: list[Instance], steps: int, precision: int = 1, warmup: int = 0) -> dict:
    """The same instances run in sequence, each as its own graph-launched
    context (the comparison the batch is measured against)."""
    import torch
    total = 0.0
    worst = 0
    for inst in instances:
        g = open_instance(inst, precision, tune=True)
        if warmup:
            g.step(warmup)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = g.step(steps)
        torch.cuda.synchronize()
        total += time.perf_counter() - t0
        worst = min(worst, rc)
        g.close()
    return {"seconds": total, "rc": worst}
