#!/usr/bin/env python
"""Throughput of the TPLS per-timestep hot path on GB300.

Default workload: the FP64 form on the 256x128x192 channel (m=2, Re=200,
4-mode seeded interface, mom_u/v/w = 30, levelset = 10, PETSc's default
pressure rtol 1e-5), K timed steps after W warm-up steps, FP64 throughout
(--mg-fp32: FP32 multigrid levels in the CG preconditioner, with CG, its
residuals and the solution still FP64).

Arms
  (default) the CUDA library through its C ABI, device-resident state;
            value = cell-steps/s over the timed steps (CUDA events on the
            library's stream, max over ranks); e2e = the same metric through
            the per-step host-buffer path (state uploaded from pinned host
            memory and downloaded every step).
  --impl reference
            the reference's CPU algorithm on this host's cores: the C
            restatement of the Fortran routines (oracle/), OpenMP over all
            cores, same workload and metric.  The Fortran/MPI/PETSc reference
            itself cannot be built on these machines.

Multi-GPU: the path is not sharded (one channel per GPU); --gpus N under
torchrun runs N independent replicas and reports the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

HEADLINE_METRIC = "cell-steps/s FP64 vs FP32-mixed at stated phi/u error; jobs/s, p50/p99 latency"


def _peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            pass
    return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, gpu_index: int):
        self.proc = None
        self.path = None
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(gpu_index), "-lms", "200"], stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def max_over_ranks(values, dist=None, device="cpu"):
    """Element-wise maximum of `values` over all ranks (one all-reduce): the
    slowest replica's timings, which set the job's throughput."""
    if dist is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def replica_throughput(ws: int, units_per_rank: float, ms: float) -> float:
    """Whole-job rate of ws independent replicas that each processed
    units_per_rank units, over the slowest replica's time (ms)."""
    return ws * units_per_rank / (ms / 1e3)


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _algorithmic_bytes(nx, ny, nz, mom, esz=8):
    """Compulsory bytes of the momentum-sweep launches, per point of the
    component grid.  FP64 (esz 8): Jacobi 32 B (x_old, RHS, mu read, x
    written), a red-black half-sweep 28 B (x and mu read in full, RHS of the
    relaxed colour, that colour written).  FP32 sweeps (esz 4; x, mu and the
    defect b in FP32): Jacobi 16 B, half-sweep 12 B.  Returns (Jacobi bytes,
    odd half-sweep bytes, Jacobi launches, odd half-sweep launches) of one
    step."""
    pts = [(nx - 1) * ny * nz, nx * ny * nz, nx * ny * (nz - 1)]
    outer = mom // 2
    n_odd = (outer + 1) // 2  # outer iterations 1, 3, 5, ... use the odd sweep
    jac_pt, half_pt = (32.0, 28.0) if esz == 8 else (16.0, 12.0)
    jac = sum(jac_pt * p for p in pts) * outer
    sor_odd = sum(half_pt * p for p in pts) * 2 * n_odd
    return jac, sor_odd, 3 * outer, 6 * n_odd


def _profile_figure(tag: str, kernel: str, workload: str | None) -> dict | None:
    """A figure from the committed ncu summaries: lines
    '<tag> <kernel> <workload>: <number> build <digest>' (tag 'traffic' =
    DRAM bytes per launch, 'fp64pipe' = FP64 pipe active % of peak; digest =
    tpls_gb300.build.source_digest() of the build the capture was taken of;
    workload None: the first line of any workload).
    Returns {"value", "file", "build", "current", "workload"}: `current`
    says whether the capture is of the sources this run was built from.
    ncu figures are not measured by this run; a figure whose build differs
    is reported only under its capture record."""
    import re
    from tpls_gb300.build import source_digest
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for line in f.read_text().splitlines():
            m = re.match(r"(\S+) (\S+) (\S+): ([0-9.]+) build ([0-9a-f]+)", line.strip())
            if m and m.group(1) == tag and m.group(2) == kernel and workload in (None, m.group(3)):
                return {"value": float(m.group(4)), "file": f"profiles/{f.name}", "build": m.group(5),
                        "current": m.group(5) == source_digest(), "workload": m.group(3)}
    return None


def run_gpu(args, ws, rank, local) -> dict | None:
    import torch
    from tpls_gb300.api import TPLS_FLAG_NO_TMA, TPLS_FLAG_ODD_COLUMNS, TplsGpu
    from tpls_gb300.channel import WORKLOADS, make_case

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w = WORKLOADS[args.config]
    precision = _precision(args)
    parts = args.fp64_parts if precision == 1 else 0
    nx, ny, nz = args.grid if args.grid else (w.nx, w.ny, w.nz)
    params, uin, st = make_case(args.config, nx=nx, ny=ny, nz=nz, p_rtol=args.p_rtol, precision=precision,
                                fp64_parts=parts, mg_fp32=1 if (precision == 0 and args.mg_fp32) else 0,
                                idm=args.idm, pe=args.dim_pe,
                                flags=(TPLS_FLAG_NO_TMA if args.no_tma else 0)
                                | (TPLS_FLAG_ODD_COLUMNS if args.odd_columns else 0))
    cells = nx * ny * nz
    g = TplsGpu(nx, ny, nz, params, uin)
    g.set_state(st)
    # the library's sweep-tile autotuner, on request (results do not depend on
    # its choice; timed on single kernels, it can pick tiles slower in the step)
    tiles = g.autotune(5) if args.autotune else None
    rc = g.step(args.warmup)
    g.sync()
    if rc != 0:
        raise SystemExit(f"tpls_step returned {rc} during warm-up")
    ext = torch.cuda.ExternalStream(g.stream_ptr())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = g.kernel_launches()
    sampler = ClockSampler(local) if rank == 0 else None
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    # timed region: tpls_step, one CUDA-graph launch per step
    ev0.record(ext)
    rc = g.step(args.steps)
    ev1.record(ext)
    torch.cuda.synchronize()
    if rc != 0:
        raise SystemExit(f"tpls_step returned {rc} in the timed region: the run is not a valid measurement")
    if dist:
        dist.barrier()
    clocks = sampler.stop() if sampler else None
    ms = ev0.elapsed_time(ev1)
    launches = g.kernel_launches() - l0
    stats = g.stats()
    # phase breakdown: a separate, shorter pass launched kernel by kernel
    # with CUDA events between phases (not part of the timed region)
    nph = max(1, min(args.steps, args.phase_steps))
    g.timing_enable(True)
    g.timing_read(reset=True)
    if g.step(nph) != 0:
        raise SystemExit("tpls_step failed in the phase-timing pass")
    phases = g.timing_read(reset=True)
    g.timing_enable(False)
    ms = max_over_ranks([ms], dist, "cuda")[0]
    value = replica_throughput(ws, cells * args.steps, ms)

    # e2e: the per-step host-buffer path through the C ABI (pinned host state
    # uploaded, one step, state downloaded), CUDA events on the same stream
    ke = max(1, min(args.steps, args.e2e_steps))
    host = {}
    state_fields = g.state_fields()
    for k in state_fields:
        a = g.get_field(k)
        buf = torch.empty(tuple(reversed(a.shape)), dtype=torch.float64, pin_memory=True).numpy().T
        buf[...] = a
        host[k] = buf
    bi = sum(a.nbytes for a in host.values())
    # untimed round trip: the batched transfers' streams, events and staging
    # buffer are created on first use (the state is set to itself)
    g.get_fields_into(host)
    g.set_fields(host)
    g.sync()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(ke):
        g.set_fields(host)  # the whole state from pinned host memory
        g.step_async(1)
        g.get_fields_into(host)  # and back; the next upload waits for it on the device
    g.xfer_join()
    e1.record(ext)
    torch.cuda.synchronize()
    g.sync()
    if g.stats()["p_worst"] != 0:
        raise SystemExit("a pressure solve failed in the end-to-end region")
    ems = e0.elapsed_time(e1)
    ems = max_over_ranks([ems], dist, "cuda")[0]
    e2e = replica_throughput(ws, cells * ke, ems)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        g.close()
        return None

    peaks = _peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    esz = 4 if precision == 1 and not (parts & 4) else 8  # FP32 sweeps unless momentum is kept in FP64
    jac_b, sor_b, jac_n, sor_n = _algorithmic_bytes(nx, ny, nz, params.mom_u, esz)
    # dominant kernel of the step: the odd-iteration red-black half-sweep
    # (k_sor_odd_c4), its launches timed with CUDA events on the library's
    # stream in the phase pass
    sor_ms, sor_l = phases["sor_odd"]
    # (one block per 64-level segment for columns of 3 or more segments)
    dominant = "k_sor_odd_seg" if (not args.odd_columns and (nz - 1) // 64 + 1 >= 3) else "k_sor_odd_c4"
    per_launch_b = sor_b / sor_n
    avg_ms = sor_ms / max(sor_l, 1)
    achieved = per_launch_b / (avg_ms / 1e3) / 1e9
    wl = f"{nx}x{ny}x{nz}-{'fp64' if precision == 0 else 'mixed'}"
    traffic_cap = _profile_figure("traffic", dominant, wl)
    # FP64 pipe utilisation from a --set full capture (a smaller case of the
    # same kernel: a full set is not captured at this size)
    fp64_cap = _profile_figure("fp64pipe", dominant, None) if precision == 0 else None
    traffic = traffic_cap["value"] if traffic_cap and traffic_cap["current"] else None
    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.config, args.cpu_seconds, (nx, ny, nz))
    out = {
        "metric": "cell-steps/s",
        "value": value,
        "unit": "cell-steps/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if precision == 0 else "f32 stencils/sweeps/smoothing + f64 state/dots/coarse solve",
        "data": "synthetic: seeded two-layer channel (4-mode interface, +-1e-3 velocity noise), no dataset",
        "config": {"workload": w.name if not args.grid else f"{w.name}, resized to {nx}x{ny}x{nz}",
                   "grid": [nx, ny, nz], "cells": cells, "m": w.m, "re": w.re,
                   "mom_uvw": params.mom_u, "levelset": params.levelset, "p_rtol": params.p_rtol,
                   "precision": "fp64" if precision == 0 else "fp32-mixed",
                   "fp64_parts": parts,
                   "mg_fp32": params.mg_fp32,
                   "odd_half_sweep": ("one block per 64-level segment, chained up the column"
                                      if dominant == "k_sor_odd_seg" else "one block per column"),
                   "advect_phi": ("read through the caches" if (args.no_tma or precision == 0)
                                  else "tiles staged by TMA (cp.async.bulk.tensor)"),
                   "idm": args.idm,
                   "dim_pe": args.dim_pe if args.idm == "dim" else None,
                   "sweep_tiles": tiles,
                   "parallelism": f"{ws} independent replica(s), no sharding",
                   "l2": f"working set ~{cells * 500 / 1e9:.0f} GB per step >> 129 MB L2 (no flush needed)",
                   "launch": "two CUDA-graph launches per step, front and back (device-side WHILE node for the "
                             "pressure CG)",
                   "grid_geometry": "cubic cells dx=dy=dz=1/nz (the reference's initialisation grid)",
                   "headline_metric": HEADLINE_METRIC},
        "e2e": {"value": e2e, "unit": "cell-steps/s", "h2d_bytes_per_step": bi, "d2h_bytes_per_step": bi,
                "steps": ke, "path": f"tpls_set_fields ({len(state_fields)} fields) -> tpls_step_async(1) -> "
                                     f"tpls_get_fields ({len(state_fields)} fields) per step, pinned host "
                                     f"arrays, one wait after the last step"},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": dominant, "bytes_per_launch": per_launch_b,
                     "avg_launch_ms": avg_ms,
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "traffic_capture": traffic_cap,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback",
                     "note": "achieved = algorithmic bytes (28 B per component point per half-sweep in FP64, "
                             "12 B in the FP32 sweeps) / CUDA-event time measured in this run; traffic = ncu "
                             "DRAM bytes per launch from the committed capture named in traffic_capture, "
                             "given only when that capture is of this run's sources (null otherwise)"},
        "fp64_pipe_capture": fp64_cap,
        "phases_ms_per_step": {k: v[0] / nph for k, v in phases.items()},
        "phases_note": f"eager pass of {nph} steps with events between phases",
        "pressure": {"its_last": stats["p_its"], "reason_last": stats["p_reason"]},
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    if dist:
        dist.destroy_process_group()
    g.close()
    return out


def run_accuracy(args) -> dict:
    """Error of the FP32-mixed form against the FP64 form on one workload.

    Both forms start from the same seeded state and step side by side (FP64
    pressure solves at rtol 1e-10 in both, so the solver tolerance does not
    mask the arithmetic); at each checkpoint the relative max-norm difference
    of phi, u, v, w and p over the interior rows, and each form's liquid-volume
    drift from the initial volume, are recorded.  Not a throughput line."""
    import numpy as np
    import torch
    from tpls_gb300.api import TplsGpu
    from tpls_gb300.channel import WORKLOADS, make_case

    torch.cuda.set_device(0)
    w = WORKLOADS[args.config]
    nx, ny, nz = args.grid if args.grid else (w.nx, w.ny, w.nz)

    def open_form(prec, parts, rtol=1e-10):
        p, u, st = make_case(args.config, nx=nx, ny=ny, nz=nz, precision=prec, fp64_parts=parts,
                             p_rtol=rtol, p_maxits=400)
        g = TplsGpu(nx, ny, nz, p, u)
        g.set_state(st)
        return g

    def rel(a, b):
        a, b = a[:, 1:ny + 1, :], b[:, 1:ny + 1, :]
        den = float(np.max(np.abs(b))) or 1.0
        return float(np.max(np.abs(a - b))) / den

    ref = open_form(0, 0)
    if args.compare_rtol > 0.0:  # the FP64 form at another pressure tolerance (the reference's is 1e-5)
        mix = open_form(0, 0, args.compare_rtol)
    elif args.perturb > 0.0:  # the FP64 form against itself with u perturbed: the workload's own sensitivity
        mix = open_form(0, 0)
        u = mix.get_field(args.perturb_field)
        rng = np.random.default_rng(7)
        mix.set_field(args.perturb_field, np.asfortranarray(u * (1.0 + args.perturb * rng.standard_normal(u.shape))))
    else:
        mix = open_form(1, args.fp64_parts)
    v0 = ref.stats()["liquid_volume"]
    if args.accuracy_every > 0:
        marks = list(range(args.accuracy_every, args.accuracy + 1, args.accuracy_every))
    else:
        marks = sorted({m for m in (20, 50, 100, 200, 500, 1000) if m < args.accuracy} | {args.accuracy})
    rows, done = [], 0
    for m in marks:
        for g in (ref, mix):
            if g.step(m - done) != 0:
                raise SystemExit(f"tpls_step failed before step {m}")
        done = m
        row = {"step": m}
        for f in ("PHI2", "U2", "V2", "W2", "PRES"):
            a, b = mix.get_field(f), ref.get_field(f)
            row[f.rstrip("2").lower()] = rel(a, b)
            if f in ("PHI2", "U2"):  # where the largest difference sits (i, j, k of the field's array)
                d = np.abs(a[:, 1:ny + 1, :] - b[:, 1:ny + 1, :])
                i, j, k = np.unravel_index(int(np.argmax(d)), d.shape)
                row[f.rstrip("2").lower() + "_at"] = [int(i), int(j) + 1, int(k)]
            if f == "PHI2":  # near the interface (|phi| < 3 dz), where curvature amplifies it: in units of dz
                band = np.abs(b[:, 1:ny + 1, :]) < 3.0 / nz
                row["phi_band_dz"] = float(np.max(d[band])) * nz if band.any() else 0.0
        row["volume_drift_fp64"] = (ref.stats()["liquid_volume"] - v0) / v0
        row["volume_drift_mixed"] = (mix.stats()["liquid_volume"] - v0) / v0
        rows.append(row)
    ref.close()
    mix.close()
    if args.compare_rtol > 0.0:
        what = f"fp64 at pressure rtol {args.compare_rtol:g} vs fp64 at rtol 1e-10"
    elif args.perturb > 0.0:
        what = f"fp64 with {args.perturb_field} perturbed by {args.perturb:g} (relative, seeded normal) vs fp64"
    else:
        what = "fp32-mixed relative max-norm error vs fp64"
    return {"metric": what, "workload": w.name,
            "grid": [nx, ny, nz], "fp64_parts": args.fp64_parts, "p_rtol": 1e-10,
            "region": "interior rows j=1..ny, every i and z plane", "checkpoints": rows}


def run_batch(args, ws, rank, local) -> dict | None:
    """The batched workload: 48 seeded instances of uneven grids, FP32-mixed,
    all advanced by one CUDA-graph launch per batch step; compared with the
    same instances run one by one."""
    import torch
    from tpls_gb300.api import STATE_FIELDS
    from tpls_gb300.batch import Batch, draw_instances, open_instance, run_one_by_one

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from tpls_gb300.api import TPLS_FLAG_ODD_COLUMNS
    precision = _precision(args)
    insts = draw_instances(args.instances)
    cells = sum(i.cells for i in insts)
    fl = TPLS_FLAG_ODD_COLUMNS if args.odd_columns else 0
    # e2e: states uploaded from host, the batch run, states downloaded
    hosts = []
    members = []
    for inst in insts:
        g = open_instance(inst, precision, tune=True, flags=fl)  # sweep tile shapes per grid (cached per shape)
        hosts.append(g.get_state())
        members.append(g)
    # the other launch form of the same members, timed first for comparison
    # (graph branches per member vs multi-instance sweep launches)
    def timed(multi: bool, mem, st0, steps):
        for m, h in zip(mem, st0):
            m.set_state(h)
        bb = Batch(mem, multi_sweeps=multi)
        if bb.step(args.warmup) != 0:
            raise SystemExit("batch warm-up failed")
        torch.cuda.synchronize()
        ta = time.perf_counter()
        if bb.step(steps) != 0:
            raise SystemExit("batch step failed")
        torch.cuda.synchronize()
        dt = time.perf_counter() - ta
        bb.close()
        return dt
    other = timed(not args.multi_sweeps, members, hosts, args.steps)
    small = None
    if args.small_instances > 0:  # many small grids, where per-launch overhead dominates
        sm_insts = draw_instances(args.small_instances, max_dims=(64, 32, 32))
        sm_mem = [open_instance(i, precision, tune=True, flags=fl) for i in sm_insts]
        sm_st = [g.get_state() for g in sm_mem]
        sm_cells = sum(i.cells for i in sm_insts)
        t_br, t_mu = timed(False, sm_mem, sm_st, args.steps), timed(True, sm_mem, sm_st, args.steps)
        small = {"instances": len(sm_insts), "grid": [64, 32, 32], "steps": args.steps,
                 "branches_cell_steps_per_s": sm_cells * args.steps / t_br,
                 "multi_sweeps_cell_steps_per_s": sm_cells * args.steps / t_mu}
        for g in sm_mem:
            g.close()
    for m, h in zip(members, hosts):
        m.set_state(h)
    b = Batch(members, multi_sweeps=args.multi_sweeps)
    if b.step(args.warmup) != 0:
        raise SystemExit("batch warm-up failed")
    ext = torch.cuda.ExternalStream(members[0].stream_ptr())
    sampler = ClockSampler(local) if rank == 0 else None
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rc = b.step(args.steps)
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    if dist:
        dist.barrier()
    clocks = sampler.stop() if sampler else None
    if rc != 0:
        raise SystemExit(f"batch step returned {rc}: not a valid measurement")
    launches = sum(m.kernel_launches() for m in members)
    # e2e through the API: every batch step uploads every member's whole
    # state from pinned host arrays, runs, and downloads it (batched
    # transfers, enqueued without host waits; one wait after the last step)
    ke = max(1, min(args.steps, args.e2e_steps))
    pins = []
    for h in hosts:
        pd = {}
        for k, a in h.items():
            buf = torch.empty(tuple(reversed(a.shape)), dtype=torch.float64, pin_memory=True).numpy().T
            buf[...] = a
            pd[k] = buf
        pins.append(pd)
    bi = sum(sum(a.nbytes for a in h.values()) for h in pins)
    for m, h in zip(members, pins):  # untimed round trip: transfer streams and staging on first use
        m.get_fields_into(h)
        m.set_fields(h)
    for m in members:
        m.sync()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(ke):
        for m, h in zip(members, pins):
            m.set_fields(h)
        b.step_async(1)
        for m, h in zip(members, pins):
            m.get_fields_into(h)
    for m in members:
        m.xfer_join()
        m.sync()
    torch.cuda.synchronize()
    e2e_sec = time.perf_counter() - t1
    if b.step(0) != 0:
        raise SystemExit("batch e2e run failed")
    b.close()
    for m in members:
        m.close()
    del ext
    solo = None
    if not args.no_one_by_one:
        solo = run_one_by_one(insts, args.steps, precision, warmup=args.warmup)
    sec, e2e_sec = max_over_ranks([sec, e2e_sec], dist, "cuda")
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return None
    value = replica_throughput(ws, cells * args.steps, sec * 1e3)
    out = {
        "metric": "cell-steps/s",
        "value": value,
        "unit": "cell-steps/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": sec * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if precision == 0 else "f32 stencils/sweeps/smoothing + f64 state/dots/coarse solve",
        "data": "synthetic: 48 seeded channel instances, no dataset",
        "config": {"workload": f"D: {len(insts)} batched instances, uneven grids, "
                               f"{'fp64' if precision == 0 else 'fp32-mixed'}",
                   "instances": len(insts), "total_cells": cells,
                   "grids": [[i.nx, i.ny, i.nz] for i in insts],
                   "launch": "one CUDA graph per batch step: every member's step as a branch" +
                             ("; the FP32 momentum sweeps as one multi-instance launch per sweep over all "
                              "members' tiles (atomic ticket)" if args.multi_sweeps else ""),
                   "timing": "host wall clock around synchronised batch steps",
                   "l2": f"working set ~{cells * 300 / 1e9:.0f} GB per step >> 129 MB L2",
                   "headline_metric": HEADLINE_METRIC},
        "jobs_per_s": ws * len(insts) / sec,
        "e2e": {"value": ws * cells * ke / e2e_sec, "unit": "cell-steps/s",
                "h2d_bytes_per_step": bi, "d2h_bytes_per_step": bi, "steps": ke,
                "path": "per batch step: tpls_set_fields (20 fields) per member -> tpls_batch_step_async(1) -> "
                        "tpls_get_fields (20 fields) per member, pinned host arrays, one wait after the last step"},
        "gpu_launches": launches,
        "other_launch_form": {"form": "branches" if args.multi_sweeps else "multi_sweeps",
                              "cell_steps_per_s": ws * cells * args.steps / other},
        "small_grids": small,
        "one_by_one": None if solo is None else {
            "seconds": solo["seconds"], "value": cells * args.steps / solo["seconds"],
            "batched_speedup": solo["seconds"] / sec},
        "roofline": None,
        "cpu_baseline": None,
        "clocks": clocks,
    }
    if dist:
        dist.destroy_process_group()
    return out


def run_serve(args, ws, rank, local) -> dict | None:
    """The served job stream: the first --jobs jobs of the seeded 2000-job
    Poisson stream (arrival rate --rate jobs/s), admitted under a 160 GB
    footprint budget, run once in the FP32-mixed form and once in FP64."""
    import torch
    from tpls_gb300.serve import GpuBackend, Server, draw_jobs, summarize
    torch.cuda.set_device(local)
    if rank != 0:
        return None
    forms = {}
    clocks = None
    njobs = {"fp32_mixed": args.jobs, "fp64": args.jobs_fp64 if args.jobs_fp64 is not None else args.jobs}
    for name, prec in (("fp32_mixed", 1), ("fp64", 0)):
        if njobs[name] <= 0:
            continue
        jobs = draw_jobs(2000, rate=args.rate, precision=prec)[:njobs[name]]
        sampler = ClockSampler(local)
        srv = Server(GpuBackend(), budget_bytes=160e9, max_active=64)
        res = srv.run(jobs, time_scale=args.time_scale)
        c = sampler.stop()
        clocks = clocks or c
        sm = summarize(res)
        sm["peak_admitted_gb"] = srv.peak_bytes / 1e9
        sm["peak_active_jobs"] = srv.peak_active
        sm["clocks"] = c
        forms[name] = sm
    mx = forms["fp32_mixed"]
    return {
        "metric": "jobs/s",
        "value": mx["jobs_per_s"],
        "unit": "jobs/s",
        "n_gpus": ws,
        "steps": sum(j.steps for j in draw_jobs(2000, rate=args.rate)[:args.jobs]),
        "warmup": 0,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32-mixed (fp64 form alongside)",
        "data": "synthetic: seeded Poisson job stream, no dataset",
        "config": {"workload": f"E: first {args.jobs} jobs (FP32-mixed; {njobs['fp64']} in FP64) of the seeded "
                               f"2000-job stream, Poisson arrivals at {args.rate} jobs/s scaled by "
                               f"{args.time_scale}, grids up to 384x192x192, budgets 50-1000 steps, 160 GB "
                               f"admission, snapshots every 50 steps",
                   "timing": "host wall clock from the first arrival to the last completion",
                   "headline_metric": HEADLINE_METRIC},
        "serve": forms,
        "p50_latency_s": mx["p50_latency_s"],
        "p99_latency_s": mx["p99_latency_s"],
        "cell_steps_per_s": mx["cell_steps_per_s"],
        "clocks": clocks,
    }


def run_routine_costs(args) -> dict:
    """What a driver that adopts the per-routine entries pays per timestep:
    each entry of one step of the reference's loop (main_ns_hybrid.F90:
    583-913) called on this workload's arrays, once with plain (pageable)
    host arrays, copied in and out around every call, and once with the
    same arrays registered (tpls_register_host: device-resident behind the
    same addresses).  Host wall clock per call (every entry waits for its
    kernels), times the calls a step makes; the device-resident tpls_step
    beside it.  The driver's own host loops between the calls (boundary
    rows, the AB3 sums) are not included."""
    import torch
    from tpls_gb300.api import TplsGpu
    from tpls_gb300.channel import WORKLOADS, make_case
    torch.cuda.set_device(0)
    w = WORKLOADS[args.config]
    nx, ny, nz = args.grid if args.grid else (w.nx, w.ny, w.nz)
    p, uin, st = make_case(args.config, nx=nx, ny=ny, nz=nz, p_rtol=args.p_rtol)
    g = TplsGpu(nx, ny, nz, p, uin)
    g.set_state(st)
    g.step(1)  # every field of the state holds a step's values
    f = g.get_field
    a = {k.lower(): f(k) for k in ("PHI2", "U2", "V2", "W2", "U3", "V3", "W3", "PRES", "PRES_OLD", "CONV0_PHI",
                                   "CONV1_PHI", "CONV2_PHI")}
    a.update(phi3=g.zeros("p"), fx=g.zeros("p"), fy=g.zeros("p"), fz=g.zeros("p"), rhs_p=g.zeros("p"),
             va=np.zeros(g.shape("va"), order="F"))
    for k in ("u", "v"):
        a.update({f"{k}3_old": g.zeros("uv"), f"rhs_{k}": g.zeros("uv"), f"conv_{k}": g.zeros("uv"),
                  f"diff_{k}": g.zeros("uv")})
    a.update(w3_old=g.zeros("w"), rhs_w=g.zeros("w"), conv_w=g.zeros("w"), diff_w=g.zeros("w"))
    dx, dy, dz, dt = p.dx, p.dy, p.dz, p.dt
    x3 = {0: ("u3", "u3_old", "rhs_u"), 1: ("v3", "v3_old", "rhs_v"), 2: ("w3", "w3_old", "rhs_w")}
    jac = {0: g.do_jacobi_u, 1: g.do_jacobi_v, 2: g.do_jacobi_w}
    sor = {0: g.do_sor_u, 1: g.do_sor_v, 2: g.do_sor_w}
    mom = p.mom_u // 2
    # (name, calls per step, call)
    entries = [
        ("do_advect_phi", 1, lambda: g.do_advect_phi(a["phi2"], a["u2"], a["v2"], a["w2"], dx, dy, dz,
                                                     conv2_phi=a["conv2_phi"])),
        ("do_tpls", 1, lambda: g.do_tpls(a["phi2"], a["conv0_phi"], a["conv1_phi"], a["conv2_phi"], p.levelset,
                                         p.height, dx, dz, dt, phi3=a["phi3"])),
        ("get_csf", 1, lambda: g.get_csf(a["phi3"], dx, dy, dz, p.scap, p.smooth_width, a["fx"], a["fy"],
                                         a["fz"])),
        ("get_viscosity", 1, lambda: g.get_viscosity(a["phi2"], p.smooth_width, p.re, p.mu_minus, p.mu_plus,
                                                     viscosity_aug=a["va"])),
        ("get_conv_all", 1, lambda: g.get_conv_all(a["va"], a["u2"], a["v2"], a["w2"], dx, dy, dz,
                                                   out=(a["conv_u"], a["conv_v"], a["conv_w"]))),
        ("get_diffusion_all", 1, lambda: g.get_diffusion_all(a["va"], a["u2"], a["v2"], a["w2"], dx, dy, dz,
                                                             out=(a["diff_u"], a["diff_v"], a["diff_w"]))),
    ]
    for c, nm in ((0, "u"), (1, "v"), (2, "w")):
        x, xo, r = x3[c]
        entries.append((f"do_jacobi_{nm}", mom, lambda c=c, x=x, xo=xo, r=r: jac[c](a[x], a[xo], a[r], a["va"],
                                                                                   dx, dy, dz, dt)))
        entries.append((f"do_sor_{nm}", 2 * mom, lambda c=c, x=x, r=r: sor[c](a[x], a[r], a["va"], dx, dy, dz,
                                                                             dt, 0, 1)))
        entries.append((f"get_difference ({nm})", 1, lambda x=x, xo=xo: g.get_difference(a[x], a[xo])))
    entries += [
        ("exchange2d", 3 * 3 * mom + 11, lambda: g.exchange2d(a["u3"])),
        ("get_source_pres", 1, lambda: g.get_source_pres(a["u3"], a["v3"], a["w3"], dx, dy, dz, dt,
                                                         rhs=a["rhs_p"])),
        ("pressure_solve", 1, lambda: g.pressure_solve(a["pres_old"], a["rhs_p"], a["u3"], uin, dx, dy, dz, dt,
                                                       rtol=p.p_rtol, maxits=p.p_maxits, pres=a["pres"])),
        ("get_uvw_pres", 1, lambda: g.get_uvw_pres(a["u2"], a["v2"], a["w2"], a["pres"], dx, dy, dz, dt, uin)),
    ]
    reps = max(1, args.routine_reps)
    table = {}
    for form in ("host", "registered"):
        if form == "registered":
            for x in a.values():
                g.register_host(x)
        for name, n, fn in entries:
            fn()  # warm-up (scratch allocation on the first call)
            t0 = time.perf_counter()
            for _ in range(reps):
                fn()
            table.setdefault(name, {"calls_per_step": n})[f"{form}_ms"] = (time.perf_counter() - t0) / reps * 1e3
        if form == "registered":
            g.download_host()
    tot = {f: sum(v["calls_per_step"] * v[f"{f}_ms"] for v in table.values()) for f in ("host", "registered")}
    g.set_state(st)
    g.step(3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g.step(5)
    torch.cuda.synchronize()
    step_ms = (time.perf_counter() - t0) / 5 * 1e3
    g.close()
    return {"routine_costs": True, "config": {"workload": f"{args.config}: {nx}x{ny}x{nz} FP64 channel",
                                              "calls": "one timestep of main_ns_hybrid.F90:583-913 "
                                                       f"(mom_uvw {p.mom_u}, levelset {p.levelset})",
                                              "host_arrays": "pageable numpy, Fortran order"},
            "per_entry": {k: {x: (round(y, 4) if isinstance(y, float) else y) for x, y in v.items()}
                          for k, v in table.items()},
            "ms_per_step": {"per_routine_host_arrays": tot["host"], "per_routine_registered": tot["registered"],
                            "tpls_step_device_resident": step_ms}}


def _precision(args) -> int:
    if args.precision is not None:
        return 0 if args.precision == "fp64" else 1
    return 1 if args.config in ("C", "D") else 0


def cpu_baseline(config: str, seconds: float, grid=None) -> dict:
    """The oracle (C restatement of the reference routines, OpenMP over all
    host cores) on the same workload, as many whole timesteps as fit in
    about `seconds` (at least one)."""
    from oracle.oracle import Oracle, set_threads
    from tpls_gb300.channel import WORKLOADS, make_case
    cores = os.cpu_count() or 1
    set_threads(cores)
    w = WORKLOADS[config]
    nx, ny, nz = grid if grid else (w.nx, w.ny, w.nz)
    params, uin, st = make_case(config, nx=nx, ny=ny, nz=nz)
    o = Oracle(nx, ny, nz, params, uin)
    o.set_state(st)
    n = 0
    t0 = time.perf_counter()
    while True:
        o.step(1)
        n += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    o.close()
    return {"value": nx * ny * nz * n / dt, "unit": "cell-steps/s", "cores": cores, "kind": "port",
            "sample": f"{n} full timestep(s) of the {nx}x{ny}x{nz} channel of {w.name.split(':')[0]} "
                      f"from the seeded initial state"}


def run_reference(args, ws, rank) -> dict | None:
    if rank != 0:
        return None
    from oracle.oracle import Oracle, base_profile, set_threads
    from tpls_gb300.channel import WORKLOADS, make_case
    cores = os.cpu_count() or 1
    set_threads(cores)
    w = WORKLOADS[args.config if args.config in WORKLOADS else "B"]
    # the CPU arm builds its initial state with the oracle's base profile, so
    # it never maps the CUDA library
    params, uin, st = make_case(w, p_rtol=args.p_rtol, profile=base_profile)
    o = Oracle(w.nx, w.ny, w.nz, params, uin)
    o.set_state(st)
    o.step(min(args.warmup, 1))
    # bounded sample: up to --steps steps or --ref-seconds of CPU time
    n = 0
    t0 = time.perf_counter()
    while n < args.steps:
        o.step(1)
        n += 1
        if time.perf_counter() - t0 > args.ref_seconds:
            break
    dt = time.perf_counter() - t0
    o.close()
    v = w.nx * w.ny * w.nz * n / dt
    return {"impl": "reference", "metric": "cell-steps/s", "value": v, "unit": "cell-steps/s", "n_gpus": ws,
            "steps": n, "warmup": min(args.warmup, 1), "ms_per_step": dt * 1e3 / n,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded two-layer channel (4-mode interface, +-1e-3 velocity noise), no dataset",
            "config": {"workload": w.name, "grid": [w.nx, w.ny, w.nz], "mom_uvw": params.mom_u,
                       "levelset": params.levelset, "precision": "fp64",
                       "implementation": "C restatement of the reference's Fortran routines (oracle/), OpenMP; "
                                         "the Fortran/MPI/PETSc reference cannot be built here"},
            "cpu_baseline": {"value": v, "unit": "cell-steps/s", "cores": cores, "kind": "port",
                             "sample": f"{n} full timesteps (of {args.steps} requested, bounded to "
                                       f"{args.ref_seconds:.0f} s) after {min(args.warmup, 1)} warm-up"},
            "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--config", default="B")
    ap.add_argument("--p-rtol", type=float, default=1e-5)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default=None,
                    help="default: fp64 for A/B/M, mixed for C/D")
    ap.add_argument("--phase-steps", type=int, default=20)
    ap.add_argument("--fp64-parts", type=int, default=2,
                    help="FP32-mixed form: TPLS_PART_* bits kept in FP64 (default 2: the redistancing "
                         "iterations, the setting that holds phi/u within 1e-7 of the FP64 form over 500 "
                         "steps)")
    ap.add_argument("--ref-seconds", type=float, default=120.0)
    ap.add_argument("--instances", type=int, default=48)
    ap.add_argument("--multi-sweeps", action="store_true",
                    help="batched workload: the FP32 momentum sweeps as multi-instance launches")
    ap.add_argument("--small-instances", type=int, default=0,
                    help="batched workload: also time this many 64x32x32 instances in both launch forms")
    ap.add_argument("--no-one-by-one", action="store_true")
    ap.add_argument("--grid", type=int, nargs=3, default=None, metavar=("NX", "NY", "NZ"),
                    help="resize the workload (small cases for profiling captures)")
    ap.add_argument("--jobs", type=int, default=16, help="served stream: jobs in the FP32-mixed run")
    ap.add_argument("--jobs-fp64", type=int, default=None, help="served stream: jobs in the FP64 run (default --jobs)")
    ap.add_argument("--rate", type=float, default=1.0)
    ap.add_argument("--time-scale", type=float, default=1.0,
                    help="served stream: arrival times multiplied by this factor")
    ap.add_argument("--autotune", action="store_true", help="run the sweep-tile autotuner before timing")
    ap.add_argument("--idm", choices=["lsm", "dim"], default="lsm",
                    help="interface method: level set (default) or diffuse interface (FP64 form)")
    ap.add_argument("--dim-pe", type=float, default=1000.0, help="diffuse interface: Peclet number Pe")
    ap.add_argument("--routine-costs", action="store_true",
                    help="per-routine entries' cost per timestep, host arrays vs registered arrays (not a "
                         "bench line)")
    ap.add_argument("--routine-reps", type=int, default=3)
    ap.add_argument("--odd-columns", action="store_true",
                    help="odd half-sweep: one block walks each whole column instead of one block per 64-level "
                         "segment chained up the column (tpls_params.flags = TPLS_FLAG_ODD_COLUMNS; bit-identical)")
    ap.add_argument("--no-tma", action="store_true",
                    help="FP32-mixed form: advection reads phi through the caches instead of TMA-staged tiles "
                         "(tpls_params.flags = TPLS_FLAG_NO_TMA; bit-identical)")
    ap.add_argument("--mg-fp32", action="store_true",
                    help="FP64 form: FP32 multigrid levels in the CG preconditioner (tpls_params.mg_fp32 = 1; "
                         "CG stays FP64 and meets p_rtol on its FP64 residual). Default: FP64 throughout")
    ap.add_argument("--accuracy", type=int, default=0, metavar="STEPS",
                    help="instead of timing: step the FP64 and FP32-mixed forms side by side for STEPS "
                         "steps and print their differences (one JSON line)")
    ap.add_argument("--accuracy-every", type=int, default=0, metavar="N",
                    help="with --accuracy: a checkpoint every N steps")
    ap.add_argument("--perturb-field", default="U2", choices=["U2", "PHI2"])
    ap.add_argument("--compare-rtol", type=float, default=0.0,
                    help="with --accuracy: compare the FP64 form at this pressure rtol with the FP64 form at 1e-10")
    ap.add_argument("--perturb", type=float, default=0.0,
                    help="with --accuracy: compare the FP64 form with itself started from u perturbed by this "
                         "relative amount (how far the workload amplifies a rounding-sized difference)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3  # timing rule: at least 3 warm-up steps
    ws, rank, local = _dist()
    if args.routine_costs:
        out = run_routine_costs(args) if rank == 0 else None
    elif args.accuracy > 0:
        out = run_accuracy(args) if rank == 0 else None
    elif args.impl == "reference":
        out = run_reference(args, ws, rank)
    elif args.config == "D":
        out = run_batch(args, ws, rank, local)
    elif args.config == "E":
        out = run_serve(args, ws, rank, local)
    else:
        out = run_gpu(args, ws, rank, local)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
