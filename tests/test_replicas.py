"""Multi-GPU is replicas only: each rank runs its own channel, and the only
communication is the timing reduction (max over ranks) and barriers.  The
reduction and the aggregation are exercised here with world_size-2 gloo
process groups on the CPU; the reference arm's rank handling (rank 0 runs,
the others exit 0 without output) as a subprocess."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, q):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    times = [10.0 + rank, 3.0 - rank]  # rank 1 slower in the first, faster in the second
    got = bench.max_over_ranks(times, dist, "cpu")
    dist.barrier()
    q.put((rank, got, bench.replica_throughput(ws, 1000.0, got[0])))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world_size_2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, thr in out:
        assert got == [11.0, 3.0]
        assert thr == pytest.approx(2 * 1000.0 / 0.011)


def test_single_process_aggregation():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks([1.5, 2.0]) == [1.5, 2.0]
    assert bench.replica_throughput(1, 6291456 * 200, 31240.0) == pytest.approx(6291456 * 200 / 31.24)


def test_reference_arm_non_zero_rank_exits_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1"],
                       capture_output=True, text=True, env=env, timeout=300, cwd=ROOT)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_rank0_prints_the_contract_line():
    """Rank 0 of the reference arm prints one JSON line with the main arm's
    metric, unit and config, the CPU baseline it describes and an e2e figure
    with no host-device bytes (one 256x128x192 step on the host cores)."""
    import json
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    # run bench.py's main in a process that afterwards reports whether the
    # CUDA library was ever mapped: the CPU arm must not load the product
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '1']; "
            "runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPS', int('libtpls_gb300' in maps), int('liboracle' in maps), file=sys.stderr)")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    maps = [ln.split() for ln in r.stderr.splitlines() if ln.startswith("MAPS ")]
    assert maps == [["MAPS", "0", "1"]], r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "cell-steps/s" and d["unit"] == "cell-steps/s"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["grid"] == [256, 128, 192]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
