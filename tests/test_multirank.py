"""The N > 1 paths of bench.py on CPU: point sharding across ranks, the
max-over-ranks reduction over a world-size-2 gloo group, and the reference
arm under torchrun (rank 0 alone reports)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_point_shards_are_disjoint_and_cover():
    """Rank r evaluates rows [r P, (r + 1) P) of one seeded stream, so the
    shards of a weak-scaling run are the single-rank workload cut in pieces."""
    P = 1000
    whole = bench.config3_points(2 * P, 1)
    parts = [bench.config3_points(P, 1, offset=r * P) for r in range(2)]
    assert np.array_equal(np.concatenate(parts), whole)


def _gloo_worker(rank, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    dist.init_process_group("gloo", rank=rank, world_size=2)
    bench.barrier(2)
    m = bench.max_over_ranks(1.5 + rank, 2)
    out.put((rank, m))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_gloo_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2.5), (1, 2.5)]


def test_reference_arm_under_torchrun():
    pytest.importorskip("torch")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--cpu-points", "2"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["cpu_baseline"]["kind"] == "port" and d["value"] > 0


def test_config5_lpt_shards_partition_the_batch():
    """Config 5 on N GPUs splits the 512 MPS by longest-processing-time-first
    on their apply+truncate flop estimates: every MPS exactly once, loads
    within 4/3 of the ideal split."""
    sys.path.insert(0, str(ROOT / "itensornumericalanalysis.jl_gb300"))
    from itensornumericalanalysis.workloads import lpt_shards, mps_apply_truncate_cost, uneven_mps_batch

    batch = uneven_mps_batch(n=512, seed=3)
    costs = [mps_apply_truncate_cost(s, ts) for s, ts in batch]
    assert min(costs) > 0
    for n in (1, 2, 4, 8):
        shards = lpt_shards(costs, n)
        flat = sorted(i for sh in shards for i in sh)
        assert flat == list(range(len(batch)))
        loads = [sum(costs[i] for i in sh) for sh in shards]
        assert max(loads) <= 4.0 / 3.0 * max(sum(costs) / n, max(costs)) + 1e-6
    assert lpt_shards(costs, 1) == [list(range(len(batch)))]
