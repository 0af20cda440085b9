"""The benchmark's multi-rank path on the CPU (gloo, world size 2).

The step loop does not shard: `bench.py --gpus N` runs N independent replicas,
one per rank, and reports the units of all ranks over the slowest rank's time
(max over ranks).  These tests exercise that reduction and the reference arm's
rank handling without a GPU.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import REPO


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=2)
    ms = [12.5, 20.0][rank]                      # each replica's own timed region
    ms_max = bench._max_over_ranks(ms, dist)
    steps = 100
    value = 2 * steps / (ms_max * 1e-3)          # whole-job rate: all ranks' steps
    q.put((rank, ms_max, value))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_with_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [20.0, 20.0]          # both ranks see the slowest time
    assert out[0][2] == out[1][2] == pytest.approx(2 * 100 / 0.020)


def test_reference_arm_two_ranks_prints_once():
    """Under torchrun with two ranks, rank 0 alone times the CPU reference and
    prints one JSON line; rank 1 exits 0 without work."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "2", "--warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600, env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    # the reference's own solver where its sources are here, else the oracle port
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("reference", "port")
