"""Multi-rank plumbing of bench.py on CPU with the gloo backend, world size 2:
replicas render their own random streams, the job's time is the slowest
rank's, and under torchrun only rank 0 prints the reference arm's line.
No GPU is needed (the GPU arm's data path has no collective)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _ranks(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        worst = bench.max_over_ranks(1.5 + rank, dist, "cpu")
        seeds = [None] * world
        dist.all_gather_object(seeds, bench.replica_seed(rank))
        out.put((rank, worst, seeds))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_replica_seeds_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_ranks, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.5, 2.5]          # both ranks see the slowest time
    seeds = res[0][2]
    assert len(set(seeds)) == 2 and res[1][2] == seeds  # distinct streams per replica


def test_max_over_ranks_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, None, "cpu") == 3.25


def test_reference_arm_under_torchrun(tmp_path):
    """`bench.py --impl reference` launched as the driver launches it for
    N = 2: one JSON line, from rank 0, every rank exiting 0."""
    pytest.importorskip("torch.distributed.run")
    from hastyrenderer_gb300 import scenes
    scenes.cornell_box(str(tmp_path), seed=0, width=128, height=64, spp=4)
    env = dict(os.environ, HASTY_BENCH_DIR=str(tmp_path))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
