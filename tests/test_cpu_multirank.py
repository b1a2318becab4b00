"""The N > 1 path of bench.py on CPU: world-size-2 gloo process group.

bench.py runs independent replicas, one per GPU (the path shards into
independent systems; no data-path collective): each rank times its own
steps between barriers, the job time is the max over ranks, and the job
rate counts every rank's interactions.  The reference arm prints from rank 0
only; other ranks exit 0 without work.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    dist.barrier()
    local_seconds = [2.0, 3.5][rank]
    m = bench.max_over_ranks(local_seconds)
    rate = bench.job_rate(100.0, world, m)
    q.put((rank, m, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_job_rate_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29000 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, m, rate in res:
        assert m == 3.5
        assert abs(rate - 2 * 100.0 / 3.5) < 1e-12


def test_reference_arm_other_ranks_exit_without_output():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "512",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_rank0_prints_one_json_line():
    import json
    env = dict(os.environ, OMP_NUM_THREADS="2")
    env.pop("RANK", None)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "1024",
                        "--steps", "2", "--warmup", "1"], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
