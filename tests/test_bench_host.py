"""The benchmark's reference arm on the host: one JSON line with the keys
the benchmark contract names, on a small matrix (no GPU needed)."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_json_line():
    env = dict(os.environ, OPENBLAS_NUM_THREADS="2")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "256",
                          "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=600, env=env,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "matrices/s"
    for key in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "config", "cpu_baseline",
                "e2e"):
        assert key in line, key
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


def _replica_worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        # rank r pretends to have taken 1 + r seconds for 4 steps
        q.put((rank, bench.replica_rate(1.0 + rank, 4, world)))
    finally:
        dist.destroy_process_group()


def test_replica_rate_gloo_two_ranks():
    """bench.py's replica mode (--gpus N under torchrun): every rank runs its
    own matrix; the whole-job rate is N * steps over the slowest rank's
    time, agreed on by a MAX all-reduce (here over gloo, two CPU ranks)."""
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(2))
    for r in range(2):
        elapsed, value = got[r]
        assert elapsed == 2.0 and value == 2 * 4 / 2.0


def test_replica_rate_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_rate(0.5, 5, 1) == (0.5, 10.0)
