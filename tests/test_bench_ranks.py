"""The multi-process path of bench.py on CPU: two gloo ranks (one process per
GPU on a GPU machine; here plain processes). The job's time is the slowest
rank's, the value counts every replica's work, and only rank 0 of the
reference arm prints."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seconds = bench.max_over_ranks(1.5 + rank, dist)
        value = bench.replica_rate(world, 2e9, 10, seconds)
        out.put((rank, seconds, value))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_and_value():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, seconds, value in got:
        assert seconds == 2.5                      # the slowest rank's time
        assert abs(value - 2 * 2.0 * 10 / 2.5) < 1e-9  # both replicas' samples


def test_single_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.25) == 3.25
    assert bench.replica_rate(1, 1e9, 4, 2.0) == 2.0


def test_reference_arm_other_ranks_print_nothing():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
