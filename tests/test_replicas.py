"""The multi-GPU path of bench.py is replicas: every rank runs the whole
workload and only the timed interval is reduced (MAX over ranks). Checked
here with two gloo ranks on the CPU, and the reference arm's rank rule
(rank 0 alone prints) without any process group."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out.put((rank, bench.replica_throughput(1.0 + rank, 100, "cpu")))
    finally:
        dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    results = dict(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # the job took the slower rank's 2 s; both ranks processed 100 units
    assert results[0] == results[1] == (2.0, 100.0)


def test_single_process_throughput():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.replica_throughput(0.5, 100, "cpu") == (0.5, 200.0)


@pytest.mark.parametrize("rank", ["1"])
def test_reference_arm_other_ranks_print_nothing(rank):
    env = dict(os.environ, RANK=rank, WORLD_SIZE="2", LOCAL_RANK=rank)
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "3", "--quick"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
