"""The benchmark's multi-rank logic on CPU: two gloo ranks (replicas, no collective on the data path)
read their place from the launcher's environment, take the slowest rank's time as the job's time,
and report the whole job's rate from it."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out: str) -> None:
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    w, r, local = bench.dist_env()
    dist.init_process_group("gloo", rank=r, world_size=w)
    try:
        # each rank's own step time; the job's is the slowest
        slowest = bench.max_over_ranks(10.0 + 5.0 * r, w, "cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()
    with open(f"{out}.{rank}", "w") as f:
        f.write(f"{w} {r} {local} {slowest!r}")


def test_two_ranks_slowest_time_and_job_rate(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world, port, out = 2, _free_port(), str(tmp_path / "rank")
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(world):
        w, rr, local, slowest = open(f"{out}.{r}").read().split()
        assert (int(w), int(rr), int(local)) == (world, r, r)
        assert float(slowest) == 15.0  # rank 1's time, on both ranks

    import bench

    # every rank's units over the slowest rank's time: 2 x 1e9 units in 15 ms
    assert bench.job_rate(1e9, 2, 15.0) == pytest.approx(2e9 / 0.015)
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5


def test_reference_arm_other_ranks_exit_without_work():
    """Under torchrun the reference arm runs on rank 0 alone; another rank exits 0 at once and
    prints nothing."""
    import subprocess

    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2", MASTER_ADDR="127.0.0.1")
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2"],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == ""
