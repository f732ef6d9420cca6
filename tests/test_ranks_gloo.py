"""The multi-rank side of bench.py on CPU: two gloo ranks (world_size 2,
127.0.0.1) run the same cross-rank reduction the GPU bench runs over NCCL.
The workload is replicas only -- each rank transforms its own polynomial --
so the one collective is the max over ranks of the timings."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r is slower in the first timing, faster in the second
        times = [10.0 + 5.0 * rank, 40.0 - 10.0 * rank, 7.5]
        got = bench.reduce_max_over_ranks(times, dist, "cpu")
        rate = bench.whole_job_rate(1 << 24, 100, world, got[0])
        dist.barrier()
    finally:
        dist.destroy_process_group()
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"max": got, "rate": rate}, f)


def test_max_over_ranks_gloo(tmp_path):
    world, port = 2, _free_port()
    ctx = torch.multiprocessing.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    for p in procs:
        if p.is_alive():
            p.kill()
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(world)]
    want = [15.0, 40.0, 7.5]  # element-wise max over the two ranks
    for r in res:
        assert r["max"] == want
        # two replicas of 2^24 elements x 100 steps in the slowest rank's 15 ms
        assert r["rate"] == pytest.approx((1 << 24) * 100 * 2 / 15e-3 / 1e6)


def test_single_process_reduction_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.reduce_max_over_ranks([3.0, 1.5], None, "cpu") == [3.0, 1.5]
    assert bench.whole_job_rate(1000, 10, 1, 2.0) == pytest.approx(5.0)


def test_reference_arm_other_ranks_exit_quietly():
    """Under torchrun only rank 0 times the reference's CPU path and prints;
    the other ranks exit 0 without work or output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, env=env,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
