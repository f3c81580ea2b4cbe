"""The multi-rank logic of bench.py (replicas only) on two gloo ranks on the CPU: the step time is the maximum
over ranks on every rank, only rank 0 runs the reference arm, and the other ranks exit without work."""
import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, outdir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, REPO)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
        buf = io.StringIO()

        class A:
            gpus, steps, warmup = world, 1, 0

        if rank != 0:
            with redirect_stdout(buf):
                bench.run_reference(A, rank, world)  # ranks other than 0 return at once
        dist.barrier()
        with open(os.path.join(outdir, f"rank{rank}.json"), "w") as fh:
            json.dump([got, buf.getvalue()], fh)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_and_only_rank0_prints(tmp_path):
    world = 2
    port = _free_port()
    mp.spawn(_rank, args=(world, port, str(tmp_path)), nprocs=world, join=True)  # spawn start method
    res = {}
    for r in range(world):
        with open(tmp_path / f"rank{r}.json") as fh:
            res[r] = json.load(fh)
    assert res[0][0] == res[1][0] == 15.0
    assert res[1][1] == ""


def test_single_rank_is_the_identity():
    sys.path.insert(0, REPO)
    import bench

    assert bench.max_over_ranks(3.5, 1) == 3.5
