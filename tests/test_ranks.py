"""The multi-rank timing of bench.py on CPU ranks (gloo, world size 2): each
rank times its own replica of the work, the reported time is the slowest
rank's, taken after a common barrier.  No GPU is involved."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench._barrier(world)
        q.put((rank, bench._max_over_ranks(times[rank], world)))
        bench._barrier(world)
    finally:
        dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [0.25, 0.75]
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = dict(q.get(timeout=5) for _ in range(2))
    assert got == {0: 0.75, 1: 0.75}


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench._max_over_ranks(1.5, 1) == 1.5
    bench._barrier(1)


def test_faust_x_arms_divide_the_same_bytes():
    """Every Faust x dense line (GPU value, e2e, CPU baseline, reference arm)
    divides the problem's bytes: X read, Y written and the factor arrays,
    charged to a column sample in proportion, so that two lines' ratio is the
    ratio of their times.  BSR operands count as BF16."""
    import types
    sys.path.insert(0, ROOT)
    import numpy as np
    import bench
    W = types.SimpleNamespace(name="csr_butterfly", n=4096, ncols=8192, np_dtype=np.float32,
                              factor_bytes=lambda: [100, 200, 300])
    full = 2 * 4096 * 8192 * 4 + 600
    assert bench._problem_bytes(W) == full
    assert bench._problem_bytes(W, 512) == full * 512 / 8192
    B = types.SimpleNamespace(name="bsr", n=16384, ncols=4096, np_dtype=np.float32, factor_bytes=lambda: [1000])
    assert bench._problem_bytes(B) == 2 * 16384 * 4096 * 2 + 1000
