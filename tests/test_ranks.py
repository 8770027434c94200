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


def test_reference_arm_line_on_cpu():
    """`bench.py --impl reference` runs on the host cores only and prints one
    JSON line with the arm's value, its CPU baseline description and an e2e
    entry without copies (the Faust x dense workload of 5 CSR 1024^2 FP64
    factors, one bounded sample)."""
    import json
    import subprocess
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "csr_random", "--steps", "1", "--warmup", "0"], cwd=ROOT, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "GB/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["config"]["workload"] == "csr_random"
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
