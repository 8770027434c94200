"""Benchmark of the faust_gb300 hot paths on one GB300 (or N ranks, weak
scaling: every rank runs its own copy of the workload, no collective on the
data path).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload palm|csr_butterfly|csr_random|csr_random_f32|bsr|
                              batched|warmstart|product]

One JSON line is printed by rank 0.  Workloads (all inputs seeded, synthetic):
  palm           palm4msa2 FP64, target = Sylvester Hadamard 1024 / 32,
                 10 factors 1024^2 with prox_sp k=2048, identity init,
                 200 iterations, power-iteration tolerance 1e-8 (default)
  csr_butterfly  12 CSR factors 4096^2 on butterfly supports (2 nnz/row),
                 FP32, times X 4096 x 8192
  csr_random     5 CSR factors 1024^2 with 10 random nnz/row, FP64, times
                 X 1024 x 512
  csr_random_f32 12 CSR factors 4096^2 with 2 random nnz/row, FP32, times
                 X 4096 x 8192 (the butterfly chain's shape without its
                 structure: the generic kernels where HBM is the bound)
  bsr            4 BSR factors 16384^2, 64x64 BF16 blocks, 8 blocks per block
                 row, times X 16384 x 4096 BF16 (FP32 accumulation)
  product        dense product (get_product, DEFAULT_L2R) of the 12 CSR
                 butterfly factors 4096^2, FP32 (the csr_butterfly Faust)
--impl reference times the CPU restatement of the reference algorithm
(oracle/, all host threads) on a bounded sample of the same workload; the
reference itself cannot be compiled here (it needs Eigen 3.4).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PALM4MSA time-to-rel-err (learned vs plain init, GB300); Faust·X GB/s vs HBM"


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- workloads
class FaustX:
    """Faust x dense: one step = F @ X over the whole X."""

    def __init__(self, name, rng):
        import torch
        from faust_gb300 import synth
        self.name = name
        self.torch = torch
        if name == "csr_butterfly":
            self.facs = synth.butterfly_faust_factors(12, rng, np.float32)
            self.n, self.ncols, self.np_dtype, self.tdtype = 4096, 8192, np.float32, torch.float32
            self.desc = "12 CSR butterfly factors 4096^2 (2 nnz/row) FP32 x X 4096x8192"
            self.dtype = "f32"
        elif name == "csr_random_f32":
            self.facs = [synth.random_csr(4096, 4096, 2, rng, np.float32) for _ in range(12)]
            self.n, self.ncols, self.np_dtype, self.tdtype = 4096, 8192, np.float32, torch.float32
            self.desc = "12 CSR 4096^2 (2 random nnz/row) FP32 x X 4096x8192"
            self.dtype = "f32"
        elif name == "csr_random":
            self.facs = [synth.random_csr(1024, 1024, 10, rng) for _ in range(5)]
            self.n, self.ncols, self.np_dtype, self.tdtype = 1024, 512, np.float64, torch.float64
            self.desc = "5 CSR 1024^2 (10 random nnz/row) FP64 x X 1024x512"
            self.dtype = "f64"
        elif name == "bsr":
            import faust_gb300 as fg
            self.n, self.ncols, self.np_dtype, self.tdtype = 16384, 4096, None, torch.bfloat16
            self.bsr, self.bsr_f32 = [], []
            sigma = 1.0 / np.sqrt(8 * 64)
            for _ in range(4):
                bp, bc, blocks = synth.random_bsr(16384, 64, 8, rng, sigma)
                bits = synth.bf16_bits(blocks)
                self.bsr.append(fg.BSRFactor(16384, 16384, bp, bc, bits))
                self.bsr_f32.append((bp, bc, synth.bf16_to_f32(bits).reshape(blocks.shape)))
            self.desc = "4 BSR 16384^2, 64x64 BF16 blocks, 8 blocks/block-row, x X 16384x4096 BF16"
            self.dtype = "bf16"
        else:
            raise ValueError(name)

    def factor_bytes(self):
        if self.name == "bsr":
            return [f.nnz_blocks * 64 * 64 * 2 + f.nnz_blocks * 4 + f.browptr.size * 4 for f in self.bsr]
        es = np.dtype(self.np_dtype).itemsize
        return [f.nnz * (es + 4) + (f.shape[0] + 1) * 4 for f in self.facs]

    def setup(self, ctx):
        import faust_gb300 as fg
        torch = self.torch
        self.F = fg.Faust(self.bsr if self.name == "bsr" else self.facs, ctx=ctx)
        g = torch.Generator(device="cuda").manual_seed(1234)
        self.X = torch.randn((self.ncols, self.n), generator=g, device="cuda", dtype=torch.float32).to(self.tdtype).t()
        self.Y = torch.empty((self.ncols, self.n), device="cuda", dtype=self.tdtype).t()
        self.es = self.X.element_size()
        self.xy_bytes = 2 * self.n * self.ncols * self.es
        # algorithmic bytes per step: every factor reads X-sized input and
        # writes a Y-sized output plus its own arrays (one launch per factor)
        self.step_bytes = sum(b + self.xy_bytes for b in self.factor_bytes())
        # the fused chain kernel (one launch) reads X once, writes Y once and
        # reads each factor
        self.fused_bytes = self.xy_bytes + sum(self.factor_bytes())
        self.flops = (sum(2 * f.nnz * self.ncols for f in self.facs) if self.name != "bsr" else
                      sum(2 * f.nnz_blocks * 64 * 64 * self.ncols for f in self.bsr))

    def step(self, mode=0):
        self.F.matmul_device(self.X, self.Y, mode=mode)

    def kernel_bytes(self, fused):
        return self.fused_bytes if fused else self.step_bytes / len(self.factor_bytes())

    def host_step(self, Xh, Yh):
        from faust_gb300 import _ffi
        _ffi.check(_ffi.lib().fgb_faust_mul_host(self.F.handle, Xh.data_ptr(), self.ncols, Yh.data_ptr()),
                   self.F.ctx.handle)


def run_faust_x(args, rank, world):
    import torch
    import faust_gb300 as fg
    from faust_gb300 import _ffi
    torch.cuda.set_device(rank % max(1, torch.cuda.device_count()))
    rng = np.random.default_rng(2024)
    W = FaustX(args.workload, rng)
    stream = torch.cuda.current_stream()
    ctx = fg.Context(torch.cuda.current_device(), stream=stream.cuda_stream)
    W.setup(ctx)
    fused = False
    if W.name != "bsr":
        # the path automatic mode takes: the fused chain when the
        # intermediates would not stay in L2 (a quarter of it), else one launch
        # per factor
        l2 = torch.cuda.get_device_properties(torch.cuda.current_device()).L2_cache_size
        fused = len(W.facs) > 1 and W.n * W.ncols * np.dtype(W.np_dtype).itemsize > l2 // 4
    # butterfly supports on every factor: automatic mode runs the butterfly
    # chain kernel (several factors per shared-memory pass) instead
    bfly = W.name == "csr_butterfly"
    chain_kernel = "k_bfly_radix" if bfly else "k_csr_chain_fused"
    fused = fused or bfly
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        W.step()
    torch.cuda.synchronize()
    _barrier(world)
    times = []
    launches0 = ctx.kernel_launches()
    with ClockSampler(torch.cuda.current_device()) as clk:
        for _ in range(args.steps):
            flush.zero_()  # L2 flush between timed iterations
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            W.step()
            e.record(stream)
            times.append((s, e))
        torch.cuda.synchronize()
    launches = ctx.kernel_launches() - launches0
    ms = [a.elapsed_time(b) for a, b in times]
    step_ms = float(np.mean(ms))
    step_ms = _max_over_ranks(step_ms, world)
    # end to end through the host-memory C-ABI entry point (pinned buffers)
    Xh = W.X.t().contiguous().cpu().pin_memory()  # (ncols, n) row-major == column-major n x ncols
    Yh = torch.empty((W.ncols, W.n), dtype=W.tdtype).pin_memory()
    W.host_step(Xh, Yh)
    e2e = []
    for _ in range(max(3, min(args.steps, 10))):
        t0 = time.perf_counter()
        W.host_step(Xh, Yh)
        e2e.append(time.perf_counter() - t0)
    e2e_ms = float(np.median(e2e)) * 1e3
    hbm, tflops, peak_kind = _peaks()
    kb = W.kernel_bytes(fused)
    launch_s = step_ms / 1e3 / (1 if fused else len(W.factor_bytes()))
    achieved = kb / launch_s / 1e9
    if W.name == "csr_random":
        # FP64 on L2-resident operands: the scalar FP64 pipe bounds the
        # per-factor products (10 dependent FMAs per entry)
        peak = fp64_peak(ctx)
        fl = W.flops / len(W.facs)
        roof = {"bound": "fp64", "achieved": round(fl / launch_s / 1e12, 4), "peak": round(peak, 4),
                "unit": "TFLOP/s", "frac": round(fl / launch_s / 1e12 / peak, 4), "traffic": None,
                "peak_kind": "measured in this run (FP64 FMA loop on all SMs)",
                "kernel": chain_kernel if fused else "k_csr_spmm",
                "algorithmic_flops_per_launch": int(fl), "algorithmic_bytes_per_launch": int(kb)}
    elif W.name == "bsr":
        fl = W.flops / len(W.bsr)
        roof = {"bound": "tensor", "achieved": round(fl / launch_s / 1e12, 1), "peak": tflops, "unit": "TFLOP/s",
                "frac": round(fl / launch_s / 1e12 / tflops, 4), "traffic": 259319552,
                "traffic_note": "dram read + write bytes of one launch, ncu capture", "peak_kind": peak_kind,
                "kernel": "k_bsr_tc", "algorithmic_flops_per_launch": int(fl), "algorithmic_bytes_per_launch": int(kb)}
    else:
        # dram read + write bytes of one launch from one ncu capture (the butterfly chain)
        traffic = 212645376 if bfly else None
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "traffic": traffic, "peak_kind": peak_kind,
                "kernel": chain_kernel if fused else "k_csr_spmm", "algorithmic_bytes_per_launch": int(kb)}
    # the problem's bytes (X read, Y written, factor arrays read once) per
    # second, the same count for every arm and path
    path_bytes = _problem_bytes(W)
    value = path_bytes * world / (step_ms / 1e3) / 1e9
    out = {
        "metric": METRIC, "submetric": "Faust.X GB/s (X read + Y written + factor arrays, per second)",
        "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(step_ms, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": W.dtype, "data": "synthetic (seeded)",
        "config": {"workload": W.name, "desc": W.desc, "l2": "flushed (256 MB write) before every timed step",
                   "path": ("butterfly chain kernel" if bfly else "fused chain kernel") if fused
                   else "one launch per factor"},
        "roofline": roof,
        "per_factor_gbs": round(W.step_bytes * world / (step_ms / 1e3) / 1e9, 2),
        "e2e": {"value": round(path_bytes / (e2e_ms / 1e3) / 1e9, 2), "unit": "GB/s",
                "ms_per_step": round(e2e_ms, 3),
                "h2d_bytes_per_step": int(W.n * W.ncols * W.es), "d2h_bytes_per_step": int(W.n * W.ncols * W.es)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if W.name == "bsr" and rank == 0 and not args.no_cpu_baseline:
        out["config"]["error_vs_fp64"] = bsr_error_vs_fp64(W)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_faust_x(W)
    return out


def _bsr_oracle_chain(W, Xs):
    """FP64 oracle of the BSR chain (BSRMat::mul per factor, right to left) on
    the columns Xs (n x c, FP64) with the BF16-rounded blocks."""
    from oracle import oracle as O
    Z = np.asfortranarray(Xs)
    for bp, bc, blocks in reversed(W.bsr_f32):
        flat = np.ascontiguousarray(blocks.transpose(0, 2, 1).reshape(len(bc), -1), np.float64)
        Z = O.bsr_mul_f64(W.n, W.n, 64, 64, bp, bc, flat, Z)
    return Z


def bsr_error_vs_fp64(W, ncols=32):
    """Relative Frobenius error of the GPU result (BF16 storage, FP32
    accumulation, BF16 intermediates) against the FP64 oracle of the same
    BF16 inputs, on a seeded subset of the columns of X."""
    import torch
    from oracle import oracle as O
    O.set_threads(os.cpu_count() or 1)
    W.step()
    torch.cuda.synchronize()
    cols = np.sort(np.random.default_rng(5).choice(W.ncols, ncols, replace=False))
    ci = torch.from_numpy(cols).cuda()
    Xs = W.X.index_select(1, ci).float().cpu().numpy().astype(np.float64)
    Ys = W.Y.index_select(1, ci).float().cpu().numpy().astype(np.float64)
    ref = _bsr_oracle_chain(W, Xs)
    return {"rel_frobenius": float(np.linalg.norm(Ys - ref) / np.linalg.norm(ref)),
            "max_abs": float(np.abs(Ys - ref).max()), "ref_rms": float(np.sqrt(np.mean(ref * ref))),
            "columns": ncols, "oracle": "FP64 BSR chain of the BF16-rounded blocks and X (no intermediate rounding)"}


def _problem_bytes(W, cols=None):
    """X read, Y written and the factor arrays of the Faust x X product on
    `cols` columns (all of X by default), the factor arrays charged to the
    columns in proportion, so that every arm divides the same work."""
    es = 2 if W.name == "bsr" else np.dtype(W.np_dtype).itemsize
    full = 2 * W.n * W.ncols * es + sum(W.factor_bytes())
    return full * (cols if cols is not None else W.ncols) / W.ncols


def cpu_baseline_faust_x(W, sample_cols=None):
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    if W.name == "bsr":
        cols = sample_cols or 32
        Xs = np.random.default_rng(7).standard_normal((W.n, cols))
        _bsr_oracle_chain(W, Xs[:, :2])
        t0 = time.perf_counter()
        _bsr_oracle_chain(W, Xs)
        dt = time.perf_counter() - t0
        bytes_ = _problem_bytes(W, cols)
        flops = sum(2 * f.nnz_blocks * 64 * 64 * cols for f in W.bsr)
        return {"value": round(bytes_ / dt / 1e9, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                "gflops": round(flops / dt / 1e9, 2),
                "sample": "FP64 oracle chain on %d of %d columns of X (%.2f s); bytes counted as BF16 like the "
                          "GPU line" % (cols, W.ncols, dt)}
    cols = sample_cols or (512 if W.name in ("csr_butterfly", "csr_random_f32") else W.ncols)
    rng = np.random.default_rng(7)
    X = np.asfortranarray(rng.standard_normal((W.n, cols)).astype(W.np_dtype))
    O.chain_mul(W.facs, X[:, :8])
    t0 = time.perf_counter()
    reps = 0
    while True:
        O.chain_mul(W.facs, X)
        reps += 1
        if time.perf_counter() - t0 > 3.0:
            break
    dt = (time.perf_counter() - t0) / reps
    bytes_ = _problem_bytes(W, cols)
    return {"value": round(bytes_ / dt / 1e9, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": "%d of %d columns of X, %d repetitions" % (cols, W.ncols, reps)}


# ---------------------------------------------------------------- dense product
PROD_N, PROD_J = 4096, 12


def _product_faust(rng):
    from faust_gb300 import synth
    return synth.butterfly_faust_factors(PROD_J, rng, np.float32)


def _product_bytes(facs, es):
    """Algorithmic bytes of get_product in the default order: the dense image
    of the last factor (one write), then per applied factor one read of its
    input, one write of its output and its CSR arrays."""
    n = facs[0].shape[0]
    plane = n * facs[-1].shape[1] * es
    fb = [f.nnz * (es + 4) + (f.shape[0] + 1) * 4 for f in facs[:-1]]
    per_factor = plane + sum(b + 2 * plane for b in fb)
    chain_launch = 2 * plane + sum(fb)  # the fused chain: image in, product out, factors
    return per_factor, chain_launch


def run_product(args, rank, world):
    import torch
    import faust_gb300 as fg
    torch.cuda.set_device(rank % max(1, torch.cuda.device_count()))
    rng = np.random.default_rng(2024)
    facs = _product_faust(rng)
    stream = torch.cuda.current_stream()
    ctx = fg.Context(torch.cuda.current_device(), stream=stream.cuda_stream)
    F = fg.Faust(facs, ctx=ctx)
    n = PROD_N
    Y = torch.empty((n, n), dtype=torch.float32, device="cuda").t()
    es = 4
    step_bytes, chain_bytes = _product_bytes(facs, es)
    path_bytes = n * n * es + chain_bytes
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        F.product_device("N", "DEFAULT_L2R", Y=Y)
    torch.cuda.synchronize()
    _barrier(world)
    times = []
    launches0 = ctx.kernel_launches()
    with ClockSampler(torch.cuda.current_device()) as clk:
        for _ in range(args.steps):
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            F.product_device("N", "DEFAULT_L2R", Y=Y)
            e.record(stream)
            times.append((s, e))
        torch.cuda.synchronize()
    launches = ctx.kernel_launches() - launches0
    step_ms = _max_over_ranks(float(np.mean([a.elapsed_time(b) for a, b in times])), world)
    # the dominant kernel alone on the same operands: the fused chain of the
    # first 11 factors applied to the dense image of the last one
    F11 = fg.Faust(facs[:-1], ctx=ctx)
    img = torch.from_numpy(np.ascontiguousarray(facs[-1].toarray().T)).cuda().t()
    Y2 = torch.empty_like(Y)
    for _ in range(3):
        F11.matmul_device(img, Y2)
    ch = []
    for _ in range(max(3, args.steps)):
        flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        F11.matmul_device(img, Y2)
        e.record(stream)
        ch.append((s, e))
    torch.cuda.synchronize()
    chain_ms = float(np.mean([a.elapsed_time(b) for a, b in ch]))
    # DYNPROG order (right-to-left leaf pairs for equal-cost butterflies);
    # its first call also builds the factors' transposes, so warm up first
    for _ in range(3):
        F.product_device("N", "DYNPROG", Y=Y2)
    dp = []
    for _ in range(max(3, args.steps)):
        flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        F.product_device("N", "DYNPROG", Y=Y2)
        e.record(stream)
        dp.append((s, e))
    torch.cuda.synchronize()
    dyn_ms = float(np.mean([a.elapsed_time(b) for a, b in dp]))
    # end to end through the public API: toarray() = product + copy to host
    F.toarray()
    e2e = []
    for _ in range(max(3, min(args.steps, 10))):
        t0 = time.perf_counter()
        F.toarray()
        e2e.append(time.perf_counter() - t0)
    e2e_ms = float(np.median(e2e)) * 1e3
    hbm, _, peak_kind = _peaks()
    achieved = chain_bytes / (chain_ms / 1e3) / 1e9
    out = {
        "metric": METRIC, "submetric": "Faust dense product GB/s (algorithmic bytes of the path: the dense image "
        "of the last factor written, then the chain kernel's image in, product out and factor arrays / step time)",
        "value": round(path_bytes * world / (step_ms / 1e3) / 1e9, 2), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": "product", "desc": "get_product (DEFAULT_L2R) of 12 CSR butterfly factors 4096^2 "
                   "(2 nnz/row) FP32 -> dense 4096x4096", "l2": "flushed (256 MB write) before every timed step",
                   "path": "dense image of the last factor + butterfly chain kernel over the other 11",
                   "dynprog_ms_per_step": round(dyn_ms, 4)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "traffic": None, "peak_kind": peak_kind,
                     "kernel": "k_bfly_chain", "kernel_ms": round(chain_ms, 4),
                     "algorithmic_bytes_per_launch": int(chain_bytes)},
        "per_factor_gbs": round(step_bytes * world / (step_ms / 1e3) / 1e9, 2),
        "e2e": {"value": round(path_bytes / (e2e_ms / 1e3) / 1e9, 2), "unit": "GB/s", "ms_per_step": round(e2e_ms, 3),
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": int(n * n * es)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_product(facs)
    F11.close()
    F.close()
    return out


def cpu_baseline_product(facs, budget_s=3.0):
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    _, chain_bytes = _product_bytes(facs, 4)
    n = facs[0].shape[0]
    step_bytes = n * facs[-1].shape[1] * 4 + chain_bytes  # the GPU line's count
    t0 = time.perf_counter()
    reps = 0
    while True:
        O.faust_product(facs, "N", 0)
        reps += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = (time.perf_counter() - t0) / reps
    return {"value": round(step_bytes / dt / 1e9, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": "the whole product, %d repetitions" % reps}


# ---------------------------------------------------------------- PALM4MSA
PALM_N, PALM_J, PALM_K, PALM_ITS, PALM_THR = 1024, 10, 2048, 200, 1e-8
_palm_its = PALM_ITS  # --palm-its shortens the run for profiling captures only


def _palm_problem():
    from faust_gb300 import fact, synth
    H = synth.hadamard(PALM_N) / 32.0
    cons = [fact.ConstraintInt("sp", PALM_N, PALM_N, PALM_K) for _ in range(PALM_J)]
    params = fact.ParamsPalm4MSA(cons, _palm_its, norm2_threshold=PALM_THR, norm2_max_iter=100)
    return H, cons, params


def run_palm(args, rank, world):
    import ctypes
    import torch
    import faust_gb300 as fg
    from faust_gb300 import _ffi, fact
    torch.cuda.set_device(rank % max(1, torch.cuda.device_count()))
    H, cons, params = _palm_problem()
    ctx = fg.Context(torch.cuda.current_device())
    Hd = torch.from_numpy(np.ascontiguousarray(H.T)).cuda().t()  # column-major, device resident
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    res = None
    for _ in range(args.warmup):
        res = fact.palm4msa(Hd, cons, params, ctx=ctx)
        res.faust.close()
    torch.cuda.synchronize()
    _barrier(world)
    times = []
    launches0 = ctx.kernel_launches()
    with ClockSampler(torch.cuda.current_device()) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = fact.palm4msa(Hd, cons, params, ctx=ctx)
            times.append(time.perf_counter() - t0)
            if _ != args.steps - 1:
                res.faust.close()
    launches = (ctx.kernel_launches() - launches0) // max(1, args.steps)
    step_s = float(np.mean(times))
    step_s = _max_over_ranks(step_s, world)
    # relative error of the result (outside the timed region)
    err = ctypes.c_double()
    _ffi.check(_ffi.lib().fgb_rel_err(res.faust.handle, Hd.data_ptr(), res.lambda_, ctypes.byref(err)), ctx.handle)
    run_factors = [res.faust.factors(i) for i in range(PALM_J)]
    res.faust.close()
    # end to end through the host-memory C-ABI entry point, under the same
    # conditions as the device-resident runs (L2 flushed before each, mean of
    # the same number of runs): A from host memory in, every factor back to
    # host memory
    Hh = np.asfortranarray(H)
    e2e = []
    d2h = 0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fact.palm4msa(Hh, cons, params, ctx=ctx)
        facs = [r.faust.factors(i) for i in range(PALM_J)]
        e2e.append(time.perf_counter() - t0)
        d2h = sum(f.nnz * 12 + (f.shape[0] + 1) * 4 for f in facs)
        r.faust.close()
    e2e_s = _max_over_ranks(float(np.mean(e2e)), world)
    hbm, tflops, peak_kind = _peaks()
    roof_spmm, roof_pi = palm_roofline(ctx, run_factors)
    out = {
        "metric": METRIC, "submetric": "palm4msa2 FP64 time to the plain 200-iteration relative error (s per run)",
        "value": round(step_s, 5), "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(step_s * 1e3, 3), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (Sylvester Hadamard 1024 / 32)",
        "config": {"workload": "palm4msa2 Hadamard 1024/32, 10 factors sp k=2048, identity init, 200 its, "
                               "power-iteration tol 1e-8 (max 100), FP64",
                   "l2": "flushed (256 MB write) before every timed run", "rel_err": err.value,
                   "lambda": res.lambda_},
        "roofline": roof_spmm,
        "roofline_power_iteration": roof_pi,
        "e2e": {"value": round(e2e_s, 5), "unit": "s", "h2d_bytes_per_step": int(H.nbytes),
                "d2h_bytes_per_step": int(d2h), "runs": len(e2e)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_palm(single_core=args.cpu_single_core)
    return out


def fp64_peak(ctx):
    """Scalar FP64 FMA throughput of the device in TFLOP/s, measured in this
    run (fgb_probe_fp64_fma: dependent-FMA loops on every SM)."""
    import ctypes
    from faust_gb300 import _ffi
    out = ctypes.c_double()
    _ffi.check(_ffi.lib().fgb_probe_fp64_fma(ctx.handle, ctypes.byref(out)), ctx.handle)
    return out.value / 1e12


def palm_roofline(ctx, run_factors):
    """Rooflines of the two FP64 kernels of the PALM run, each timed alone with
    CUDA events on the run's own final factors.

    * The gradient product (the main stream's largest share): one factor of
      the run times a 1024 x 1024 FP64 block, as an update launches it
      (k_csr_spmm for rows of at most 16 entries beside k_csr_spmm_long for
      the longer rows on a forked side stream), over each of the 10 factors;
      against the device FP64 FMA rate.
    * The power iteration (one CTA per chain, on a side stream in the run) on
      the run's chain S_1 ... S_9: against one SM's share of the FP64 FMA
      rate (it is one CTA) and against the whole device.
    Both work on L2-resident data: the scalar FP64 pipe, not HBM, bounds them."""
    import ctypes
    import torch
    import faust_gb300 as fg
    from faust_gb300 import _ffi
    peak = fp64_peak(ctx)
    sm_count = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    stream = torch.cuda.current_stream()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # --- gradient products: each factor of the run times a 1024^2 block
    X = torch.randn((PALM_N, PALM_N), device="cuda", dtype=torch.float64).t()
    Y = torch.empty((PALM_N, PALM_N), device="cuda", dtype=torch.float64).t()
    singles = [fg.Faust([f], ctx=ctx) for f in run_factors]
    for G in singles:
        G.matmul_device(X, Y, mode=1)
    torch.cuda.synchronize()
    calls = 20
    s.record(stream)
    for _ in range(calls):
        for G in singles:
            G.matmul_device(X, Y, mode=1)
    e.record(stream)
    torch.cuda.synchronize()
    us = s.elapsed_time(e) * 1e3 / (calls * len(singles))
    nnz = float(np.mean([f.nnz for f in run_factors]))
    longest = max(int(np.diff(f.indptr).max()) for f in run_factors)
    flops = 2.0 * nnz * PALM_N
    spmm = {"bound": "fp64", "achieved": round(flops / (us * 1e-6) / 1e12, 4), "peak": round(peak, 4),
            "unit": "TFLOP/s", "frac": round(flops / (us * 1e-6) / 1e12 / peak, 4),
            "traffic": None, "traffic_note": "L2-resident operands (8 MB blocks); see profiles/",
            "peak_kind": "measured in this run (FP64 FMA loop on all SMs; MEASURED_PEAKS.json has no FP64 figure)",
            "kernel": "k_csr_spmm + k_csr_spmm_long (one gradient product: a factor of the run, %d entries on "
                      "average, rows up to %d, x a 1024^2 FP64 block)" % (nnz, longest),
            "algorithmic_flops_per_launch": int(flops), "us_per_launch": round(us, 3),
            "timing": "CUDA events, %d back-to-back products of each of the 10 factors" % calls}
    for G in singles:
        G.close()
    # --- power iteration on the run's chain S_1 ... S_9 (one CTA)
    G = fg.Faust(run_factors[1:], ctx=ctx)
    out, flag = ctypes.c_double(), ctypes.c_int()

    def norm():
        _ffi.check(_ffi.lib().fgb_faust_spectral_norm(G.handle, 100, PALM_THR, ctypes.byref(out),
                                                      ctypes.byref(flag)), ctx.handle)
    norm()
    reps = 5
    s.record(stream)
    for _ in range(reps):
        norm()
    e.record(stream)
    torch.cuda.synchronize()
    pi_us = s.elapsed_time(e) * 1e3 / reps
    G.close()
    its = 100 if flag.value < 0 else max(1, flag.value)
    # per iteration: F F^H x over 2 x 9 products (2 flops per entry) and two
    # length-n dot products
    chain_nnz = float(sum(f.nnz for f in run_factors[1:]))
    pi_flops = its * (2 * 2.0 * chain_nnz + 4.0 * PALM_N)
    achieved = pi_flops / (pi_us * 1e-6) / 1e12
    sm_peak = peak / sm_count
    pi = {"bound": "fp64", "achieved": round(achieved, 5), "peak": round(peak, 4), "unit": "TFLOP/s",
          "frac": round(achieved / peak, 5), "peak_one_sm": round(sm_peak, 5),
          "frac_of_one_sm": round(achieved / sm_peak, 4), "traffic": None,
          "peak_kind": "the device FP64 FMA rate measured in this run; frac_of_one_sm against one SM's share "
                       "(the kernel is one CTA per chain)",
          "kernel": "k_power_iteration (the run's chain S_1..S_9, %d entries, %d iterations to tol 1e-8)"
                    % (chain_nnz, its),
          "algorithmic_flops_per_launch": int(pi_flops), "us_per_launch": round(pi_us, 1)}
    return spmm, pi


def cpu_baseline_palm(single_core=False):
    """The oracle's palm4msa2 over the whole 200-iteration run on all host
    cores (and, with single_core, the whole run again on one core: the
    reference's default CPU build is single-threaded)."""
    from oracle import oracle as O
    H, cons, params = _palm_problem()
    threads = os.cpu_count() or 1
    runs = [(threads, "all host threads")] + ([(1, "one thread")] if single_core else [])
    out = None
    for th, what in runs:
        O.set_threads(th)
        t0 = time.perf_counter()
        O.palm4msa2(H, [c.oracle_dict() for c in cons], _palm_its, norm2_threshold=PALM_THR, norm2_max_iter=100)
        dt = time.perf_counter() - t0
        rec = {"value": round(dt, 3), "unit": "s", "cores": th, "kind": "port",
               "sample": "the whole %d-iteration run once on %s" % (_palm_its, what)}
        if out is None:
            out = rec
        else:
            out["single_core"] = rec
    O.set_threads(threads)
    return out


# ---------------------------------------------------------------- batched PALM4MSA
def batched_problem(rng, count=512):
    from faust_gb300 import synth
    return synth.batched_palm_targets(rng, count)


def run_batched(args, rank, world):
    """512 independent palm4msa2 instances (splincol k=4, 4 factors, 100
    iterations, FP32 with FP64 step-size norms) in one persistent launch;
    value = instances per second (all ranks)."""
    import torch
    import faust_gb300 as fg
    from faust_gb300 import fact
    torch.cuda.set_device(rank % max(1, torch.cuda.device_count()))
    rng = np.random.default_rng(4 + rank)
    ns, mats = batched_problem(rng, args.batch_count)
    ctx = fg.default_context(torch.cuda.current_device())
    dev = [torch.from_numpy(np.ascontiguousarray(A.T)).cuda().t() for A in mats]
    cons_by_n = {}
    probs = []
    for A, n in zip(dev, ns):
        if n not in cons_by_n:
            cons_by_n[n] = [fact.ConstraintInt("splincol", int(n), int(n), 4) for _ in range(4)]
        probs.append((A, cons_by_n[n]))
    params = fact.ParamsPalm4MSA(probs[0][1], 100, norm2_fp64=True)
    for _ in range(args.warmup):
        res = fact.palm4msa_batched(probs[:32], params, ctx=ctx, ctas_per_sm=args.ctas_per_sm)
        for r in res:
            r.faust.close()
    torch.cuda.synchronize()
    _barrier(world)
    times = []
    with ClockSampler(torch.cuda.current_device()) as clk:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = fact.palm4msa_batched(probs, params, ctx=ctx, ctas_per_sm=args.ctas_per_sm)
            times.append(time.perf_counter() - t0)
            bad = sum(1 for r in res if r.status)
            cycles = np.array([r.cycles for r in res], np.float64)
            for r in res:
                r.faust.close()
    step_s = _max_over_ranks(float(np.mean(times)), world)
    # per-instance time on its CTA (SM cycles at the sampled clock): the
    # largest instances bound the launch
    mhz = clk.summary().get("sm_mhz") or 2070.0
    inst_s = cycles / (mhz * 1e6)
    by_n = {}
    lo = 0
    for hi in (64, 128, 256, 384, 512):
        sel = (ns > lo) & (ns <= hi)
        if sel.any():
            by_n["%d-%d" % (lo + 1, hi)] = round(float(np.median(inst_s[sel])), 4)
        lo = hi
    per_instance = {"max_s": round(float(inst_s.max()), 4), "median_s": round(float(np.median(inst_s)), 4),
                    "sum_over_ctas_s": round(float(inst_s.sum()), 2), "median_s_by_n_bucket": by_n}
    # end to end: host matrices in, every factor back to host memory
    t0 = time.perf_counter()
    dev2 = [torch.from_numpy(np.ascontiguousarray(A.T)).cuda().t() for A in mats]
    res = fact.palm4msa_batched([(A, c) for A, (_, c) in zip(dev2, probs)], params, ctx=ctx,
                                ctas_per_sm=args.ctas_per_sm)
    d2h = 0
    for r in res:
        for i in range(4):
            f = r.faust.factors(i)
            d2h += f.nnz * 8 + (f.shape[0] + 1) * 4
        r.faust.close()
    e2e_s = time.perf_counter() - t0
    out = {
        "metric": METRIC, "submetric": "batched palm4msa2 instances per second (one persistent launch)",
        "value": round(len(mats) * world / step_s, 2), "unit": "instances/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(step_s * 1e3, 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (FP64 step-size norms)", "data": "synthetic (seeded)",
        "config": {"workload": "%d palm4msa2 instances, n in [64, 512] log-uniform (multiples of 16), "
                               "target P1P2P3 + 1e-3 noise, 4 factors splincol k=4, 100 iterations" % len(mats),
                   "sum_n2": int(np.sum(ns.astype(np.int64) ** 2)), "failed_instances": bad,
                   "ctas_per_sm": args.ctas_per_sm or fact.tuned_ctas_per_sm(int(ns.max()), len(ns), np.float32),
                   "ctas_per_sm_from": "argument" if args.ctas_per_sm else "faust_gb300/tuning/batched_palm.json",
                   "instance_time_on_its_cta": per_instance},
        "e2e": {"value": round(len(mats) / e2e_s, 2), "unit": "instances/s",
                "h2d_bytes_per_step": int(sum(A.nbytes for A in mats)), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": 1,
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_batched(ns, mats)
    return out


def cpu_baseline_batched(ns, mats, sample=16):
    """The oracle on a sample of instances, one instance per host core."""
    import concurrent.futures
    import multiprocessing
    from oracle import oracle as O
    idx = np.random.default_rng(0).choice(len(mats), size=min(sample, len(mats)), replace=False)
    threads = os.cpu_count() or 1
    O.set_threads(1)
    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda i: O.palm4msa2(mats[i], [dict(kind=O.SPLINCOL, k=4, rows=int(ns[i]), cols=int(ns[i]))
                                                    for _ in range(4)], 100, norm2_fp64=True), idx))
    dt = time.perf_counter() - t0
    scale = float(np.sum(ns.astype(np.float64) ** 2) / np.sum(ns[idx].astype(np.float64) ** 2))
    return {"value": round(len(mats) / (dt * scale), 3), "unit": "instances/s", "cores": threads, "kind": "port",
            "sample": "%d of %d instances on %d threads (%.1f s), scaled by sum n^2" % (len(idx), len(mats),
                                                                                      threads, dt)}


# ---------------------------------------------------------------- learned warm start
def run_warmstart(args, rank, world):
    """Gaussian-kernel butterfly factorizations: plain palm4msa2 (200
    iterations) against MLP-predicted factors refined by palm4msa2, on
    held-out draws.  Every held-out matrix is compared with its OWN plain
    200-iteration relative error.  value = wall time, for the whole held-out
    set, of the MLP inference plus the seeded refinement (the device writes
    the predicted values into the supports and the optimal starting lambda)
    at the smallest iteration count where every instance is at or below its
    own plain error; if no count in the sweep gets every instance there, the
    largest share of 0.99, 0.95 and 0.9 that some count reaches (config names
    the share, and time_to_share gives every level)."""
    import torch
    import faust_gb300 as fg
    from faust_gb300 import warmstart as ws
    torch.cuda.set_device(rank % max(1, torch.cuda.device_count()))
    rng = np.random.default_rng(11 + rank)
    ctx = fg.default_context(torch.cuda.current_device())
    prob = ws.ButterflyProblem()
    ntrain, ntest = args.ws_train, args.ws_test
    t0 = time.perf_counter()
    Ktr, _ = ws.kernel_matrices(ntrain, rng)
    Y = []
    for s0 in range(0, ntrain, 2048):
        res, _ = ws.run_plain(prob, Ktr[s0:s0 + 2048], 200)
        Y.append(np.stack([prob.factor_values(r.faust) for r in res]))
        for r in res:
            r.faust.close()
    Y = torch.from_numpy(np.concatenate(Y)).cuda()
    t_gen = time.perf_counter() - t0
    X = ws.to_inputs(torch, Ktr)
    net = ws.MLP(batch=256, seed=1)
    t0 = time.perf_counter()
    losses = []
    for epoch in range(args.ws_epochs):
        perm = torch.randperm(ntrain, device="cuda")
        for s0 in range(0, ntrain - 255, 256):
            idx = perm[s0:s0 + 256]
            losses.append(net.train_step(X[idx].contiguous(), Y[idx].contiguous(), lr=3e-4))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del X, Y
    Kte, _ = ws.kernel_matrices(ntest, rng)
    Kd = ws.to_device(Kte)
    Xte = ws.to_inputs(torch, Kte)
    for _ in range(args.warmup):
        r, _t = ws.run_plain(prob, Kd[:64], 5)
        for x in r:
            x.faust.close()
        for x in ws.run_warm(prob, Kd[:64], net.predict(Xte[:64]), 5):
            x.faust.close()
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        plain, t_plain = ws.run_plain(prob, Kd, 200)
        e_plain = ws.rel_errors(plain, Kd)
        for r in plain:
            r.faust.close()
        sweep = {}
        for its in (1, 2, 5, 10, 20, 50, 100, 200):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            pred = net.predict(Xte)
            warm = ws.run_warm(prob, Kd, pred, its)
            t_w = time.perf_counter() - t0
            e_w = ws.rel_errors(warm, Kd)
            for r in warm:
                r.faust.close()
            ok = e_w <= e_plain
            sweep[its] = {"s": round(t_w, 4), "frac_at_or_below_own_plain": float(np.mean(ok)),
                          "median_rel_err": float(np.median(e_w)),
                          "median_ratio_to_own_plain": float(np.median(e_w / e_plain))}
    # time (inference + refinement) at the smallest iteration count where a
    # given share of the held-out instances is at or below its own plain error
    reach = {}
    for share in (1.0, 0.99, 0.95, 0.9, 0.5):
        ok = [k for k, v in sweep.items() if v["frac_at_or_below_own_plain"] >= share]
        reach["%g" % share] = {"iterations": ok[0], "s": sweep[ok[0]]["s"]} if ok else None
    crit = next((sh for sh in ("1", "0.99", "0.95", "0.9") if reach[sh]), None)
    its_needed = reach[crit]["iterations"] if crit else None
    value = reach[crit]["s"] if crit else None
    out = {
        "metric": METRIC, "submetric": "time for %d held-out kernel matrices to reach their own plain palm4msa2 "
                                       "200-iteration relative error from the learned start (s)" % ntest,
        "value": round(value, 4) if value else None, "unit": "s", "n_gpus": world, "steps": 1,
        "warmup": args.warmup, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+bf16", "data": "synthetic Gaussian kernel matrices (256 points U[0,1]^3, sigma log-U[0.05,0.5])",
        "config": {"workload": "warmstart: 8 butterfly supp factors of 256x256, MLP 65536-1024-1024-4096 BF16",
                   "train_instances": ntrain, "test_instances": ntest, "epochs": args.ws_epochs,
                   "timed": "MLP inference + seeded batched refinement (values and starting lambda set on the "
                            "device), matrices already on the device; plain: the batched 200-iteration run",
                   "plain_200_s": round(t_plain, 4), "plain_median_rel_err": float(np.median(e_plain)),
                   "criterion": ("share of instances at or below their own plain 200-iteration error >= %s"
                                 % crit) if crit else None,
                   "iterations_needed": its_needed, "time_to_share": reach,
                   "speedup_vs_plain": round(t_plain / value, 3) if value else None, "sweep": sweep,
                   "data_gen_s": round(t_gen, 2), "train_s": round(t_train, 2),
                   "final_train_loss": losses[-1] if losses else None},
        "clocks": clk.summary(),
    }
    return out


# ---------------------------------------------------------------- helpers
def _barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(x, world):
    """The slowest rank's time: every rank's timed region ends at the same
    barrier, so the job's time is the maximum (NCCL on the GPUs; gloo keeps
    the tensor on the host)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="palm",
                    choices=["palm", "batched", "csr_butterfly", "csr_random", "csr_random_f32", "bsr", "warmstart",
                             "product"])
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--ctas-per-sm", type=int, default=0,
                    help="batched: resident instances per SM (0 = the tuned table's choice)")
    ap.add_argument("--ws-train", type=int, default=20000)
    ap.add_argument("--ws-test", type=int, default=1024)
    ap.add_argument("--ws-epochs", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-single-core", action="store_true",
                    help="palm: also time the CPU baseline's whole run on one core (about 75 s)")
    ap.add_argument("--palm-its", type=int, default=PALM_ITS,
                    help="iterations of the PALM workload (profiling captures only; the bench uses 200)")
    args = ap.parse_args()
    global _palm_its
    _palm_its = args.palm_its
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    if args.impl == "reference":
        if rank == 0:
            out = reference_arm(args, world)
            print(json.dumps(out), flush=True)
        return
    if args.workload == "palm":
        out = run_palm(args, rank, world)
    elif args.workload == "warmstart":
        out = run_warmstart(args, rank, world)
    elif args.workload == "batched":
        out = run_batched(args, rank, world)
    elif args.workload == "product":
        out = run_product(args, rank, world)
    else:
        out = run_faust_x(args, rank, world)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def reference_arm_palm(args, world):
    """The oracle's palm4msa2 (CPU restatement of the reference, all host
    threads) on the PALM workload.  The K timed steps walk through ONE whole
    run: step i runs iterations [i*m, (i+1)*m) with m = ceil(200 / K),
    starting from the factors and lambda step i-1 ended with (the first step
    from the identity initialisation), so every iteration of the run is timed
    once; the value is the total time scaled to 200 iterations (exactly the
    run's time when K divides 200).  The W warm-up steps run the first m
    iterations untimed."""
    from oracle import oracle as O
    H, cons, params = _palm_problem()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    ocons = [c.oracle_dict() for c in cons]
    K = max(1, args.steps)
    m = -(-_palm_its // K)
    for _ in range(args.warmup):
        O.palm4msa2(H, ocons, m, norm2_threshold=PALM_THR, norm2_max_iter=100)
    facts, lam = None, 1.0
    total = 0.0
    for _ in range(K):
        t0 = time.perf_counter()
        facts, lam, _tr = O.palm4msa2(H, ocons, m, norm2_threshold=PALM_THR, norm2_max_iter=100,
                                      init_facts=facts, init_lambda=lam)
        total += time.perf_counter() - t0
    its = K * m
    v = round(total * _palm_its / its, 3)
    rel = O.rel_err(H, facts, lam)
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total / K * 1e3, 1),
            "higher_is_better": False,
            "config": {"workload": "palm4msa2 Hadamard 1024/32, 10 factors sp k=2048, identity init, 200 its, "
                                   "power-iteration tol 1e-8 (max 100), FP64",
                       "rel_err": rel, "lambda": lam},
            "cpu_baseline": {"value": v, "unit": "s", "cores": threads, "kind": "port",
                             "sample": "one whole run: %d steps of %d consecutive iterations (%d timed), each "
                                       "resuming from the previous step's factors" % (K, m, its)},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def reference_arm(args, world):
    import faust_gb300.synth  # noqa: F401  (generators only)
    rng = np.random.default_rng(2024)
    if args.workload == "palm":
        return reference_arm_palm(args, world)

    if args.workload == "product":
        facs = _product_faust(rng)
        vals = [cpu_baseline_product(facs) for _ in range(max(1, args.steps))]
        v = float(np.median([x["value"] for x in vals]))
        cb = dict(vals[0])
        cb["value"] = v
        return {"impl": "reference", "metric": METRIC, "value": v, "unit": "GB/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "config": {"workload": "product"}, "cpu_baseline": cb,
                "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}

    if args.workload == "warmstart":
        return {"impl": "reference", "unavailable": "the learned warm start has no reference counterpart; "
                "its line times plain palm4msa2 initialisation beside it"}

    if args.workload == "batched":
        ns, mats = batched_problem(np.random.default_rng(4), args.batch_count)
        vals = [cpu_baseline_batched(ns, mats) for _ in range(max(1, args.steps))]
        v = float(np.median([x["value"] for x in vals]))
        cb = dict(vals[0])
        cb["value"] = v
        return {"impl": "reference", "metric": METRIC, "value": v, "unit": "instances/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "config": {"workload": "batched"}, "cpu_baseline": cb,
                "e2e": {"value": v, "unit": "instances/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}

    class _W:
        pass

    from faust_gb300 import synth
    W = _W()
    W.name = args.workload
    if W.name == "bsr":
        import types
        W.n, W.ncols = 16384, 4096
        sigma = 1.0 / np.sqrt(8 * 64)
        W.bsr_f32 = []
        for _ in range(4):
            bp, bc, blocks = synth.random_bsr(16384, 64, 8, rng, sigma)
            W.bsr_f32.append((bp, bc, synth.bf16_to_f32(synth.bf16_bits(blocks)).reshape(blocks.shape)))
        W.bsr = [types.SimpleNamespace(nnz_blocks=len(bc)) for _, bc, _ in W.bsr_f32]
        W.factor_bytes = lambda: [len(bc) * 64 * 64 * 2 + len(bc) * 4 + len(bp) * 4 for bp, bc, _ in W.bsr_f32]
        vals = [cpu_baseline_faust_x(W) for _ in range(max(1, args.steps))]
        v = float(np.median([x["value"] for x in vals]))
        cb = dict(vals[0])
        cb["value"] = v
        return {"impl": "reference", "metric": METRIC, "value": v, "unit": "GB/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "config": {"workload": "bsr"}, "cpu_baseline": cb,
                "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if W.name == "csr_butterfly":
        W.facs = synth.butterfly_faust_factors(12, rng, np.float32)
        W.n, W.ncols, W.np_dtype = 4096, 8192, np.float32
    elif W.name == "csr_random_f32":
        W.facs = [synth.random_csr(4096, 4096, 2, rng, np.float32) for _ in range(12)]
        W.n, W.ncols, W.np_dtype = 4096, 8192, np.float32
    else:
        W.facs = [synth.random_csr(1024, 1024, 10, rng) for _ in range(5)]
        W.n, W.ncols, W.np_dtype = 1024, 512, np.float64
    es = np.dtype(W.np_dtype).itemsize
    W.factor_bytes = lambda: [f.nnz * (es + 4) + (f.shape[0] + 1) * 4 for f in W.facs]
    vals = []
    for _ in range(max(1, args.steps)):
        vals.append(cpu_baseline_faust_x(W))
    v = float(np.median([x["value"] for x in vals]))
    cb = dict(vals[0])
    cb["value"] = v
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "config": {"workload": W.name}, "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


if __name__ == "__main__":
    main()
