"""Learned warm start for palm4msa2 on butterfly supports.

A BF16 MLP (65536 -> 1024 -> 1024 -> 4096, ReLU) maps a 256 x 256 Gaussian
kernel matrix K_ij = exp(-|x_i - x_j|^2 / (2 sigma^2)) to the 4096 values of
its 8 butterfly-support factors (2 entries per row each).  It is trained on
factorizations produced by plain palm4msa2 (the batched GPU driver) and its
prediction seeds a shorter palm4msa2 refinement; plain initialisation stays
the fallback and plain palm4msa2's 200-iteration error is the target.

Every GEMM runs in the project's tcgen05 kernel (fgb_gemm_bf16) and every
elementwise training step in its own kernels (include/fgb_mlp.h); torch only
holds device memory.
"""
import ctypes
import math
import time

import numpy as np

from . import _ffi, fact, synth
from ._ffi import check
from .faust import default_context

N_POINTS = 256
N_FACTORS = 8
N_VALUES = N_FACTORS * 2 * N_POINTS  # 4096
VALUE_SCALE = math.sqrt(2 * N_POINTS)  # factors have unit Frobenius norm


def _torch():
    import torch
    return torch


# ---------------------------------------------------------------- data
def kernel_matrices(count, rng, n=N_POINTS, sig_lo=0.05, sig_hi=0.5):
    """count Gaussian kernel matrices over n points uniform in [0,1]^3, sigma
    log-uniform in [sig_lo, sig_hi] (FP32, (count, n, n))."""
    x = rng.random((count, n, 3))
    sig = np.exp(rng.uniform(np.log(sig_lo), np.log(sig_hi), size=count))
    d2 = ((x[:, :, None, :] - x[:, None, :, :]) ** 2).sum(-1)
    return np.exp(-d2 / (2 * sig[:, None, None] ** 2)).astype(np.float32), sig


def supports():
    return synth.butterfly_supports(N_FACTORS, np.float32)


def support_positions():
    """(factor, row, col) of the 4096 support entries in CSR order."""
    pos = []
    for f, s in enumerate(supports()):
        for r in range(s.shape[0]):
            for p in range(s.indptr[r], s.indptr[r + 1]):
                pos.append((f, r, s.indices[p]))
    return np.array(pos, np.int64)


class ButterflyProblem:
    """Constraint objects shared by every instance (their supports go to the
    device once per batched call)."""

    def __init__(self):
        self.sups = supports()
        self.cons = [fact.ConstraintMat("supp", s.toarray()) for s in self.sups]
        self.pos = support_positions()

    def params(self, its, init_lambda=1.0):
        return fact.ParamsPalm4MSA(self.cons, its, init_lambda=init_lambda)

    def factor_values(self, faust):
        """4096 support values of a palm4msa2 result (scaled to O(1))."""
        dense = np.stack([faust.factors(i).toarray() for i in range(N_FACTORS)])
        return (dense[self.pos[:, 0], self.pos[:, 1], self.pos[:, 2]] * VALUE_SCALE).astype(np.float32)

    def init_factors(self, values):
        """Dense factors on the supports from 4096 predicted values, as the
        seeded batched run forms them (value / VALUE_SCALE, rounded once to
        FP32)."""
        facs = np.zeros((N_FACTORS, N_POINTS, N_POINTS), np.float32)
        v = (np.asarray(values, np.float32).astype(np.float64) * (1.0 / VALUE_SCALE)).astype(np.float32)
        facs[self.pos[:, 0], self.pos[:, 1], self.pos[:, 2]] = v
        return list(facs)


def _colmajor(torch, M):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(M).T)).cuda().t()


def to_device(Ks):
    """Column-major CUDA copies of host kernel matrices."""
    torch = _torch()
    return [_colmajor(torch, K) for K in Ks]


def run_plain(problem, Ks, its, ctx=None, ctas_per_sm=0):
    """Plain palm4msa2 (default zero/identity initialisation) on each K in one
    batched launch; Ks host arrays or column-major CUDA tensors.  Returns
    (results, wall seconds of the batched call)."""
    torch = _torch()
    mats = [K if isinstance(K, torch.Tensor) else _colmajor(torch, K) for K in Ks]
    probs = [(M, problem.cons) for M in mats]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = fact.palm4msa_batched(probs, problem.params(its), ctx=ctx, ctas_per_sm=ctas_per_sm)
    return res, time.perf_counter() - t0


def rel_errors(results, Ks, ctx=None):
    torch = _torch()
    out = []
    for r, K in zip(results, Ks):
        A = K if isinstance(K, torch.Tensor) else _colmajor(torch, K)
        e = ctypes.c_double()
        check(_ffi.lib().fgb_rel_err(r.faust.handle, A.data_ptr(), r.lambda_, ctypes.byref(e)),
              (ctx or default_context()).handle)
        out.append(e.value)
    return np.array(out)


# ---------------------------------------------------------------- MLP
class MLP:
    """dims[0] -> dims[1] -> ... (ReLU between layers, linear output).
    FP32 master weights + BF16 copies (W and W^T) on the device."""

    def __init__(self, dims=(N_POINTS * N_POINTS, 1024, 1024, N_VALUES), batch=256, seed=0, ctx=None):
        torch = _torch()
        self.torch = torch
        self.ctx = ctx or default_context()
        self.dims = list(dims)
        self.batch = batch
        g = torch.Generator(device="cuda").manual_seed(seed)
        self.W, self.Wb, self.WTb, self.b, self.mW, self.vW, self.mb, self.vb = ([] for _ in range(8))
        for fin, fout in zip(dims[:-1], dims[1:]):
            std = math.sqrt(2.0 / fin)
            W = torch.randn((fout, fin), generator=g, device="cuda", dtype=torch.float32) * std
            self.W.append(W)
            self.Wb.append(torch.empty((fout, fin), device="cuda", dtype=torch.bfloat16))
            self.WTb.append(torch.empty((fin, fout), device="cuda", dtype=torch.bfloat16))
            self.b.append(torch.zeros(fout, device="cuda", dtype=torch.float32))
            self.mW.append(torch.zeros_like(W))
            self.vW.append(torch.zeros_like(W))
            self.mb.append(torch.zeros(fout, device="cuda", dtype=torch.float32))
            self.vb.append(torch.zeros(fout, device="cuda", dtype=torch.float32))
        for i in range(len(self.W)):
            self._refresh(i)
        self.step_no = 0
        B = batch
        self.act = [torch.empty((B, d), device="cuda", dtype=torch.bfloat16) for d in dims[1:-1]]
        self.out = torch.empty((B, dims[-1]), device="cuda", dtype=torch.float32)
        self.work = torch.empty(B * max(dims[1:]), device="cuda", dtype=torch.float32)
        self.gW = [torch.empty_like(W) for W in self.W]
        self.gb = [torch.empty_like(b) for b in self.b]
        self.dact = [torch.empty((B, d), device="cuda", dtype=torch.bfloat16) for d in dims[1:]]
        self.dz = [torch.empty((B, d), device="cuda", dtype=torch.bfloat16) for d in dims[1:]]
        self.dzT = [torch.empty((d, B), device="cuda", dtype=torch.bfloat16) for d in dims[1:]]
        self.xT = [torch.empty((d, B), device="cuda", dtype=torch.bfloat16) for d in dims[:-1]]
        self.loss = torch.zeros(1, device="cuda", dtype=torch.float32)

    def _lib(self):
        return _ffi.lib()

    def _refresh(self, i):
        L = self._lib()
        W = self.W[i]
        check(L.fgb_mlp_f32_to_bf16(self.ctx.handle, W.numel(), W.data_ptr(), self.Wb[i].data_ptr()), self.ctx.handle)
        fout, fin = W.shape
        check(L.fgb_mlp_transpose_bf16(self.ctx.handle, fout, fin, self.Wb[i].data_ptr(), fin, self.WTb[i].data_ptr(),
                                       fout), self.ctx.handle)

    def _gemm(self, M, N, K, A, lda, B, ldb, C, ldc, c_f32, bias=None, relu=False, split_k=1):
        check(self._lib().fgb_gemm_bf16(self.ctx.handle, M, N, K, A.data_ptr(), lda, B.data_ptr(), ldb, C.data_ptr(),
                                        ldc, _ffi.F32 if c_f32 else _ffi.BF16,
                                        bias.data_ptr() if bias is not None else None, int(relu), split_k,
                                        self.work.data_ptr()), self.ctx.handle)

    @staticmethod
    def _split(M, N, K, sm=152):
        tiles = (M // 128) * (N // 128)
        if tiles >= sm:
            return 1
        return max(1, min(K // 64, sm // max(1, tiles)))

    def forward(self, X):
        """X: (B, dims[0]) BF16 CUDA tensor -> FP32 (B, dims[-1])."""
        B = X.shape[0]
        h = X
        nl = len(self.W)
        for i in range(nl):
            fout, fin = self.W[i].shape
            last = i == nl - 1
            C = self.out if last else self.act[i]
            self._gemm(B, fout, fin, h, fin, self.Wb[i], fin, C, fout, last, bias=self.b[i], relu=not last,
                       split_k=self._split(B, fout, fin))
            h = C
        self._x = X
        return self.out

    def train_step(self, X, T, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        """One Adam step on the mean squared error to T (FP32 (B, out)); returns the loss."""
        torch = self.torch
        L = self._lib()
        h = self.ctx.handle
        B = X.shape[0]
        self.forward(X)
        self.loss.zero_()
        nl = len(self.W)
        check(L.fgb_mlp_mse_grad(h, self.out.numel(), self.out.data_ptr(), T.data_ptr(), 1.0 / B,
                                 self.dz[-1].data_ptr(), self.loss.data_ptr()), h)
        for i in reversed(range(nl)):
            fout, fin = self.W[i].shape
            dz = self.dz[i]
            if i < nl - 1:  # ReLU backward from the layer's output
                check(L.fgb_mlp_relu_grad(h, dz.numel(), self.dact[i].data_ptr(), self.act[i].data_ptr(),
                                          dz.data_ptr()), h)
            x = self._x if i == 0 else self.act[i - 1]
            check(L.fgb_mlp_colsum(h, B, fout, dz.data_ptr(), fout, self.gb[i].data_ptr()), h)
            # dW = dz^T x : (fout x B) (fin x B)^T
            check(L.fgb_mlp_transpose_bf16(h, B, fout, dz.data_ptr(), fout, self.dzT[i].data_ptr(), B), h)
            check(L.fgb_mlp_transpose_bf16(h, B, fin, x.data_ptr(), fin, self.xT[i].data_ptr(), B), h)
            self._gemm(fout, fin, B, self.dzT[i], B, self.xT[i], B, self.gW[i], fin, True)
            if i > 0:  # dx = dz W : (B x fout) (fin x fout)^T
                self._gemm(B, fin, fout, dz, fout, self.WTb[i], fout, self.dact[i - 1], fin, False,
                           split_k=self._split(B, fin, fout))
        self.step_no += 1
        for i in range(nl):
            W = self.W[i]
            check(L.fgb_mlp_adam(h, W.numel(), W.data_ptr(), self.gW[i].data_ptr(), self.mW[i].data_ptr(),
                                 self.vW[i].data_ptr(), None, lr, b1, b2, eps, self.step_no), h)
            check(L.fgb_mlp_adam(h, self.b[i].numel(), self.b[i].data_ptr(), self.gb[i].data_ptr(),
                                 self.mb[i].data_ptr(), self.vb[i].data_ptr(), None, lr, b1, b2, eps, self.step_no), h)
            self._refresh(i)
        return float(self.loss.item())

    def predict(self, X):
        """Predictions for any number of rows (padded to the batch size)."""
        torch = self.torch
        n = X.shape[0]
        out = torch.empty((n, self.dims[-1]), device="cuda", dtype=torch.float32)
        for s in range(0, n, self.batch):
            xb = X[s:s + self.batch]
            if xb.shape[0] < self.batch:
                pad = torch.zeros((self.batch - xb.shape[0], xb.shape[1]), device="cuda", dtype=X.dtype)
                xb = torch.cat([xb, pad])
            y = self.forward(xb.contiguous())
            out[s:s + self.batch] = y[:min(self.batch, n - s)]
        return out


def to_inputs(torch, Ks):
    return torch.from_numpy(np.ascontiguousarray(Ks.reshape(len(Ks), -1))).cuda().to(torch.bfloat16)


def run_warm(problem, Ks_dev, values_dev, its, ctx=None, ctas_per_sm=0):
    """palm4msa2 seeded with predicted factor values, all on the device: the
    batched driver writes the values (values_dev, (instances, 4096) FP32 CUDA
    tensor, divided by VALUE_SCALE) into the butterfly supports and starts
    each instance from lambda = <K, S> / ||S||^2 of its seeded factors.
    Ks_dev: column-major CUDA tensors.  Returns the results."""
    probs = [(K, problem.cons) for K in Ks_dev]
    return fact.palm4msa_batched(probs, problem.params(max(1, its)), ctx=ctx, ctas_per_sm=ctas_per_sm,
                                 init_values=values_dev.contiguous(), values_scale=1.0 / VALUE_SCALE,
                                 lambda_from_init=True)
