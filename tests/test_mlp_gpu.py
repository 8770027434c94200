"""The warm-start MLP's kernels: the tcgen05 BF16 GEMM against a PyTorch FP32
reference of the same op, the backward pass against an FP64 NumPy
restatement (gradient check), and the gain of the learned warm start over
plain initialisation on a small training set."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gemm(torch, A, B, c_f32=True, bias=None, relu=False, split_k=1):
    import faust_gb300 as fg
    from faust_gb300 import _ffi
    ctx = fg.default_context()
    M, K = A.shape
    N = B.shape[0]
    C = torch.empty((M, N), device="cuda", dtype=torch.float32 if c_f32 else torch.bfloat16)
    work = torch.empty(M * N, device="cuda", dtype=torch.float32)
    _ffi.check(_ffi.lib().fgb_gemm_bf16(ctx.handle, M, N, K, A.data_ptr(), K, B.data_ptr(), K, C.data_ptr(), N,
                                        _ffi.F32 if c_f32 else _ffi.BF16,
                                        bias.data_ptr() if bias is not None else None, int(relu), split_k,
                                        work.data_ptr()), ctx.handle)
    torch.cuda.synchronize()
    return C


@pytest.mark.parametrize("M,N,K,split", [(128, 128, 64, 1), (256, 384, 192, 1), (256, 1024, 4096, 8),
                                         (512, 256, 1024, 3)])
def test_gemm_bf16_matches_torch_fp32(M, N, K, split):
    """Tolerance: FP32 accumulation of BF16 products vs torch FP32 matmul of
    the same BF16 values, relative Frobenius 1e-5 (FP32 output)."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn((M, K), generator=g, device="cuda").to(torch.bfloat16)
    B = torch.randn((N, K), generator=g, device="cuda").to(torch.bfloat16)
    C = _gemm(torch, A, B, split_k=split)
    ref = A.float() @ B.float().t()
    rel = (torch.linalg.norm(C - ref) / torch.linalg.norm(ref)).item()
    assert rel < 1e-5, rel


def test_gemm_bias_relu_bf16_output():
    import torch
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn((256, 512), generator=g, device="cuda").to(torch.bfloat16)
    B = torch.randn((256, 512), generator=g, device="cuda").to(torch.bfloat16)
    bias = torch.randn(256, generator=g, device="cuda")
    for split in (1, 4):
        C = _gemm(torch, A, B, c_f32=False, bias=bias, relu=True, split_k=split).float()
        ref = torch.relu(A.float() @ B.float().t() + bias)
        rel = (torch.linalg.norm(C - ref) / torch.linalg.norm(ref)).item()
        assert rel < 8e-3, rel  # one BF16 rounding of the output


def test_mlp_gradients_match_fp64_restatement():
    """Gradient check: one backward pass of a small MLP (256-128-128-128,
    batch 128) against NumPy FP64 on the same BF16 weights and inputs.
    Tolerance 3e-2 relative per weight matrix (BF16 activations and
    gradients between layers)."""
    import torch
    from faust_gb300.warmstart import MLP
    net = MLP(dims=(256, 128, 128, 128), batch=128, seed=1)
    g = torch.Generator(device="cuda").manual_seed(2)
    X = torch.randn((128, 256), generator=g, device="cuda").to(torch.bfloat16)
    T = torch.randn((128, 128), generator=g, device="cuda")
    Ws = [W.detach().to(torch.bfloat16).double().cpu().numpy() for W in net.W]
    bs = [b.double().cpu().numpy() for b in net.b]
    net.train_step(X, T, lr=0.0)  # lr 0: gradients only
    # FP64 restatement
    x = X.double().cpu().numpy()
    hs, zs = [x], []
    for i, (W, b) in enumerate(zip(Ws, bs)):
        z = hs[-1] @ W.T + b
        zs.append(z)
        hs.append(np.maximum(z, 0) if i < len(Ws) - 1 else z)
    t = T.double().cpu().numpy()
    d = (hs[-1] - t) / x.shape[0]
    grads = [None] * len(Ws)
    for i in reversed(range(len(Ws))):
        if i < len(Ws) - 1:
            d = d * (zs[i] > 0)
        grads[i] = d.T @ hs[i]
        d = d @ Ws[i]
    for i in range(len(Ws)):
        got = net.gW[i].double().cpu().numpy()
        rel = np.linalg.norm(got - grads[i]) / np.linalg.norm(grads[i])
        assert rel < 3e-2, (i, rel)


def test_learned_warm_start_gains_over_plain_init():
    """Small version of the warm-start workload: train on plain palm4msa2
    factorizations of 384 kernel matrices, then compare, on 32 held-out
    matrices, palm4msa2 after a few iterations from the predicted factors with
    the same number of iterations from the plain initialisation."""
    import torch
    from faust_gb300 import warmstart as ws
    rng = np.random.default_rng(0)
    prob = ws.ButterflyProblem()
    Ktr, _ = ws.kernel_matrices(384, rng)
    Kte, _ = ws.kernel_matrices(32, rng)
    res, _ = ws.run_plain(prob, Ktr, 60)
    Y = torch.from_numpy(np.stack([prob.factor_values(r.faust) for r in res])).cuda()
    for r in res:
        r.faust.close()
    X = ws.to_inputs(torch, Ktr)
    net = ws.MLP(batch=128, seed=3)
    for epoch in range(40):
        perm = torch.randperm(len(Ktr), device="cuda")
        for s in range(0, len(Ktr), 128):
            idx = perm[s:s + 128]
            net.train_step(X[idx].contiguous(), Y[idx].contiguous(), lr=3e-4)
    pred = net.predict(ws.to_inputs(torch, Kte))
    Kd = ws.to_device(Kte)
    its = 5
    plain, _ = ws.run_plain(prob, Kd, its)
    warm = ws.run_warm(prob, Kd, pred, its)
    e_plain = ws.rel_errors(plain, Kd)
    e_warm = ws.rel_errors(warm, Kd)
    # each held-out matrix against its own plain run
    assert np.median(e_warm) < np.median(e_plain), (np.median(e_warm), np.median(e_plain))
    assert np.mean(e_warm < e_plain) >= 0.75, (e_warm, e_plain)
