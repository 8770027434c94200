"""GPU parity of the Faust x dense path through the C ABI against the oracle.

CSR chains are compared BIT FOR BIT (both sides use the same sequential fma
order per output entry).  BSR (BF16 operands, FP32 accumulation) is compared
against the FP64 oracle with a stated tolerance.
"""
import numpy as np
import pytest

from faust_gb300 import synth

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def _colmajor_cuda(X):
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(X.T)).cuda().t()


def _to_np(Yt):
    return Yt.t().contiguous().cpu().numpy().T


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_csr_chain_config1_bitexact(fgb, oracle, mode):
    """5 CSR 1024x1024 (10 nnz/row) FP64 factors x X 1024x512."""
    rng = np.random.default_rng(11)
    facs = [synth.random_csr(1024, 1024, 10, rng) for _ in range(5)]
    X = synth.dense_colmajor(1024, 512, rng)
    ref = oracle.chain_mul(facs, X)
    F = fgb.Faust(facs)
    Y = _to_np(F.matmul_device(_colmajor_cuda(X), mode=mode))
    assert np.array_equal(Y, ref)
    rel = np.linalg.norm(Y - ref) / np.linalg.norm(ref)
    assert rel <= 1e-12


def test_csr_chain_host_entry_point(fgb, oracle):
    rng = np.random.default_rng(12)
    facs = [synth.random_csr(300, 200, 7, rng), synth.random_csr(200, 450, 3, rng), synth.random_csr(450, 450, 9, rng)]
    X = synth.dense_colmajor(450, 33, rng)
    F = fgb.Faust(facs)
    Y = F @ X
    assert np.array_equal(Y, oracle.chain_mul(facs, X))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("ncols", [1, 3, 8, 129])
def test_csr_chain_ragged(fgb, oracle, dtype, ncols):
    rng = np.random.default_rng(ncols)
    dims = [64, 100, 37, 250, 64]
    facs = []
    for a, b in zip(dims[:-1], dims[1:]):
        m = synth.random_csr(a, b, min(4, b), rng, dtype).tolil()
        m[a // 2, :] = 0  # an empty row
        facs.append(m.tocsr())
    X = synth.dense_colmajor(dims[-1], ncols, rng, dtype)
    F = fgb.Faust(facs, dtype=dtype)
    ref = oracle.chain_mul(facs, X)
    for mode in (0, 1):
        Y = _to_np(F.matmul_device(_colmajor_cuda(X), mode=mode))
        assert np.array_equal(Y, ref)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("ncols", [1, 5, 64])
def test_csr_chain_transposed(fgb, oracle, dtype, ncols):
    """F^T X (op 'T' and 'H') against the oracle chain of the transposed
    factors in reverse order, per-factor and fused paths, ragged shapes."""
    rng = np.random.default_rng(100 + ncols)
    dims = [64, 100, 37, 250, 64]
    facs = []
    for a, b in zip(dims[:-1], dims[1:]):
        m = synth.random_csr(a, b, min(4, b), rng, dtype).tolil()
        m[a // 2, :] = 0
        facs.append(m.tocsr())
    X = synth.dense_colmajor(dims[0], ncols, rng, dtype)
    F = fgb.Faust(facs, dtype=dtype)
    tfacs = []
    for f in reversed(facs):
        t = f.T.tocsr()
        t.sort_indices()
        tfacs.append(t)
    ref = oracle.chain_mul(tfacs, X)
    for op in ("T", "H"):
        for mode in (0, 1):
            Y = _to_np(F.matmul_op_device(op, _colmajor_cuda(X), mode=mode))
            assert Y.shape == (dims[-1], ncols)
            assert np.array_equal(Y, ref), (op, mode)
    Xn = synth.dense_colmajor(dims[-1], ncols, rng, dtype)
    assert np.array_equal(_to_np(F.matmul_op_device("N", _colmajor_cuda(Xn))), oracle.chain_mul(facs, Xn))


def test_csr_butterfly_fp32_bitexact(fgb, oracle):
    rng = np.random.default_rng(13)
    facs = synth.butterfly_faust_factors(10, rng, np.float32)
    X = synth.dense_colmajor(1024, 256, rng, np.float32)
    F = fgb.Faust(facs)
    ref = oracle.chain_mul(facs, X)
    for mode in (0, 1):
        assert np.array_equal(_to_np(F.matmul_device(_colmajor_cuda(X), mode=mode)), ref)


def _bfly_perm_factors(nf, order, rng, dtype):
    """Butterfly factors of size 2^nf applied with strides in a given order
    (repeats allowed): factor q has stride 2^order[q]."""
    import scipy.sparse as sp
    n = 1 << nf
    r = np.arange(n)
    out = []
    for b in order:
        h = 1 << b
        cols = np.stack([r & ~h, r | h], axis=1).ravel().astype(np.int32)
        vals = rng.standard_normal(2 * n).astype(dtype)
        out.append(sp.csr_matrix((vals, cols, np.arange(0, 2 * n + 1, 2, dtype=np.int32)), shape=(n, n)))
    return out


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("nf,ncols", [(4, 7), (7, 130), (10, 1000), (12, 301), (10, 1301), (11, 2500)])
def test_butterfly_kernel_bitexact(fgb, oracle, dtype, nf, ncols):
    """The butterfly chain kernel (mode 3) against the oracle's CSR chain,
    for F and F^T, ragged column counts."""
    rng = np.random.default_rng(nf * 100 + ncols)
    facs = synth.butterfly_faust_factors(nf, rng, dtype)
    F = fgb.Faust(facs, dtype=dtype)
    X = synth.dense_colmajor(1 << nf, ncols, rng, dtype)
    assert np.array_equal(_to_np(F.matmul_device(_colmajor_cuda(X), mode=3)), oracle.chain_mul(facs, X))
    assert np.array_equal(_to_np(F.matmul_device(_colmajor_cuda(X), mode=0)), oracle.chain_mul(facs, X))
    ref_t = oracle.chain_mul([f.T.tocsr() for f in facs[::-1]], X)
    assert np.array_equal(_to_np(F.matmul_op_device("T", _colmajor_cuda(X), mode=3)), ref_t)
    F.close()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_butterfly_kernel_shuffled_and_repeated_strides(fgb, oracle, dtype):
    """Strides in any order, repeated strides and chains whose length is not
    a multiple of the pass size."""
    rng = np.random.default_rng(3)
    for order in ([0, 5, 3, 3, 9, 1, 2, 2, 2, 8, 7], [9, 9], [4], [1, 0, 1, 0, 1]):
        facs = _bfly_perm_factors(10, order, rng, dtype)
        F = fgb.Faust(facs, dtype=dtype)
        X = synth.dense_colmajor(1024, 97, rng, dtype)
        assert np.array_equal(_to_np(F.matmul_device(_colmajor_cuda(X), mode=3)), oracle.chain_mul(facs, X)), order
        F.close()


@pytest.mark.parametrize("nf,order,ncols", [
    (10, [3, 0, 4, 1, 2, 7, 5, 9, 6, 8], 1000),     # shuffled strides
    (11, [0, 0, 2, 1, 4, 3, 5, 8, 6, 10, 7, 9], 37),  # a repeated stride, ragged columns
    (12, list(range(12)), 5),                          # fewer columns than one tile
    (13, list(range(13)), 129),                        # 8192 rows (128 KB tile rows of 16 bytes)
])
def test_butterfly_kernel_orders_and_sizes(fgb, oracle, nf, order, ncols):
    """FP32 butterfly chains in given application orders (order[0] applied
    first), against the oracle's CSR chain bit for bit."""
    rng = np.random.default_rng(nf * 7 + ncols)
    facs = _bfly_perm_factors(nf, order[::-1], rng, np.float32)
    F = fgb.Faust(facs, dtype=np.float32)
    X = synth.dense_colmajor(1 << nf, ncols, rng, np.float32)
    assert np.array_equal(_to_np(F.matmul_device(_colmajor_cuda(X), mode=3)), oracle.chain_mul(facs, X))
    F.close()


def test_bounded_wait_kernels_leave_no_timeout(fgb, oracle):
    """The radix butterfly kernel and the tcgen05 BSR kernel record an expired
    bounded wait in the context's error word; after ordinary products
    fgb_ctx_synchronize reports none, and the host-buffer product (which
    reads the word after its own synchronisation) returns the oracle's
    result."""
    rng = np.random.default_rng(91)
    facs = synth.butterfly_faust_factors(10, rng, np.float32)
    F = fgb.Faust(facs, dtype=np.float32)
    X = synth.dense_colmajor(1024, 96, rng, np.float32)
    Y = F.matmul_device(_colmajor_cuda(X), mode=3)
    F.ctx.synchronize()
    assert np.array_equal(_to_np(Y), oracle.chain_mul(facs, X))
    assert np.array_equal(F @ np.asfortranarray(X), oracle.chain_mul(facs, X))
    bfacs, _ = _bsr_factors(fgb, 512, 2, rng)
    B = fgb.Faust(bfacs)
    torch = _torch()
    Xb = torch.randn((256, 512), device="cuda", dtype=torch.float32).to(torch.bfloat16).t()
    B.matmul_device(Xb)
    B.ctx.synchronize()
    F.close()
    B.close()


def test_butterfly_kernel_rejects_other_supports(fgb):
    rng = np.random.default_rng(4)
    facs = [synth.random_csr(64, 64, 2, rng) for _ in range(3)]
    F = fgb.Faust(facs)
    X = _colmajor_cuda(synth.dense_colmajor(64, 8, rng))
    with pytest.raises(Exception):
        F.matmul_device(X, mode=3)
    F.close()


def test_csr_butterfly_config3b_column_subset(fgb, oracle):
    """Full size (12 factors of 4096^2, X 4096 x 8192 FP32): columns of Y
    depend only on the same columns of X, so a column subset is checked
    bit for bit against the oracle."""
    torch = _torch()
    rng = np.random.default_rng(14)
    facs = synth.butterfly_faust_factors(12, rng, np.float32)
    F = fgb.Faust(facs)
    g = torch.Generator(device="cuda").manual_seed(0)
    Xt = torch.randn((8192, 4096), generator=g, device="cuda", dtype=torch.float32).t()
    Yt = F.matmul_device(Xt)
    cols = [0, 1, 7, 4095, 4096, 8191]
    Xs = Xt[:, cols].t().contiguous().cpu().numpy().T
    ref = oracle.chain_mul(facs, np.asfortranarray(Xs))
    got = Yt[:, cols].t().contiguous().cpu().numpy().T
    assert np.array_equal(got, ref)


def _bsr_factors(fgb, n, nfac, rng):
    sigma = 1.0 / np.sqrt(8 * 64)
    out, f32 = [], []
    for _ in range(nfac):
        bp, bc, blocks = synth.random_bsr(n, 64, 8 if n >= 512 else 2, rng, sigma)
        bits = synth.bf16_bits(blocks)
        out.append(fgb.BSRFactor(n, n, bp, bc, bits))
        f32.append((bp, bc, synth.bf16_to_f32(bits).reshape(blocks.shape)))
    return out, f32


def _oracle_bsr_chain(oracle, n, f32, X, round_bf16):
    Y = X.astype(np.float64)
    for bp, bc, blocks in reversed(f32):
        flat = np.ascontiguousarray(blocks.transpose(0, 2, 1).reshape(len(bc), -1), np.float64)
        Y = oracle.bsr_mul_f64(n, n, 64, 64, bp, bc, flat, Y)
        if round_bf16:
            Y = synth.bf16_to_f32(synth.bf16_bits(Y.astype(np.float32))).reshape(Y.shape).astype(np.float64)
    return Y


@pytest.mark.parametrize("n,ncols", [(512, 256), (1024, 384), (512, 512), (1024, 1536)])
def test_bsr_chain_bf16(fgb, oracle, n, ncols):
    """BF16 blocks, FP32 accumulation; tolerance: 1e-2 relative Frobenius
    against the FP64 oracle with BF16 rounding of each intermediate product
    (the kernel stores intermediates in BF16), which bounds FP32-vs-FP64
    accumulation plus one BF16 rounding per factor."""
    torch = _torch()
    rng = np.random.default_rng(n)
    facs, f32 = _bsr_factors(fgb, n, 3, rng)
    F = fgb.Faust(facs)
    X = rng.standard_normal((n, ncols)).astype(np.float32)
    Xb = synth.bf16_to_f32(synth.bf16_bits(X)).reshape(X.shape)
    Xt = torch.from_numpy(np.ascontiguousarray(Xb.T)).to(torch.bfloat16).cuda().t()
    Yt = F.matmul_device(Xt)
    Y = Yt.t().float().cpu().numpy().T.astype(np.float64)
    ref = _oracle_bsr_chain(oracle, n, f32, Xb, round_bf16=True)
    rel = np.linalg.norm(Y - ref) / np.linalg.norm(ref)
    assert rel < 1e-2, rel


def test_spectral_norm_matches_oracle(fgb, oracle):
    rng = np.random.default_rng(21)
    facs = [synth.random_csr(128, 128, 5, rng) for _ in range(4)]
    F = fgb.Faust(facs)
    got = F.norm(2, max_iter=200, threshold=1e-10)
    ref, _ = oracle.spectral_norm(facs, max_iter=200, thr=1e-10)
    assert got == ref


def _long_row_factors(rng, dims, dtype, lengths):
    """CSR factors with a few rows of the given lengths (beyond the 16-entry
    chunk, past 256 entries = one chunk group round of 8 warps, past 4096 =
    several rounds of 64 chunk groups) on top of 3 random entries per row."""
    import scipy.sparse as sp
    facs = []
    for q in range(len(dims) - 1):
        r, c = dims[q], dims[q + 1]
        A = synth.random_csr(r, c, 3, rng, dtype).tolil()
        rows = rng.choice(r, len(lengths), replace=False)
        for i, L in zip(rows, lengths):
            L = min(L, c)
            cols = rng.choice(c, L, replace=False)
            A[i, cols] = rng.standard_normal(L).astype(dtype)
        facs.append(sp.csr_matrix(A, dtype=dtype))
    return facs


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_long_rows_products_bitexact(fgb, oracle, dtype):
    """Products with rows (and columns, for F^T) of 17 to 6000 entries: the
    long-row kernels follow the chunked row order of the oracle bit for bit,
    for F X and F^T X and in both product modes."""
    rng = np.random.default_rng(31)
    dims = [6200, 6100, 6300]
    facs = _long_row_factors(rng, dims, dtype, [17, 33, 255, 257, 1000, 4096, 4097, 6000])
    F = fgb.Faust(facs, dtype=dtype)
    X = synth.dense_colmajor(dims[-1], 45, rng, dtype)
    ref = oracle.chain_mul(facs, X)
    for mode in (0, 1):
        assert np.array_equal(_to_np(F.matmul_device(_colmajor_cuda(X), mode=mode)), ref), mode
    Xt = synth.dense_colmajor(dims[0], 40, rng, dtype)
    ref_t = oracle.chain_mul([f.T.tocsr() for f in facs[::-1]], Xt)
    assert np.array_equal(_to_np(F.matmul_op_device("T", _colmajor_cuda(Xt))), ref_t)
    F.close()


@pytest.mark.parametrize("shape", [(1024, 1024), (700, 900)])
def test_spectral_norm_long_rows_matches_oracle(fgb, oracle, shape):
    """Rows and columns far longer than the 16-entry chunk of the power
    iteration's row order (up to 1000 entries: several rounds of 32 chunks),
    square and rectangular chains: the norm equals the oracle's bit for bit."""
    import scipy.sparse as sp
    rng = np.random.default_rng(22)
    m, n = shape
    facs = []
    for (r, c) in [(m, n), (n, n), (n, m)]:
        A = synth.random_csr(r, c, 3, rng).tolil()
        for i in rng.choice(r, 12, replace=False):
            cols = rng.choice(c, int(rng.integers(17, min(c, 1000))), replace=False)
            A[i, cols] = rng.standard_normal(len(cols))
        facs.append(sp.csr_matrix(A))
    F = fgb.Faust(facs)
    got = F.norm(2, max_iter=100, threshold=1e-12)
    ref, _ = oracle.spectral_norm(facs, max_iter=100, thr=1e-12)
    assert got == ref
    F.close()


def test_invalid_factor_is_rejected(fgb):
    import scipy.sparse as sp
    m = sp.csr_matrix(np.eye(4))
    m.indices[1] = 7  # column out of range
    with pytest.raises(Exception):
        fgb.Faust([m])


def test_bsr_tensor_core_matches_cuda_core_path(fgb, monkeypatch):
    """The tcgen05 kernel (whole 128-column tiles) against the CUDA-core
    kernel on the same BF16 inputs: both accumulate in FP32, in different
    orders, so agreement is within BF16 output rounding (2^-8 relative)."""
    torch = _torch()
    rng = np.random.default_rng(31)
    n = 1024
    facs, _ = _bsr_factors(fgb, n, 1, rng)
    F = fgb.Faust(facs)
    X = torch.randn((512, n), device="cuda", dtype=torch.float32).to(torch.bfloat16).t()
    Yt = F.matmul_device(X).float()
    monkeypatch.setenv("FGB_BSR_SIMT", "1")
    Ys = F.matmul_device(X).float()
    rel = (torch.linalg.norm(Yt - Ys) / torch.linalg.norm(Ys)).item()
    assert rel < 8e-3, rel


def test_bsr_ragged_columns_use_cuda_core_path(fgb, oracle):
    torch = _torch()
    rng = np.random.default_rng(32)
    n = 512
    facs, f32 = _bsr_factors(fgb, n, 2, rng)
    F = fgb.Faust(facs)
    X = rng.standard_normal((n, 77)).astype(np.float32)
    Xb = synth.bf16_to_f32(synth.bf16_bits(X)).reshape(X.shape)
    Yt = F.matmul_device(torch.from_numpy(np.ascontiguousarray(Xb.T)).to(torch.bfloat16).cuda().t())
    Y = Yt.t().float().cpu().numpy().T.astype(np.float64)
    ref = _oracle_bsr_chain(oracle, n, f32, Xb, round_bf16=True)
    assert np.linalg.norm(Y - ref) / np.linalg.norm(ref) < 1e-2
