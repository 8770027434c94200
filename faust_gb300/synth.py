"""Seeded synthetic inputs for the Faust x dense and PALM4MSA workloads.

No public data set is involved: every input is generated here from a seed
with the shapes and value distributions of the benchmark configurations.
"""
import numpy as np
import scipy.sparse as sp


def random_csr(n, m, nnz_per_row, rng, dtype=np.float64):
    """n x m CSR with exactly nnz_per_row distinct uniformly random columns per
    row (sorted), values N(0, 1)."""
    k = nnz_per_row
    # distinct columns per row: argsort of uniform keys, first k
    cols = np.empty((n, k), np.int32)
    chunk = max(1, (1 << 22) // max(m, 1))
    for r0 in range(0, n, chunk):
        r1 = min(n, r0 + chunk)
        keys = rng.random((r1 - r0, m))
        cols[r0:r1] = np.argpartition(keys, k - 1, axis=1)[:, :k]
    cols.sort(axis=1)
    vals = rng.standard_normal((n, k)).astype(dtype)
    indptr = np.arange(0, n * k + 1, k, dtype=np.int32)
    return sp.csr_matrix((vals.ravel(), cols.ravel(), indptr), shape=(n, m))


def hadamard(n, dtype=np.float64):
    """Sylvester Hadamard matrix of order n (a power of 2), unscaled."""
    H = np.ones((1, 1), dtype)
    while H.shape[0] < n:
        H = np.block([[H, H], [H, -H]])
    return H


def butterfly_supports(nfactors, dtype=np.float64):
    """Supports of butterfly_support(nfactors)
    (src/algorithm/factorization/faust_butterfly.hpp:459-492): factor i is
    kron(I_{2^i}, kron(ones(2,2), I_{2^(n-i-1)})), two entries per row: row r
    of a block of size b = 2^(n-i) touches columns (r mod b/2) and
    (r mod b/2) + b/2 of that block."""
    n = 1 << nfactors
    out = []
    r = np.arange(n)
    for i in range(nfactors):
        b = 1 << (nfactors - i)
        h = b // 2
        start = (r // b) * b
        c0 = start + (r % h)
        cols = np.stack([c0, c0 + h], axis=1).astype(np.int32)
        indptr = np.arange(0, 2 * n + 1, 2, dtype=np.int32)
        out.append(sp.csr_matrix((np.ones(2 * n, dtype), cols.ravel(), indptr), shape=(n, n)))
    return out


def butterfly_faust_factors(nfactors, rng, dtype=np.float32):
    """Butterfly-support CSR factors with N(0,1) values."""
    facs = []
    for s in butterfly_supports(nfactors, dtype):
        s = s.copy()
        s.data = rng.standard_normal(s.nnz).astype(dtype)
        facs.append(s)
    return facs


def dense_colmajor(rows, cols, rng, dtype=np.float64):
    return np.asfortranarray(rng.standard_normal((rows, cols)).astype(dtype))


def bf16_bits(x):
    """float32 array -> bfloat16 bit patterns (round to nearest even)."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    rounded = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return rounded.astype(np.uint16)


def bf16_to_f32(bits):
    return (np.asarray(bits, np.uint16).astype(np.uint32) << 16).view(np.float32)


def random_bsr(n, bs, blocks_per_row, rng, sigma):
    """n x n BSR, bs x bs blocks, blocks_per_row distinct uniform block columns
    per block row, block values N(0, sigma) (sigma a standard deviation).
    Returns (browptr, bcolind, blocks float32 (nblk, bs, bs) C-ordered [r][c])."""
    nb = n // bs
    k = blocks_per_row
    keys = rng.random((nb, nb))
    bcol = np.argpartition(keys, k - 1, axis=1)[:, :k]
    bcol.sort(axis=1)
    browptr = np.arange(0, nb * k + 1, k, dtype=np.int32)
    blocks = (rng.standard_normal((nb * k, bs, bs)) * sigma).astype(np.float32)
    return browptr, bcol.ravel().astype(np.int32), blocks


def batched_palm_targets(rng, count=512):
    """Targets of the batched palm4msa2 workload: `count` instances of size
    n = round16(exp(U[ln 64, ln 512])), each P1 P2 P3 + 1e-3 N(0,1) with every
    Pi an n x n matrix of 4 distinct random columns per row with N(0,1)
    values; FP32.  Returns (sizes, matrices)."""
    ns = (np.round(np.exp(rng.uniform(np.log(64), np.log(512), size=count)) / 16) * 16).astype(int)
    ns = np.clip(ns, 64, 512)
    mats = []
    for n in ns:
        P = [random_csr(int(n), int(n), 4, rng, np.float64) for _ in range(3)]
        A = (P[0] @ (P[1] @ P[2].toarray())) + 1e-3 * rng.standard_normal((n, n))
        mats.append(np.asarray(A, np.float32))
    return ns, mats


def gaussian_kernel(npts, sigma, rng, dim=3):
    """K_ij = exp(-||x_i - x_j||^2 / (2 sigma^2)) over npts points uniform in
    [0, 1]^dim, FP32."""
    x = rng.random((npts, dim))
    d2 = ((x[:, None, :] - x[None, :, :]) ** 2).sum(-1)
    return np.exp(-d2 / (2.0 * sigma * sigma)).astype(np.float32)
