"""CPU tests of the oracle (test infrastructure): products against dense
numpy, the top-k tie rule against an independent restatement of libstdc++'s
heap selection, projection properties from the reference's own tests
(wrapper/python/pyfaust/tests/test_FaustPy.py:1904-2030), the power-iteration
start vector, and palm4msa2 on the reference's config_compared_palm2 fixture.
"""
import ctypes
import os

import numpy as np
import pytest
import scipy.sparse as sp

from faust_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


# ---------------------------------------------------------------- heap select
def heap_select_set(v, k):
    """Positions kept by std::partial_sort(first, first+k, last, |a|>|b|):
    make_heap on the first k, then every later element strictly larger in
    magnitude than the heap top replaces it (pop_heap semantics).  Written
    from the documented algorithm (hole moved to a leaf along the preferred
    child, then sifted up), independent of the oracle's call into libstdc++."""
    mag = [abs(x) for x in v]
    comp = lambda a, b: mag[a] > mag[b]  # "a before b" = larger magnitude
    heap = list(range(k))

    def adjust(hole, length, value):
        top = hole
        child = hole
        while child < (length - 1) // 2:
            child = 2 * (child + 1)
            if comp(heap[child], heap[child - 1]):
                child -= 1
            heap[hole] = heap[child]
            hole = child
        if (length & 1) == 0 and child == (length - 2) // 2:
            child = 2 * (child + 1)
            heap[hole] = heap[child - 1]
            hole = child - 1
        parent = (hole - 1) // 2
        while hole > top and comp(heap[parent], value):
            heap[hole] = heap[parent]
            hole = parent
            parent = (hole - 1) // 2
        heap[hole] = value

    if k >= 2:
        parent = (k - 2) // 2
        while True:
            adjust(parent, k, heap[parent])
            if parent == 0:
                break
            parent -= 1
    for i in range(k, len(v)):
        if comp(i, heap[0]):
            adjust(0, k, i)
    return sorted(heap)


@pytest.mark.parametrize("seed", range(12))
def test_topk_matches_heap_restatement_on_ties(oracle, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(5, 400))
    k = int(rng.integers(1, n))
    levels = rng.integers(1, 5)
    v = rng.integers(-levels, levels + 1, size=n).astype(np.float64)
    got = sorted(oracle.topk(v, k).tolist())
    assert got == heap_select_set(v.tolist(), k)


def test_topk_all_ties_keeps_first_positions(oracle):
    v = np.ones(1000)
    assert sorted(oracle.topk(v, 4).tolist()) == [0, 1, 2, 3]
    assert sorted(oracle.topk(-v, 37).tolist()) == list(range(37))


def test_topk_tie_order_is_not_lowest_index(oracle):
    # A larger element after the heap is full evicts the tie that the heap
    # layout puts on top, which is not the last position.
    v = np.array([1, 1, 1, 1, 2, 1, 1, 2], np.float64)
    got = sorted(oracle.topk(v, 4).tolist())
    assert got == heap_select_set(v.tolist(), 4)
    assert 4 in got and 7 in got
    assert got != [0, 1, 4, 7]


def test_topk_distinct_values_are_the_k_largest(oracle):
    rng = np.random.default_rng(5)
    v = rng.standard_normal(10000)
    k = 321
    got = set(oracle.topk(v, k).tolist())
    assert got == set(np.argsort(-np.abs(v))[:k].tolist())


# ---------------------------------------------------------------- products
@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-13), (np.float32, 1e-5)])
def test_chain_product_matches_dense(oracle, dtype, tol):
    rng = np.random.default_rng(1)
    facs = [synth.random_csr(96, 96, 5, rng, dtype) for _ in range(4)]
    X = synth.dense_colmajor(96, 17, rng, dtype)
    Y = oracle.chain_mul(facs, X)
    ref = X.astype(np.float64)
    for f in reversed(facs):
        ref = f.toarray().astype(np.float64) @ ref
    assert np.linalg.norm(Y - ref) / np.linalg.norm(ref) < tol


def test_bsr_product_matches_dense(oracle):
    rng = np.random.default_rng(2)
    n, bs = 256, 64
    bp, bc, blocks = synth.random_bsr(n, bs, 2, rng, 0.1)
    X = rng.standard_normal((n, 7))
    # column-major per block
    flat = np.ascontiguousarray(blocks.transpose(0, 2, 1).reshape(len(bc), -1), np.float64)
    Y = oracle.bsr_mul_f64(n, n, bs, bs, bp, bc, flat, X)
    dense = np.zeros((n, n))
    for br in range(n // bs):
        for p in range(bp[br], bp[br + 1]):
            dense[br * bs:(br + 1) * bs, bc[p] * bs:(bc[p] + 1) * bs] = blocks[p]
    assert np.allclose(Y, dense @ X, rtol=1e-12, atol=1e-12)


def test_butterfly_support_structure():
    sups = synth.butterfly_supports(5)
    assert len(sups) == 5
    for s in sups:
        assert s.shape == (32, 32)
        assert np.all(np.diff(s.indptr) == 2)
    # the product of the supports is dense (every entry reachable)
    P = sups[0].toarray()
    for s in sups[1:]:
        P = P @ s.toarray()
    assert np.all(P > 0)


# ---------------------------------------------------------------- projections
def _nnz_cols(M):
    return (M != 0).sum(axis=0)


def _nnz_rows(M):
    return (M != 0).sum(axis=1)


def test_prox_properties(oracle):
    rng = np.random.default_rng(3)
    M = rng.standard_normal((40, 30))
    k = 5
    sp_ = oracle.prox(oracle.SP, M, k=k)
    assert np.count_nonzero(sp_) <= k and abs(np.linalg.norm(sp_) - 1) < 1e-12
    spcol = oracle.prox(oracle.SPCOL, M, k=k)
    assert _nnz_cols(spcol).max() <= k and abs(np.linalg.norm(spcol) - 1) < 1e-12
    splin = oracle.prox(oracle.SPLIN, M, k=k)
    assert _nnz_rows(splin).max() <= k and abs(np.linalg.norm(splin) - 1) < 1e-12
    slc = oracle.prox(oracle.SPLINCOL, M, k=k)
    # every entry kept by spcol or splin, union semantics
    a = oracle.prox(oracle.SPCOL, M, k=k, normalized=False)
    b = oracle.prox(oracle.SPLIN, M, k=k, normalized=False)
    assert np.array_equal(slc != 0, (a != 0) | (b != 0))
    nc = oracle.prox(oracle.NORMCOL, M, s=2.0, normalized=False)
    assert np.allclose(np.linalg.norm(nc, axis=0), 2.0)
    nl = oracle.prox(oracle.NORMLIN, M, s=3.0, normalized=False)
    assert np.allclose(np.linalg.norm(nl, axis=1), 3.0)
    supp = (rng.random((40, 30)) < 0.2).astype(np.float64)
    sup = oracle.prox(oracle.SUPP, M, supp=supp)
    assert np.all(sup[supp == 0] == 0) and abs(np.linalg.norm(sup) - 1) < 1e-12
    pos = oracle.prox(oracle.SP_POS, M, k=k)
    assert np.all(pos >= 0)


def test_prox_sp_keeps_everything_when_k_large(oracle):
    M = np.arange(12, dtype=np.float64).reshape(3, 4) - 5
    out = oracle.prox(oracle.SP, M, k=12, normalized=False)
    assert np.array_equal(out, M)


def test_prox_k_bounds(oracle):
    """The k bounds of faust_prox.hpp: k <= 0 gives zeros (:78-79, :119-120,
    :153-154); sp keeps everything unless k < rows*cols (:82), spcol unless
    k < rows (:123), splin unless k < cols (:157)."""
    rng = np.random.default_rng(11)
    M = rng.standard_normal((7, 5))
    for kind in (oracle.SP, oracle.SPCOL, oracle.SPLIN):
        assert not np.any(oracle.prox(kind, M, k=0, normalized=False))
    assert np.array_equal(oracle.prox(oracle.SP, M, k=35, normalized=False), M)
    assert np.array_equal(oracle.prox(oracle.SPCOL, M, k=7, normalized=False), M)
    assert np.array_equal(oracle.prox(oracle.SPLIN, M, k=5, normalized=False), M)
    assert np.count_nonzero(oracle.prox(oracle.SP, M, k=34, normalized=False)) == 34
    assert _nnz_cols(oracle.prox(oracle.SPCOL, M, k=6, normalized=False)).max() == 6
    assert _nnz_rows(oracle.prox(oracle.SPLIN, M, k=4, normalized=False)).max() == 4


def test_prox_normcol_zero_s_and_zero_columns(oracle):
    """prox_normcol (faust_prox.hpp:204-246): s == 0 gives zeros; a zero
    column stays zero (its scale factor stays 0); the others get norm s."""
    rng = np.random.default_rng(12)
    M = rng.standard_normal((6, 4))
    assert not np.any(oracle.prox(oracle.NORMCOL, M, s=0.0, normalized=False))
    M[:, 2] = 0
    out = oracle.prox(oracle.NORMCOL, M, s=1.5, normalized=False)
    assert not np.any(out[:, 2])
    assert np.allclose(np.linalg.norm(out[:, [0, 1, 3]], axis=0), 1.5)


def test_prox_pos_clamps_before_selection(oracle):
    """pre_prox_pos (faust_prox.hpp:307-320) runs first: with every entry
    negative the projection keeps only zeros, which the normalisation
    rejects."""
    M = -np.abs(np.random.default_rng(13).standard_normal((5, 5))) - 0.1
    assert not np.any(oracle.prox(oracle.SP, M, k=4, normalized=False, pos=True))
    with pytest.raises(RuntimeError):
        oracle.prox(oracle.SP, M, k=4, normalized=True, pos=True)


def test_prox_normcol_negative_s_is_an_error(oracle):
    with pytest.raises(RuntimeError):
        oracle.prox(oracle.NORMCOL, np.ones((3, 3)), s=-1.0)


def test_prox_zero_norm_is_an_error(oracle):
    with pytest.raises(RuntimeError):
        oracle.prox(oracle.SP, np.zeros((4, 4)), k=3)


# ---------------------------------------------------------------- power iteration
def test_power_iteration_start_vector_is_srand_418(oracle):
    libc = ctypes.CDLL(None)
    libc.srand(418)
    r = np.array([libc.rand() for _ in range(64)], np.float64)
    expect = -1.0 + (2.0 * r) / 2147483647.0
    assert np.array_equal(oracle.rand_start(64), expect)


def test_spectral_norm_matches_svd(oracle):
    rng = np.random.default_rng(4)
    facs = [synth.random_csr(64, 64, 6, rng) for _ in range(3)]
    nrm, flag = oracle.spectral_norm(facs, max_iter=1000, thr=1e-14)
    P = facs[0].toarray() @ facs[1].toarray() @ facs[2].toarray()
    assert flag > 0
    assert abs(nrm - np.linalg.norm(P, 2)) / np.linalg.norm(P, 2) < 1e-6


# ---------------------------------------------------------------- palm4msa2
def test_palm_hadamard_small(oracle):
    n = 32
    H = synth.hadamard(n) / np.sqrt(n)
    cons = [dict(kind=oracle.SP, k=2 * n, rows=n, cols=n) for _ in range(5)]
    facts, lam, tr = oracle.palm4msa2(H, cons, 30, norm2_threshold=1e-8)
    for f in facts:
        assert np.count_nonzero(f) <= 2 * n
        assert abs(np.linalg.norm(f) - 1) < 1e-12
    err = oracle.rel_err(H, facts, lam)
    assert 0 <= err < 1.0
    assert np.all(tr["lambdas"] > 0)


def test_palm_fixture_config_compared_palm2(oracle):
    """palm4msa_2020.cpp.in:81-121 settings on its own fixture data."""
    data = np.load(os.path.join(GOLDEN, "config_compared_palm2_data.npy"))
    cons = [dict(kind=oracle.SPLIN, k=5, rows=500, cols=32),
            dict(kind=oracle.NORMCOL, s=1.0, rows=32, cols=32)]
    facts, lam, _ = oracle.palm4msa2(data, cons, 200, packing_RL=False, norm2_threshold=1e-15,
                                     norm2_max_iter=1000)
    assert _nnz_rows(facts[0]).max() <= 5
    err = oracle.rel_err(data, facts, lam)
    assert 0 < err < 0.8
    # exact reproducibility of the restatement
    facts2, lam2, _ = oracle.palm4msa2(data, cons, 200, packing_RL=False, norm2_threshold=1e-15,
                                       norm2_max_iter=1000)
    assert lam2 == lam and all(np.array_equal(a, b) for a, b in zip(facts, facts2))


# ---------------------------------------------------------------- hierarchical
def _wht_cons(oracle, n):
    d = 2 ** n
    fc = [dict(kind=oracle.SPLINCOL, k=2, rows=d, cols=d) for _ in range(n - 1)]
    rc = [dict(kind=oracle.SPLINCOL, k=d // 2 ** (i + 1), rows=d, cols=d) for i in range(n - 1)]
    return fc, rc


@pytest.mark.parametrize("n", [4, 5])
def test_hierarchical_wht_factorizes_hadamard(oracle, n):
    """pyfaust's ParamsHierarchicalWHT (factparams.py:1605-1638: splincol k=2
    factors, residuals splincol d/2^(i+1), 30 iterations each, R2L, no
    packing): the Hadamard matrix comes out exactly as n butterfly-like
    factors with 2 entries per row and column."""
    d = 2 ** n
    A = synth.hadamard(d).astype(np.float64)
    fc, rc = _wht_cons(oracle, n)
    S, lam = oracle.hierarchical(A, fc, rc, 30, 30, is_update_way_R2L=True, packing_RL=False)
    assert len(S) == n
    for f in S:
        assert _nnz_rows(f).max() <= 2 and np.count_nonzero(f) == 2 * d
    assert oracle.rel_err(A, S, lam) < 1e-12


def _hadamard32_config(oracle):
    """The hierarchical configuration of the reference's Hadamard tests
    (misc/config_file/mat/config_HADAMARD_32.mat, extracted by
    tests/golden/make_golden.py) as oracle constraint dicts."""
    import json
    with open(os.path.join(GOLDEN, "config_HADAMARD_32_params.json")) as f:
        p = json.load(f)
    kinds = {"sp": oracle.SP, "spcol": oracle.SPCOL, "splin": oracle.SPLIN, "splincol": oracle.SPLINCOL}
    fc, rc = [[dict(kind=kinds[c[0]], k=c[1], rows=c[2], cols=c[3]) for c in row] for row in p["cons"]]
    return p, fc, rc


def test_hierarchical_hadamard32_reference_config(oracle):
    """config_HADAMARD_32.mat equals pyfaust's WHT parameters for n = 5, and
    with it (update_way 1 = right-to-left, faust_init_from_matio_params.hpp:142-148)
    the 32 x 32 Hadamard matrix factorizes exactly into nfacts factors."""
    p, fc, rc = _hadamard32_config(oracle)
    assert (p["nfacts"], p["nrow"], p["ncol"]) == (5, 32, 32)
    assert (fc, rc) == _wht_cons(oracle, 5)
    A = synth.hadamard(p["nrow"]).astype(np.float64)
    S, lam = oracle.hierarchical(A, fc, rc, p["niter1"], p["niter2"],
                                 is_update_way_R2L=bool(p["update_way"]), packing_RL=False)
    assert len(S) == p["nfacts"]
    assert all(np.count_nonzero(f) == 2 * 32 for f in S)
    assert oracle.rel_err(A, S, lam) < 1e-12


def test_hierarchical_left_side_shapes(oracle):
    """is_fact_side_left: the residual is split on the left; factor shapes
    and the global constraint order follow faust_hierarchical.hpp:101-121."""
    rng = np.random.default_rng(5)
    A = rng.standard_normal((40, 24))
    fc = [dict(kind=oracle.SP, k=60, rows=24, cols=24), dict(kind=oracle.SP, k=60, rows=32, cols=24)]
    rc = [dict(kind=oracle.SP, k=400, rows=40, cols=24), dict(kind=oracle.SP, k=300, rows=40, cols=32)]
    S, lam = oracle.hierarchical(A, fc, rc, 10, 10, is_fact_side_left=True)
    assert [f.shape for f in S] == [(40, 32), (32, 24), (24, 24)]
    assert np.count_nonzero(S[0]) <= 300 and np.count_nonzero(S[1]) <= 60 and np.count_nonzero(S[2]) <= 60
    assert 0 < oracle.rel_err(A, S, lam) < 1


def _fma(a, b, c):
    from fractions import Fraction
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _row_value(vals, xs, chunk=16):
    """Independent restatement of the canonical row order: 16-entry chunks
    of sequential fma from +0, partials added by the recursive-halving tree."""
    parts = []
    for m in range(0, len(vals), chunk):
        acc = 0.0
        for v, x in zip(vals[m:m + chunk], xs[m:m + chunk]):
            acc = _fma(v, x, acc)
        parts.append(acc)
    s = 1
    while s < len(parts):
        for l in range(0, len(parts) - s, 2 * s):
            parts[l] = parts[l] + parts[l + s]
        s *= 2
    return parts[0] if parts else 0.0


def test_row_order_chunked_tree(oracle):
    """Sparse-row products (chain products and the power iteration's) follow
    the chunked tree order: rows of 1..200 entries, including lengths around
    the 16-entry chunk and the powers of two of the tree."""
    import scipy.sparse as sps
    rng = np.random.default_rng(17)
    lens = [1, 2, 15, 16, 17, 31, 32, 33, 48, 63, 64, 65, 100, 127, 128, 129, 200]
    ncol = 256
    rows, cols, vals = [], [], []
    for i, L in enumerate(lens):
        c = np.sort(rng.choice(ncol, L, replace=False))
        rows += [i] * L
        cols += list(c)
        vals += list(rng.standard_normal(L) * 10.0 ** rng.integers(-3, 4, L))
    S = sps.csr_matrix((vals, (rows, cols)), shape=(len(lens), ncol))
    S.sort_indices()
    x = rng.standard_normal((ncol, 1))
    got = oracle.pi_spmv(S, x[:, 0])
    seq = oracle.chain_mul([S], x)[:, 0]
    for i in range(len(lens)):
        p0, p1 = S.indptr[i], S.indptr[i + 1]
        vals, xs = list(S.data[p0:p1]), [x[c, 0] for c in S.indices[p0:p1]]
        assert got[i] == _row_value(vals, xs), lens[i]
        assert seq[i] == got[i], lens[i]


def test_palm_resumed_in_segments_equals_one_run(oracle):
    """The CPU baseline of the PALM workload times one run as consecutive
    segments, each resuming from the factors and lambda the previous one
    ended with: the result equals the uninterrupted run bit for bit."""
    import numpy as np
    from faust_gb300 import synth
    n = 64
    H = synth.hadamard(n) / 8.0
    cons = [dict(kind=oracle.SP, k=2 * n, s=1.0, normalized=True, pos=False, rows=n, cols=n, supp=None)
            for _ in range(6)]
    f1, l1, _ = oracle.palm4msa2(H, cons, 30, norm2_threshold=1e-8)
    facts, lam = None, 1.0
    for _ in range(3):
        facts, lam, _ = oracle.palm4msa2(H, cons, 10, norm2_threshold=1e-8, init_facts=facts, init_lambda=lam)
    assert lam == l1
    assert all(np.array_equal(a, b) for a, b in zip(f1, facts))
