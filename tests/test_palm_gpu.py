"""GPU parity of the projections and of palm4msa2 against the oracle.

Supports (integer/index work) are compared bit for bit; values too, since
GPU and oracle follow the same floating-point operation order.  The top-k
inputs include heavy ties, where the heap order of std::partial_sort
decides which entries stay.
"""
import os

import numpy as np
import pytest

from faust_gb300 import fact, synth

pytestmark = pytest.mark.gpu


def _cuda_colmajor(M):
    import torch
    return torch.from_numpy(np.ascontiguousarray(M.T)).cuda().t()


def _host(Mt):
    return Mt.t().contiguous().cpu().numpy().T


def _gpu_prox(M, c):
    Mt = _cuda_colmajor(M)
    fact.prox(Mt, c)
    return _host(Mt)


def _tie_matrix(rng, rows, cols, levels, dtype=np.float64):
    return rng.integers(-levels, levels + 1, size=(rows, cols)).astype(dtype) / 8.0


@pytest.mark.parametrize("seed", range(8))
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_prox_sp_ties_bitexact(oracle, seed, dtype):
    rng = np.random.default_rng(seed)
    rows, cols = [(64, 64), (100, 37), (257, 129), (1024, 64)][seed % 4]
    M = _tie_matrix(rng, rows, cols, 1 + seed % 4, dtype)
    k = int(rng.integers(1, rows * cols))
    c = fact.ConstraintInt("sp", rows, cols, k, normalized=bool(seed % 2), pos=bool(seed % 3 == 0))
    got = _gpu_prox(M, c)
    ref = oracle.prox(oracle.SP, M, k=k, normalized=c.normalized, pos=c.pos)
    assert np.array_equal(got, ref)


def test_prox_sp_heap_order_case(oracle):
    """Ties at the threshold with larger entries after the k-th tie: the
    heap layout decides (the replay path)."""
    rng = np.random.default_rng(99)
    found = 0
    for trial in range(40):
        n = 200
        v = np.where(rng.random(n) < 0.5, 1.0, rng.choice([0.5, 2.0, 3.0], size=n))
        k = int(rng.integers(5, 60))
        M = v.reshape(20, 10)
        got = _gpu_prox(M, fact.ConstraintInt("sp", 20, 10, k, normalized=False))
        ref = oracle.prox(oracle.SP, M, k=k, normalized=False)
        assert np.array_equal(got, ref), trial
        found += 1
    assert found == 40


@pytest.mark.parametrize("rows,cols,k,levels", [(1024, 1024, 2048, 6), (1024, 1024, 2048, 400),
                                                 (512, 384, 30000, 50), (777, 301, 9000, 3)])
def test_prox_sp_heap_order_large(oracle, rows, cols, k, levels):
    """Large selections through the pre-filtered replay: 1M entries with
    k = 2048 (heap on chip) and k = 30000 (heap in device memory), few or
    many distinct magnitudes; bit-exact against std::partial_sort."""
    rng = np.random.default_rng(rows + k + levels)
    M = _tie_matrix(rng, rows, cols, levels)
    # a few large entries late in the order force heap evictions of ties
    tail = rng.integers(rows * cols // 2, rows * cols, size=64)
    M.reshape(-1, order="F")[tail] = (levels + 1) / 8.0
    for pos in (False, True):
        c = fact.ConstraintInt("sp", rows, cols, k, normalized=False, pos=pos)
        got = _gpu_prox(M, c)
        ref = oracle.prox(oracle.SP, M, k=k, normalized=False, pos=pos)
        assert np.array_equal(got, ref), pos


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("espan,levels", [(40, 0), (20, 0), (40, 5), (3, 0)])
def test_prox_sp_radix_key_list(oracle, dtype, espan, levels):
    """1M entries whose magnitudes spread over `espan` binades, so the radix
    select finishes in one block over its key list: after the first digit
    when the k-th key's bucket holds at most 32,768 keys (espan 40: ~26,000
    in FP64), after the second when it does not (espan 20 and 3: 52,000 and
    349,000 after the first digit); `levels` > 0 puts ties inside the bucket
    (thousands of equal keys).  Heavy ties that keep the bucket above the
    list's size to the last digit are the tie tests above.  Support and
    normalised values bit-exact against the oracle."""
    rng = np.random.default_rng(espan * 10 + levels + (dtype == np.float32))
    n = 1024
    e = rng.integers(0, espan, size=(n, n))
    frac = rng.integers(0, levels + 1, size=(n, n)) / 8.0 if levels else rng.random((n, n))
    M = (np.where(rng.random((n, n)) < 0.5, -1.0, 1.0) * np.ldexp(1.0 + frac, -e)).astype(dtype)
    for k, normalized, pos in [(2048, True, False), (int(rng.integers(1000, 100000)), True, True),
                               (int(rng.integers(100000, 400000)), False, False)]:
        c = fact.ConstraintInt("sp", n, n, k, normalized=normalized, pos=pos)
        got = _gpu_prox(M, c)
        ref = oracle.prox(oracle.SP, M, k=k, normalized=normalized, pos=pos)
        assert np.array_equal(got, ref), (k, normalized, pos)
        assert np.count_nonzero(got) == min(k, np.count_nonzero(np.maximum(M, 0) if pos else M))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("espan,levels", [(40, 0), (3, 0), (20, 5)])
def test_prox_sp_radix_select_beyond_registers(oracle, dtype, espan, levels):
    """1,572,864 entries: more than the 16 keys per thread the register-
    resident radix select holds on a full cooperative grid of a GB300, so the
    select that re-reads the keys per digit runs (its key list and one-block
    finish included); bit-exact against the oracle."""
    rng = np.random.default_rng(espan + 7 * levels + (dtype == np.float32))
    rows, cols = 1536, 1024
    e = rng.integers(0, espan, size=(rows, cols))
    frac = rng.integers(0, levels + 1, size=(rows, cols)) / 8.0 if levels else rng.random((rows, cols))
    M = (np.where(rng.random((rows, cols)) < 0.5, -1.0, 1.0) * np.ldexp(1.0 + frac, -e)).astype(dtype)
    for k, normalized, pos in [(2048, True, False), (int(rng.integers(20000, 200000)), False, True)]:
        c = fact.ConstraintInt("sp", rows, cols, k, normalized=normalized, pos=pos)
        got = _gpu_prox(M, c)
        ref = oracle.prox(oracle.SP, M, k=k, normalized=normalized, pos=pos)
        assert np.array_equal(got, ref), (k, normalized, pos)


@pytest.mark.parametrize("name,kind", [("spcol", 1), ("splin", 2), ("splincol", 3)])
@pytest.mark.parametrize("seed", range(4))
def test_prox_lines_bitexact(oracle, name, kind, seed):
    rng = np.random.default_rng(100 + seed)
    rows, cols = [(40, 30), (64, 64), (17, 200), (512, 33)][seed]
    M = _tie_matrix(rng, rows, cols, 2) if seed % 2 else rng.standard_normal((rows, cols))
    k = [1, 4, 5, 7][seed]
    c = fact.ConstraintInt(name, rows, cols, k, pos=(seed == 2))
    got = _gpu_prox(M, c)
    ref = oracle.prox(kind, M, k=k, pos=c.pos)
    assert np.array_equal(got, ref)


def test_prox_norms_supp_bitexact(oracle):
    rng = np.random.default_rng(7)
    M = rng.standard_normal((50, 20))
    for name, kind, s in [("normcol", 4, 2.0), ("normlin", 5, 0.5)]:
        for normalized in (False, True):
            c = fact.ConstraintReal(name, 50, 20, s, normalized=normalized)
            assert np.array_equal(_gpu_prox(M, c), oracle.prox(kind, M, s=s, normalized=normalized))
    supp = (rng.random((50, 20)) < 0.3).astype(np.float64)
    c = fact.ConstraintMat("supp", supp)
    assert np.array_equal(_gpu_prox(M, c), oracle.prox(6, M, supp=supp))


def test_prox_zero_norm_is_an_error():
    with pytest.raises(Exception):
        _gpu_prox(np.zeros((8, 8)), fact.ConstraintInt("sp", 8, 8, 3))


def _factors_dense(res):
    F = res.faust
    return [F.factors(i).toarray() for i in range(F.numfactors())]


def _compare_palm(oracle, A, cons, its, **kw):
    params = fact.ParamsPalm4MSA(cons, its, **kw)
    res = fact.palm4msa(A, cons, params)
    okw = dict(kw)
    okw.pop("init_facts", None)
    facts_o, lam_o, _ = oracle.palm4msa2(A, [c.oracle_dict() for c in cons], its,
                                         init_facts=kw.get("init_facts"), **okw)
    got = _factors_dense(res)
    for g, o in zip(got, facts_o):
        assert np.array_equal(g.astype(o.dtype), o)
    assert res.lambda_ == lam_o
    return res, facts_o, lam_o


@pytest.mark.parametrize("n", [32, 64])
def test_palm_hadamard_bitexact(oracle, n):
    J = int(np.log2(n))
    H = synth.hadamard(n) / np.sqrt(n)
    cons = [fact.ConstraintInt("sp", n, n, 2 * n) for _ in range(J)]
    _compare_palm(oracle, H, cons, 60, norm2_threshold=1e-8)


def test_palm_hadamard_r2l_bitexact(oracle):
    n = 32
    H = synth.hadamard(n) / np.sqrt(n)
    cons = [fact.ConstraintInt("sp", n, n, 2 * n) for _ in range(5)]
    _compare_palm(oracle, H, cons, 20, norm2_threshold=1e-8, is_update_way_R2L=True)


def test_palm_fixture_config_compared_palm2_bitexact(oracle):
    """The reference's own palm4msa2 test settings and fixture
    (misc/test/src/C++/palm4msa_2020.cpp.in:81-121)."""
    import os
    data = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                "config_compared_palm2_data.npy"))
    cons = [fact.ConstraintInt("splin", 500, 32, 5), fact.ConstraintReal("normcol", 32, 32, 1.0, normalized=True)]
    _compare_palm(oracle, data, cons, 200, packing_RL=False, norm2_threshold=1e-15, norm2_max_iter=1000)


def test_palm_splincol_fp32_fp64_norms(oracle):
    """Batched-PALM instance shape: splincol k=4, FP32, FP64 step-size norms."""
    rng = np.random.default_rng(5)
    n = 96
    P = [synth.random_csr(n, n, 4, rng, np.float64).toarray() for _ in range(3)]
    A = (P[0] @ P[1] @ P[2] + 1e-3 * rng.standard_normal((n, n))).astype(np.float32)
    cons = [fact.ConstraintInt("splincol", n, n, 4) for _ in range(4)]
    _compare_palm(oracle, A, cons, 30, norm2_fp64=True)


def test_palm_butterfly_supp_fp32(oracle):
    """Learned-warm-start shape: 8 butterfly supp factors of a 256 x 256
    Gaussian kernel matrix, FP32."""
    rng = np.random.default_rng(6)
    x = rng.random((256, 3))
    d2 = ((x[:, None, :] - x[None, :, :]) ** 2).sum(-1)
    K = np.exp(-d2 / (2 * 0.2 ** 2)).astype(np.float32)
    sups = synth.butterfly_supports(8, np.float32)
    cons = [fact.ConstraintMat("supp", s.toarray()) for s in sups]
    init = [s.toarray() for s in sups]
    _compare_palm(oracle, K, cons, 25, init_facts=init)


def test_palm_config2_first_iterations_bitexact(oracle):
    """Full-size Hadamard 1024 / 32, 10 factors, sp k=2048: the first three
    iterations against the oracle."""
    n = 1024
    H = synth.hadamard(n) / 32.0
    cons = [fact.ConstraintInt("sp", n, n, 2048) for _ in range(10)]
    oracle.set_threads(16)
    _compare_palm(oracle, H, cons, 3, norm2_threshold=1e-8)


def test_palm_cancel_flag_is_honoured():
    """fgb_cancel set before the run stops it at the first check."""
    import faust_gb300 as fg
    ctx = fg.Context(0)
    n = 32
    H = synth.hadamard(n) / np.sqrt(n)
    cons = [fact.ConstraintInt("sp", n, n, 2 * n) for _ in range(5)]
    ctx.cancel()
    with pytest.raises(Exception) as e:
        fact.palm4msa(H, cons, fact.ParamsPalm4MSA(cons, 50), ctx=ctx)
    assert "CANCELLED" in str(e.value)


def _config4_instance(rng, n):
    P = [synth.random_csr(n, n, 4, rng, np.float64).toarray() for _ in range(3)]
    return (P[0] @ P[1] @ P[2] + 1e-3 * rng.standard_normal((n, n))).astype(np.float32)


def test_palm_batched_matches_oracle_per_instance(oracle):
    """Uneven splincol instances (the batched configuration's shape, smaller
    n) in one persistent launch; each instance bit-identical to its oracle run."""
    import torch
    rng = np.random.default_rng(40)
    sizes = [64, 144, 80, 112, 96, 128]
    probs, host = [], []
    for n in sizes:
        A = _config4_instance(rng, n)
        cons = [fact.ConstraintInt("splincol", n, n, 4) for _ in range(4)]
        probs.append((_cuda_colmajor(A), cons))
        host.append((A, cons))
    params = fact.ParamsPalm4MSA(probs[0][1], 15, norm2_fp64=True)
    res = fact.palm4msa_batched(probs, params, ctas_per_sm=1)
    for r, (A, cons) in zip(res, host):
        assert r.status == 0
        facts_o, lam_o, _ = oracle.palm4msa2(A, [c.oracle_dict() for c in cons], 15, norm2_fp64=True)
        got = [r.faust.factors(i).toarray() for i in range(4)]
        for g, o in zip(got, facts_o):
            assert np.array_equal(g.astype(np.float32), o)
        assert r.lambda_ == lam_o


def test_palm_batched_equals_single_instance_gpu():
    rng = np.random.default_rng(41)
    n = 96
    A = _config4_instance(rng, n)
    cons = [fact.ConstraintInt("splincol", n, n, 4) for _ in range(4)]
    params = fact.ParamsPalm4MSA(cons, 12, norm2_fp64=True)
    single = fact.palm4msa(A, cons, params)
    batched = fact.palm4msa_batched([(_cuda_colmajor(A), cons)] * 3, params)
    for r in batched:
        assert r.lambda_ == single.lambda_
        for i in range(4):
            assert (r.faust.factors(i) != single.faust.factors(i)).nnz == 0


def test_palm_batched_butterfly_supp(oracle):
    rng = np.random.default_rng(42)
    sups = synth.butterfly_supports(6, np.float32)
    probs, host = [], []
    for _ in range(4):
        x = rng.random((64, 3))
        d2 = ((x[:, None, :] - x[None, :, :]) ** 2).sum(-1)
        K = np.exp(-d2 / (2 * 0.3 ** 2)).astype(np.float32)
        cons = [fact.ConstraintMat("supp", s.toarray()) for s in sups]
        init = [s.toarray() for s in sups]
        probs.append((_cuda_colmajor(K), cons, init))
        host.append((K, cons, init))
    params = fact.ParamsPalm4MSA(probs[0][1], 10)
    res = fact.palm4msa_batched(probs, params)
    for r, (K, cons, init) in zip(res, host):
        facts_o, lam_o, _ = oracle.palm4msa2(K, [c.oracle_dict() for c in cons], 10, init_facts=init)
        assert r.lambda_ == lam_o
        for i in range(6):
            assert np.array_equal(r.faust.factors(i).toarray().astype(np.float32), facts_o[i])


# ---------------------------------------------------------------- hierarchical
def _dense_factors(F):
    return [F.factors(i).toarray() for i in range(F.numfactors())]


def test_hierarchical_wht_bitexact(oracle):
    """hierarchical with pyfaust's ParamsHierarchicalWHT on the 32 x 32
    Hadamard matrix: factors and lambda equal to the oracle's composition of
    palm4msa2 runs, and the factorization is exact."""
    n, d = 5, 32
    A = synth.hadamard(d).astype(np.float64)
    fc = [fact.ConstraintInt("splincol", d, d, 2) for _ in range(n - 1)]
    rc = [fact.ConstraintInt("splincol", d, d, d // 2 ** (i + 1)) for i in range(n - 1)]
    p = fact.ParamsHierarchical(fc, rc, 30, 30, is_update_way_R2L=True, packing_RL=False)
    res = fact.hierarchical(A, p)
    got = _dense_factors(res.faust)
    ref, lam = oracle.hierarchical(A, [c.oracle_dict() for c in fc], [c.oracle_dict() for c in rc], 30, 30,
                                   is_update_way_R2L=True, packing_RL=False)
    assert res.lambda_ == lam
    assert len(got) == len(ref) and all(np.array_equal(a, b) for a, b in zip(got, ref))
    assert oracle.rel_err(A, got, res.lambda_) < 1e-12
    res.faust.close()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_hierarchical_hadamard32_reference_config(oracle, dtype):
    """The reference's Hadamard test configuration (config_HADAMARD_32.mat,
    committed as JSON): factors and lambda equal the oracle's in double and
    float, and the float factorization is exact to float rounding."""
    import json
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                           "config_HADAMARD_32_params.json")) as f:
        p = json.load(f)
    fc, rc = [[fact.ConstraintInt(c[0], c[2], c[3], c[1]) for c in row] for row in p["cons"]]
    A = synth.hadamard(p["nrow"]).astype(dtype)
    r2l = bool(p["update_way"])
    res = fact.hierarchical(A, fact.ParamsHierarchical(fc, rc, p["niter1"], p["niter2"],
                                                       is_update_way_R2L=r2l, packing_RL=False))
    got = _dense_factors(res.faust)
    ref, lam = oracle.hierarchical(A, [c.oracle_dict() for c in fc], [c.oracle_dict() for c in rc],
                                   p["niter1"], p["niter2"], is_update_way_R2L=r2l, packing_RL=False)
    assert np.float64(res.lambda_) == np.float64(lam)
    assert len(got) == p["nfacts"] and all(np.array_equal(a, b) for a, b in zip(got, ref))
    assert oracle.rel_err(A, got, res.lambda_) < (1e-12 if dtype == np.float64 else 1e-5)
    res.faust.close()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_hierarchical_left_side_sp_bitexact(oracle, dtype):
    rng = np.random.default_rng(5)
    A = rng.standard_normal((40, 24)).astype(dtype)
    fc = [fact.ConstraintInt("sp", 24, 24, 60), fact.ConstraintInt("sp", 32, 24, 60)]
    rc = [fact.ConstraintInt("sp", 40, 24, 400), fact.ConstraintInt("sp", 40, 32, 300)]
    p = fact.ParamsHierarchical(fc, rc, 10, 10, is_fact_side_left=True, norm2_fp64=dtype == np.float32)
    res = fact.hierarchical(A, p)
    got = _dense_factors(res.faust)
    ref, lam = oracle.hierarchical(A, [c.oracle_dict() for c in fc], [c.oracle_dict() for c in rc], 10, 10,
                                   is_fact_side_left=True, norm2_fp64=dtype == np.float32)
    assert [g.shape for g in got] == [(40, 32), (32, 24), (24, 24)]
    assert np.float64(res.lambda_) == np.float64(lam)
    assert all(np.array_equal(a, b) for a, b in zip(got, ref))
    res.faust.close()


def test_palm_batched_seeded_from_device_values(oracle):
    """Starting values given on the device (the learned warm start's path):
    factors seeded on shared butterfly supports from a values tensor, lambda
    started at <K, S> / ||S||^2 of the seeded factors; every instance equals
    the oracle run from the same dense factors and lambda."""
    import torch
    rng = np.random.default_rng(43)
    J, n = 6, 64
    sups = synth.butterfly_supports(J, np.float32)
    cons = [fact.ConstraintMat("supp", s.toarray()) for s in sups]
    V = sum(s.nnz for s in sups)
    Ks = [synth.gaussian_kernel(n, s, rng) for s in (0.1, 0.2, 0.3, 0.45, 0.07)]
    vals = rng.standard_normal((len(Ks), V)).astype(np.float32)
    scale = 0.5
    res = fact.palm4msa_batched([(_cuda_colmajor(K), cons) for K in Ks], fact.ParamsPalm4MSA(cons, 15),
                                init_values=torch.from_numpy(vals).cuda(), values_scale=scale,
                                lambda_from_init=True)
    for i, (K, r) in enumerate(zip(Ks, res)):
        init, q = [], 0
        for s in sups:
            d = np.zeros((n, n), np.float32)
            rows = np.repeat(np.arange(n), np.diff(s.indptr))
            d[rows, s.indices] = (scale * vals[i, q:q + s.nnz].astype(np.float64)).astype(np.float32)
            q += s.nnz
            init.append(d)
        lam0 = oracle.lambda_of_factors(K, init)
        facts_o, lam_o, _ = oracle.palm4msa2(K, [c.oracle_dict() for c in cons], 15, init_facts=init,
                                             init_lambda=lam0)
        assert r.status == 0
        assert r.lambda_ == lam_o, i
        for f in range(J):
            assert np.array_equal(r.faust.factors(f).toarray().astype(np.float32), facts_o[f]), (i, f)
        r.faust.close()


def test_palm_batched_graph_launch_on_created_stream():
    """The batched launch (queue reset, seeding, the persistent kernel) runs as
    one captured CUDA graph on a created stream and, through a private stream,
    for a context on the legacy default stream; the results are the same in
    both and for every CTAs-per-SM variant (1, 2, and 3 with the 80-register
    kernel)."""
    import torch
    import faust_gb300 as fg
    rng = np.random.default_rng(44)
    sizes = [64, 96, 80, 128]
    probs = []
    for n in sizes:
        A = _config4_instance(rng, n)
        probs.append((_cuda_colmajor(A), [fact.ConstraintInt("splincol", n, n, 4) for _ in range(4)]))
    params = fact.ParamsPalm4MSA(probs[0][1], 10, norm2_fp64=True)
    ref = fact.palm4msa_batched(probs, params, ctx=fg.Context(0, stream=0), ctas_per_sm=2)
    s = torch.cuda.Stream()
    ctx = fg.Context(0, stream=s.cuda_stream)
    for cps in (1, 2, 3):
        got = fact.palm4msa_batched(probs, params, ctx=ctx, ctas_per_sm=cps)
        for a, b in zip(ref, got):
            assert a.lambda_ == b.lambda_ and b.status == 0 and b.cycles > 0
            for i in range(4):
                assert (a.faust.factors(i) != b.faust.factors(i)).nnz == 0
            b.faust.close()
    for a in ref:
        a.faust.close()
