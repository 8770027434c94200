"""Dense product of a Faust (TransformHelper::get_product,
src/faust_linear_operator/CPU/faust_TransformHelper.hpp:1132-1178) in the
DEFAULT_L2R and DYNPROG orders (dynprog_multiply, faust_prod_opt_gen.hpp:80-202),
and the DYNPROG-ordered Faust x dense product, against the oracle's
restatement.  The reference tests DYNPROG by comparing the product to the
plain one (misc/test/src/C++/test_dynprog_mul_cpu.cpp.in); here the split
table, then every bit of the result, is compared."""
import numpy as np
import pytest
import scipy.sparse as sp

from faust_gb300 import synth
from faust_gb300.faust import dynprog_plan


def _chain(rng, dims, dens, dtype):
    return [sp.random(dims[q], dims[q + 1], density=dens[q], format="csr", dtype=dtype, random_state=rng)
            for q in range(len(dims) - 1)]


def _leaves(rng, n, with_dense):
    dims = rng.integers(1, 400, n + 1)
    out = []
    for q in range(n):
        r, c = int(dims[q]), int(dims[q + 1])
        out.append((r, c, int(rng.integers(0, r * c + 1)), 0))
    if with_dense:
        out.append((int(dims[n]), int(rng.integers(1, 300)), 0, 1))
        out[-1] = (out[-1][0], out[-1][1], out[-1][0] * out[-1][1], 1)
    return out


@pytest.mark.parametrize("op", ["N", "T"])
@pytest.mark.parametrize("with_dense", [False, True])
def test_dynprog_plan_matches_oracle(oracle, op, with_dense):
    """The library's split table (host code) equals the oracle's restatement
    of the reference's dynamic program on random chains."""
    rng = np.random.default_rng(11)
    for trial in range(60):
        n = int(rng.integers(2, 9))
        leaves = _leaves(rng, n, with_dense)
        want = oracle.dynprog_splits([(a, b, c, bool(d)) for a, b, c, d in leaves], op)
        assert dynprog_plan(leaves, op) == want, (trial, leaves)


def test_dynprog_plan_int32_wrap(oracle):
    """Costs past 2^31 wrap as the reference's int arithmetic does."""
    leaves = [(60000, 60000, 3000000, 0), (60000, 60000, 2500000, 0), (60000, 50000, 2000000, 0),
              (50000, 70000, 1000000, 0)]
    want = oracle.dynprog_splits([(a, b, c, bool(d)) for a, b, c, d in leaves], "N")
    assert dynprog_plan(leaves, "N") == want


def test_dynprog_butterfly_is_right_to_left(oracle):
    """Equal-cost butterfly factors: the first minimiser (k = i) everywhere,
    i.e. the right-to-left chain."""
    n = 6
    leaves = [(1024, 1024, 2048, False)] * n
    s = oracle.dynprog_splits(leaves, "N")
    assert all(k == i for (i, j), k in s.items())


def test_oracle_product_matches_numpy(oracle):
    rng = np.random.default_rng(2)
    f = _chain(rng, [30, 50, 20, 60, 40], [0.2, 0.5, 0.05, 0.3], np.float64)
    D = (f[0] @ f[1] @ f[2] @ f[3]).toarray()
    for order in (0, 5):
        assert np.allclose(oracle.faust_product(f, "N", order), D, rtol=0, atol=1e-12)
        assert np.allclose(oracle.faust_product(f, "T", order), D.T, rtol=0, atol=1e-12)
    X = rng.standard_normal((40, 9))
    assert np.allclose(oracle.faust_product(f, "N", 5, X), D @ X, atol=1e-12)


# ---------------------------------------------------------------- GPU parity
def _faust(facs, dtype):
    from faust_gb300 import Faust
    return Faust(facs, dtype=dtype)


CHAINS = [
    # (dims, densities): butterfly-like equal costs; uneven densities that
    # make DYNPROG split in the middle (dense x dense products); thin and wide
    ([64, 64, 64, 64, 64], [0.05, 0.05, 0.05, 0.05]),
    ([179, 233, 45, 100, 220, 66], [0.02, 0.8, 0.005, 0.8, 0.8]),
    ([17, 300, 5, 400, 33], [0.1, 0.9, 0.2, 0.05]),
    ([128, 96], [0.1]),
]


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("op", ["N", "T", "H"])
@pytest.mark.parametrize("ci", range(len(CHAINS)))
def test_product_bitexact(oracle, dtype, op, ci):
    dims, dens = CHAINS[ci]
    rng = np.random.default_rng(100 + ci)
    facs = _chain(rng, dims, dens, dtype)
    F = _faust(facs, dtype)
    for order, code in (("DEFAULT_L2R", 0), ("DYNPROG", 5)):
        got = F.product_device(op, order).cpu().numpy()
        want = oracle.faust_product(facs, op, code)
        assert got.dtype == want.dtype and got.shape == want.shape
        assert np.array_equal(got, want), (order, op)
    F.close()


def test_dynprog_takes_dense_dense_path(oracle):
    """The second GPU chain's DYNPROG plan multiplies two computed products
    (so the dense x dense kernel is covered)."""
    dims, dens = CHAINS[1]
    rng = np.random.default_rng(101)
    facs = _chain(rng, dims, dens, np.float64)
    leaves = [(f.shape[0], f.shape[1], f.nnz, False) for f in facs]
    s = oracle.dynprog_splits(leaves, "N")

    def has_dd(i, j):
        if j - i < 1:
            return False
        k = s[(i, j)]
        return (k > i and k + 1 < j) or has_dd(i, k) or has_dd(k + 1, j)
    assert has_dd(0, len(facs) - 1)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("op", ["N", "T"])
def test_mul_dynprog_bitexact(oracle, dtype, op):
    import torch
    dims, dens = CHAINS[1]
    rng = np.random.default_rng(7)
    facs = _chain(rng, dims, dens, dtype)
    F = _faust(facs, dtype)
    rows_in = F.shape[1] if op == "N" else F.shape[0]
    for ncols in (1, 37, 300):
        X = rng.standard_normal((rows_in, ncols)).astype(dtype)
        Xd = torch.from_numpy(np.ascontiguousarray(X.T)).cuda().t()
        got = F.matmul_dynprog_device(Xd, op).cpu().numpy()
        want = oracle.faust_product(facs, op, 5, X)
        assert np.array_equal(got, want), ncols
    F.close()


@pytest.mark.gpu
def test_toarray_butterfly_and_ldy(oracle):
    """toarray of a 1024 butterfly Faust and a product into a padded Y."""
    import torch
    rng = np.random.default_rng(9)
    facs = [sp.csr_matrix(f) for f in synth.butterfly_faust_factors(10, rng, np.float64)]
    F = _faust(facs, np.float64)
    want = oracle.faust_product(facs, "N", 0)
    assert np.array_equal(F.toarray(), want)
    assert np.array_equal(F.toarray("DYNPROG"), oracle.faust_product(facs, "N", 5))
    Ypad = torch.full((1024, 1030), 7.0, dtype=torch.float64, device="cuda").t()  # ld 1030
    Y = Ypad[:1024, :]
    F.product_device("N", "DEFAULT_L2R", Y=Y)
    assert np.array_equal(Y.cpu().numpy(), want)
    assert torch.all(Ypad[1024:, :] == 7.0)
    F.close()


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_product_long_rows_bitexact(oracle, dtype):
    """DYNPROG products that multiply a dense intermediate by sparse factors
    with long rows and columns (dense x CSR^T long-row kernel) and the default
    order, bit for bit against the oracle."""
    import scipy.sparse as sps
    rng = np.random.default_rng(41)
    facs = []
    for (r, c) in [(300, 1200), (1200, 900), (900, 1300), (1300, 500)]:
        A = sps.random(r, c, density=0.004, format="lil", dtype=dtype, random_state=rng)
        for i in rng.choice(r, 6, replace=False):
            L = int(rng.integers(17, c))
            A[i, rng.choice(c, L, replace=False)] = rng.standard_normal(L).astype(dtype)
        for j in rng.choice(c, 6, replace=False):
            L = int(rng.integers(17, r))
            A[rng.choice(r, L, replace=False), j] = rng.standard_normal(L).astype(dtype)
        facs.append(sps.csr_matrix(A))
    F = _faust(facs, dtype)
    for order, code in (("DEFAULT_L2R", 0), ("DYNPROG", 5)):
        for op in ("N", "T"):
            got = F.product_device(op, order).cpu().numpy()
            assert np.array_equal(got, oracle.faust_product(facs, op, code)), (order, op)
    F.close()
