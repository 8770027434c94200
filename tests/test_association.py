"""The reference's packed-dense association of the palm4msa2 gradient against
the sparse-chain association the oracle and the GPU use
(oracle/association_study.py; compute_n_apply_grad2,
src/algorithm/factorization/faust_palm4msa2020.hpp:362-439).

On Hadamard targets the two associations keep different sets of entries
whose values are rounding residue (|v| below 1e-12 of the factor's largest
entry: an exact cancellation in one order is a 1-ulp remainder in the
other); every entry above that is kept by both, and lambda, the product
lambda * S_0 ... S_{J-1} and the relative error agree to 1e-12."""
import numpy as np
import pytest


@pytest.mark.parametrize("n,its", [(32, 40), (64, 30)])
def test_dense_association_agrees_with_sparse_chain(oracle, n, its):
    from oracle import association_study as AS
    J = int(np.log2(n))
    k = 2 * n
    A = np.asfortranarray(AS.hadamard(n) / np.sqrt(n))
    cons = [dict(kind=oracle.SP, k=k, s=1.0, normalized=True, pos=False, rows=n, cols=n, supp=None)
            for _ in range(J)]
    fo, lo, tro = oracle.palm4msa2(A, cons, its, norm2_threshold=1e-8)
    fd, ld, trd = AS.palm4msa2_dense(A, J, k, its)
    lam_o, lam_d = np.asarray(tro["lambdas"]), np.asarray(trd["lambdas"])
    assert np.max(np.abs(lam_o - lam_d) / np.abs(lam_o)) < 1e-12
    Po, Pd = fo[-1], fd[-1]
    for Mo, Md in zip(reversed(fo[:-1]), reversed(fd[:-1])):
        Po, Pd = Mo @ Po, Md @ Pd
    assert np.linalg.norm(lo * Po - ld * Pd) / np.linalg.norm(lo * Po) < 1e-12
    for a, b in zip(fo, fd):
        ma, mb = np.abs(a), np.abs(b)
        assert np.array_equal(ma > 1e-12 * ma.max(), mb > 1e-12 * mb.max())
    assert abs(oracle.rel_err(A, fo, lo) - AS.rel_err(A, fd, ld)) < 1e-12
