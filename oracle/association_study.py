"""Association study for palm4msa2 (TEST INFRASTRUCTURE ONLY).

The oracle (faust_oracle.cpp) and the GPU evaluate the gradient of each
factor update as a chain of sparse products:

    E = lambda * S_0 ... S_f * pR_f - A,   G = S_0^H ... S_{f-1}^H * E * S_{J-1}^H ... S_{f+1}^H

The reference instead packs the left and right parts into dense matrices and
multiplies dense matrices (compute_n_apply_grad2,
src/algorithm/factorization/faust_palm4msa2020.hpp:362-439):

    pR[i] = pack(S[i+1] * pR[i+1])        init_ite, :198-211
    pL[f+1] = pack(pL[f] * S[f])          next_fid, :212-222
    E = lambda * L * (D * R) - A          multiply_order_opt_all_ends on {L, D, R}
                                          (faust_prod_opt.hpp:49-86: equal costs
                                          take the right-end product first)
    G = (lambda / c) * L^H * (E * R^H)    same function, flags {H, N, H}
    D = D - G
    c = 1.001 * lambda^2 * ||R||^2 * ||L||^2, with ||M|| = sqrt of the power
        iteration on M M^H (Transform::spectralNorm of the packed factor,
        CPU/faust_Transform.hpp:683-708; power_iteration,
        faust_linear_algebra.hpp:806-899)
    lambda = tr(A^H * (pL[J-1] * S[J-1])) / ||pL[J-1] * S[J-1]||_F^2
        (update_lambda, :441-493, with the packed reuse rule)

This module restates that association with NumPy (BLAS GEMMs, whose
summation order is OpenBLAS's, not Eigen's) and runs it next to the oracle
on the same problem.  Both use the oracle's projection (std::partial_sort
tie rule).  It reports, for every factor update, whether the support chosen
by the two associations is the same, the lambda of every iteration, and the
final relative error of each run (calc_rel_err, :35-44).

    python oracle/association_study.py --n 1024 --its 200 --out result.json

runs the Hadamard 1024 / 32 configuration (10 factors, sp k = 2048,
norm2_threshold 1e-8, 200 iterations).
"""
import argparse
import json
import os
import sys
import time

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# run as a script, this folder comes first on the path and its oracle.py
# would shadow the package of the same name
sys.path = [ROOT] + [q for q in sys.path if os.path.abspath(q or ".") != HERE]

from oracle import oracle as O  # noqa: E402


def hadamard(n):
    H = np.array([[1.0]])
    while H.shape[0] < n:
        H = np.block([[H, H], [H, -H]])
    return H


def spectral_norm_packed(M, max_iter, thr, x0, transposed_gemm=False):
    """sqrt of power_iteration on M M^H (square packed factor)."""
    xk = x0.copy()
    lam_old, lam = 1.0, 0.0
    i = 0
    while (abs(lam_old - lam) > abs(thr) or abs(lam) <= abs(thr)) and i < max_iter:
        i += 1
        lam_old = lam
        nrm = np.sqrt(xk @ xk)
        if nrm == 0:
            raise FloatingPointError("power iteration: zero vector")
        xn = xk / nrm
        xk = M @ (M.T @ xn)
        if not xk.any():
            return 0.0, i
        lam = float(xn @ xk)
    return float(abs(np.sqrt(lam))), (i if i < max_iter else -1)


def gemm(a, b, transposed):
    """a @ b, or the same product evaluated as (b^T a^T)^T (another BLAS
    kernel order), to see how much the supports depend on GEMM rounding."""
    return (b.T @ a.T).T if transposed else a @ b


def palm4msa2_dense(A, J, k, nb_it, thr=1e-8, max_iter=100, transposed_gemm=False, log=None):
    """palm4msa2 (L2R, packing_RL, sp constraints, identity init) in the
    reference's packed-dense association.  Returns (factors, lambda, trace)."""
    n = A.shape[0]
    S = [np.zeros((n, n))] + [np.eye(n) for _ in range(J - 1)]
    lam = 1.0
    x0 = O.rand_start(n)
    hashes, nnzs, lams = [], [], []
    for it in range(nb_it):
        t0 = time.time()
        # init_ite: pR[J-1] empty, pR[i] = S[i+1] * pR[i+1] packed
        pR = [None] * J
        pR[J - 2] = S[J - 1].copy()
        for i in range(J - 3, -1, -1):
            pR[i] = np.asarray(sp.csr_matrix(S[i + 1]) @ pR[i + 1])
        pL = [None] * J
        for f in range(J):
            hasL, hasR = f > 0, f + 1 < J
            nR = nL = 1.0
            if hasR:
                nR, _ = spectral_norm_packed(pR[f], max_iter, thr, x0)
            if hasL:
                nL, _ = spectral_norm_packed(pL[f], max_iter, thr, x0)
            if nR == 0 or (nL == 0 and it > 0):
                raise FloatingPointError("zero 2-norm at it %d f %d" % (it, f))
            c = 1.001 * lam * lam * nR * nR * nL * nL
            D = S[f]
            if hasL and hasR:
                E = lam * gemm(pL[f], gemm(D, pR[f], transposed_gemm), transposed_gemm) - A
                G = (lam / c) * gemm(pL[f].T, gemm(E, pR[f].T, transposed_gemm), transposed_gemm)
            elif hasR:
                E = lam * gemm(D, pR[f], transposed_gemm) - A
                G = (lam / c) * gemm(E, pR[f].T, transposed_gemm)
            else:
                E = lam * gemm(pL[f], D, transposed_gemm) - A
                G = (lam / c) * gemm(pL[f].T, E, transposed_gemm)
            D = D - G
            D = O.prox(O.SP, D, k=k, normalized=True, pos=False)
            S[f] = np.asarray(D, dtype=np.float64, order="C")
            h, nz = O.support_hash(S[f])
            hashes.append(h)
            nnzs.append(nz)
            # next_fid: pL[f+1] = pack(pL[f] * S[f])
            if f + 1 < J:
                pL[f + 1] = S[f].copy() if f == 0 else np.asarray((sp.csr_matrix(S[f]).T @ pL[f].T).T)
        # update_lambda with the packed reuse rule: S = pL[J-1] * S[J-1]
        S_mat = np.asarray((sp.csr_matrix(S[J - 1]).T @ pL[J - 1].T).T)
        tr = np.trace(gemm(A.T, S_mat, transposed_gemm))
        nS = np.sqrt((S_mat * S_mat).sum())
        lam = float(tr / (nS * nS))
        lams.append(lam)
        if log:
            log("it %d lambda %.17g (%.1f s)" % (it, lam, time.time() - t0))
    return S, lam, {"supp_hash": hashes, "supp_nnz": nnzs, "lambdas": lams}


def rel_err(A, S, lam):
    P = S[-1]
    for M in reversed(S[:-1]):
        P = M @ P
    return float(np.linalg.norm(lam * P - A) / np.linalg.norm(A))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--its", type=int, default=200)
    ap.add_argument("--transposed-gemm", action="store_true")
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    n = a.n
    J = int(np.log2(n))
    k = 2 * n
    A = np.asfortranarray(hadamard(n) / np.sqrt(n))
    O.set_threads(a.threads)
    t0 = time.time()
    cons = [dict(kind=O.SP, k=k, s=1.0, normalized=True, pos=False, rows=n, cols=n, supp=None) for _ in range(J)]
    fo, lo, tro = O.palm4msa2(A, cons, a.its, norm2_threshold=1e-8)
    t_oracle = time.time() - t0
    print("oracle (sparse chain): lambda %.17g in %.1f s" % (lo, t_oracle), flush=True)
    t0 = time.time()
    fd, ld, trd = palm4msa2_dense(A, J, k, a.its, transposed_gemm=a.transposed_gemm,
                                  log=lambda s: print(s, flush=True) if a.its <= 20 else None)
    t_dense = time.time() - t0
    print("dense association: lambda %.17g in %.1f s" % (ld, t_dense), flush=True)
    ho = [int(x) for x in tro["supp_hash"]]
    hd = [int(x) for x in trd["supp_hash"]]
    same = [x == y for x, y in zip(ho, hd)]
    first_diff = next((i for i, s in enumerate(same) if not s), None)
    lo_traj = [float(x) for x in tro["lambdas"]]
    ld_traj = [float(x) for x in trd["lambdas"]]
    rel_lam = [abs(x - y) / abs(x) if x else 0.0 for x, y in zip(lo_traj, ld_traj)]
    Po, Pd = fo[-1], fd[-1]
    for Mo, Md in zip(reversed(fo[:-1]), reversed(fd[:-1])):
        Po, Pd = Mo @ Po, Md @ Pd
    prod_diff = float(np.linalg.norm(lo * Po - ld * Pd) / np.linalg.norm(lo * Po))

    def significant(M, rel=1e-12):
        m = np.abs(M)
        return m > rel * m.max() if m.max() > 0 else m > 0

    sig_same = [bool(np.array_equal(significant(a_), significant(b_))) for a_, b_ in zip(fo, fd)]
    noise = [int(np.count_nonzero((a_ != 0) & ~significant(a_))) for a_ in fo]
    res = {
        "problem": "Hadamard %d / sqrt(%d), %d sp factors k=%d, L2R, packing_RL, norm2_threshold 1e-8, %d its"
                   % (n, n, J, k, a.its),
        "dense_gemm": "transposed (B^T A^T)^T" if a.transposed_gemm else "A @ B",
        "updates": len(same),
        "updates_same_support": int(sum(same)),
        "first_differing_update": first_diff,
        "first_differing_iteration": None if first_diff is None else first_diff // J,
        "lambda_oracle": lo, "lambda_dense": ld,
        "max_rel_lambda_diff": max(rel_lam) if rel_lam else 0.0,
        "final_product_rel_diff": prod_diff,
        "final_factors_same_significant_support": sig_same,
        "final_factors_oracle_noise_entries": noise,
        "rel_err_oracle": O.rel_err(A, fo, lo),
        "rel_err_dense": rel_err(A, fd, ld),
        "seconds_oracle": t_oracle, "seconds_dense": t_dense,
        "lambda_oracle_per_it": lo_traj, "lambda_dense_per_it": ld_traj,
        "same_support_per_update": [int(s) for s in same],
    }
    print(json.dumps({k2: v for k2, v in res.items() if not k2.endswith(("_per_it", "_per_update"))}, indent=1))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(res, f)
            f.write("\n")


if __name__ == "__main__":
    main()
