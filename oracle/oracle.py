"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this
module; the product package never does.  The oracle restates FAuST's
Faust x dense chain (src/faust_linear_operator/CPU/faust_Transform.hpp:1713-1855)
and palm4msa2 (src/algorithm/factorization/faust_palm4msa2020.hpp:46-676) on the
CPU; see faust_oracle.cpp for the operation order it fixes.  Parity against
the reference's own numerical outputs is unpinned (the reference needs Eigen,
which is absent); the top-k tie rule is pinned by calling std::partial_sort.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liborc.so")
_lib = None

# Constraint kinds (same values as include/fgb.h).
SP, SPCOL, SPLIN, SPLINCOL, NORMCOL, NORMLIN, SUPP, SP_POS = range(8)


class PalmParams(ctypes.Structure):
    _fields_ = [
        ("nb_it", ctypes.c_int),
        ("is_update_way_R2L", ctypes.c_int),
        ("packing_RL", ctypes.c_int),
        ("no_normalization", ctypes.c_int),
        ("no_lambda", ctypes.c_int),
        ("norm2_threshold", ctypes.c_double),
        ("norm2_max_iter", ctypes.c_int),
        ("constant_step_size", ctypes.c_int),
        ("step_size", ctypes.c_double),
        ("no_lambda_error", ctypes.c_int),
        ("norm2_fp64", ctypes.c_int),
    ]


def build():
    subprocess.check_call(["sh", os.path.join(_HERE, "build_oracle.sh")])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = ctypes.CDLL(_LIB_PATH)
        _lib.orc_last_error.restype = ctypes.c_char_p
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _check(rc):
    if rc != 0:
        raise RuntimeError("oracle error %d: %s" % (rc, lib().orc_last_error().decode()))


def set_threads(n):
    return lib().orc_set_threads(int(n))


def _pack_chain(factors, dtype):
    """factors: list of scipy.sparse CSR matrices (sorted indices)."""
    dims, rp, ci, vv = [], [], [], []
    for f in factors:
        f = f.tocsr()
        f.sort_indices()
        dims += [f.shape[0], f.shape[1], f.nnz]
        rp.append(f.indptr.astype(np.int32))
        ci.append(f.indices.astype(np.int32))
        vv.append(f.data.astype(dtype))
    cat = lambda xs, dt: np.ascontiguousarray(np.concatenate(xs) if xs else np.zeros(0, dt), dtype=dt)
    return (np.asarray(dims, np.int32), cat(rp, np.int32), cat(ci, np.int32), cat(vv, dtype))


def chain_mul(factors, X):
    """Y = S_0 ... S_{J-1} X, right to left (Transform::multiply)."""
    dtype = X.dtype
    assert dtype in (np.float32, np.float64)
    dims, rp, ci, vv = _pack_chain(factors, dtype)
    Xf = np.asfortranarray(X)
    Y = np.zeros((factors[0].shape[0], X.shape[1]), dtype=dtype, order="F")
    fn = lib().orc_chain_mul_f64 if dtype == np.float64 else lib().orc_chain_mul_f32
    _check(fn(len(factors), _p(dims), _p(rp), _p(ci), _p(vv), _p(Xf), X.shape[0], X.shape[1], _p(Y)))
    return Y


def pi_spmv(S, x):
    """y = S x with the power iteration's row order (16-entry chunks, pairwise
    tree over the chunk partials), FP64."""
    S = _csr(S).astype(np.float64)
    x = np.ascontiguousarray(x, np.float64).ravel()
    y = np.zeros(S.shape[0], np.float64)
    rp, ci = S.indptr.astype(np.int32), S.indices.astype(np.int32)
    _check(lib().orc_pi_spmv_f64(S.shape[0], S.shape[1], _p(rp), _p(ci), _p(np.ascontiguousarray(S.data)), _p(x),
                                 _p(y)))
    return y


def bsr_mul_f64(m, n, bm, bn, browptr, bcolind, blocks, X):
    """Y = B X in FP64 (BSRMat::mul); blocks is (bnnz, bm*bn) column-major per block."""
    Xf = np.asfortranarray(X, dtype=np.float64)
    Y = np.zeros((m, X.shape[1]), np.float64, order="F")
    bp = np.ascontiguousarray(browptr, np.int32)
    bc = np.ascontiguousarray(bcolind, np.int32)
    bl = np.ascontiguousarray(blocks, np.float64)
    _check(lib().orc_bsr_mul_f64(m, n, bm, bn, _p(bp), _p(bc), _p(bl), _p(Xf), Xf.shape[0], X.shape[1], _p(Y), m))
    return Y


def topk(v, k):
    """Indices kept by sort_idx: std::partial_sort with comparator |a| > |b|."""
    v = np.ascontiguousarray(v)
    out = np.zeros(k, np.int32)
    fn = lib().orc_topk_f64 if v.dtype == np.float64 else lib().orc_topk_f32
    _check(fn(ctypes.c_long(v.size), _p(v), k, _p(out)))
    return out


def prox(kind, M, k=0, s=1.0, normalized=True, pos=False, supp=None):
    M = np.array(M, order="F", copy=True)
    sup = None if supp is None else np.asfortranarray(supp, dtype=M.dtype)
    fn = lib().orc_prox_f64 if M.dtype == np.float64 else lib().orc_prox_f32
    _check(fn(kind, ctypes.c_long(k), ctypes.c_double(s), int(normalized), int(pos), _p(M), M.shape[0], M.shape[1],
              _p(sup)))
    return M


def spectral_norm(factors, max_iter=100, thr=1e-6):
    dims, rp, ci, vv = _pack_chain(factors, np.float64)
    out = ctypes.c_double()
    flag = ctypes.c_int()
    _check(lib().orc_spectral_norm_f64(len(factors), _p(dims), _p(rp), _p(ci), _p(vv), max_iter,
                                       ctypes.c_double(thr), ctypes.byref(out), ctypes.byref(flag)))
    return out.value, flag.value


def rand_start(n):
    out = np.zeros(n, np.float64)
    _check(lib().orc_rand_start_f64(n, _p(out)))
    return out


def canonical_dot(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b, dtype=a.dtype)
    if a.dtype == np.float64:
        out = ctypes.c_double()
        _check(lib().orc_canonical_dot_f64(ctypes.c_long(a.size), _p(a), _p(b), ctypes.byref(out)))
    else:
        out = ctypes.c_float()
        _check(lib().orc_canonical_dot_f32(ctypes.c_long(a.size), _p(a), _p(b), ctypes.byref(out)))
    return out.value


def _pack_cons(cons, dtype):
    J = len(cons)
    kind = np.array([c["kind"] for c in cons], np.int32)
    k = np.array([c.get("k", 0) for c in cons], np.int64)
    s = np.array([c.get("s", 1.0) for c in cons], np.float64)
    flags = np.array(sum([[int(c.get("normalized", True)), int(c.get("pos", False))] for c in cons], []), np.int32)
    cdims = np.array(sum([[c["rows"], c["cols"]] for c in cons], []), np.int32)
    supps = [np.asfortranarray(c["supp"], dtype=dtype).ravel(order="F") for c in cons if c["kind"] == SUPP]
    supp = np.ascontiguousarray(np.concatenate(supps) if supps else np.zeros(1, dtype), dtype=dtype)
    return J, kind, k, s, flags, cdims, supp


def palm4msa2(A, cons, nb_it, is_update_way_R2L=False, packing_RL=True, no_normalization=False, no_lambda=False,
              norm2_threshold=1e-6, norm2_max_iter=100, constant_step_size=False, step_size=1e-16,
              no_lambda_error=False, norm2_fp64=False, init_facts=None, init_lambda=1.0):
    """palm4msa2 restatement.  cons: list of dicts(kind,k,s,normalized,pos,rows,cols,supp).

    Returns (factors as dense column-major arrays, lambda, trace dict)."""
    dtype = A.dtype
    Af = np.asfortranarray(A)
    J, kind, k, s, flags, cdims, supp = _pack_cons(cons, dtype)
    p = PalmParams(nb_it, int(is_update_way_R2L), int(packing_RL), int(no_normalization), int(no_lambda),
                   norm2_threshold, norm2_max_iter, int(constant_step_size), step_size, int(no_lambda_error),
                   int(norm2_fp64))
    sizes = [c["rows"] * c["cols"] for c in cons]
    out = np.zeros(sum(sizes), dtype)
    init = None
    if init_facts is not None:
        init = np.ascontiguousarray(np.concatenate([np.asfortranarray(f, dtype=dtype).ravel(order="F")
                                                    for f in init_facts]))
    lam = ctypes.c_double()
    lambdas = np.zeros(max(nb_it, 1), np.float64)
    cvals = np.zeros(max(nb_it * J, 1), np.float64)
    niters = np.zeros(max(2 * nb_it * J, 1), np.int32)
    tcase = np.full(max(nb_it * J, 1), -1, np.int32)
    shash = np.zeros(max(nb_it * J, 1), np.uint64)
    snnz = np.zeros(max(nb_it * J, 1), np.int64)
    fn = lib().orc_palm4msa2_f64 if dtype == np.float64 else lib().orc_palm4msa2_f32
    _check(fn(_p(Af), A.shape[0], A.shape[1], J, _p(kind), _p(k), _p(s), _p(flags), _p(cdims), _p(supp),
              ctypes.byref(p), _p(init), ctypes.c_double(init_lambda), _p(out), ctypes.byref(lam), _p(lambdas),
              _p(cvals), _p(niters), _p(tcase), _p(shash), _p(snnz)))
    facts, off = [], 0
    for c, sz in zip(cons, sizes):
        facts.append(out[off:off + sz].reshape((c["rows"], c["cols"]), order="F"))
        off += sz
    return facts, lam.value, {"lambdas": lambdas[:nb_it], "c": cvals[:nb_it * J], "norm_iters": niters,
                               "topk_case": tcase[tcase >= 0], "supp_hash": shash[:nb_it * J],
                               "supp_nnz": snnz[:nb_it * J]}


def support_hash(M):
    """The oracle's support fingerprint of a dense matrix: the wrapping sum of
    splitmix64 of the column-major linear indices of its non-zero entries."""
    idx = np.flatnonzero(np.asarray(M).ravel(order="F") != 0).astype(np.uint64)
    with np.errstate(over="ignore"):
        z = idx + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return int(z.sum(dtype=np.uint64)), int(idx.size)


def rel_err(A, facts, lam, dtype=np.float64):
    """calc_rel_err (faust_palm4msa2020.hpp:35-44) evaluated in `dtype`
    (float64 or float32), the scalar type of the factorization."""
    Af = np.asfortranarray(A, dtype=dtype)
    cd = np.array(sum([[f.shape[0], f.shape[1]] for f in facts], []), np.int32)
    fl = np.ascontiguousarray(np.concatenate([np.asfortranarray(f, dtype=dtype).ravel(order="F")
                                              for f in facts]))
    out = ctypes.c_double()
    fn = lib().orc_rel_err_f64 if np.dtype(dtype) == np.float64 else lib().orc_rel_err_f32
    _check(fn(_p(Af), A.shape[0], A.shape[1], len(facts), _p(cd), _p(fl), ctypes.c_double(lam), ctypes.byref(out)))
    return out.value


def lambda_of_factors(A, facts, lam_in=1.0):
    """<A, S> / ||S||_F^2 with S the product of the dense factors `facts`, in
    A's dtype (lam_in when S is zero or NaN): the starting lambda of a seeded
    batched run."""
    dtype = A.dtype
    Af = np.asfortranarray(A)
    cd = np.array(sum([[f.shape[0], f.shape[1]] for f in facts], []), np.int32)
    fl = np.ascontiguousarray(np.concatenate([np.asfortranarray(f, dtype=dtype).ravel(order="F") for f in facts]))
    out = ctypes.c_double()
    fn = lib().orc_lambda_of_factors_f64 if dtype == np.float64 else lib().orc_lambda_of_factors_f32
    _check(fn(_p(Af), A.shape[0], A.shape[1], len(facts), _p(cd), _p(fl), ctypes.c_double(lam_in),
              ctypes.byref(out)))
    return out.value


def hierarchical(A, fac_cons, res_cons, its_2facts, its_global, is_fact_side_left=False, is_update_way_R2L=False,
                 **palm_kw):
    """Faust::hierarchical, 2020 version (src/algorithm/factorization/
    faust_hierarchical.hpp:1-121), composed from this oracle's palm4msa2.

    Step i splits the current residual (last factor, or first on the left
    side) with the constraints (fac_i, res_i) -- (res_i, fac_i) on the left --
    from the default start and lambda 1 (:42-97); the global lambda is
    multiplied by the local one (:99); the two factors replace the residual
    (:101-111); palm4msa2 refines all factors against A from them and the
    global lambda, with the constraints fac_0..fac_i, res_i in factor order
    (:114-121).  Returns (dense factors, lambda)."""
    A = np.asfortranarray(A)
    S = None
    glo = 1.0
    for i in range(len(fac_cons)):
        if i == 0:
            Si = A
        else:
            Si = np.asfortranarray(S[0] if is_fact_side_left else S[-1])
        lc = [res_cons[i], fac_cons[i]] if is_fact_side_left else [fac_cons[i], res_cons[i]]
        two, lam, _ = palm4msa2(Si, lc, its_2facts, is_update_way_R2L=is_update_way_R2L, init_lambda=1.0, **palm_kw)
        glo *= lam
        if i == 0:
            S = list(two)
        elif is_fact_side_left:
            S = list(two) + S[1:]
        else:
            S = S[:-1] + list(two)
        if is_fact_side_left:
            gc = [res_cons[i]] + [fac_cons[j] for j in range(i, -1, -1)]
        else:
            gc = [fac_cons[j] for j in range(i + 1)] + [res_cons[i]]
        S, glo, _ = palm4msa2(A, gc, its_global, is_update_way_R2L=is_update_way_R2L, init_facts=S,
                              init_lambda=glo, **palm_kw)
        S = list(S)
    return S, glo


# ---------------------------------------------------------------- dense product
def _csr(S):
    import scipy.sparse as sps
    S = sps.csr_matrix(S)
    S.sort_indices()
    return S


def _csr_op(S, op):
    """CSR of op(S); a transposed row lists entries by increasing original row."""
    return _csr(S) if op == "N" else _csr(_csr(S).T)


def _spmm(S, X):
    S = _csr(S)
    X = np.asfortranarray(X, dtype=S.dtype)
    Y = np.zeros((S.shape[0], X.shape[1]), S.dtype, order="F")
    fn = lib().orc_spmm_f64 if S.dtype == np.float64 else lib().orc_spmm_f32
    rp, ci = S.indptr.astype(np.int32), S.indices.astype(np.int32)
    _check(fn(S.shape[0], S.shape[1], _p(rp), _p(ci), _p(np.ascontiguousarray(S.data)), _p(X), X.shape[1], _p(Y)))
    return Y


def _dense_csrT(X, S):
    """Y = X S^T given the CSR of S: y[r, c] = sequential fma over row c of S."""
    S = _csr(S)
    X = np.asfortranarray(X, dtype=S.dtype)
    Y = np.zeros((X.shape[0], S.shape[0]), S.dtype, order="F")
    fn = lib().orc_dense_csrT_f64 if S.dtype == np.float64 else lib().orc_dense_csrT_f32
    rp, ci = S.indptr.astype(np.int32), S.indices.astype(np.int32)
    _check(fn(X.shape[0], _p(X), S.shape[0], S.shape[1], _p(rp), _p(ci), _p(np.ascontiguousarray(S.data)), _p(Y)))
    return Y


def _gemm_seq(A, B):
    A = np.asfortranarray(A)
    B = np.asfortranarray(B, dtype=A.dtype)
    C = np.zeros((A.shape[0], B.shape[1]), A.dtype, order="F")
    fn = lib().orc_gemm_seq_f64 if A.dtype == np.float64 else lib().orc_gemm_seq_f32
    _check(fn(A.shape[0], B.shape[1], A.shape[1], _p(A), _p(B), _p(C)))
    return C


def _w32(v):
    """C int arithmetic of the reference's cost model: two's complement wrap."""
    v &= 0xFFFFFFFF
    return v - (1 << 32) if v >= (1 << 31) else v


def _div32(a, b):
    if b == 0:
        return 0
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b > 0) else -q  # C division truncates toward zero


def dynprog_splits(leaves, op):
    """Split table of dynprog_multiply (src/faust_linear_operator/
    faust_prod_opt_gen.hpp:113-190) over the cost model of
    CPU/faust_prod_opt.cpp:1-80.  leaves: list of (rows, cols, nnz, dense)
    with stored dimensions.  Returns {(i, j): k}: leaves i..j multiply as
    (i..k)(k+1..j); k is the first minimiser (strict <)."""
    n = len(leaves)
    INT_MAX = 2 ** 31 - 1
    c = {(i, i): 0 for i in range(n)}
    split = {}
    tr = op != "N"
    for p in range(1, n):
        for i in range(n - p):
            j = p + i
            li, lj = leaves[i], leaves[j]
            best, arg = INT_MAX, None
            for k in range(i, j):
                rf_init = k + 1 == j
                cost = _w32(c[(i, k)] + c[(k + 1, j)])
                mf_ncols = leaves[k][1]
                if li[3] and lj[3]:
                    add = _w32(_w32(li[0] * mf_ncols) * (lj[0] if tr and rf_init else lj[1]))
                elif li[3]:
                    add = _w32((mf_ncols if tr and k == i else li[0]) * lj[2])
                elif lj[3]:
                    add = _w32(li[2] * (lj[0] if tr and rf_init else lj[1]))
                else:
                    add = _div32(_w32(li[2] * lj[2]), li[1] if tr else li[0])
                cost = _w32(cost + add)
                if cost < best:
                    best, arg = cost, k
            c[(i, j)] = best
            split[(i, j)] = i if arg is None else arg
    return split


def faust_product(factors, op="N", order=0, X=None):
    """Dense product of a Faust of CSR factors (TESTING ONLY).

    X None: TransformHelper::get_product (CPU/faust_TransformHelper.hpp:
    1132-1178); order 0 (DEFAULT_L2R) = Transform::get_product
    (CPU/faust_Transform.hpp:598-656): dense image of the last factor of
    op(F), then sparse x dense products right to left; order 5 (DYNPROG) =
    dynprog_multiply.  X given: op(F) X in the DYNPROG order
    (TransformHelper::multiply, CPU/faust_TransformHelper.hpp:373-379).
    Pairwise products: sparse x sparse = S x dense image; sparse x dense;
    dense x sparse through the CSR of the right operand's transpose; dense x
    dense with a sequential fma over k."""
    op = "N" if op in ("N", "n") else "T"
    facs = [_csr(f) for f in factors]
    J = len(facs)
    G = facs if op == "N" else facs[::-1]
    if X is None and (order == 0 or J == 1):
        if J == 1:
            return np.asfortranarray(_csr_op(G[0], op).toarray())
        cur = np.asfortranarray(_csr_op(G[-1], op).toarray())
        for q in range(J - 2, -1, -1):
            cur = _spmm(_csr_op(G[q], op), cur)
        return cur
    if order != 5:
        raise ValueError("only DEFAULT_L2R (0) and DYNPROG (5)")
    leaves = [(g.shape[0], g.shape[1], g.nnz, False) for g in G]
    ops = [op] * J
    data = list(G)
    last_op = op
    if X is not None:
        X = np.asfortranarray(X, dtype=facs[0].dtype)
        leaves.append((X.shape[0], X.shape[1], _w32(X.shape[0] * X.shape[1]), True))
        data.append(X)
        last_op = "N"
    n = len(leaves)
    split = dynprog_splits(leaves, op)

    def mult(L, opl, R, opr):
        lsp, rsp = not isinstance(L, np.ndarray), not isinstance(R, np.ndarray)
        if lsp:
            A = _csr_op(L, opl)
            D = np.asfortranarray(_csr_op(R, opr).toarray()) if rsp else R
            return _spmm(A, D)
        if rsp:
            return _dense_csrT(L, _csr_op(R, "T" if opr == "N" else "N"))
        return _gemm_seq(L, R)

    def rec(i, j):
        if i == j:
            return data[i]
        if j - i == 1:
            return mult(data[i], op, data[j], op if j < n - 1 else last_op)
        k = split[(i, j)]
        p1, p2 = rec(i, k), rec(k + 1, j)
        opl = op if i == k else "N"
        opr = (last_op if j == n - 1 else op) if k + 1 == j else "N"
        return mult(p1, opl, p2, opr)

    if n == 1:
        return _spmm(_csr_op(data[0], op), X)
    return rec(0, n - 1)
