"""palm4msa on the GPU, with the parameter surface of pyfaust.fact.palm4msa
(wrapper/python/pyfaust/fact.py:798-874, backend=2020) and its constraint
classes (wrapper/python/pyfaust/factparams.py: ConstraintInt :507,
ConstraintReal :709, ConstraintMat :582, ParamsPalm4MSA :1933-1959).

The returned Faust holds the factors S_0..S_{J-1} on the device; lambda is
returned beside it (pyfaust folds it into the first factor).
"""
import ctypes

import numpy as np

from . import _ffi
from ._ffi import check
from .faust import Faust, default_context

_KINDS = {"sp": _ffi.SP, "spcol": _ffi.SPCOL, "splin": _ffi.SPLIN, "splincol": _ffi.SPLINCOL,
          "normcol": _ffi.NORMCOL, "normlin": _ffi.NORMLIN, "supp": _ffi.SUPP, "sppos": _ffi.SP_POS}


class ConstraintGeneric:
    def __init__(self, name, num_rows, num_cols, cons_value, normalized, pos):
        if name not in _KINDS:
            raise ValueError("unsupported constraint %r" % (name,))
        self.name = name
        self.kind = _KINDS[name]
        self.shape = (int(num_rows), int(num_cols))
        self.cons_value = cons_value
        self.normalized = bool(normalized)
        self.pos = bool(pos)

    def _c(self, dtype, keep):
        k, s, supp = 0, 1.0, None
        if self.kind in (_ffi.NORMCOL, _ffi.NORMLIN):
            s = float(self.cons_value)
        elif self.kind == _ffi.SUPP:
            # one host copy per constraint object and dtype, so instances that
            # share a constraint share its device copy in batched runs
            cache = self.__dict__.setdefault("_supp_cache", {})
            key = np.dtype(dtype).str
            if key not in cache:
                cache[key] = np.asfortranarray(self.cons_value, dtype=dtype)
            a = cache[key]
            keep.append(a)
            supp = a.ctypes.data
        else:
            k = int(self.cons_value)
        return _ffi.Constraint(self.kind, self.shape[0], self.shape[1], k, s, int(self.normalized), int(self.pos),
                               supp)

    def oracle_dict(self):
        d = dict(kind=self.kind, rows=self.shape[0], cols=self.shape[1], normalized=self.normalized, pos=self.pos)
        if self.kind in (_ffi.NORMCOL, _ffi.NORMLIN):
            d["s"] = float(self.cons_value)
        elif self.kind == _ffi.SUPP:
            d["supp"] = np.asarray(self.cons_value)
        else:
            d["k"] = int(self.cons_value)
        return d


class ConstraintInt(ConstraintGeneric):
    """sp, spcol, splin, splincol, sppos; normalized=True by default."""

    def __init__(self, name, num_rows, num_cols, cons_value, normalized=True, pos=False):
        super().__init__(name, num_rows, num_cols, cons_value, normalized, pos)


class ConstraintReal(ConstraintGeneric):
    """normcol, normlin; normalized=False by default."""

    def __init__(self, name, num_rows, num_cols, cons_value, normalized=False, pos=False):
        super().__init__(name, num_rows, num_cols, cons_value, normalized, pos)


class ConstraintMat(ConstraintGeneric):
    """supp (cons_value = support matrix); normalized=True by default."""

    def __init__(self, name, cons_value, normalized=True, pos=False):
        cons_value = np.asarray(cons_value)
        super().__init__(name, cons_value.shape[0], cons_value.shape[1], cons_value, normalized, pos)


class ParamsPalm4MSA:
    def __init__(self, constraints, num_its=200, is_update_way_R2L=False, init_lambda=1.0, step_size=1e-16,
                 constant_step_size=False, init_facts=None, packing_RL=True, no_normalization=False, no_lambda=False,
                 norm2_max_iter=100, norm2_threshold=1e-6, norm2_fp64=False, no_lambda_error=False):
        self.constraints = list(constraints)
        self.num_its = int(num_its)
        self.is_update_way_R2L = is_update_way_R2L
        self.init_lambda = float(init_lambda)
        self.step_size = float(step_size)
        self.constant_step_size = constant_step_size
        self.init_facts = init_facts
        self.packing_RL = packing_RL
        self.no_normalization = no_normalization
        self.no_lambda = no_lambda
        self.norm2_max_iter = int(norm2_max_iter)
        self.norm2_threshold = float(norm2_threshold)
        self.norm2_fp64 = norm2_fp64
        self.no_lambda_error = no_lambda_error

    def _c(self):
        return _ffi.PalmParams(self.num_its, int(self.is_update_way_R2L), int(self.packing_RL),
                               int(self.no_normalization), int(self.no_lambda), self.norm2_threshold,
                               self.norm2_max_iter, int(self.constant_step_size), self.step_size,
                               int(self.no_lambda_error), int(self.norm2_fp64))


class PalmResult:
    def __init__(self, faust, lambda_):
        self.faust = faust
        self.lambda_ = lambda_


def palm4msa(M, constraints, params=None, ret_lambda=True, ctx=None):
    """Runs palm4msa2 on the GPU.  M: numpy array (host) or a column-major
    CUDA tensor.  Returns a PalmResult (faust, lambda_)."""
    ctx = ctx or default_context()
    if params is None:
        params = ParamsPalm4MSA(constraints)
    on_device = hasattr(M, "is_cuda") and M.is_cuda
    if on_device:
        import torch
        dtype = np.float64 if M.dtype == torch.float64 else np.float32
        rows, cols = M.shape
        Mc = M if (M.stride(0) == 1 and (cols == 1 or M.stride(1) == rows)) else M.t().contiguous().t()
    else:
        dtype = np.dtype(M.dtype)
        if dtype not in (np.float32, np.float64):
            dtype = np.dtype(np.float64)
        Mc = np.asfortranarray(M, dtype=dtype)
        rows, cols = Mc.shape
    code = _ffi.F64 if dtype == np.float64 else _ffi.F32
    keep = []
    J = len(constraints)
    cons = (_ffi.Constraint * J)()
    for i, c in enumerate(constraints):
        cons[i] = c._c(dtype, keep)
    init = None
    if params.init_facts is not None:
        arrs = [np.asfortranarray(f, dtype=dtype) for f in params.init_facts]
        keep += arrs
        init = (ctypes.c_void_p * J)(*[a.ctypes.data for a in arrs])
    p = params._c()
    lam = ctypes.c_double(params.init_lambda)
    h = ctypes.c_void_p()
    if on_device:
        st = _ffi.lib().fgb_palm4msa2_device(ctx.handle, code, Mc.data_ptr(), rows, cols, J, cons, ctypes.byref(p),
                                             init, ctypes.byref(lam), ctypes.byref(h))
    else:
        st = _ffi.lib().fgb_palm4msa2(ctx.handle, code, Mc.ctypes.data, rows, cols, J, cons, ctypes.byref(p), init,
                                      ctypes.byref(lam), ctypes.byref(h))
    check(st, ctx.handle)
    F = Faust._from_handle(h, ctx, dtype)
    return PalmResult(F, lam.value)


class ParamsHierarchical:
    """pyfaust.factparams.ParamsHierarchical: fact_constraints[i] and
    res_constraints[i] split the residual at step i; stop_crit1 (iterations
    of each two-factor palm4msa2), stop_crit2 (iterations of each global
    palm4msa2); the rest as ParamsPalm4MSA."""

    def __init__(self, fact_constraints, res_constraints, stop_crit1, stop_crit2, is_update_way_R2L=False,
                 init_lambda=1.0, step_size=1e-16, constant_step_size=False, is_fact_side_left=False,
                 packing_RL=True, no_normalization=False, no_lambda=False, norm2_max_iter=100,
                 norm2_threshold=1e-6, norm2_fp64=False):
        if len(fact_constraints) != len(res_constraints):
            raise ValueError("fact_constraints and res_constraints must have the same length")
        self.fact_constraints = list(fact_constraints)
        self.res_constraints = list(res_constraints)
        self.is_fact_side_left = is_fact_side_left

        def mk(its):
            return ParamsPalm4MSA([], int(its), is_update_way_R2L=is_update_way_R2L, init_lambda=init_lambda,
                                  step_size=step_size, constant_step_size=constant_step_size, packing_RL=packing_RL,
                                  no_normalization=no_normalization, no_lambda=no_lambda,
                                  norm2_max_iter=norm2_max_iter, norm2_threshold=norm2_threshold,
                                  norm2_fp64=norm2_fp64)
        self.params_2facts = mk(stop_crit1)
        self.params_global = mk(stop_crit2)


def hierarchical(M, p, ret_lambda=True, ctx=None):
    """hierarchical (2020 backend) on the GPU: Faust::hierarchical.  M: numpy
    array (host).  Returns a PalmResult (faust with len(fact_constraints) + 1
    factors, lambda_)."""
    ctx = ctx or default_context()
    dtype = np.dtype(M.dtype)
    if dtype not in (np.float32, np.float64):
        dtype = np.dtype(np.float64)
    Mc = np.asfortranarray(M, dtype=dtype)
    rows, cols = Mc.shape
    n = len(p.fact_constraints)
    keep = []
    fc = (_ffi.Constraint * n)()
    rc = (_ffi.Constraint * n)()
    for i in range(n):
        fc[i] = p.fact_constraints[i]._c(dtype, keep)
        rc[i] = p.res_constraints[i]._c(dtype, keep)
    p2, pg = p.params_2facts._c(), p.params_global._c()
    lam = ctypes.c_double(1.0)
    h = ctypes.c_void_p()
    check(_ffi.lib().fgb_hierarchical(ctx.handle, _ffi.F64 if dtype == np.float64 else _ffi.F32, Mc.ctypes.data, rows,
                                      cols, n, fc, rc, ctypes.byref(p2), ctypes.byref(pg), int(p.is_fact_side_left),
                                      ctypes.byref(lam), ctypes.byref(h)), ctx.handle)
    return PalmResult(Faust._from_handle(h, ctx, dtype), lam.value)


def palm4msa_batched(problems, params, ctx=None, ctas_per_sm=0, init_values=None, values_scale=1.0,
                     lambda_from_init=False):
    """Runs many palm4msa2 instances in one persistent launch.

    problems: list of (M, constraints[, init_facts]) with M a column-major
    CUDA tensor (float32 or float64, all the same dtype).  params: one
    ParamsPalm4MSA for every instance (its constraints are ignored).
    init_values: optional CUDA tensor (instances x values) of starting values
    on the SUPP supports shared by every instance (factor by factor, row-major
    order), multiplied by values_scale; lambda_from_init starts each instance
    from the optimal scale <M, S> / ||S||^2 of its starting factors.
    ctas_per_sm = 0 takes the tuned table's choice for the batch.
    Returns a list of PalmResult; an instance that failed carries .status."""
    import torch
    ctx = ctx or default_context()
    n = len(problems)
    dtype = np.float64 if problems[0][0].dtype == torch.float64 else np.float32
    keep = []
    arr = (_ffi.PalmProblem * n)()
    for i, prob in enumerate(problems):
        M, cons = prob[0], prob[1]
        init = prob[2] if len(prob) > 2 else None
        rows, cols = M.shape
        if not (M.is_cuda and M.stride(0) == 1 and (cols == 1 or M.stride(1) == rows)):
            raise ValueError("instance %d: M must be a column-major CUDA tensor" % i)
        ca = (_ffi.Constraint * len(cons))()
        for f, c in enumerate(cons):
            ca[f] = c._c(dtype, keep)
        keep.append(ca)
        ip = None
        if init is not None:
            arrs = [np.asfortranarray(x, dtype=dtype) for x in init]
            keep += arrs
            ip = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
            keep.append(ip)
        arr[i] = _ffi.PalmProblem(rows, cols, M.data_ptr(), len(cons), ca, ip, float(params.init_lambda))
    out = (_ffi.PalmResultC * n)()
    p = params._c()
    if not ctas_per_sm:
        ctas_per_sm = tuned_ctas_per_sm(max(max(p[0].shape) for p in problems), len(problems), dtype)
    vals, nv = None, 0
    if init_values is not None:
        tdt = torch.float64 if dtype == np.float64 else torch.float32
        if not (init_values.is_cuda and init_values.dtype == tdt and init_values.shape[0] == n
                and init_values.is_contiguous()):
            raise ValueError("init_values: a contiguous (instances x values) CUDA tensor of the run's dtype")
        vals, nv = init_values.data_ptr(), int(init_values.shape[1])
    opts = _ffi.BatchOpts(int(ctas_per_sm), vals, nv, float(values_scale), int(bool(lambda_from_init)))
    check(_ffi.lib().fgb_palm4msa2_batched(ctx.handle, _ffi.F64 if dtype == np.float64 else _ffi.F32, n, arr,
                                           ctypes.byref(p), ctypes.byref(opts), out), ctx.handle)
    results = []
    for i in range(n):
        F = Faust._from_handle(ctypes.c_void_p(out[i].faust), ctx, dtype)
        r = PalmResult(F, out[i].lambda_)
        r.status = out[i].status
        r.cycles = out[i].cycles
        results.append(r)
    return results


def tuned_ctas_per_sm(maxdim, count, dtype):
    """Resident instances per SM for a batched launch, from the table the
    offline sweep wrote (faust_gb300/tuning/batched_palm.json, keyed by the
    batch's largest dimension); 2 when no entry covers the batch."""
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning", "batched_palm.json")
    try:
        with open(path) as f:
            table = json.load(f)
    except OSError:
        return 2
    key = "f64" if np.dtype(dtype) == np.float64 else "f32"
    best = None
    for e in table.get(key, []):
        if maxdim <= e["maxdim"] and (best is None or e["maxdim"] < best["maxdim"]):
            best = e
    return int(best["ctas_per_sm"]) if best else 2


def prox(M, constraint, ctx=None):
    """In-place projection of a column-major CUDA tensor M (ConstraintGeneric
    project).  Returns M."""
    import torch
    ctx = ctx or default_context()
    rows, cols = M.shape
    assert M.is_cuda and (M.stride(0) == 1 and (cols == 1 or M.stride(1) == rows))
    dtype = np.float64 if M.dtype == torch.float64 else np.float32
    keep = []
    c = constraint._c(dtype, keep)
    check(_ffi.lib().fgb_prox(ctx.handle, _ffi.F64 if dtype == np.float64 else _ffi.F32, ctypes.byref(c),
                              M.data_ptr()), ctx.handle)
    return M
