"""ctypes binding of the C ABI in include/fgb.h (libfaust_gb300.so).

The library is built in-tree by faust_gb300/build.py.  There is no CPU
fallback: when the shared library is missing or cannot be loaded every entry
point raises, so a missing CUDA build fails loudly.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libfaust_gb300.so")

FGB_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA", 4: "NAN", 5: "ZERO_NORM", 6: "CANCELLED",
                7: "TIMEOUT", 8: "NOT_SUPPORTED"}
F32, F64, BF16 = 0, 1, 2
CSR, BSR = 0, 1
ORDER_DEFAULT_L2R, ORDER_DYNPROG = 0, 5
# Constraint kinds (fgb_cons_kind).
SP, SPCOL, SPLIN, SPLINCOL, NORMCOL, NORMLIN, SUPP, SP_POS = range(8)


class FactorDesc(ctypes.Structure):
    _fields_ = [("format", ctypes.c_int), ("rows", ctypes.c_int), ("cols", ctypes.c_int), ("nnz", ctypes.c_int),
                ("bm", ctypes.c_int), ("bn", ctypes.c_int), ("rowptr", ctypes.c_void_p),
                ("colind", ctypes.c_void_p), ("values", ctypes.c_void_p)]


class Constraint(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("rows", ctypes.c_int), ("cols", ctypes.c_int), ("k", ctypes.c_longlong),
                ("s", ctypes.c_double), ("normalized", ctypes.c_int), ("pos", ctypes.c_int),
                ("supp", ctypes.c_void_p)]


class PalmParams(ctypes.Structure):
    _fields_ = [("nb_it", ctypes.c_int), ("is_update_way_R2L", ctypes.c_int), ("packing_RL", ctypes.c_int),
                ("no_normalization", ctypes.c_int), ("no_lambda", ctypes.c_int),
                ("norm2_threshold", ctypes.c_double), ("norm2_max_iter", ctypes.c_int),
                ("constant_step_size", ctypes.c_int), ("step_size", ctypes.c_double),
                ("no_lambda_error", ctypes.c_int), ("norm2_fp64", ctypes.c_int)]


class PalmProblem(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int), ("cols", ctypes.c_int), ("A", ctypes.c_void_p), ("nfacts", ctypes.c_int),
                ("cons", ctypes.POINTER(Constraint)), ("init_facts", ctypes.POINTER(ctypes.c_void_p)),
                ("init_lambda", ctypes.c_double)]


class PalmResultC(ctypes.Structure):
    _fields_ = [("faust", ctypes.c_void_p), ("lambda_", ctypes.c_double), ("status", ctypes.c_int),
                ("cycles", ctypes.c_longlong)]


class BatchOpts(ctypes.Structure):
    _fields_ = [("ctas_per_sm", ctypes.c_int), ("init_values", ctypes.c_void_p),
                ("values_per_instance", ctypes.c_int), ("init_values_scale", ctypes.c_double),
                ("lambda_from_init", ctypes.c_int)]


class FgbError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


_lib = None

# name -> (restype, argtypes)
_P, _I, _D, _LL = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_longlong
_SIGS = {
    "fgb_ctx_create": (_I, [_I, _P, ctypes.POINTER(_P)]),
    "fgb_ctx_destroy": (_I, [_P]),
    "fgb_last_error": (ctypes.c_char_p, [_P]),
    "fgb_ctx_synchronize": (_I, [_P]),
    "fgb_cancel": (_I, [_P]),
    "fgb_ctx_kernel_launches": (_LL, [_P]),
    "fgb_faust_create": (_I, [_P, _I, _I, ctypes.POINTER(FactorDesc), ctypes.POINTER(_P)]),
    "fgb_faust_destroy": (_I, [_P]),
    "fgb_faust_shape": (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "fgb_faust_mul": (_I, [_P, _P, _I, _I, _P, _I, _I]),
    "fgb_faust_mul_op": (_I, [_P, ctypes.c_char, _P, _I, _I, _P, _I, _I]),
    "fgb_faust_product": (_I, [_P, ctypes.c_char, _I, _P, _I]),
    "fgb_faust_mul_dynprog": (_I, [_P, ctypes.c_char, _P, _I, _I, _P, _I]),
    "fgb_dynprog_plan": (_I, [_I, _P, _P, _P, _P, ctypes.c_char, _P]),
    "fgb_faust_mul_host": (_I, [_P, _P, _I, _P]),
    "fgb_faust_spectral_norm": (_I, [_P, _I, _D, ctypes.POINTER(_D), ctypes.POINTER(_I)]),
    "fgb_faust_factor_info": (_I, [_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                                   ctypes.POINTER(_I)]),
    "fgb_faust_factor_to_dense": (_I, [_P, _I, _P]),
    "fgb_faust_factor_to_csr": (_I, [_P, _I, _P, _P, _P]),
    "fgb_faust_factor_to_bsr": (_I, [_P, _I, _P, _P, _P]),
    "fgb_prox": (_I, [_P, _I, ctypes.POINTER(Constraint), _P]),
    "fgb_prox_noalloc": (_I, [_P, _I, ctypes.POINTER(Constraint), _P, _P]),
    "fgb_palm_params_default": (_I, [ctypes.POINTER(PalmParams)]),
    "fgb_palm4msa2": (_I, [_P, _I, _P, _I, _I, _I, ctypes.POINTER(Constraint), ctypes.POINTER(PalmParams),
                           ctypes.POINTER(_P), ctypes.POINTER(_D), ctypes.POINTER(_P)]),
    "fgb_palm4msa2_device": (_I, [_P, _I, _P, _I, _I, _I, ctypes.POINTER(Constraint),
                                  ctypes.POINTER(PalmParams), ctypes.POINTER(_P), ctypes.POINTER(_D),
                                  ctypes.POINTER(_P)]),
    "fgb_rel_err": (_I, [_P, _P, _D, ctypes.POINTER(_D)]),
    "fgb_hierarchical": (_I, [_P, _I, _P, _I, _I, _I, ctypes.POINTER(Constraint), ctypes.POINTER(Constraint),
                              ctypes.POINTER(PalmParams), ctypes.POINTER(PalmParams), _I, ctypes.POINTER(_D),
                              ctypes.POINTER(_P)]),
    "fgb_palm4msa2_batched": (_I, [_P, _I, _I, ctypes.POINTER(PalmProblem), ctypes.POINTER(PalmParams),
                                   ctypes.POINTER(BatchOpts), ctypes.POINTER(PalmResultC)]),
    # include/fgb_diag.h
    "fgb_probe_fp64_fma": (_I, [_P, ctypes.POINTER(_D)]),
    # include/fgb_mlp.h
    "fgb_gemm_bf16": (_I, [_P, _I, _I, _I, _P, ctypes.c_long, _P, ctypes.c_long, _P, ctypes.c_long, _I, _P, _I, _I,
                           _P]),
    "fgb_mlp_transpose_bf16": (_I, [_P, _I, _I, _P, ctypes.c_long, _P, ctypes.c_long]),
    "fgb_mlp_relu_grad": (_I, [_P, ctypes.c_long, _P, _P, _P]),
    "fgb_mlp_colsum": (_I, [_P, _I, _I, _P, ctypes.c_long, _P]),
    "fgb_mlp_mse_grad": (_I, [_P, ctypes.c_long, _P, _P, ctypes.c_float, _P, _P]),
    "fgb_mlp_adam": (_I, [_P, ctypes.c_long, _P, _P, _P, _P, _P, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                          ctypes.c_float, _I]),
    "fgb_mlp_f32_to_bf16": (_I, [_P, ctypes.c_long, _P, _P]),
    "fgb_mlp_bf16_to_f32": (_I, [_P, ctypes.c_long, _P, _P]),
}


def exported_symbols():
    """Entry points declared by include/fgb.h (the ones bound here)."""
    return sorted(_SIGS)


def lib():
    """Loads libfaust_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libfaust_gb300.so is not built (run faust_gb300/build.py or __graft_entry__.build())")
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def check(status, ctx=None):
    if status != FGB_OK:
        msg = lib().fgb_last_error(ctx).decode() if ctx else ""
        raise FgbError(status, msg)
