"""faust_gb300 — FAuST's Faust x dense product and palm4msa2 factor update,
rebuilt for one GB300 (sm_103a) behind the C ABI of include/fgb.h.

Python API (mirrors pyfaust):
  Faust(factors)            device-resident product of CSR / BSR factors
  F @ X                     Faust x dense (host arrays or CUDA tensors)
  F.norm(2)                 FP64 power-iteration 2-norm
  F.save(path) / Faust.load(path)  MAT5 'faust_factors' files
  fact.palm4msa(M, cons, params)   palm4msa2 on the GPU
  fact.hierarchical(M, params)     hierarchical factorization (PALM chain)
  proj.sp / splincol / ...  constraint descriptions
"""
from . import _ffi
from .faust import BSRFactor, Context, Faust, default_context

__all__ = ["Faust", "BSRFactor", "Context", "default_context", "lib_path", "load"]

lib_path = _ffi.LIB_PATH


def load():
    """Loads the CUDA library; raises when it is missing (no CPU fallback)."""
    return _ffi.lib()
