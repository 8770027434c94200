"""fgb_prox_noalloc: the projection for callers that cannot allocate device
memory (applications that reserve all GPU memory up front, loops that must
not reach cudaMalloc / cudaFree because those can synchronise the device).
It must give the same result as the allocating entry point fgb_prox, call
after call, although its scratch is one fixed device array that keeps
whatever the previous call left.

This file is collected last on purpose: a failure here stops a -x run only
after every other test has run."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(name, ctx, dtype_code, cons, M, supp=None):
    from faust_gb300 import _ffi
    lib = _ffi.lib()
    if name == "fgb_prox":
        st = lib.fgb_prox(ctx.handle, dtype_code, ctypes.byref(cons), M.data_ptr())
    else:
        st = lib.fgb_prox_noalloc(ctx.handle, dtype_code, ctypes.byref(cons), M.data_ptr(),
                                  supp.data_ptr() if supp is not None else None)
    _ffi.check(st, ctx.handle)


def _cases(rng):
    """(dtype, kind, rows, cols, k, s, matrix) covering the top-k paths:
    unique thresholds, ties decided by the prefix rule and by the heap replay
    (on-chip and, for large k, in the scratch array), per-line selection,
    column norms and supports."""
    from faust_gb300 import _ffi
    ties = lambda r, c, lv: rng.integers(-lv, lv + 1, size=(r, c)).astype(np.float64) / 8.0
    return [
        (np.float64, _ffi.SP, 256, 128, 1000, 1.0, ties(256, 128, 3)),
        (np.float64, _ffi.SP, 1024, 64, 30000, 1.0, ties(1024, 64, 2)),
        (np.float32, _ffi.SP, 300, 200, 777, 1.0, rng.standard_normal((300, 200))),
        (np.float32, _ffi.SPLINCOL, 128, 96, 4, 1.0, ties(128, 96, 2)),
        (np.float64, _ffi.NORMCOL, 64, 80, 0, 2.0, rng.standard_normal((64, 80))),
        (np.float64, _ffi.SUPP, 40, 60, 0, 1.0, rng.standard_normal((40, 60))),
        # pos clamping before the selection, and the normalisation, whose
        # partial sums sit in the scratch array
        (np.float64, _ffi.SP_POS, 200, 150, 500, 1.0, ties(200, 150, 3)),
        (np.float32, _ffi.SPCOL, 96, 70, 5, 1.0, ties(96, 70, 2)),
        (np.float64, _ffi.SPLIN, 50, 300, 7, 1.0, rng.standard_normal((50, 300))),
    ]


def test_noalloc_matches_fgb_prox_on_consecutive_calls():
    import torch
    import faust_gb300 as fg
    from faust_gb300 import _ffi
    ctx = fg.Context(0)
    rng = np.random.default_rng(2024)
    for rep in range(2):  # two rounds of calls in a row over the shared scratch
        for dtype, kind, rows, cols, k, s, M in _cases(rng):
            tdt = torch.float64 if dtype == np.float64 else torch.float32
            code = _ffi.F64 if dtype == np.float64 else _ffi.F32
            supp_h = (rng.random((rows, cols)) < 0.3).astype(dtype)
            supp_f = np.asfortranarray(supp_h)
            cons = _ffi.Constraint(kind, rows, cols, k, s, 1, 0, supp_f.ctypes.data if kind == _ffi.SUPP else None)
            a = torch.from_numpy(np.ascontiguousarray(M.astype(dtype).T)).cuda().t()
            b = a.clone()
            _call("fgb_prox", ctx, code, cons, a)
            supp_d = torch.from_numpy(np.ascontiguousarray(supp_h.T)).cuda().t() if kind == _ffi.SUPP else None
            _call("fgb_prox_noalloc", ctx, code, cons, b, supp_d)
            torch.cuda.synchronize()
            # same kernels and operation order: identical results (tolerance 0)
            assert torch.equal(a, b), (rep, kind, rows, cols, k)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch
    import faust_gb300 as fg
    from faust_gb300 import _ffi
    ctx = fg.Context(0)
    M = torch.zeros((4096, 2048), device="cuda", dtype=torch.float32).t()
    cons = _ffi.Constraint(_ffi.SP, 2048, 4096, 10, 1.0, 0, 0, None)
    st = _ffi.lib().fgb_prox_noalloc(ctx.handle, _ffi.F32, ctypes.byref(cons), M.data_ptr(), None)
    assert st == 1 and b"exceeds the fixed scratch" in _ffi.lib().fgb_last_error(ctx.handle)
    # rows + cols above 65536 with few entries
    M1 = torch.zeros((65536, 1), device="cuda", dtype=torch.float32).t()
    cons = _ffi.Constraint(_ffi.SPLIN, 1, 65536, 4, 1.0, 0, 0, None)
    st = _ffi.lib().fgb_prox_noalloc(ctx.handle, _ffi.F32, ctypes.byref(cons), M1.data_ptr(), None)
    assert st == 1 and b"exceeds the fixed scratch" in _ffi.lib().fgb_last_error(ctx.handle)
    # sp with k above the replay heap (k < rows * cols)
    M2 = torch.zeros((512, 512), device="cuda", dtype=torch.float64).t()
    for kind in (_ffi.SP, _ffi.SP_POS):
        cons = _ffi.Constraint(kind, 512, 512, 65537, 1.0, 0, 0, None)
        st = _ffi.lib().fgb_prox_noalloc(ctx.handle, _ffi.F64, ctypes.byref(cons), M2.data_ptr(), None)
        assert st == 1 and b"exceeds the fixed scratch" in _ffi.lib().fgb_last_error(ctx.handle)
    # the rejected calls left nothing behind: a valid call still matches fgb_prox
    rng = np.random.default_rng(7)
    M = rng.standard_normal((64, 48))
    a = torch.from_numpy(np.ascontiguousarray(M.T)).cuda().t()
    b = a.clone()
    cons = _ffi.Constraint(_ffi.SP, 64, 48, 100, 1.0, 1, 0, None)
    _call("fgb_prox", ctx, _ffi.F64, cons, a)
    _call("fgb_prox_noalloc", ctx, _ffi.F64, cons, b)
    torch.cuda.synchronize()
    assert torch.equal(a, b)


def test_noalloc_restores_the_current_device():
    import torch
    import faust_gb300 as fg
    from faust_gb300 import _ffi
    ctx = fg.Context(0)
    before = torch.cuda.current_device()
    M = torch.from_numpy(np.ascontiguousarray(np.random.default_rng(3).standard_normal((32, 16)).T)).cuda().t()
    cons = _ffi.Constraint(_ffi.SP, 32, 16, 40, 1.0, 1, 0, None)
    _call("fgb_prox_noalloc", ctx, _ffi.F64, cons, M)
    assert torch.cuda.current_device() == before
