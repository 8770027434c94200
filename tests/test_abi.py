"""CPU checks of the C ABI: the library loads and exports every entry point
that include/fgb.h declares (no compute call: there may be no GPU here)."""
import os
import re

from faust_gb300 import _ffi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"^\s*(?:fgb_status|const char\*|long long|int|void)\s+(fgb_\w+)\s*\(", txt,
                                    re.M))
    return names


def test_library_exports_every_declared_symbol():
    lib = _ffi.lib()
    declared = _declared()
    assert len(declared) >= 20
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert _declared() <= set(_ffi.exported_symbols())


def test_ctx_create_without_gpu_fails_cleanly():
    import ctypes
    try:
        import torch
        if torch.cuda.is_available():
            return
    except Exception:
        pass
    h = ctypes.c_void_p()
    st = _ffi.lib().fgb_ctx_create(0, None, ctypes.byref(h))
    assert st != 0 and not h.value


def test_params_default_mirror_reference():
    p = _ffi.PalmParams()
    assert _ffi.lib().fgb_palm_params_default(p) == 0
    # palm4msa2 defaults (faust_palm4msa2020.h:45-72, pyfaust ParamsPalm4MSA)
    assert p.is_update_way_R2L == 0 and p.packing_RL == 1 and p.norm2_max_iter == 100
    assert abs(p.norm2_threshold - 1e-6) < 1e-18 and p.no_normalization == 0 and p.no_lambda == 0


def test_tuned_ctas_per_sm_table_lookup():
    """fact.tuned_ctas_per_sm reads the sweep's table: the entry of the
    smallest size bucket that covers the batch's largest dimension, 2 when no
    bucket covers it or the table is missing."""
    import json
    import numpy as np
    from faust_gb300 import fact
    with open(os.path.join(ROOT, "faust_gb300", "tuning", "batched_palm.json")) as f:
        table = json.load(f)
    buckets = sorted(table["f32"], key=lambda e: e["maxdim"])
    assert buckets and all(1 <= e["ctas_per_sm"] <= 3 for e in buckets)
    for e in buckets:
        assert fact.tuned_ctas_per_sm(e["maxdim"], 512, np.float32) == e["ctas_per_sm"]
    assert fact.tuned_ctas_per_sm(buckets[0]["maxdim"] - 1, 512, np.float32) == buckets[0]["ctas_per_sm"]
    assert fact.tuned_ctas_per_sm(buckets[-1]["maxdim"] + 1, 512, np.float32) == 2
    assert fact.tuned_ctas_per_sm(64, 512, np.float64) == 2  # no FP64 entries
