"""The C ABI library loads and exports every function include/hsr_gb300.h declares,
and the ctypes mirrors have the header's struct sizes. No compute calls (no GPU here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "hsr_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hsr_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("hsr_scene_create", "hsr_backend_run", "hsr_simulate_batch", "hsr_simulate_batch_device",
                 "hsr_intersect", "hsr_visible", "hsr_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(product_lib):
    missing = [n for n in declared_functions() if not hasattr(product_lib, n)]
    assert not missing, missing


def test_struct_layouts():
    from hussar_gb300 import _lib
    assert ctypes.sizeof(_lib.RFConfigC) == 24
    assert ctypes.sizeof(_lib.FrameConfigC) == 12
    assert ctypes.sizeof(_lib.AntennaC) == 48
    assert ctypes.sizeof(_lib.FlagsC) == 11 * 4 + 3 * 4


def test_default_flags_match_reference(product_lib):
    from hussar_gb300 import _lib, PathTracer
    f = _lib.FlagsC()
    product_lib.hsr_default_flags(ctypes.byref(f))
    t = PathTracer()
    for name, _ in _lib.FlagsC._fields_:
        assert getattr(f, name) == pytest.approx(float(getattr(t, name))), name


def test_no_device_reports_error_not_fallback(product_lib):
    """Without a GPU the library refuses to compute (no CPU fallback)."""
    import numpy as np
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    from hussar_gb300 import _lib
    h = ctypes.c_void_p()
    v = np.zeros((3, 3), np.float32)
    i = np.array([[0, 1, 2]], np.int32)
    st = product_lib.hsr_scene_create(_lib.ptr(v), 3, _lib.ptr(i), 1, ctypes.byref(h))
    assert st == _lib.HSR_ERR_NO_DEVICE


def test_invalid_indices_rejected_before_device(product_lib):
    import numpy as np
    from hussar_gb300 import _lib
    h = ctypes.c_void_p()
    v = np.zeros((3, 3), np.float32)
    i = np.array([[0, 1, 3]], np.int32)
    st = product_lib.hsr_scene_create(_lib.ptr(v), 3, _lib.ptr(i), 1, ctypes.byref(h))
    assert st == _lib.HSR_ERR_INVALID_ARGUMENT
    assert b"outside" in product_lib.hsr_last_error()


def test_build_setters_validate_without_device(product_lib):
    """The process-wide BVH settings check their range before anything else."""
    from hussar_gb300 import _lib
    for bad in (0, 9, -1):
        assert product_lib.hsr_set_bvh_leaf_size(bad) == _lib.HSR_ERR_INVALID_ARGUMENT
    assert product_lib.hsr_set_bvh_builder(2) == _lib.HSR_ERR_INVALID_ARGUMENT
    for bad in (-1, 65):
        assert product_lib.hsr_set_bvh_optimize(bad) == _lib.HSR_ERR_INVALID_ARGUMENT
    assert product_lib.hsr_set_bvh_optimize(32) == _lib.HSR_OK
    for good in (1, 8, 4):  # ends at the default
        assert product_lib.hsr_set_bvh_leaf_size(good) == _lib.HSR_OK


def test_sincos_sweep_validates_without_device(product_lib):
    from hussar_gb300 import _lib
    n = ctypes.c_int64()
    for lo, hi in ((1.0, 0.5), (-1.0, 1.0), (0.0, float("inf")), (float("nan"), 1.0)):
        assert product_lib.hsr_debug_sincos_sweep(lo, hi, ctypes.byref(n), ctypes.byref(n),
                                                  ctypes.byref(n)) == _lib.HSR_ERR_INVALID_ARGUMENT


def test_abi_version_matches_the_mirrors(product_lib):
    """The header's HSR_ABI_VERSION, the library's and the ctypes mirrors' agree."""
    from hussar_gb300 import _lib
    src = open(os.path.join(ROOT, "include", "hsr_gb300.h")).read()
    m = re.search(r"#define HSR_ABI_VERSION (\d+)", src)
    assert m and int(m.group(1)) == _lib.ABI_VERSION == product_lib.hsr_abi_version()
