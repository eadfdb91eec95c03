"""The C-ABI library builds, loads without a GPU and exports its header."""
import ctypes
import os
import re

import numpy as np

from lpm_cases import pkg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "lpm_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lpm_[A-Za-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    path = pkg.build.build()
    L = ctypes.CDLL(path)
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(pkg.capi.exported_symbols()) <= set(names)


def test_bad_arguments_are_rejected_before_any_device_work():
    L = pkg.capi.load()
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    h = ctypes.c_void_p()
    xyz = np.zeros((2, 3))
    xyz[1, 0] = 1.0
    p1 = np.array([0], np.int32)
    p2 = np.array([1], np.int32)
    lay = np.array([0], np.int32)
    kn = np.ones(1)
    tv = np.zeros(1)
    args = lambda a: a.ctypes.data_as(dp if a.dtype == np.float64 else ip)
    # a bond 0 -> 1 without 1 -> 0
    st = L.lpm_create(2, 2, 1, args(xyz), args(p1), args(p2), args(lay), args(kn), args(tv), 1.0, 12, ctypes.byref(h))
    assert st == pkg.capi.ERR_TOPOLOGY and not h.value
    assert b"opposite" in L.lpm_last_error(None)
    # particle id out of range
    p2b = np.array([5], np.int32)
    st = L.lpm_create(2, 2, 1, args(xyz), args(p1), args(p2b), args(lay), args(kn), args(tv), 1.0, 12, ctypes.byref(h))
    assert st == pkg.capi.ERR_ARG
    # bad dimension
    st = L.lpm_create(4, 2, 1, args(xyz), args(p1), args(p2), args(lay), args(kn), args(tv), 1.0, 12, ctypes.byref(h))
    assert st == pkg.capi.ERR_ARG
    # NULL handle calls
    assert L.lpm_update_geometry_force(None) == pkg.capi.ERR_ARG


def handle_entry_points():
    """Entry points of the header whose first parameter is the handle."""
    text = open(os.path.join(ROOT, "include", "lpm_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lpm_[A-Za-z0-9_]+)\s*\(\s*(?:const\s+)?lpm_handle\s*\*", text)))


def test_every_handle_entry_point_rejects_a_null_handle():
    """Each entry point tests its handle before anything else, so a NULL
    handle returns LPM_ERR_ARG (lpm_destroy: a no-op; lpm_last_error: the
    library-wide message) and no other argument is read.  A CDLL of its own
    gives function objects without the binding's argument types."""
    pkg.capi.load()
    L = ctypes.CDLL(pkg.build.build())
    names = handle_entry_points()
    assert len(names) >= 40
    for name in names:
        fn = getattr(L, name)
        if name == "lpm_last_error":
            fn.restype = ctypes.c_char_p
            assert isinstance(fn(None), bytes)
        elif name == "lpm_destroy":
            assert fn(None) == pkg.capi.OK
        else:
            fn.restype = ctypes.c_int
            assert fn(None) == pkg.capi.ERR_ARG, name
