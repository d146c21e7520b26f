"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/mhd_gb300.h declares.  No GPU work is issued here."""
import ctypes
import os
import re

import pytest

from code_tohoku_gb300 import build, native
from code_tohoku_gb300.problems import MhdParams

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"^\s*(?:int|long long|void|double)\s+\**(mhd_\w+)\s*\(", txt, re.M))
    return names


def test_library_exports_header_symbols():
    lib = build.build()
    L = ctypes.CDLL(lib)
    names = declared_symbols()
    assert names >= set(native.EXPORTS)
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_binary_targets_sm103a():
    lib = build.build()
    data = open(lib, "rb").read()
    assert b"sm_103a" in data or b"sm_103" in data


def test_create_rejects_bad_arguments():
    L = native.load()
    h = ctypes.c_void_p()
    p = native.params_struct(MhdParams(8, 8, 8, bc=(3, 3, 3, 3, 3, 2)))
    assert L.mhd_create(ctypes.byref(p), ctypes.byref(h)) == 1   # MHD_ERR_ARG: BC code 2
    p = native.params_struct(MhdParams(2, 8, 8))
    assert L.mhd_create(ctypes.byref(p), ctypes.byref(h)) == 1   # grid too small
    assert L.mhd_create(None, ctypes.byref(h)) == 1
    p = native.params_struct(MhdParams(8, 8, 8, ifchem=1))
    assert L.mhd_create(ctypes.byref(p), ctypes.byref(h)) == 1   # ifchem is 0 or 2
    p = native.params_struct(MhdParams(8, 8, 8, ifchem=2), precision=native.PREC_FP32,
                             cooling=native.COOL_SURROGATE)
    assert L.mhd_create(ctypes.byref(p), ctypes.byref(h)) == 1   # surrogate is KI-only


def test_create_without_gpu_reports_no_device():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    L = native.load()
    h = ctypes.c_void_p()
    p = native.params_struct(MhdParams(16, 16, 16))
    assert L.mhd_create(ctypes.byref(p), ctypes.byref(h)) == 6   # MHD_ERR_NO_DEVICE
    with pytest.raises(native.MhdError):
        native.Mhd3D(MhdParams(16, 16, 16))
