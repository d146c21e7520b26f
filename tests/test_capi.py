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


def test_null_handle_is_an_argument_error():
    """Every entry point that takes a handle rejects NULL with MHD_ERR_ARG
    before touching the device (mhd_destroy(NULL) is a no-op, like free)."""
    L = ctypes.CDLL(build.build())   # untyped: plain C calls
    buf = (ctypes.c_double * 64)()
    d, i = ctypes.c_double(), ctypes.c_int()
    dt = ctypes.c_double(0.1)
    calls = {
        "mhd_upload": lambda: L.mhd_upload(None, buf, buf, buf, buf, buf, buf, buf, buf),
        "mhd_download": lambda: L.mhd_download(None, buf, buf, buf),
        "mhd_download_columns": lambda: L.mhd_download_columns(None, buf),
        "mhd_timestep": lambda: L.mhd_timestep(None, ctypes.byref(d), ctypes.byref(i)),
        "mhd_source": lambda: L.mhd_source(None, dt),
        "mhd_sweep": lambda: L.mhd_sweep(None, 0, dt),
        "mhd_ct": lambda: L.mhd_ct(None, dt),
        "mhd_dissip": lambda: L.mhd_dissip(None),
        "mhd_advance": lambda: L.mhd_advance(None, dt),
        "mhd_step": lambda: L.mhd_step(None, ctypes.c_double(1e30), ctypes.byref(d), ctypes.byref(i)),
        "mhd_step_host": lambda: L.mhd_step_host(None, buf, buf, buf, buf, ctypes.c_double(1e30),
                                                 ctypes.byref(d), ctypes.byref(i)),
        "mhd_evolve": lambda: L.mhd_evolve(None, 1, ctypes.c_double(1e30), ctypes.byref(i)),
        "mhd_set_inflow": lambda: L.mhd_set_inflow(None, None, None, ctypes.c_double(1.0)),
        "mhd_get_time": lambda: L.mhd_get_time(None, ctypes.byref(d), ctypes.byref(i)),
        "mhd_set_time": lambda: L.mhd_set_time(None, ctypes.c_double(0.0), 1),
        "mhd_diagnostics": lambda: L.mhd_diagnostics(None, buf),
        "mhd_synchronize": lambda: L.mhd_synchronize(None),
        "mhd_set_stream": lambda: L.mhd_set_stream(None, None),
        "mhd_last_error": lambda: L.mhd_last_error(None, ctypes.create_string_buffer(64), 64),
        "mhd_reset_counters": lambda: L.mhd_reset_counters(None),
        "mhd_surrogate_load": lambda: L.mhd_surrogate_load(None, None, ctypes.c_float(1e-3)),
    }
    bad = {k: r for k, r in ((k, f()) for k, f in calls.items()) if r != 1}
    assert not bad, bad
    assert L.mhd_destroy(None) == 0
