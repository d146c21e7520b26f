"""ctypes binding of libmhd_gb300.so (the C ABI of include/mhd_gb300.h).

This is the Python face of the same entry points a Fortran driver binds
with iso_c_binding.  There is no CPU fallback: if the CUDA library cannot
be loaded or no GPU is present, every constructor raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build
from .problems import MhdParams, MhdState

MHD_OK = 0
ERRORS = {1: "MHD_ERR_ARG", 2: "MHD_ERR_CUDA", 3: "MHD_ERR_NONFINITE", 4: "MHD_ERR_DT",
          5: "MHD_ERR_STATE", 6: "MHD_ERR_NO_DEVICE", 7: "MHD_ERR_TOO_LARGE"}
NOALLOC_MAX_CELLS = 16777216
PREC_FP64, PREC_FP32 = 0, 1
COOL_EXACT, COOL_SURROGATE, COOL_NEWTON = 0, 1, 2

# every symbol the header declares (checked by the CPU test suite)
EXPORTS = ("mhd_create", "mhd_destroy", "mhd_upload", "mhd_download", "mhd_timestep", "mhd_source",
           "mhd_sweep", "mhd_ct", "mhd_dissip", "mhd_gravity", "mhd_advance", "mhd_step", "mhd_step_host", "mhd_evolve",
           "mhd_download_columns", "mhd_download_potential", "mhd_get_time",
           "mhd_set_time", "mhd_set_inflow", "mhd_diagnostics", "mhd_synchronize", "mhd_set_stream", "mhd_last_error",
           "mhd_kernel_launches", "mhd_reset_counters", "mhd_surrogate_nparams", "mhd_surrogate_load",
           "mhd_surrogate_train", "mhd_surrogate_label", "mhd_surrogate_eval", "mhd_surrogate_grad",
           "mhd_timestep_noalloc", "mhd_fp64_peak")


class MhdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class _Params(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("cfl", ctypes.c_double), ("facdep", ctypes.c_double), ("tfinal", ctypes.c_double),
                ("bc", ctypes.c_int * 6),
                ("pmin", ctypes.c_double), ("pmax", ctypes.c_double), ("rmin", ctypes.c_double),
                ("kb", ctypes.c_double), ("kcond", ctypes.c_double),
                ("ifthrm", ctypes.c_int), ("dissip", ctypes.c_int), ("precision", ctypes.c_int),
                ("cooling", ctypes.c_int), ("device", ctypes.c_int), ("ifchem", ctypes.c_int), ("ifrad", ctypes.c_int),
                ("ifgrv", ctypes.c_int)]


class _Diag(ctypes.Structure):
    _fields_ = [("mass", ctypes.c_double), ("momentum", ctypes.c_double * 3), ("energy", ctypes.c_double),
                ("divb_max", ctypes.c_double), ("time", ctypes.c_double), ("steps", ctypes.c_longlong),
                ("imc_cells", ctypes.c_longlong), ("surrogate_cells", ctypes.c_longlong),
                ("fallback_cells", ctypes.c_longlong)]


class DeviceState(ctypes.Structure):
    """Device pointers (as integers) of arrays in the mhd_upload layout."""
    _fields_ = [("U", ctypes.c_void_p), ("species", ctypes.c_void_p), ("bcc", ctypes.c_void_p),
                ("dx", ctypes.c_void_p), ("dy", ctypes.c_void_p), ("dz", ctypes.c_void_p),
                ("nde", ctypes.c_void_p), ("ndtot", ctypes.c_void_p), ("columns", ctypes.c_void_p)]


_lib = None
_P = ctypes.POINTER(ctypes.c_double)


def library_path():
    return _build.LIB


class _Inflow(ctypes.Structure):
    _fields_ = [("rho_ref", ctypes.c_double), ("v", (ctypes.c_double * 3) * 2), ("p", ctypes.c_double * 2),
                ("b", (ctypes.c_double * 3) * 2), ("species", ctypes.c_double * 8)]


def load(build_if_missing=True):
    """Load libmhd_gb300.so, compiling it first when it is missing or stale."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError(f"{_build.LIB} is missing; run code_tohoku_gb300.build.build()")
    L = ctypes.CDLL(_build.LIB)
    H = ctypes.c_void_p
    sig = {
        "mhd_create": [ctypes.POINTER(_Params), ctypes.POINTER(H)],
        "mhd_destroy": [H],
        "mhd_upload": [H, _P, _P, _P, _P, _P, _P, _P, _P],
        "mhd_download": [H, _P, _P, _P],
        "mhd_download_columns": [H, _P],
        "mhd_download_potential": [H, _P],
        "mhd_timestep": [H, _P, ctypes.POINTER(ctypes.c_int)],
        "mhd_source": [H, ctypes.c_double],
        "mhd_sweep": [H, ctypes.c_int, ctypes.c_double],
        "mhd_ct": [H, ctypes.c_double],
        "mhd_dissip": [H],
        "mhd_gravity": [H, ctypes.c_double, ctypes.c_int],
        "mhd_advance": [H, ctypes.c_double],
        "mhd_step": [H, ctypes.c_double, _P, ctypes.POINTER(ctypes.c_int)],
        "mhd_step_host": [H, _P, _P, _P, _P, ctypes.c_double, _P, ctypes.POINTER(ctypes.c_int)],
        "mhd_evolve": [H, ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_int)],
        "mhd_get_time": [H, _P, ctypes.POINTER(ctypes.c_int)],
        "mhd_set_time": [H, ctypes.c_double, ctypes.c_int],
        "mhd_diagnostics": [H, ctypes.POINTER(_Diag)],
        "mhd_synchronize": [H],
        "mhd_set_stream": [H, ctypes.c_void_p],
        "mhd_last_error": [H, ctypes.c_char_p, ctypes.c_int],
        "mhd_set_inflow": [H, ctypes.POINTER(_Inflow), ctypes.c_void_p, ctypes.c_double],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.mhd_kernel_launches.argtypes = [H]
    L.mhd_kernel_launches.restype = ctypes.c_longlong
    F = ctypes.POINTER(ctypes.c_float)
    L.mhd_reset_counters.argtypes = [H]
    L.mhd_reset_counters.restype = ctypes.c_int
    L.mhd_surrogate_nparams.argtypes = []
    L.mhd_surrogate_nparams.restype = ctypes.c_int
    L.mhd_surrogate_load.argtypes = [H, F, ctypes.c_float]
    L.mhd_surrogate_load.restype = ctypes.c_int
    L.mhd_surrogate_train.argtypes = [F, ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                      ctypes.c_ulonglong, F, ctypes.c_int]
    L.mhd_surrogate_train.restype = ctypes.c_int
    L.mhd_surrogate_label.argtypes = [F, F, ctypes.c_longlong, ctypes.c_double, ctypes.c_int]
    L.mhd_surrogate_label.restype = ctypes.c_int
    L.mhd_surrogate_eval.argtypes = [F, F, F, ctypes.c_longlong, ctypes.c_int]
    L.mhd_surrogate_eval.restype = ctypes.c_int
    L.mhd_surrogate_grad.argtypes = [F, F, F, ctypes.c_longlong, F, F, ctypes.c_int]
    L.mhd_surrogate_grad.restype = ctypes.c_int
    L.mhd_timestep_noalloc.argtypes = [ctypes.POINTER(_Params), ctypes.POINTER(DeviceState), _P,
                                       ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]
    L.mhd_timestep_noalloc.restype = ctypes.c_int
    L.mhd_fp64_peak.argtypes = [ctypes.c_int, _P, _P, _P]
    L.mhd_fp64_peak.restype = ctypes.c_int
    _lib = L
    return L


def _ptr(a):
    return a.ctypes.data_as(_P)


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _sck(r, what):
    if r != MHD_OK:
        raise MhdError(r, what)


def surrogate_nparams():
    return load().mhd_surrogate_nparams()


def surrogate_train(params, n_data=1 << 24, batch=65536, steps=4000, lr=1e-3, seed=1, device=0):
    """Trains in place on the GPU; returns (params, per-step batch MSE)."""
    p = np.ascontiguousarray(params, dtype=np.float32).copy()
    hist = np.zeros(max(steps, 1), dtype=np.float32)
    _sck(load().mhd_surrogate_train(_fptr(p), n_data, batch, steps, lr, seed, _fptr(hist), device),
         "mhd_surrogate_train")
    return p, hist[:steps]


def surrogate_label(x, kb=8.63359, device=0):
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.zeros(len(x), dtype=np.float32)
    _sck(load().mhd_surrogate_label(_fptr(x), _fptr(y), len(x), kb, device), "mhd_surrogate_label")
    return y


def surrogate_eval(params, x, device=0):
    p = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.zeros((len(x), 2), dtype=np.float32)
    _sck(load().mhd_surrogate_eval(_fptr(p), _fptr(x), _fptr(out), len(x), device), "mhd_surrogate_eval")
    return out


def surrogate_grad(params, x, y, device=0):
    p = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    g = np.zeros(len(p), dtype=np.float32)
    loss = np.zeros(1, dtype=np.float32)
    _sck(load().mhd_surrogate_grad(_fptr(p), _fptr(x), _fptr(y), len(x), _fptr(g), _fptr(loss), device),
         "mhd_surrogate_grad")
    return g, float(loss[0])


def timestep_noalloc(params: MhdParams, dev_state: DeviceState, stream=None, device=0, precision=PREC_FP64):
    """mhd_timestep_noalloc: (dt, limiter) from device arrays the caller owns;
    no device memory is allocated by the library."""
    ps = params_struct(params, precision=precision, device=device)
    dt = ctypes.c_double()
    st = ctypes.c_int()
    r = load().mhd_timestep_noalloc(ctypes.byref(ps), ctypes.byref(dev_state), ctypes.byref(dt),
                                    ctypes.byref(st), ctypes.c_void_p(stream) if stream else None)
    _sck(r, "mhd_timestep_noalloc")
    return dt.value, st.value


def fp64_peak(device=0):
    """mhd_fp64_peak: measured FP64 FMA GFLOP/s, divisions and square roots
    in billions per second."""
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    _sck(load().mhd_fp64_peak(device, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), "mhd_fp64_peak")
    return {"fma_gflops": a.value, "div_per_ns": b.value, "sqrt_per_ns": c.value}


def params_struct(p: MhdParams, precision=PREC_FP64, cooling=COOL_EXACT, device=0):
    s = _Params()
    s.nx, s.ny, s.nz = p.nx, p.ny, p.nz
    s.cfl, s.facdep, s.tfinal = p.cfl, p.facdep, p.tfinal
    for q in range(6):
        s.bc[q] = p.bc[q]
    s.pmin, s.pmax, s.rmin = p.pmin, p.pmax, p.rmin
    s.kb, s.kcond = p.kb, p.kcond
    s.ifthrm, s.dissip = p.ifthrm, p.dissip
    s.precision, s.cooling, s.device = precision, cooling, device
    s.ifchem = getattr(p, "ifchem", 0)
    s.ifrad = getattr(p, "ifrad", 0)
    s.ifgrv = getattr(p, "ifgrv", 0)
    return s


class Mhd3D:
    """GPU-resident 3D MHD + KI cooling state driven through the C ABI."""

    def __init__(self, params: MhdParams, precision=PREC_FP64, cooling=COOL_EXACT, device=0):
        self.L = load()
        self.params = params
        self.shape = (params.nz + 4, params.ny + 4, params.nx + 4)
        self.h = ctypes.c_void_p()
        ps = params_struct(params, precision, cooling, device)
        r = self.L.mhd_create(ctypes.byref(ps), ctypes.byref(self.h))
        if r != MHD_OK:
            raise MhdError(r, "mhd_create failed")

    def _ck(self, r):
        if r != MHD_OK:
            buf = ctypes.create_string_buffer(512)
            self.L.mhd_last_error(self.h, buf, 512)
            raise MhdError(r, buf.value.decode(errors="replace"))

    def upload(self, st: MhdState):
        U = np.ascontiguousarray(st.U, dtype=np.float64)
        sp = np.ascontiguousarray(st.species, dtype=np.float64)
        co = [np.ascontiguousarray(a, dtype=np.float64) for a in (st.x, st.dx, st.y, st.dy, st.z, st.dz)]
        self._ck(self.L.mhd_upload(self.h, _ptr(U), _ptr(sp), *[_ptr(c) for c in co]))

    def download(self, with_bcc=True, out=None):
        """Copy the state to host arrays: new ones, or `out` = (U, species, bcc)
        of shapes (8,)+shape, (8,)+shape and (3,)+shape (bcc may be None),
        C-contiguous float64 (pinned host memory makes the copy faster)."""
        if out is None:
            U = np.empty((8,) + self.shape)
            sp = np.empty((8,) + self.shape)
            bcc = np.empty((3,) + self.shape) if with_bcc else None
        else:
            U, sp, bcc = out
            for a, lead in ((U, 8), (sp, 8), (bcc, 3)):
                if a is not None and (a.dtype != np.float64 or not a.flags.c_contiguous
                                      or a.shape != (lead,) + self.shape):
                    raise ValueError("download: output arrays must be C-contiguous float64 of the state shape")
        self._ck(self.L.mhd_download(self.h, _ptr(U), _ptr(sp), _ptr(bcc) if bcc is not None else None))
        return U, sp, bcc

    def timestep(self):
        dt = ctypes.c_double()
        st = ctypes.c_int()
        self._ck(self.L.mhd_timestep(self.h, ctypes.byref(dt), ctypes.byref(st)))
        return dt.value, st.value

    def source(self, dt):
        self._ck(self.L.mhd_source(self.h, dt))

    def sweep(self, d, dt):
        self._ck(self.L.mhd_sweep(self.h, d, dt))

    def ct(self, dt):
        self._ck(self.L.mhd_ct(self.h, dt))

    def dissip(self):
        self._ck(self.L.mhd_dissip(self.h))

    def gravity(self, dt, mode):
        """GRAVTY(dt, mode): 2 the potential, 3 the half kick (ifgrv = 2)."""
        self._ck(self.L.mhd_gravity(self.h, dt, mode))

    def advance(self, dt):
        self._ck(self.L.mhd_advance(self.h, dt))

    def step(self, tsave=1e30):
        dt = ctypes.c_double()
        st = ctypes.c_int()
        self._ck(self.L.mhd_step(self.h, tsave, ctypes.byref(dt), ctypes.byref(st)))
        return dt.value, st.value

    def columns(self):
        """SHIELD's ten column arrays (ifrad = 2), padded layout."""
        out = np.zeros((10,) + self.shape)
        self._ck(self.L.mhd_download_columns(self.h, _ptr(out)))
        return out

    def potential(self):
        """The gravitational potential (ifgrv = 2), padded layout."""
        out = np.zeros(self.shape)
        self._ck(self.L.mhd_download_potential(self.h, _ptr(out)))
        return out

    def step_host(self, U_in, species_in, U_out, species_out, tsave=1e30):
        """mhd_step_host: one step from host arrays to host arrays (same
        layout as upload/download; all four C-contiguous float64)."""
        for a in (U_in, species_in, U_out, species_out):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.shape != (8,) + self.shape:
                raise ValueError("step_host: arrays must be C-contiguous float64 of shape (8,) + padded grid")
        dt = ctypes.c_double()
        st = ctypes.c_int()
        self._ck(self.L.mhd_step_host(self.h, _ptr(U_in), _ptr(species_in), _ptr(U_out), _ptr(species_out),
                                      tsave, ctypes.byref(dt), ctypes.byref(st)))
        return dt.value, st.value

    def evolve(self, nsteps, tsave=1e30):
        n = ctypes.c_int()
        self._ck(self.L.mhd_evolve(self.h, nsteps, tsave, ctypes.byref(n)))
        return n.value

    def set_inflow(self, inflow, reservoir=None, uniform_density=0.0):
        """BC=4 data (problems.Inflow); reservoir: DTF as float32 of the padded
        state shape, or None for a uniform reservoir.  Call before upload."""
        c = _Inflow()
        c.rho_ref = inflow.rho_ref
        for s_ in range(2):
            c.p[s_] = inflow.p[s_]
            for q in range(3):
                c.v[s_][q] = inflow.v[s_][q]
                c.b[s_][q] = inflow.b[s_][q]
        for q in range(8):
            c.species[q] = inflow.species[q]
        if reservoir is None:
            self._ck(self.L.mhd_set_inflow(self.h, ctypes.byref(c), None, float(uniform_density)))
        else:
            r = np.ascontiguousarray(reservoir, dtype=np.float32)
            if r.shape != self.shape:
                raise ValueError(f"reservoir shape {r.shape}, expected {self.shape}")
            self._ck(self.L.mhd_set_inflow(self.h, ctypes.byref(c), r.ctypes.data_as(ctypes.c_void_p),
                                           float(uniform_density)))

    def set_time(self, time, ifevo=1):
        self._ck(self.L.mhd_set_time(self.h, time, ifevo))

    @property
    def time(self):
        t = ctypes.c_double()
        o = ctypes.c_int()
        self._ck(self.L.mhd_get_time(self.h, ctypes.byref(t), ctypes.byref(o)))
        return t.value

    def diagnostics(self):
        d = _Diag()
        self._ck(self.L.mhd_diagnostics(self.h, ctypes.byref(d)))
        return dict(mass=d.mass, momentum=tuple(d.momentum), energy=d.energy, divb_max=d.divb_max,
                    time=d.time, steps=d.steps, imc_cells=d.imc_cells, surrogate_cells=d.surrogate_cells,
                    fallback_cells=d.fallback_cells)

    def synchronize(self):
        self._ck(self.L.mhd_synchronize(self.h))

    def set_stream(self, stream_ptr):
        self._ck(self.L.mhd_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    def surrogate_load(self, params, tol=1e-3):
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._ck(self.L.mhd_surrogate_load(self.h, _fptr(p), tol))

    def reset_counters(self):
        self._ck(self.L.mhd_reset_counters(self.h))

    @property
    def kernel_launches(self):
        return self.L.mhd_kernel_launches(self.h)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.L.mhd_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
