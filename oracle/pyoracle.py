"""ctypes wrapper of the oracle library (test infrastructure only).

The oracle is the CPU restatement of the reference algorithm; tests, the
smoke check and the CPU-baseline leg of bench.py load it as the checker.
Nothing on the product path imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_P = ctypes.POINTER(ctypes.c_double)


def build(force=False):
    """Compile oracle/_build/liboracle.so with the committed Makefile."""
    srcs = [os.path.join(_HERE, f) for f in ("mhd1d.cpp", "mhd3d.cpp")]
    if not force and os.path.exists(_LIB) and all(
            os.path.getmtime(_LIB) >= os.path.getmtime(s) for s in srcs):
        return _LIB
    subprocess.run(["make", "-C", _HERE, "-B" if force else "all"], check=True,
                   stdout=subprocess.DEVNULL)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        L.o1d_create.restype = ctypes.c_void_p
        L.o1d_create.argtypes = [_P]
        L.o1d_ncell.argtypes = [ctypes.c_void_p]
        L.o1d_time.restype = ctypes.c_double
        L.o1d_time.argtypes = [ctypes.c_void_p]
        L.o1d_step.restype = ctypes.c_double
        L.o1d_step.argtypes = [ctypes.c_void_p]
        L.o1d_step_dt.restype = ctypes.c_double
        L.o1d_step_dt.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.o1d_set_riemann_iterations.restype = None
        L.o1d_set_riemann_iterations.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.o1d_run_trace.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]
        L.o1d_state.argtypes = [ctypes.c_void_p, _P]
        L.o1d_destroy.argtypes = [ctypes.c_void_p]
        L.o3d_create.restype = ctypes.c_void_p
        L.o3d_create.argtypes = [_P]
        L.o3d_upload.argtypes = [ctypes.c_void_p, _P, _P, _P]
        L.o3d_download.argtypes = [ctypes.c_void_p, _P, _P, _P]
        L.o3d_timestep.restype = ctypes.c_double
        L.o3d_timestep.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        for n in ("o3d_source", "o3d_ct", "o3d_advance"):
            getattr(L, n).argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.o3d_sweep.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
        L.o3d_dissip.argtypes = [ctypes.c_void_p]
        L.o3d_time.restype = ctypes.c_double
        L.o3d_time.argtypes = [ctypes.c_void_p]
        L.o3d_set_order.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.o3d_step.restype = ctypes.c_double
        L.o3d_step.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.POINTER(ctypes.c_int)]
        L.o3d_destroy.argtypes = [ctypes.c_void_p]
        L.o3d_set_inflow.argtypes = [ctypes.c_void_p, _P, ctypes.c_void_p, ctypes.c_double]
        L.o3d_columns.argtypes = [ctypes.c_void_p, _P]
        L.o3d_potential.argtypes = [ctypes.c_void_p, _P]
        L.o3d_gravity_solve.argtypes = [ctypes.c_void_p]
        L.o3d_chem_probe.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_longlong, _P]
        L.o3d_chem_cell_probe.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_double, _P]
        L.o3d_ct_probe.argtypes = [ctypes.c_void_p, ctypes.c_double, _P]
        L.o3d_detmath.argtypes = [ctypes.c_int, _P, _P, _P, ctypes.c_longlong]
        L.o3d_ki_label.restype = ctypes.c_double
        L.o3d_ki_label.argtypes = [ctypes.c_double] * 4
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(_P)


class Oracle1D:
    """KIcool/1DMHDwCC3.f90 (or the Brio-Wu variant) on the CPU."""

    def __init__(self, deck_vector):
        d = np.ascontiguousarray(deck_vector, dtype=np.float64)
        self.h = lib().o1d_create(_ptr(d))
        self.ncell = lib().o1d_ncell(self.h)

    def run_trace(self, nsteps, probe_n=512, probe_b=510):
        tr = np.zeros((nsteps, 4))
        lib().o1d_run_trace(self.h, nsteps, probe_n, probe_b, _ptr(tr))
        return tr

    def step(self):
        return lib().o1d_step(self.h)

    def step_dt(self, dt):
        """One step of the given length instead of the Couran/Stblty one."""
        return lib().o1d_step_dt(self.h, float(dt))

    def set_riemann_iterations(self, n):
        """RHS's RIEMAN iteration count (5 in the 1D codes, 4 in the 3D one)."""
        lib().o1d_set_riemann_iterations(self.h, int(n))

    @property
    def time(self):
        return lib().o1d_time(self.h)

    def state(self):
        out = np.zeros((self.ncell, 17))
        lib().o1d_state(self.h, _ptr(out))
        return out

    def __del__(self):
        if getattr(self, "h", None):
            lib().o1d_destroy(self.h)
            self.h = None


class Oracle3D:
    """One-block restatement of the 3D step (MCF3DSGincfca3.f90 + KI cooling)."""

    def __init__(self, params):
        p = params
        v = [p.nx, p.ny, p.nz, p.cfl, p.facdep, p.tfinal, *p.bc, p.pmin, p.pmax, p.rmin,
             p.kb, p.kcond, p.ifthrm, p.dissip, getattr(p, "ifchem", 0), getattr(p, "ifrad", 0),
             getattr(p, "ifgrv", 0)]
        self.params = p
        self.shape = (p.nz + 4, p.ny + 4, p.nx + 4)
        self.h = lib().o3d_create(_ptr(np.array(v, dtype=np.float64)))

    def upload(self, state):
        U = np.ascontiguousarray(state.U, dtype=np.float64)
        sp = np.ascontiguousarray(state.species, dtype=np.float64)
        co = np.ascontiguousarray(state.coords_vector(), dtype=np.float64)
        lib().o3d_upload(self.h, _ptr(U), _ptr(sp), _ptr(co))

    def download(self):
        U = np.zeros((8,) + self.shape)
        sp = np.zeros((8,) + self.shape)
        bcc = np.zeros((3,) + self.shape)
        lib().o3d_download(self.h, _ptr(U), _ptr(sp), _ptr(bcc))
        return U, sp, bcc

    def timestep(self):
        st = ctypes.c_int(0)
        dt = lib().o3d_timestep(self.h, ctypes.byref(st))
        return dt, st.value

    def source(self, dt):
        lib().o3d_source(self.h, dt)

    def columns(self):
        """SHIELD's ten column arrays (Ntot, NH2, NnC, NCO, tCII; each from
        the left and the right), padded layout."""
        out = np.zeros((10,) + self.shape)
        lib().o3d_columns(self.h, _ptr(out))
        return out

    def chem_probe(self, T, c):
        """Species Fcool and the 21 RATES at temperature T for padded cell c,
        with the cell's species, nde, ndtot and columns (see o3d_chem_probe)."""
        out = np.zeros(42)
        lib().o3d_chem_probe(self.h, float(T), int(c), _ptr(out))
        return out

    def chem_cell_probe(self, c, dt):
        """The chemistry network of padded cell c over dt, with the cell's
        inputs and results (see o3d_chem_cell_probe)."""
        out = np.zeros(32)
        lib().o3d_chem_cell_probe(self.h, int(c), float(dt), _ptr(out))
        return out

    def ct_probe(self, dt):
        """Constrained transport over dt with its intermediates (see
        o3d_ct_probe): U(1..8) as CCT read them, Vfc(1..3), EMF(1..3) and
        U(6..8) after the face update, each padded."""
        out = np.zeros((17,) + self.shape)
        lib().o3d_ct_probe(self.h, float(dt), _ptr(out))
        return out[0:8], out[8:11], out[11:14], out[14:17]

    def potential(self):
        """Phi (self-gravity, ifgrv = 2) in the padded layout."""
        out = np.zeros(self.shape)
        lib().o3d_potential(self.h, _ptr(out))
        return out

    def gravity_solve(self):
        lib().o3d_gravity_solve(self.h)

    def sweep(self, d, dt):
        lib().o3d_sweep(self.h, d, dt)

    def ct(self, dt):
        lib().o3d_ct(self.h, dt)

    def dissip(self):
        lib().o3d_dissip(self.h)

    def advance(self, dt):
        lib().o3d_advance(self.h, dt)

    def step(self, tsave=1e30):
        st = ctypes.c_int(0)
        dt = lib().o3d_step(self.h, tsave, ctypes.byref(st))
        return dt, st.value

    def set_order(self, ifevo):
        lib().o3d_set_order(self.h, ifevo)

    def set_inflow(self, inflow, reservoir=None, uniform=0.0):
        """BC=4 data: `inflow` is the packed vector of problems.Inflow.vector()
        and `reservoir` the DTF array (nz+4, ny+4, nx+4) float32, or None for
        a uniform reservoir of density `uniform`."""
        v = np.ascontiguousarray(inflow, dtype=np.float64)
        if reservoir is None:
            lib().o3d_set_inflow(self.h, _ptr(v), None, ctypes.c_double(uniform))
        else:
            r = np.ascontiguousarray(reservoir, dtype=np.float32)
            lib().o3d_set_inflow(self.h, _ptr(v), r.ctypes.data_as(ctypes.c_void_p), ctypes.c_double(uniform))

    @property
    def time(self):
        return lib().o3d_time(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().o3d_destroy(self.h)
            self.h = None


def ki_labels(x, kb=8.63359):
    """The oracle's IMC answer log10(T_new/T) for surrogate inputs x[n][3]."""
    L = lib()
    return np.array([L.o3d_ki_label(float(a), float(b), float(c), kb) for a, b, c in x])


def detmath(fn, x, e=None):
    """The oracle's own exp, log10, exp10 (10**x), log or pow (x**e)
    elementwise (x and e broadcast), for restatements that must agree bit
    for bit."""
    a, b = np.broadcast_arrays(np.asarray(x, dtype=np.float64), np.asarray(0.0 if e is None else e, dtype=np.float64))
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    y = np.empty_like(a)
    code = {"exp": 0, "log10": 1, "exp10": 2, "log": 3, "pow": 4}[fn]
    lib().o3d_detmath(code, _ptr(a), _ptr(b), _ptr(y), a.size)
    return y
