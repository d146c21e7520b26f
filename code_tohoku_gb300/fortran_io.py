"""The reference driver's files: the INPUT3D.DAT deck, SAVEU / SAVEU2D's
per-rank output and restart files, time.DAT / tsave.DAT and SAVEU's info
line (3DMHD-CfCA/MCF3DSGincfca3.f90:120-150, :454-465, :684-794).

The binary files are written and read by the library's host code
(include/mhd_io.h, csrc/mhd_io.cpp); this module binds it and adds the
SAVEU sequence and the deck reader.  Arrays are the padded single-domain
state of `native.Mhd3D.download()`: U (8, nz+4, ny+4, nx+4), species in the
upload order (H, p, H2, He, He+, C, C+, CO), Bcc (3, ...), Phi (optional).
"""
import ctypes
import os
import re
from dataclasses import dataclass
from typing import List, Tuple

import numpy as np

from . import native


class _Grid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("nsplit", ctypes.c_int * 3)]


_D = ctypes.POINTER(ctypes.c_double)
_SIGS = {
    "mhd_io_write_snapshot": [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(_Grid), _D, _D, _D],
    "mhd_io_write_restart": [ctypes.c_char_p, ctypes.POINTER(_Grid), _D, _D, _D],
    "mhd_io_read_restart": [ctypes.c_char_p, ctypes.POINTER(_Grid), _D, _D, _D],
    "mhd_io_write_plane": [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(_Grid), _D, _D, _D, _D],
    "mhd_io_format_d25_17": [ctypes.c_double, ctypes.c_int, ctypes.c_char_p],
    "mhd_io_write_reservoir": [ctypes.c_char_p, ctypes.POINTER(_Grid), ctypes.c_void_p],
    "mhd_io_read_reservoir": [ctypes.c_char_p, ctypes.POINTER(_Grid), ctypes.c_void_p, ctypes.c_double],
    "mhd_io_write_time_dat": [ctypes.c_char_p, _D, ctypes.c_int, ctypes.c_int],
    "mhd_io_write_tsave": [ctypes.c_char_p, ctypes.c_double, ctypes.c_int, ctypes.c_int],
    "mhd_io_format_info_line": [ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_char_p, ctypes.c_char_p],
}
_lib = None


def _L():
    global _lib
    if _lib is None:
        L = native.load()
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _lib = L
    return _lib


def _ck(rc, what):
    if rc == -1:
        raise ValueError(f"{what}: bad argument (grid, decomposition or array)")
    if rc != 0:
        raise OSError(f"{what}: I/O error")


def _grid(shape, nsplit):
    nz, ny, nx = (s - 4 for s in shape[-3:])
    return _Grid(nx, ny, nz, (ctypes.c_int * 3)(*nsplit))


def _arr(a, lead, shape):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != (lead,) + tuple(shape) and not (lead == 1 and a.shape == tuple(shape)):
        raise ValueError(f"array of shape {a.shape}, expected {(lead,) + tuple(shape)}")
    return a


def _p(a):
    return a.ctypes.data_as(_D) if a is not None else None


def write_snapshot(directory, nunit, U, species, phi=None, nsplit=(1, 1, 1)):
    """SAVEU's NNNRRR.dat (FP32, 17 fields) for every rank of `nsplit`."""
    sh = U.shape[1:]
    U, species, phi = _arr(U, 8, sh), _arr(species, 8, sh), _arr(phi, 1, sh)
    g = _grid(sh, nsplit)
    _ck(_L().mhd_io_write_snapshot(os.fsencode(directory), nunit, ctypes.byref(g), _p(U), _p(species), _p(phi)),
        "write_snapshot")


def write_restart(directory, U, species, phi=None, nsplit=(1, 1, 1)):
    """SAVEU's 000RRR.dat (FP64 restart) for every rank of `nsplit`."""
    sh = U.shape[1:]
    U, species, phi = _arr(U, 8, sh), _arr(species, 8, sh), _arr(phi, 1, sh)
    g = _grid(sh, nsplit)
    _ck(_L().mhd_io_write_restart(os.fsencode(directory), ctypes.byref(g), _p(U), _p(species), _p(phi)),
        "write_restart")


def read_restart(directory, shape, nsplit=(1, 1, 1), U=None, species=None, phi=None):
    """INITIA's restart read: the per-rank 000RRR.dat into one padded state.
    `shape` is the padded (nz+4, ny+4, nx+4); returns (U, species, phi)."""
    sh = tuple(shape)
    U = np.zeros((8,) + sh) if U is None else U
    species = np.zeros((8,) + sh) if species is None else species
    phi = np.zeros(sh) if phi is None else phi
    for a in (U, species, phi):
        if a.dtype != np.float64 or not a.flags.c_contiguous:
            raise ValueError("read_restart: arrays must be C-contiguous float64")
    g = _grid(sh, nsplit)
    _ck(_L().mhd_io_read_restart(os.fsencode(directory), ctypes.byref(g), _p(U), _p(species), _p(phi)),
        "read_restart")
    return U, species, phi


def write_plane(directory, nunit2d, U, bcc, species, phi=None, nsplit=(1, 1, 1)):
    """SAVEU2D's 2DNNNRRR.dat: plane k = 1 of every rank, cell-centred B."""
    sh = U.shape[1:]
    U, bcc, species, phi = _arr(U, 8, sh), _arr(bcc, 3, sh), _arr(species, 8, sh), _arr(phi, 1, sh)
    g = _grid(sh, nsplit)
    _ck(_L().mhd_io_write_plane(os.fsencode(directory), nunit2d, ctypes.byref(g), _p(U), _p(bcc), _p(species),
                                _p(phi)), "write_plane")


def write_reservoir(directory, dtf, nsplit=(1, 1, 1)):
    """The DTF reservoir (float32, padded state shape) as per-rank D###.dat."""
    d = np.ascontiguousarray(dtf, dtype=np.float32)
    g = _grid(d.shape, nsplit)
    _ck(_L().mhd_io_write_reservoir(os.fsencode(directory), ctypes.byref(g), d.ctypes.data_as(ctypes.c_void_p)),
        "write_reservoir")


def read_reservoir(directory, shape, nsplit=(1, 1, 1), ghost_density=0.0):
    """Per-rank D###.dat into the padded reservoir for mhd_set_inflow (periodic
    y/z ghosts, ghost_density in the x ghosts)."""
    d = np.zeros(tuple(shape), dtype=np.float32)
    g = _grid(d.shape, nsplit)
    _ck(_L().mhd_io_read_reservoir(os.fsencode(directory), ctypes.byref(g), d.ctypes.data_as(ctypes.c_void_p),
                                   float(ghost_density)), "read_reservoir")
    return d


def format_d25_17(v, with_1p=True):
    """One value as Fortran writes it with 1P,D25.17 (3D code) or D25.17 (1D)."""
    buf = ctypes.create_string_buffer(32)
    _ck(_L().mhd_io_format_d25_17(float(v), 1 if with_1p else 0, buf), "format_d25_17")
    return buf.value.decode()


def write_time_dat(path, times, with_1p=True):
    t = np.ascontiguousarray(times, dtype=np.float64)
    _ck(_L().mhd_io_write_time_dat(os.fsencode(path), _p(t), len(t), 1 if with_1p else 0), "write_time_dat")


def write_tsave(path, time, nunit, with_1p=True):
    _ck(_L().mhd_io_write_tsave(os.fsencode(path), float(time), int(nunit), 1 if with_1p else 0), "write_tsave")


def info_line(time, step, dt, limiter):
    buf = ctypes.create_string_buffer(128)
    _ck(_L().mhd_io_format_info_line(float(time), int(step), float(dt), limiter.encode(), buf), "info_line")
    return buf.value.decode()


def saveu(directory, nunit, times, time, dt, limiter, step, U, species, phi=None, nsplit=(1, 1, 1),
          tfinal=None, info_path=None):
    """SAVEU (:684-761): snapshot NNNRRR.dat, time.DAT with t(nunit) = time,
    the info line, tsave.DAT and the restart files; returns nunit + 1.
    `times` is the list t(1..) of save times (updated in place)."""
    write_snapshot(directory, nunit, U, species, phi, nsplit)
    while len(times) < nunit:
        times.append(0.0)
    times[nunit - 1] = time
    write_time_dat(os.path.join(directory, "time.DAT"), times[:nunit])
    if info_path is not None:
        with open(info_path, "a") as f:
            f.write(info_line(time, step, dt, limiter) + "\n")
            if tfinal is not None:
                f.write("Done ! Time =" + _e11_3(time) + _e11_3(tfinal) + "\n")
    nunit += 1
    write_tsave(os.path.join(directory, "tsave.DAT"), time, nunit - 1)
    write_restart(directory, U, species, phi, nsplit)
    return nunit


def _e11_3(v):
    # the info line's dt field is 1P,E11.3: reuse it through a dummy line
    s = info_line(0.0, 0, v, "")
    return s[len(s) - 11:]


# ------------------------------------------------------------ INPUT3D.DAT
@dataclass
class Deck:
    """INPUT3D.DAT, the 16 list-directed rows INITIA reads (:135-150)."""
    Np: Tuple[Tuple[int, int], ...]          # cells left/right of the origin per axis
    ql: Tuple[Tuple[float, float], ...]      # lengths left/right per axis
    vinit: Tuple[Tuple[float, float], ...]   # velocity components (side 1, side 2)
    binit: Tuple[Tuple[float, float], ...]
    cfl: float
    facdep: float
    maxstp: int
    nitera: int
    tfinal: float
    bc: Tuple[int, int, int, int, int, int]
    ifchem: int
    ifthrm: int
    ifrad: int
    ifgrv: int

    @property
    def shape(self):
        return tuple(a + b for a, b in self.Np)

    @property
    def box(self):
        return tuple(a + b for a, b in self.ql)


def _values(line: str) -> List[str]:
    return [v for v in re.split(r"[,\s]+", line.strip()) if v]


def _num(v: str) -> float:
    return float(re.sub(r"[dD]", "e", v))


def read_input3d(path) -> Deck:
    """Parse INPUT3D.DAT (Fortran list-directed values, D exponents)."""
    rows = [r for r in open(path).read().splitlines() if r.strip()]
    if len(rows) < 16:
        raise ValueError(f"{path}: INPUT3D.DAT has 16 rows, found {len(rows)}")
    v = [_values(r) for r in rows[:16]]

    def pair(r, conv=float):
        return (conv(_num(v[r][0])), conv(_num(v[r][1])))

    return Deck(Np=(pair(0, int), pair(1, int), pair(2, int)), ql=(pair(3), pair(4), pair(5)),
                vinit=(pair(6), pair(7), pair(8)), binit=(pair(9), pair(10), pair(11)),
                cfl=_num(v[12][0]), facdep=_num(v[12][1]), maxstp=int(_num(v[13][0])),
                nitera=int(_num(v[13][1])), tfinal=_num(v[13][2]),
                bc=tuple(int(_num(x)) for x in v[14][:6]),
                ifchem=int(_num(v[15][0])), ifthrm=int(_num(v[15][1])), ifrad=int(_num(v[15][2])),
                ifgrv=int(_num(v[15][3])))
