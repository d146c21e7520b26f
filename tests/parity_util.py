"""Helpers shared by the GPU parity tests: run the same state through the
oracle (CPU restatement) and the CUDA path and compare."""
import numpy as np

from code_tohoku_gb300 import native
from oracle.pyoracle import Oracle3D


def interior_views(U, sp, bcc):
    """Cells 1..N of every field, plus face n+1 of the face-centred B."""
    c = (slice(None), slice(2, -2), slice(2, -2), slice(2, -2))
    out = {"U1-5": U[0:5][c], "species": sp[c], "bcc": bcc[c]}
    out["Bx"] = U[5, 2:-2, 2:-2, 2:-1]
    out["By"] = U[6, 2:-2, 2:-1, 2:-2]
    out["Bz"] = U[7, 2:-1, 2:-2, 2:-2]
    return out


def compare(gpu, ora, exact=True, rtol=0.0):
    Ug, sg, bg = gpu.download()
    Uo, so, bo = ora.download()
    vg, vo = interior_views(Ug, sg, bg), interior_views(Uo, so, bo)
    worst = {}
    for k in vg:
        a, b = vg[k], vo[k]
        if exact:
            bad = np.argwhere(a.view(np.int64) != b.view(np.int64))
            if len(bad):
                idx = tuple(bad[0])
                raise AssertionError(f"{k}: {len(bad)} cells differ, first {idx}: gpu {a[idx]!r} oracle {b[idx]!r}")
        d = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
        worst[k] = float(d.max())
        if not exact:
            assert worst[k] <= rtol, (k, worst[k])
    return worst


def pair(state, precision=native.PREC_FP64):
    g = native.Mhd3D(state.params, precision=precision)
    g.upload(state)
    o = Oracle3D(state.params)
    o.upload(state)
    return g, o
