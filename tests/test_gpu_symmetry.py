"""Rotation and mirror symmetry of the GPU step (see test_oracle_symmetry.py
for the construction).  The plain FP64 kernels are the oracle bit for bit,
so their images agree to round-off; the chosen form's sweeps are written
per direction (the x sweep folds its ghost loads into the pencil pass, y and
z use other CTA shapes) and its EMF kernel per edge direction, so the pin
checks that each direction's FP32 kernels index the same physics: images
agree to FP32 rounding (measured ~1e-6 of each field's range), where a
mis-indexed stencil term gives ~1e-3."""
import numpy as np
import pytest

from code_tohoku_gb300 import native
from symmetry_util import ROT_ORDER, mirror_state, random_state, rot_bcc, rot_state

pytestmark = pytest.mark.gpu
C = (slice(2, -2),) * 3


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _pair(st, st2, precision):
    g1 = native.Mhd3D(st.params, precision=precision)
    g1.upload(st)
    g2 = native.Mhd3D(st2.params, precision=precision)
    g2.upload(st2)
    return g1, g2


@pytest.mark.parametrize("precision,tol", [(native.PREC_FP64, 1e-12), (native.PREC_FP32, 1e-4)])
@pytest.mark.parametrize("cooling", [False, True])
def test_rotated_steps_gpu(precision, tol, cooling):
    st = random_state(n=24, seed=11, cooling=cooling)
    g1, g2 = _pair(st, rot_state(st), precision)
    for k in range(6):
        e = k % 6 + 1
        g1.set_time(g1.time, e)
        g2.set_time(g2.time, ROT_ORDER[e])
        dt, _ = g1.timestep()
        g1.advance(dt)
        g2.advance(dt)
    U1, s1, b1 = g1.download()
    U2, _, b2 = g2.download()
    R = rot_state(st, U1, s1)
    errs = [_rel(R.U[q][C], U2[q][C]) for q in range(8)]
    rb = rot_bcc(b1)
    errs += [_rel(rb[q][C], b2[q][C]) for q in range(3)]
    assert max(errs) < tol, errs


@pytest.mark.parametrize("precision,tol", [(native.PREC_FP64, 1e-12), (native.PREC_FP32, 1e-4)])
def test_mirrored_steps_gpu(precision, tol):
    st = random_state(n=24, seed=12)
    g1, g2 = _pair(st, mirror_state(st), precision)
    for k in range(6):
        g1.set_time(g1.time, k + 1)
        g2.set_time(g2.time, k + 1)
        dt, _ = g1.timestep()
        g1.advance(dt)
        g2.advance(dt)
    U1, s1, _ = g1.download()
    U2, _, _ = g2.download()
    R = mirror_state(st, U1, s1)
    errs = [_rel(R.U[q][C], U2[q][C]) for q in range(8)]
    assert max(errs) < tol, errs
