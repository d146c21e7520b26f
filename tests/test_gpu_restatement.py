"""The CUDA FP64 path against the NumPy restatements of the Fortran
directly, not through the oracle: whole EVOLVE iterations bit for bit, on
free and periodic boundaries with KI cooling, and on the shipped deck's
configuration (inflow on both x sides from a random reservoir, the
chemistry on).  The restated steps start from the state the GPU holds after
its upload (its cell-centred field and, with the chemistry, INITIA's
species totals).  Every padded cell of U and of the cell-centred field is
compared; the species on cells 0..n+1 of every direction: the outer ghost
layer of the species (-1 and n+2) holds, in the reference, what the last
sweep's exchange copied there, which no later step reads, and the GPU's
sweeps make those exchanges in shared memory only."""
import numpy as np
import pytest

from code_tohoku_gb300 import native
from test_chem_exact_restatement import deck_state, deck_step, totals
from test_inflow_restatement import InflowX, make_inflow
from test_step_restatement import step
from test_sweep_restatement import make_state

pytestmark = pytest.mark.gpu


def same(a, b, what):
    for q in range(a.shape[0]):
        assert np.array_equal(a[q], b[q]), (what, q, np.argwhere(a[q] != b[q])[:3])


def test_gpu_steps_equal_the_restatement():
    st = make_state((20, 9, 8), (1, 1, 3, 3, 3, 3), 17)
    g = native.Mhd3D(st.params, precision=native.PREC_FP64)
    g.upload(st)
    U, sp, bcc = g.download()
    for s in range(3):
        U, sp, bcc, dt, lim = step(U, sp, bcc, st, s + 1)
        dtg, limg = g.step()
        assert (dt, lim) == (dtg, limg), s
        Ug, spg, bccg = g.download()
        same(U, Ug, "U")
        same(sp[:, 1:-1, 1:-1, 1:-1], spg[:, 1:-1, 1:-1, 1:-1], "species")
        same(bcc, bccg, "Bcc")


def test_gpu_shipped_deck_steps_equal_the_restatement():
    st = deck_state((20, 9, 8), (4, 4, 3, 3, 3, 3), 29)
    p = st.params
    inflow, dtf = make_inflow(st, 6)
    g = native.Mhd3D(p, precision=native.PREC_FP64)
    g.set_inflow(inflow, dtf, 0.0)
    g.upload(st)
    U, sp, bcc = g.download()
    col = np.zeros((10,) + U[0].shape)
    nde, ndtot = np.zeros_like(U[0]), np.zeros_like(U[0])
    Kp, Jp, Ip = slice(2, p.nz + 3), slice(2, p.ny + 3), slice(2, p.nx + 3)
    nde[Kp, Jp, Ip], ndtot[Kp, Jp, Ip] = totals([s_[Kp, Jp, Ip] for s_ in sp])
    xf = InflowX(inflow, dtf, st)
    for s in range(3):
        U, sp, bcc, nde, ndtot, dt, lim = deck_step(U, sp, bcc, nde, ndtot, col, st, s + 1, xf)
        xf.time += dt
        dtg, limg = g.step()
        assert (dt, lim) == (dtg, limg), s
        Ug, spg, bccg = g.download()
        same(U, Ug, "U")
        same(sp[:, 1:-1, 1:-1, 1:-1], spg[:, 1:-1, 1:-1, 1:-1], "species")
        same(bcc, bccg, "Bcc")
