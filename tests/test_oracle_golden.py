"""The oracle's 1D restatement against the reference's own golden output.

KIcool/1DMHDwCC3.f90 wrote cooling.dat (one row per step) and bw051.dat
(the full state after 5000 steps); the fixtures under tests/golden/ were
extracted from those files by tests/golden/make_fixtures.py.  Matching them
pins the restated Riemann solver, MOC, remap, limiter, KI cooling function,
IMC bisection and time-step control to the reference's arithmetic.
"""
import os

import numpy as np
import pytest

from code_tohoku_gb300 import problems
from oracle.pyoracle import Oracle1D


@pytest.fixture(scope="module")
def ki_run(golden_dir):
    tr = np.load(os.path.join(golden_dir, "ki_cooling_trace.npz"))
    bw = np.load(os.path.join(golden_dir, "ki_bw051.npz"))
    o = Oracle1D(problems.ki_shock_tube_deck())
    first = o.run_trace(5000, probe_n=512, probe_b=510)
    state = o.state()
    rest = o.run_trace(5080 - 5000)
    return tr, bw, np.vstack([first, rest]), state


def test_cooling_trace_first_steps_bit_exact(ki_run):
    tr, _, mine, _ = ki_run
    rows, ref = tr["rows"], tr["trace"]
    # row 0 is t=0; row k is the state after k steps.  The first ten steps
    # reproduce the reference to the last bit.
    sel = (rows >= 1) & (rows <= 10)
    assert np.array_equal(mine[rows[sel] - 1], ref[sel])


def test_cooling_trace_all_rows(ki_run):
    tr, _, mine, _ = ki_run
    rows, ref = tr["rows"], tr["trace"]
    sel = rows >= 1
    rel = np.abs(mine[rows[sel] - 1] - ref[sel]) / np.abs(ref[sel])
    # 5080 steps of a shock-compressed, thermally unstable flow: agreement
    # stays at the 1e-11 level (libm differences of the original run)
    assert rel.max() < 1e-11, rel.max()


def test_bw051_full_state(ki_run):
    _, bw, mine, state = ki_run
    assert abs(mine[4999, 0] - float(bw["time"])) <= 1e-12 * float(bw["time"])
    ref = bw["state"]
    # E19.10 output: half a unit of the 10th significant digit, plus the
    # 1e-11 drift (relative to each column's scale) of 5000 steps
    mag = np.where(ref != 0, np.floor(np.log10(np.abs(ref) + 1e-300)) + 1, 0)
    tol = 0.51e-10 * 10.0 ** mag + 1e-11 * np.abs(ref).max(axis=0)
    assert np.all(np.abs(state - ref) <= tol)


def test_brio_wu_runs_to_tfinal():
    o = Oracle1D(problems.brio_wu_deck(800, tfinal=0.1, cfl=0.5))
    n = 0
    while o.time < 0.1 - 1e-15 and n < 10000:
        o.step()
        n += 1
    s = o.state()
    assert abs(o.time - 0.1) < 1e-14
    rho, p = s[:, 1], s[:, 5]
    assert np.all(rho > 0) and np.all(p > 0)
    # the waves stay inside the tube: both ends keep their initial states
    assert abs(rho[0] - 1.0) < 1e-9 and abs(rho[-1] - 0.125) < 1e-8
    assert rho.max() <= 1.0 + 1e-5 and rho.min() >= 0.1
    By = s[:, 7]
    assert abs(By[0] - 1.0) < 1e-9 and abs(By[-1] + 1.0) < 1e-8
    # the slow compound wave leaves By reversed at the centre
    assert By[400] < -0.5 and np.all(np.abs(s[:, 6] - 0.75) == 0)
