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


def test_brio_wu_gamma_two_only_in_the_wave_speeds():
    """1DMHDmany/1DMHDwCC3bw.f90 forces gamma = 2 in the Courant limit (:752)
    and the dependency-domain sound speeds of RHS (:490, :498), while the
    energy <-> pressure conversions (:436-440, :544-546) and the Riemann
    solver (:520) keep the species gamma (5/3 for the deck's atomic gas).
    Pinned three ways: the first dt is CFL * min dx / (sqrt((2 p + B^2) /
    rho) + |vx|) bit for bit; total energy with p / (5/3 - 1) is conserved
    while the waves stay inside the tube (with p / (2 - 1) it is not); and
    the momenta change by exactly the boundary fluxes of the two uniform
    end states over t = 0.1: x by (p_L - p_R) t = 0.09, y by
    Bx (By_R - By_L) t = -0.15 (magnetic pressure B^2 / 2 in these units)."""
    o = Oracle1D(problems.brio_wu_deck(800, tfinal=0.1, cfl=0.5))
    s0 = o.state()
    dx = 0.5 / 400

    def totals(s, gamma):
        rho, vx, vy, vz, p, bx, by, bz = (s[:, q] for q in range(1, 9))
        e = p / (gamma - 1.0) + 0.5 * rho * (vx ** 2 + vy ** 2 + vz ** 2) + 0.5 * (bx ** 2 + by ** 2 + bz ** 2)
        return np.array([rho.sum(), (rho * vx).sum(), (rho * vy).sum(), e.sum()]) * dx

    rho, vx, p, bx, by, bz = s0[:, 1], s0[:, 2], s0[:, 5], s0[:, 6], s0[:, 7], s0[:, 8]
    c2 = (2.0 * p + bx * bx + by * by + bz * bz) / rho
    dt_gamma2 = 0.5 * np.min(dx / (np.sqrt(c2) + np.abs(vx)))
    c2_53 = (5.0 / 3.0 * p + bx * bx + by * by + bz * bz) / rho
    dt_gamma53 = 0.5 * np.min(dx / (np.sqrt(c2_53) + np.abs(vx)))
    dt1 = o.step()
    assert dt1 == dt_gamma2
    assert abs(dt1 / dt_gamma53 - 1.0) > 5e-3
    while o.time < 0.1 - 1e-15:
        o.step()
    s = o.state()
    m0, m1 = totals(s0, 5.0 / 3.0), totals(s, 5.0 / 3.0)
    assert abs(m1[0] - m0[0]) < 1e-10 * m0[0]               # mass
    assert abs(m1[1] - 0.09) < 1e-11 and abs(m1[2] + 0.15) < 1e-11
    assert abs(m1[3] - m0[3]) < 1e-10 * m0[3]               # energy with gamma = 5/3
    e2 = totals(s, 2.0)[3] - totals(s0, 2.0)[3]
    assert abs(e2) > 1e-3 * totals(s0, 2.0)[3]
