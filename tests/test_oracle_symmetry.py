"""Symmetry pins of the 3D-only routines on the oracle.

The reference ships no 3D output, so CC(1..4), CCT (MCF3DSGincfca3.f90
:2115-2445, with its three iwx / iwy / iwz branches), MOC's and REMAP's
per-direction index maps (:1939-2098, :1556-1686) and the ghost exchanges
between sweeps are pinned by symmetry instead: the step of a rotated state
(x -> y -> z -> x, with the rotated sweep order) must be the rotated step of
the state, and the step of an x-mirrored state the mirrored step.  The
mirror runs every interface through the other upwind branch (Bn <= 0,
vadt > 0, ...).  A mis-indexed slope, a swapped EMF candidate or a wrong
axis in one branch changes results at the 1e-3 level after one step;
what remains is round-off, because the reference sums v^2 and B^2 (E <->
p) and the conduction fluxes in a fixed x, y, z order, which a rotation
or mirror reorders.  In a single sweep, rho, v and B are bit-identical.
"""
import numpy as np
import pytest

from oracle.pyoracle import Oracle3D
from symmetry_util import ROT_ORDER, mirror_state, random_state, rot_bcc, rot_state

C = (slice(2, -2),) * 3


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _oracle(st):
    o = Oracle3D(st.params)
    o.upload(st)
    return o


@pytest.mark.parametrize("d", [0, 1, 2])
def test_rotated_single_sweep(d):
    st = random_state(seed=3)
    o1, o2 = _oracle(st), _oracle(rot_state(st))
    dt, _ = o1.timestep()
    assert o2.timestep()[0] == dt
    o1.sweep(d, dt)
    o2.sweep((d + 1) % 3, dt)
    U1, s1, _ = o1.download()
    U2, _, _ = o2.download()
    R = rot_state(st, U1, s1)
    for q in (0, 1, 2, 3, 5, 6, 7):
        assert np.array_equal(R.U[q][C], U2[q][C]), q
    assert _rel(R.U[4][C], U2[4][C]) < 1e-13


@pytest.mark.parametrize("cooling", [False, True])
def test_rotated_steps(cooling):
    """12 full steps (both orders of every sweep pair, CT, SOURCE), the same
    dt given to both states."""
    st = random_state(seed=4, cooling=cooling)
    o1, o2 = _oracle(st), _oracle(rot_state(st))
    for k in range(12):
        e = k % 6 + 1
        o1.set_order(e)
        o2.set_order(ROT_ORDER[e])
        dt, _ = o1.timestep()
        assert abs(o2.timestep()[0] / dt - 1.0) < 1e-13
        o1.advance(dt)
        o2.advance(dt)
    U1, s1, b1 = o1.download()
    U2, _, b2 = o2.download()
    R = rot_state(st, U1, s1)
    for q in range(8):
        assert _rel(R.U[q][C], U2[q][C]) < 1e-12, q
    rb = rot_bcc(b1)
    for q in range(3):
        assert _rel(rb[q][C], b2[q][C]) < 1e-12, q


def test_mirrored_steps():
    st = random_state(seed=5)
    o1, o2 = _oracle(st), _oracle(mirror_state(st))
    for k in range(6):
        o1.set_order(k + 1)
        o2.set_order(k + 1)
        dt, _ = o1.timestep()
        o1.advance(dt)
        o2.advance(dt)
    U1, s1, _ = o1.download()
    U2, _, _ = o2.download()
    R = mirror_state(st, U1, s1)
    for q in range(8):
        assert _rel(R.U[q][C], U2[q][C]) < 1e-12, q


def test_symmetry_catches_a_swapped_index():
    """The pin has teeth: the same comparison between a state and a rotated
    image whose face field is NOT rotated with it fails after one step."""
    st = random_state(seed=6)
    bad = rot_state(st)
    bad.U[5], bad.U[6] = bad.U[6].copy(), bad.U[5].copy()
    o1, o2 = _oracle(st), _oracle(bad)
    o1.set_order(1)
    o2.set_order(2)
    dt, _ = o1.timestep()
    o1.advance(dt)
    o2.advance(dt)
    U1, s1, _ = o1.download()
    U2, _, _ = o2.download()
    R = rot_state(st, U1, s1)
    assert max(_rel(R.U[q][C], U2[q][C]) for q in range(8)) > 1e-3
