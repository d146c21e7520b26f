"""Whole EVOLVE iterations (3DMHD-CfCA/MCF3DSGincfca3.f90:566-656) composed
from the NumPy restatements of its parts, against the oracle's step bit for
bit: the time step, half a SOURCE, the three sweeps in the order of ifEVO
(:612-641, the six orders in turn), CT, the second half SOURCE and DISSIP.
The composition exercises the exchanges that no single part's test does:
CC(1)'s of the velocity and face-field components before the face
velocities (:2123-2125), of Vfc (:2135) and of U5 (:2137), CC(2)'s of the
density (:2142), and CC(4)'s of the cell-centred field (:2171-2181), whose
ghosts the next step's sweeps read.  Face velocities start undefined (NaN),
as the reference allocates them afresh, so any read of a value CC(1) does
not set would show."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle3D
from test_ct_restatement import emf_edge
from test_dissip_restatement import dissip
from test_source_restatement import source_thermal, timestep
from test_sweep_restatement import exchange, local, make_state, sweep

ORDERS = ((0, 1, 2), (1, 2, 0), (2, 0, 1), (0, 2, 1), (1, 0, 2), (2, 1, 0))


def fill(a, p, dirs, kind=None, xfill=None, U1=None):
    """Two ghost layers in the given directions, in that order;
    xfill(kind, a, 2, 1, U1, None) replaces the exchange along x."""
    n = (p.nx, p.ny, p.nz)
    for d in dirs:
        if d == 0 and xfill is not None:
            xfill(kind, local(a, 0), 2, 1, local(U1, 0), None)
        else:
            exchange(local(a, d), n[d], (p.bc[2 * d], p.bc[2 * d + 1]))


def ct(U, st, dt, xfill=None):
    """CC(1), CC(2) + CCT for the three edges, CC(3), CC(4); returns U and
    the new cell-centred field."""
    p = st.params
    n = (p.nx, p.ny, p.nz)
    dx = (st.dx, st.dy, st.dz)
    U = U.copy()
    F = lambda a, dirs, kind: fill(a, p, dirs, kind, xfill, U[0])
    for d, fields in ((0, (1, 6, 7)), (1, (2, 5, 7)), (2, (3, 5, 6))):
        for f in fields:
            F(U[f], [d], ("U", f))
    Vfc = [np.full_like(U[0], np.nan) for _ in range(3)]
    for d in range(3):
        N, M, L = n[d], n[(d + 1) % 3], n[(d + 2) % 3]
        v, V, w = local(U[1 + d], d), local(Vfc[d], d), dx[d]
        dm = w[1:N + 2][:, None, None]
        d0 = w[2:N + 3][:, None, None]
        T = (slice(2, M + 2), slice(2, L + 2))
        V[(slice(2, N + 3),) + T] = (dm * v[(slice(2, N + 3),) + T] + d0 * v[(slice(1, N + 2),) + T]) / (dm + d0)
    F(Vfc[1], [0], ("Vfc", 1))
    F(Vfc[2], [0, 1], ("Vfc", 2))
    F(Vfc[0], [1, 2], ("Vfc", 0))
    F(Vfc[1], [2], ("Vfc", 1))
    F(U[4], [0, 1, 2], ("U", 4))
    F(U[0], [0, 1, 2], ("U", 0))
    E = []
    for e in range(3):
        da, db, dc = e, (e + 1) % 3, (e + 2) % 3
        full = np.zeros_like(U[0])
        local(full, e)[2:n[da] + 3, 2:n[db] + 3, 2:n[dc] + 2] = emf_edge(e, U, Vfc, dx, n, p.kb, p.facdep, dt)
        E.append(full)
    Ez, Ex, Ey = E
    nx, ny, nz = n
    K, J, I = slice(2, nz + 2), slice(2, ny + 2), slice(2, nx + 2)
    I1, J1, K1 = slice(2, nx + 3), slice(2, ny + 3), slice(2, nz + 3)
    sh = lambda s: slice(s.start + 1, s.stop + 1)
    dyj, dzk, dxi = st.dy[J][None, :, None], st.dz[K][:, None, None], st.dx[I][None, None, :]
    b1 = U[5][K, J, I1] + dt / dyj * (Ez[K, sh(J), I1] - Ez[K, J, I1]) - dt / dzk * (Ey[sh(K), J, I1] - Ey[K, J, I1])
    b2 = U[6][K, J1, I] + dt / dzk * (Ex[sh(K), J1, I] - Ex[K, J1, I]) - dt / dxi * (Ez[K, J1, sh(I)] - Ez[K, J1, I])
    b3 = U[7][K1, J, I] + dt / dxi * (Ey[K1, J, sh(I)] - Ey[K1, J, I]) - dt / dyj * (Ex[K1, sh(J), I] - Ex[K1, J, I])
    U[5][K, J, I1], U[6][K, J1, I], U[7][K1, J, I] = b1, b2, b3
    bcc = np.zeros((3,) + U[0].shape)
    bcc[0][K, J, I] = 0.5 * (U[5][K, J, I] + U[5][K, J, sh(I)])
    bcc[1][K, J, I] = 0.5 * (U[6][K, J, I] + U[6][K, sh(J), I])
    bcc[2][K, J, I] = 0.5 * (U[7][K, J, I] + U[7][sh(K), J, I])
    for c in range(3):
        F(bcc[c], [0, 1, 2], ("Bcc", c))
    return U, bcc


def step(U, sp, bcc, st, ifevo, xfill=None, dfill=None):
    """One iteration; xfill replaces the x exchanges as in the parts,
    dfill(q, v) DISSIP's exchange of velocity component q."""
    p = st.params
    dt, lim, _ = timestep(U, sp, bcc, st)
    U, sp, _ = source_thermal(U, sp, st, 0.5 * dt, xfill)
    coords = (st.x, st.dx, st.y, st.dy, st.z, st.dz)
    for d in ORDERS[ifevo - 1]:
        U, sp = sweep(d, U, sp, bcc, coords, p, dt, xfill)
    U, bcc = ct(U, st, dt, xfill)
    U, sp, _ = source_thermal(U, sp, st, 0.5 * dt, xfill)
    if p.dissip:
        U = U.copy()
        U[1:4] = dissip(U, (p.nx, p.ny, p.nz), dfill)
    return U, sp, bcc, dt, lim


@pytest.mark.parametrize("first", [1, 4])
def test_steps_match_the_composed_restatements(first):
    st = make_state((20, 9, 8), (1, 1, 3, 3, 3, 3), 17)
    o = Oracle3D(st.params)
    o.upload(st)
    o.set_order(first)
    U, sp, bcc = o.download()
    for s in range(3):
        ifevo = (first - 1 + s) % 6 + 1
        U, sp, bcc, dt, lim = step(U, sp, bcc, st, ifevo)
        dto, limo = o.step()
        Uo, spo, bcco = o.download()
        assert dt == dto and lim == limo, (s, dt, dto, lim, limo)
        assert np.all(np.isfinite(Uo))
        for f in range(8):
            assert np.array_equal(U[f], Uo[f]), (s, f)
        for q in range(8):
            assert np.array_equal(sp[q], spo[q]), (s, q)
        for c in range(3):
            assert np.array_equal(bcc[c], bcco[c]), (s, c)
