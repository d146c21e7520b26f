"""DISSIP (3DMHD-CfCA/MCF3DSGincfca3.f90:3143-3173) restated in NumPy from
the Fortran, against the oracle's C++ on the same state: the exchange of
v_x, v_y, v_z (BC_MPI, two layers, primitive mode: free copies in x,
periodic images in y and z, a pass per direction over all transverse
indices), the velocity divergence on the twelve x positions 0..11 of each
x-edge strip, and the damping of cells 1..10 of the strip by a tenth of its
centred differences.  The single-domain run damps both x edges (what every
run with two or more x ranks does).  The arithmetic is the reference's in
its order, so the two agree bit for bit."""
import numpy as np

from code_tohoku_gb300 import problems
from oracle.pyoracle import Oracle3D


def fill_free_x_periodic_yz(a, n):
    """Two ghost layers: x free (copies of cells 1 and n), then y and z
    periodic, each pass over all transverse indices (padded arrays
    [z, y, x], interior 2..n+1)."""
    nx, ny, nz = n
    a[:, :, 0] = a[:, :, 2]
    a[:, :, 1] = a[:, :, 2]
    a[:, :, nx + 2] = a[:, :, nx + 1]
    a[:, :, nx + 3] = a[:, :, nx + 1]
    a[:, 0, :] = a[:, ny, :]
    a[:, 1, :] = a[:, ny + 1, :]
    a[:, ny + 2, :] = a[:, 2, :]
    a[:, ny + 3, :] = a[:, 3, :]
    a[0, :, :] = a[nz, :, :]
    a[1, :, :] = a[nz + 1, :, :]
    a[nz + 2, :, :] = a[2, :, :]
    a[nz + 3, :, :] = a[3, :, :]


def dissip(U, n, fill=None):
    """fill(q, v), when given, replaces the free-x / periodic-y,z exchange
    of velocity component q (1..3)."""
    nx, ny, nz = n
    vx, vy, vz = (U[q].copy() for q in (1, 2, 3))
    for q, v in zip((1, 2, 3), (vx, vy, vz)):
        if fill is None:
            fill_free_x_periodic_yz(v, n)
        else:
            fill(q, v)
    out = [vx.copy(), vy.copy(), vz.copy()]
    J = slice(1, ny + 3)   # j = 0..ny+1 (padded 1..ny+2)
    K = slice(1, nz + 3)
    for off in (0, nx - 10):
        divv = np.zeros((nz + 2, ny + 2, 12))
        for i in range(12):
            ix = i + off + 1   # padded index of x position i + off
            divv[:, :, i] = (vx[K, J, ix + 1] - vx[K, J, ix - 1] + vy[K, 2:ny + 4, ix] - vy[K, 0:ny + 2, ix]
                             + vz[2:nz + 4, J, ix] - vz[0:nz + 2, J, ix]) * 0.25
        for i in range(1, 11):
            ix = i + off + 1
            c = (slice(2, nz + 2), slice(2, ny + 2), ix)
            out[0][c] = vx[c] + 0.1 * (divv[1:nz + 1, 1:ny + 1, i + 1] - divv[1:nz + 1, 1:ny + 1, i - 1])
            out[1][c] = vy[c] + 0.1 * (divv[1:nz + 1, 2:ny + 2, i] - divv[1:nz + 1, 0:ny, i])
            out[2][c] = vz[c] + 0.1 * (divv[2:nz + 2, 1:ny + 1, i] - divv[0:nz, 1:ny + 1, i])
    return out


def test_dissip_matches_an_independent_restatement():
    st = problems.colliding_flows(24)
    rng = np.random.default_rng(21)
    for q in (1, 2, 3):
        st.U[q] += rng.normal(0.0, 3.0, st.U[q].shape)   # every ghost random too
    n = (st.params.nx, st.params.ny, st.params.nz)
    o = Oracle3D(st.params)
    o.upload(st)
    U0, _, _ = o.download()
    o.dissip()
    U1, _, _ = o.download()
    want = dissip(U0, n)
    for q in range(3):
        assert np.array_equal(U1[1 + q][2:-2, 2:-2, 2:-2], want[q][2:-2, 2:-2, 2:-2]), q
    # the strips changed, the middle did not
    assert np.any(U1[1][2:-2, 2:-2, 2:12] != U0[1][2:-2, 2:-2, 2:12])
    assert np.array_equal(U1[1][2:-2, 2:-2, 13:-13], U0[1][2:-2, 2:-2, 13:-13])
