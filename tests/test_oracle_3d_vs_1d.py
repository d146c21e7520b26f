"""The 3D restatement against the 1D one on a plane-parallel problem.

The reference ships no 3D golden data; its only reference-produced numbers
are 1D (cooling.dat, bw051.dat), which pin the 1D restatement
(test_oracle_golden.py).  Here the 3D restatement of MCF3DSGincfca3.f90
runs the KI colliding flow of KIcool/INPUT.DAT (128 cells over 20 pc,
+-48.89, Bx = By = 1.57734, p/kB = 8810.8 K cm^-3) as a 128 x 4 x 4 slab,
periodic across the flow, to the time the 1D restatement reaches in 200
steps.  The two codes differ in the transverse update (MOC + constrained
transport in 3D, the 1D scheme's own MOC) and in the species floors, so the
agreement is close but not exact; the tolerances below are a few times the
observed differences (rho 0.9 %, p 1.9 %, vx 0.16 %).
"""
import numpy as np

from code_tohoku_gb300 import problems
from oracle.pyoracle import Oracle1D, Oracle3D


def _ki_deck(half_cells):
    spec = [(1.0, 1.0)] + [(0.0, 0.0)] * 7
    return problems._deck_vector(half_cells, half_cells, 10.0, 10.0, (1.0, 1.0), (48.89, -48.89), (0, 0),
                                 (0, 0), (1.0, 0.1), (1.57734, 1.57734), (1.57734, 1.57734), (0, 0), spec,
                                 0.49, 1.0, 40.0, (1, 1), 2, 0, 8.810807e3 * problems.KB * 1.0e-3)


def _slab_from_1d(s0, ny=4, nz=4):
    """The 1D initial state (x, U1..U8, 8 species per cell) as a 3D slab."""
    nx = s0.shape[0]
    dx = s0[1, 0] - s0[0, 0]
    p = problems.MhdParams(nx, ny, nz, cfl=0.49, bc=(1, 1, 3, 3, 3, 3), ifthrm=2, dissip=0)
    st = problems._empty_state(p, nx * dx, ny * dx, nz * dx)

    def col(c):   # interior profile with the free-boundary ghost copies
        return np.concatenate([[s0[0, c]] * 2, s0[:, c], [s0[-1, c]] * 2])[None, None, :]

    for q in range(5):
        st.U[q][...] = col(1 + q)
    st.U[5][...] = s0[0, 6]   # uniform Bx on the x faces
    st.U[6][...] = col(7)
    st.U[7][...] = col(8)
    for s in range(8):
        st.species[s][...] = col(9 + s)
    return st


def test_plane_parallel_slab_follows_1d():
    o1 = Oracle1D(_ki_deck(64))
    s0 = o1.state()
    o3 = Oracle3D(_slab_from_1d(s0).params)
    o3.upload(_slab_from_1d(s0))
    for _ in range(200):
        o1.step()
    t1 = o1.time
    steps = 0
    while o3.time < t1 and steps < 1000:
        o3.step(t1)
        steps += 1
    assert o3.time == t1
    U, _, _ = o3.download()
    s1 = o1.state()

    def l1(a, b):
        return np.abs(a - b).mean() / np.abs(b).mean()

    for j, k in ((2, 2), (3, 5)):   # every column of the slab carries the same solution
        rho, p, vx = U[0][k, j, 2:-2], U[4][k, j, 2:-2], U[1][k, j, 2:-2]
        assert l1(rho, s1[:, 1]) < 0.03
        assert l1(p, s1[:, 5]) < 0.06
        assert l1(vx, s1[:, 2]) < 0.01
        # the cooled layer at the collision plane: peak density within 5 %
        assert abs(rho.max() - s1[:, 1].max()) < 0.05 * s1[:, 1].max()
        assert s1[:, 1].max() > 20.0
