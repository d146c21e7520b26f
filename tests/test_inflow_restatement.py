"""The BC = 4 inflow boundary on both x sides (the shipped deck's), restated
in NumPy from the Fortran and composed with the restated parts of the step
into whole EVOLVE iterations, against the oracle's steps bit for bit.

On an inflow side there is no neighbour (LEFT / RIGT = MPI_PROC_NULL,
3DMHD-CfCA/MCF3DSG.f90:150-151), so the ghosts take only the assigned
values of BC_MPI (3DMHD-CfCA/MCF3DSGincfca3.f90:814-890) and BC_MPI_OT
(:948-1080), from INITIA's BBRV (:191-200):

* density from the DTF reservoir at the ghost's position moved back by
  v_in t and wrapped into the box (:820-826, :856-862);
* velocities, pressure and the transverse face fields at their inflow
  values — in the conservative exchanges (mode 2) momentum from the ghost's
  own density along x and from the reference density across, and total
  energy from the inflow pressure, the ghost's density and x field and
  the inflow transverse field (:833-843);
* the normal face field copied from the boundary face, the right side's
  face N+1 kept (:827-831, :863-867); the cell-centred x field and the
  face velocities copied from the edge cell; the Lagrangian fields at their
  inflow values; the Lagrangian widths at dx(0) and dx(N+1);
* the species as the inflow abundances times the ghost's density, on rows
  with interior transverse indices only (:1050-1080).

The reservoir is random and the inflow fast, so the reservoir cell a ghost
reads changes between the steps."""
import numpy as np
import pytest

from code_tohoku_gb300 import problems
from oracle.pyoracle import Oracle3D
from test_step_restatement import step
from test_sweep_restatement import exchange, local, make_state


class InflowX:
    """The x exchange of a run with BC = 4 on both x sides; arrays come in
    the x frame (x, y, z), padded along x."""

    def __init__(self, inflow, dtf, st):
        self.rho = inflow.rho_ref
        self.v, self.p, self.b, self.cm = inflow.v, inflow.p, inflow.b, inflow.species
        self.dtf = local(dtf.astype(np.float64), 0)
        self.x, self.dx = st.x, st.dx
        self.N = st.params.nx
        self.time = 0.0

    def ghosts(self, side, nol):
        """Padded x indices of the ghost layers of one side."""
        N = self.N
        return [g + 1 for g in range(1 - nol, 1)] if side == 0 else [g + 1 for g in range(N + 1, N + nol + 1)]

    def column(self, side, g):
        """The reservoir's x index II that ghost g (Fortran index) reads."""
        dx0 = self.dx[1]
        L = dx0 * self.N * 1
        if side == 0:
            xp = self.x[1] - 0.5 * dx0 + g * dx0 - self.time * self.v[0][0]
            xp = xp + L * (int(abs(xp) / L) + 1)
        else:
            xp = 0.5 * (self.x[g] + self.x[g + 1]) - self.time * self.v[1][0]
            xp = xp - L * int(abs(xp) / L)
        return int(xp / dx0) + 1

    def reservoir(self, side, g):
        return self.dtf[self.column(side, g) + 1]

    def __call__(self, kind, a, nol, mode, U1, Bcc1):
        N = self.N
        for side in (0, 1):
            v, b = self.v[side], self.b[side]
            edge = 2 if side == 0 else N + 1        # the edge cell (or face 1 / face N+1)
            for q in self.ghosts(side, nol):
                if kind == ("U", 0):
                    a[q] = self.reservoir(side, q - 1)
                elif kind == ("U", 1):
                    a[q] = v[0] if mode == 1 else U1[q] * v[0]
                elif kind in (("U", 2), ("U", 3)):
                    a[q] = v[kind[1] - 1] if mode == 1 else self.rho * v[kind[1] - 1]
                elif kind == ("U", 4):
                    a[q] = self.p[side] if mode == 1 else \
                        self.p[side] * 1.5 + 0.5 * (U1[q] * (v[0] * v[0]) + Bcc1[q] * Bcc1[q] + b[1] * b[1]
                                                    + b[2] * b[2])
                elif kind == ("U", 5):
                    if side == 0:
                        a[q] = a[2]
                    elif q >= N + 3:
                        a[q] = a[N + 2]
                elif kind in (("U", 6), ("U", 7)):
                    a[q] = b[kind[1] - 5]
                elif kind[0] == "sp":
                    a[q, 2:-2, 2:-2] = self.cm[kind[1]] * U1[q, 2:-2, 2:-2]
                elif kind == ("dxlag",):
                    a[q] = self.dx[1] if side == 0 else self.dx[N + 2]
                elif kind[0] == "Blg":
                    a[q] = b[1 + kind[1]]
                elif kind == ("Bcc", 0) or kind[0] == "Vfc":
                    a[q] = a[edge]
                elif kind[0] == "Bcc":
                    a[q] = b[kind[1]]
                else:
                    raise AssertionError(kind)


def dissip_fill(xf, p):
    """DISSIP's exchange of v_q: the inflow x ghosts, then y and z."""
    n = (p.nx, p.ny, p.nz)

    def fill(q, v):
        xf(("U", q), local(v, 0), 2, 1, None, None)
        for d in (1, 2):
            exchange(local(v, d), n[d], (p.bc[2 * d], p.bc[2 * d + 1]))
    return fill


def make_inflow(st, seed):
    rng = np.random.default_rng(seed)
    cm = np.array(problems.reference_inflow((1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 1.0, 0.0)).species)
    inflow = problems.Inflow(rho_ref=1.31, v=((30.0, 2.0, -1.0), (-28.0, 1.0, 2.0)), p=(35.0, 31.0),
                             b=((0.7, 2.2, -0.4), (0.5, 1.9, 0.3)), species=tuple(cm))
    dtf = (problems.MU * np.exp(rng.normal(0.0, 0.4, st.U[0].shape))).astype(np.float32)
    return inflow, dtf


@pytest.mark.parametrize("first", [1, 2])
def test_inflow_steps_match_the_composed_restatements(first):
    st = make_state((20, 9, 8), (4, 4, 3, 3, 3, 3), 23)
    p = st.params
    inflow, dtf = make_inflow(st, 5)
    o = Oracle3D(p)
    o.upload(st)
    o.set_inflow(inflow.vector(), dtf, 0.0)
    o.set_order(first)
    U, sp, bcc = o.download()
    xf = InflowX(inflow, dtf, st)
    reads = set()
    for s in range(4):
        ifevo = (first - 1 + s) % 6 + 1
        reads.add((xf.column(0, -1), xf.column(1, p.nx + 1)))
        U, sp, bcc, dt, lim = step(U, sp, bcc, st, ifevo, xf, dissip_fill(xf, p))
        dto, limo = o.step()
        Uo, spo, bcco = o.download()
        assert dt == dto and lim == limo, (s, dt, dto, lim, limo)
        assert np.all(np.isfinite(Uo))
        for f in range(8):
            assert np.array_equal(U[f], Uo[f]), (s, f, np.argwhere(U[f] != Uo[f])[:4])
        for q in range(8):
            assert np.array_equal(sp[q], spo[q]), (s, q)
        for c in range(3):
            assert np.array_equal(bcc[c], bcco[c]), (s, c)
        xf.time += dt
    # the ghosts read more than one reservoir column over the run
    assert len(reads) > 1, reads
