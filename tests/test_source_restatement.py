"""The thermal SOURCE with Koyama–Inutsuka cooling and the time step,
restated in NumPy from the Fortran and checked against the oracle's C++
bit for bit:

* SOURCE's ifthrm = 2 branch (3DMHD-CfCA/MCF3DSGincfca3.f90:2477-2572):
  the one-layer exchanges of U1, U5 and the species, T and the capped
  conduction fluxes (sqrt of the face-weighted T, capped at 3.873) on
  every face of cells 0..N, then two passes over the cells — half a step
  of cooling (explicit where dt <= 0.2 P / (gamma1 |CooL|), else the IMC
  bisection, :2898-2921, 30 halvings in log P to 1e-5) and of conduction
  (switched off where the conduction time, built on dx alone, is shorter
  than dt), the exchange of U5 and fresh T and fluxes, then the full step
  from the pass's input pressure — with the pressure floor and ceiling;
* the KI cooling function (KIcool/1DMHDwCC3.f90:1166-1173) of the cell's
  density;
* the time step (EVOLVE :569-596 for one rank): Couran (:1912-1930) with
  the fast-magnetosonic speed, Stblty (:2784-2822) with the conduction
  limit at T <= 15 and the cooling time floored at 2.5e-4, and the limiter
  id.

exp, log10 and 10**x are the oracle's own deterministic routines (called
through the oracle library, so that the comparison can be exact); every
other operation is NumPy's IEEE arithmetic in the Fortran's order."""
import numpy as np
import pytest

from code_tohoku_gb300 import problems
from oracle.pyoracle import Oracle3D, detmath
from test_sweep_restatement import fmax2, fmin2, local, sgn


def dexp(x):
    return detmath("exp", x)


def fcool_ki(T, NN):
    T0, absl = 1.0e3, 3.94656e1
    laml = fmin2(1.0e7 * dexp(-1.184e5 / (T * T0 + 1.0e3)), 5.e3)
    lamc = 1.4e-2 * np.sqrt(T * T0) * dexp(-9.2e1 / (T * T0))
    return (NN * NN * (laml + lamc) - NN) * absl


def imc(P, n, dt, g1c, cool, kb):
    """IMC: bisection of P_new + CooL(P_new) dt gamma1 = P in log P; cool(T)
    is the cooling function of the cells at temperatures T."""
    Pu = np.full_like(P, 1.e10)
    Pd = np.full_like(P, 1.e-10)
    Pm = np.full_like(P, 1.e1)
    Pmold = np.full_like(P, -1.0)
    nkbi = 1.0 / (kb * n)
    active = np.ones(P.shape, dtype=bool)
    for _ in range(30):
        C = cool(Pm * nkbi)
        iud = sgn(1.0, Pm + C * dt * g1c - P)
        Pd = np.where(active, fmax2(-iud * Pm, Pd), Pd)
        Pu = np.where(active, fmin2(2.0 * Pm / (iud + 1.0 + 1.e-10), Pu), Pu)
        mid = 0.5 * (detmath("log10", Pu) + detmath("log10", Pd))
        Pm = np.where(active, detmath("exp10", mid), Pm)
        done = active & (np.abs(Pm - Pmold) < 1.e-5)
        Pmold = np.where(active & ~done, Pm, Pmold)
        active &= ~done
    return Pm


def exchange1(a, N, bc, species=False):
    """One ghost layer along axis 0 on every row: the periodic image, then
    the edge cell's copy on a free side (species: interior rows only)."""
    a[1] = a[N + 1]
    a[N + 2] = a[2]
    r = a[:, 2:a.shape[1] - 2, 2:a.shape[2] - 2] if species else a
    if bc[0] == 1:
        r[1] = r[2]
    if bc[1] == 1:
        r[N + 2] = r[N + 1]


def exchange_all(a, p, species=False, kind=None, xfill=None, U1=None):
    """x, y, z in turn; xfill(kind, a, 1, 1, U1, None) replaces x's."""
    n = (p.nx, p.ny, p.nz)
    for d in range(3):
        if d == 0 and xfill is not None:
            xfill(kind, local(a, 0), 1, 1, local(U1, 0), None)
        else:
            exchange1(local(a, d), n[d], (p.bc[2 * d], p.bc[2 * d + 1]), species)


def gammi1(sp):
    h = sp[0] + sp[1] + sp[3] + sp[4]
    return (2.0 * h + 2.0 * sp[2]) / (3.0 * h + 5.0 * sp[2])


def source_thermal(U, sp, st, dt, xfill=None, cool=None):
    """cool(T, sel): the cooling function of the interior cells selected by
    the mask sel (all for None) at temperatures T; KI by default."""
    p = st.params
    U, sp = U.copy(), sp.copy()
    nx, ny, nz = p.nx, p.ny, p.nz
    K, J, I = slice(2, nz + 2), slice(2, ny + 2), slice(2, nx + 2)
    dx, dy, dz = st.dx, st.dy, st.dz
    kb, kc = p.kb, p.kcond
    with np.errstate(all="ignore"):
        exchange_all(U[0], p, False, ("U", 0), xfill, U[0])
        exchange_all(U[4], p, False, ("U", 4), xfill, U[0])
        for s in range(8):
            exchange_all(sp[s], p, True, ("sp", s), xfill, U[0])
        ntot = sp[1] + sp[0] + sp[2] + sp[3] + sp[4]          # p, H, H2, He, He+
        nimc = sp[0] + sp[1] + sp[3] + sp[4] + sp[2]          # H, p, He, He+, H2

        def temps_fluxes():
            Tn = U[4] / (kb * ntot)
            Q = []
            for ax, w in ((2, dx), (1, dy), (0, dz)):
                T0 = np.delete(Tn, -1, axis=ax)
                T1 = np.delete(Tn, 0, axis=ax)
                sh = [1, 1, 1]
                sh[ax] = -1
                d0 = w[:-1].reshape(sh)
                d1 = w[1:].reshape(sh)
                rt = np.sqrt((d0 * T1 + d1 * T0) / (d0 + d1))
                Q.append(kc * fmin2(rt, 3.873) * (T1 - T0) * 2.0 / (d0 + d1))
            Qx, Qy, Qz = Q
            div = ((Qx[K, J, 2:nx + 2] - Qx[K, J, 1:nx + 1]) / dx[I][None, None, :]
                   + (Qy[K, 2:ny + 2, I] - Qy[K, 1:ny + 1, I]) / dy[J][None, :, None]
                   + (Qz[2:nz + 2, J, I] - Qz[1:nz + 1, J, I]) / dz[K][:, None, None])
            return Tn[K, J, I], div

        Pn = U[4][K, J, I].copy()
        NN = U[0][K, J, I] / 1.27
        if cool is None:
            cool = lambda T, sel: fcool_ki(T, NN if sel is None else NN[sel])
        g1c = gammi1([s[K, J, I] for s in sp])
        n = nimc[K, J, I]
        stats = {}
        for ps in (0, 1):
            if ps == 1:
                exchange_all(U[4], p, False, ("U", 4), xfill, U[0])
            Tn, div = temps_fluxes()
            C = cool(Tn, None)
            expl = dt <= 0.2 * Pn / (g1c * np.abs(C))
            imp = ~expl
            sub = lambda T: cool(T, imp)
            if ps == 0:
                P = np.where(expl, U[4][K, J, I] - g1c * C * dt * 0.5, 0.0)
                P[imp] = imc(U[4][K, J, I][imp], n[imp], dt * 0.5, g1c[imp], sub, kb)
            else:
                P = np.where(expl, Pn - g1c * C * dt, 0.0)
                P[imp] = imc(Pn[imp], n[imp], dt, g1c[imp], sub, kb)
            tcd = g1c * kc * np.sqrt(Tn)
            tcd = 0.49 * n * kb / tcd * (dx[I] * dx[I])[None, None, :]
            tcd = sgn(0.5, tcd - dt)
            if ps == 0:
                P = P + (tcd + 0.5) * g1c * dt * 0.5 * div
            else:
                P = P + (tcd + 0.5) * g1c * dt * div
            U[4][K, J, I] = fmin2(fmax2(P, p.pmin), p.pmax)
            stats[ps] = (int(np.count_nonzero(expl)), int(np.count_nonzero(~expl)),
                         int(np.count_nonzero(tcd > 0)), int(np.count_nonzero(tcd < 0)))
    return U, sp, stats


def timestep(U, sp, bcc, st, cool=None):
    """cool(T): the cooling function of the interior cells (KI by default)."""
    p = st.params
    nx, ny, nz = p.nx, p.ny, p.nz
    K, J, I = slice(2, nz + 2), slice(2, ny + 2), slice(2, nx + 2)
    u = [f[K, J, I] for f in U]
    s = [a[K, J, I] for a in sp]
    b = [a[K, J, I] for a in bcc]
    dx = st.dx[I][None, None, :]
    dy = st.dy[J][None, :, None]
    dz = st.dz[K][:, None, None]
    h = s[0] + s[1] + s[3] + s[4]
    gam = (5.0 * h + 7.0 * s[2]) / (3.0 * h + 5.0 * s[2])
    c = np.sqrt((gam * u[4] + b[0] * b[0] + b[1] * b[1] + b[2] * b[2]) / u[0])
    tcfl = min(p.tfinal, np.min(dx / (c + np.abs(u[1]))), np.min(dy / (c + np.abs(u[2]))),
               np.min(dz / (c + np.abs(u[3]))))
    Nn = s[1] + s[0] + s[2] + s[3] + s[4]
    Tn = u[4] / (p.kb * Nn)
    dl = fmin2(fmin2(dx, dy), dz)
    g1c = gammi1(s)
    alpha = g1c * p.kcond * np.sqrt(fmin2(Tn, 15.0))
    alpha = 0.4 * Nn * p.kb / alpha * (dl * dl)
    C = fcool_ki(Tn, u[0] / 1.27) if cool is None else cool(Tn)
    tauC = fmax2(0.2 * (u[4] / g1c / np.abs(C)), 2.5e-4)
    tlmt = min(p.tfinal, np.min(tauC), np.min(alpha))
    dtm = min(p.tfinal, p.cfl * tcfl)
    stt = dtm
    dtm = min(dtm, tlmt)
    which = "cfl" if dtm == stt else ("conduction" if np.min(alpha) < np.min(tauC) else "cooling")
    return min(p.tfinal, dtm), (2 if dtm < stt else 1), which


def make_state(n, bc, seed, lengths=(0.6, 0.5, 0.4), rho=(1.0, 1.6), trange=(0.03, 20.0), vel=3.0, bmag=2.0):
    """By default cells small enough that conduction is switched off in
    the thinnest, densities (scale, lognormal width) over four decades and
    T from 30 K to 2e4 K (trange in 1e3 K), so that both the explicit and
    the implicit cooling and both conduction branches run."""
    nx, ny, nz = n
    p = problems.MhdParams(nx, ny, nz, bc=bc, ifthrm=2)
    sh = (nz + 4, ny + 4, nx + 4)
    rng = np.random.default_rng(seed)
    axes = []
    for m, length in zip(n, lengths):
        dx = np.full(m + 4, length / m) * rng.uniform(0.75, 1.25, m + 4)
        x = np.empty(m + 4)
        x[0] = -dx[1]
        for i in range(1, m + 4):
            x[i] = x[i - 1] + dx[i]
        axes += [x, dx]
    U = np.zeros((8,) + sh)
    U[0] = problems.MU * rho[0] * np.exp(rng.normal(0.0, rho[1], sh))
    U[1:4] = rng.normal(0.0, vel, (3,) + sh)
    U[5:8] = rng.normal(0.0, bmag, (3,) + sh)
    sp = np.zeros((8,) + sh)
    frac = rng.uniform(0.0, 0.4, sh)
    nH = U[0] / problems.MU
    sp[0] = 0.91 * nH * (1.0 - frac)
    sp[1] = 0.91 * nH * 0.01 * rng.uniform(0.5, 1.5, sh)
    sp[2] = 0.5 * 0.91 * nH * frac
    sp[3] = 0.09 * nH
    sp[4] = 0.09 * nH * 0.006 * rng.uniform(0.5, 1.5, sh)
    sp[5] = 1e-8 * nH
    sp[6] = 1.4e-4 * nH
    sp[7] = 1e-20 * nH
    T = np.exp(rng.uniform(np.log(trange[0]), np.log(trange[1]), sh))
    U[4] = T * problems.KB * (sp[1] + sp[0] + sp[2] + sp[3] + sp[4])
    return problems.MhdState(p, U, sp, *axes)


CASES = [((10, 9, 8), (1, 1, 3, 3, 3, 3)), ((9, 8, 10), (3, 3, 3, 3, 3, 3)), ((8, 10, 9), (3, 3, 1, 1, 1, 1))]


@pytest.mark.parametrize("n,bc", CASES)
@pytest.mark.parametrize("dt", [0.05, 0.004])
def test_source_matches_an_independent_restatement(n, bc, dt):
    st = make_state(n, bc, 7)
    o = Oracle3D(st.params)
    o.upload(st)
    U0, sp0, _ = o.download()
    o.source(dt)
    U1, sp1, _ = o.download()
    U2, sp2, stats = source_thermal(U0, sp0, st, dt)
    assert np.all(np.isfinite(U1[4]))
    for f in range(8):
        assert np.array_equal(U1[f], U2[f]), f
    for s in range(8):
        assert np.array_equal(sp1[s], sp2[s]), s
    # both cooling branches in both passes; both conduction branches
    for ps in (0, 1):
        assert min(stats[ps][:3]) > 0, stats
    assert stats[0][3] + stats[1][3] > 0, stats


TIMESTEP_STATES = [
    # cooling time at its 2.5e-4 floor: dense, cold, thin cells
    (dict(), "cooling"),
    # Courant: fast flows in warm, uniform gas
    (dict(lengths=(2.0, 2.0, 2.0), rho=(1.0, 0.1), trange=(5.0, 8.0), vel=30.0), "cfl"),
    # conduction: hot (partly above the T = 15 cap), thin, tenuous gas with
    # a weak field
    (dict(lengths=(0.05, 0.05, 0.05), rho=(0.01, 0.1), trange=(10.0, 40.0), vel=1.0, bmag=0.05), "conduction"),
]


@pytest.mark.parametrize("n,bc", CASES)
@pytest.mark.parametrize("kw,limit", TIMESTEP_STATES)
def test_timestep_matches_an_independent_restatement(n, bc, kw, limit):
    st = make_state(n, bc, 3, **kw)
    o = Oracle3D(st.params)
    o.upload(st)
    U0, sp0, bcc = o.download()
    dt, lim = o.timestep()
    want, wlim, which = timestep(U0, sp0, bcc, st)
    assert dt == want and lim == wlim, (dt, want, lim, wlim)
    assert which == limit
