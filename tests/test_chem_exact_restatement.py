"""The chemistry of the shipped deck (ifchem = 2) restated in NumPy from the
Fortran, vectorised over cells, and checked against the oracle bit for bit:
Fcool with fesc and LEVC2 (3DMHD-CfCA/MCF3DSGincfca3.f90:2825-2895),
RATES (:3040-3131), Omexp (:3134-3140), the network of SOURCE's CHEM
branch (:2576-2776), SHIELD's column densities (:2924-3036; INITIA's twenty
passes and SOURCE's one), the thermal SOURCE and the time step with the
species cooling, and whole steps of the shipped deck's configuration —
inflow on both x sides, the chemistry, KI-free species cooling — composed
from the restated parts.

exp, log and real powers are the oracle's own deterministic routines
(called through the oracle library, as in the KI restatement); integer
powers are products (x**2 = x*x, x**3 = x*x*x, x**4 = (x*x)*(x*x)), and the
REAL*4 literal 0.6 of ATN5 is single precision widened.  Every other
operation is IEEE double in the Fortran's order."""
import numpy as np
import pytest

from code_tohoku_gb300 import problems
from oracle.pyoracle import Oracle3D, detmath
from test_chem_restatement import mixed_state
from test_dissip_restatement import dissip
from test_inflow_restatement import InflowX, dissip_fill, make_inflow
from test_source_restatement import source_thermal, timestep
from test_step_restatement import ORDERS, ct
from test_sweep_restatement import fmax2, fmin2, make_state, sgn, sweep

G0, XO, DV, TGR = 1.0, 3.2e-4, 2.0, 5.0e-3        # :28
M_H, M_HE, M_H2 = 1.0, 4.0, 2.0                    # :27
F32_06 = float(np.float32(0.6))


def E(x):
    return detmath("exp", x)


def LG(x):
    return detmath("log", x)


def PW(x, e):
    return detmath("pow", x, e)


def fesc(tau):
    return ((0.5 + sgn(0.5, 0.1 - 1.e-16 - tau)) * (0.5 - 0.585 * tau + 0.4563 * (tau * tau))
            + (0.5 + sgn(0.5, 11.9025 - (tau - 3.55) * (tau - 3.55))) * (1.0 - E(-2.34 * tau)) / (4.68 * tau + 1.e-8)
            + (0.5 + sgn(0.5, tau - 7.0)) / (4.0 * tau * np.sqrt(LG(fmax2(tau * 0.56419, 4.0))) + 1.e-8))


def levc2(T, b21, H, H2, ne, Cp):
    c21 = 8.854e-8 * ne / np.sqrt(T) + 9.399e-10 * PW(T, 0.07) * (H + H2)
    c12 = 2.0 * c21 * E(-0.092 / T)
    a21 = 2.4e-6 * b21
    return Cp * (c21 + a21) / (c12 + c21 + a21), Cp * c12 / (c12 + c21 + a21)


def shld(x):
    s = 1.0 + x / DV
    return 0.965 / (s * s) + 0.035 / np.sqrt(1.0 + x) * E(-8.5e-4 * np.sqrt(1.0 + x))


def fcool(T, sp, ne, nt, col):
    H, p, H2, He, Hep, C, Cp, CO = sp
    Ntot1, Ntot2, NH21, NH22, NnC1, NnC2, NCO1, NCO2, tC1, tC2 = col
    Av1, x1 = 1.63542e-3 * Ntot1, 6.1714e3 * NH21
    Av2, x2 = 1.63542e-3 * Ntot2, 6.1714e3 * NH22
    atn1 = (E(-2.5 * Av1) + E(-2.5 * Av2)) * 0.5
    atn2 = (E(-3.77358 * Av1) + E(-3.77358 * Av2)) * 0.5
    pha = G0 * np.sqrt(1.e3 * T) * atn1 / ne
    laml = H * ne * 1.44049e9 * E(-1.184e2 / T)
    laml = laml + p * ne * 1.48e6 * E(-8.e1 / T)
    b21 = fesc(tC1) + fesc(tC2)
    _, n2 = levc2(T, b21, H, H2, ne, Cp)
    lamc = 6.0157e7 * n2 * b21
    to1, to2 = 3.40057e-6 * Ntot1 / XO, 3.40057e-6 * Ntot2 / XO
    lamo = (fmax2(nt * XO - CO, 0.0) / XO) * (H + 0.5 * H2) * 1.23916e1 * PW(T, 0.4) * E(-0.228 / T)
    lamo = lamo * (fesc(to1) + fesc(to2))
    lamd = ne * nt * 6.06236 * PW(T, 0.94) * PW(pha, 0.462628 / PW(T, 6.8e-2))
    ncr = 3.3e6 * PW(T, 0.75) / (H + p + H2 + He + Hep)
    tau1, tau2 = 1.33194e1 * NCO1 / (T * DV), 1.33194e1 * NCO2 / (T * DV)
    q1, q2 = tau1 * 0.36788, tau2 * 0.36788
    ct1, ct2 = tau1 * np.sqrt(6.283 * LG(2.13 + q1 * q1)), tau2 * np.sqrt(6.283 * LG(2.13 + q2 * q2))
    ym1, ym2 = LG(1.0 + ct1 / (1.0 + 1.e1 * ncr)), LG(1.0 + ct2 / (1.0 + 1.e1 * ncr))
    fes = ((2.0 + ym1 + 0.6 * (ym1 * ym1)) / (1.0 + ct1 + ncr + 1.5 * np.sqrt(ncr))
           + (2.0 + ym2 + 0.6 * (ym2 * ym2)) / (1.0 + ct2 + ncr + 1.5 * np.sqrt(ncr)))
    lcor = CO * 1.91505e10 * (T * T) * fes
    lcoh = H * CO * 7.96086e4 * np.sqrt(T) * E(-PW(2.0 / T, 3.43)) * E(-3.08 / T)
    lcoh2 = H2 * CO * 3.60834e4 * T * E(-PW(3.14e2 / T, 0.333)) * E(-3.08 / T)
    gampe = nt * 2.56526e3 * G0 * atn1 * (7.382e-3 * PW(T, 0.7) / (1.0 + 2.e-4 * pha)
                                          + 4.9e-2 / (1.0 + 4.e-3 * PW(pha, 0.73)))
    gamcr = (H + He + H2) * 1.89435
    gampd = H2 * 4.16362e4 * G0 * atn2 * (shld(x1) + shld(x2)) * 0.5
    return laml + lamc + lamo + lamd + lcor + lcoh + lcoh2 - gampe - gamcr - gampd


def rates(T, H2, ne, col):
    Ntot1, Ntot2, NH21, NH22, NnC1, NnC2, NCO1, NCO2, _, _ = col
    Av1, x1 = 1.63542e-3 * Ntot1, 6.1714e3 * NH21
    Av2, x2 = 1.63542e-3 * Ntot2, 6.1714e3 * NH22
    atn2 = (E(-3.77358 * Av1) + E(-3.77358 * Av2)) * 0.5
    atn3 = (E(-2.3585 * Av1) + E(-2.3585 * Av2)) * 0.5
    atn4 = (fmin2(1.0, PW(3.0857e1 * NH21, -3.e-2) * E(-1.54285e-3 * NH21))
            + fmin2(1.0, PW(3.0857e1 * NH22, -3.e-2) * E(-1.54285e-3 * NH22)))
    atn4 = atn4 * 0.5

    def atn5_terms(nco):
        s = sgn(0.5, nco - 1.40995e-3)
        return ((0.5 - s) * E(-1.0 * PW(1.02857e3 * nco, F32_06)),
                (0.5 + s) * fmin2(PW(3.75439e3 * nco + 1.e-100, -0.75), PW(7.3469e1 * nco + 1.e-100, -1.3)))

    a, b = atn5_terms(NCO1)
    atn5 = a + b
    a, b = atn5_terms(NCO2)
    atn5 = atn5 + a + b
    atn5 = atn5 * 0.5
    zeta = 9.4671e-4
    s = sgn(0.5, 15.78 - T)
    khrec = (0.5 + s) * 0.45 * LG(1.578e2 / T) + (0.5 - s) * 0.4 * np.sqrt(1.578e2 / T)
    khrec = 2.05572e1 * PW(T, -0.5) * khrec
    kherec = 6.37623e1 * PW(T, -0.672)
    kh2 = 3.4569e-3 * np.sqrt(T) / (1.0 + 1.26491 * np.sqrt(T + TGR) + 2.0 * T + 8.0 * (T * T))
    kh2ph = 1.04138e3 * G0 * atn2 * (shld(x1) + shld(x2)) * 0.5
    kh2dh = 1.07294e5 * E(-4.39e1 / T)
    kh2de = 1.133e6 * PW(T, 0.35) * E(-1.02e2 / T)
    kco = 1.57785e-2 / (1.0 + G0 * atn3 / (H2 * XO))
    kcoph = 3.155e3 * G0 * atn3 * atn4 * atn5
    shlc1 = E(-2.6 * Av1 - 3.0857e1 * NnC1 - 4.33743413e-4 * NH21) / (1.0 + 4.33743413e-4 * NH21)
    shlc2 = E(-2.6 * Av2 - 3.0857e1 * NnC2 - 4.33743413e-4 * NH22) / (1.0 + 4.33743413e-4 * NH22)
    kci = 3.97 * zeta + 6.62697e3 * G0 * (shlc1 + shlc2) * 0.5
    kcrec = 2.69267e1 * PW(T, -0.62) * (1.0 + 1.e-4 * np.sqrt(ne) / (T * T))
    kcode = 1.4e4 * PW(T, -0.5) * E(-1.14e2 / T)
    kcodh = 1.91858e3 * PW(T, -0.5) * E(-7.77e1 / T)
    khie = 5.76e4 * np.sqrt(T) * E(-1.58e2 / T)
    kheie = 2.76e4 * PW(T, 0.43) * E(-2.85e2 / T)
    kcie = 1.74e5 * PW(T, 0.4) * E(-1.31e2 / T)
    khih = 9.79 * np.sqrt(T) * E(-1.58e2 / T)
    kheih = 4.57 * PW(T, 0.43) * E(-2.85e2 / T)
    kcih = 3.01e1 * PW(T, 0.4) * E(-1.31e2 / T)
    kh2dhep = 1.1676 * E(-0.035 / T)
    kcodhep = np.full_like(T, 5.0491e4)
    return [np.full_like(T, zeta), khrec, kherec, kh2, kh2ph, kh2dh, kh2de, kco, kcoph, kci, kcrec, kcode, kcodh,
            khie, kheie, kcie, khih, kheih, kcih, kcodhep, kh2dhep]


def omexp(eps):
    e2 = eps * eps
    return ((0.5 + sgn(0.5, eps - 1.e-4)) * (1.0 - E(-eps))
            + (0.5 - sgn(0.5, eps - 1.e-4))
            * (eps - 0.5 * e2 + 0.16666666666666667 * (e2 * eps) - 4.16666666666666667e-2 * (e2 * e2)))


def network(sp, ne, nt, pres, col, dt, rmin, kb):
    """SOURCE's CHEM branch for cells (arrays), stage by stage; returns the
    species, nde, ndtot and rho."""
    H, p, H2, He, Hep, C, Cp, CO = (np.asarray(a, dtype=np.float64) for a in sp)
    T = pres / kb / (p + H + H2 + He + Hep)
    (zeta, kHrec, kHerec, kH2, kH2ph, kH2dH, kH2de, kCO, kCOph, kCi, kCrec, kCOde, kCOdH, kHie, kHeie, kCie,
     kHiH, kHeiH, kCiH, kCOdHep, kH2dHep) = rates(T, H2, ne, col)
    with np.errstate(all="ignore"):
        # H recombination and ionisation by cosmic rays
        t1 = kHrec * ne
        t2, t3, om = E(-dt * (zeta + t1)), 1.0 / (zeta + t1), omexp(dt * (zeta + t1))
        H, p = (t1 * H + zeta * H * t2 + t1 * p * om) * t3, (zeta * p + t1 * p * t2 + zeta * H * om) * t3
        ne = p + Hep + Cp
        # He recombination and ionisation by cosmic rays
        t1 = kHerec * ne
        t2, t3, om = E(-dt * (zeta + t1)), 1.0 / (zeta + t1), omexp(dt * (zeta + t1))
        He, Hep = (t1 * He + zeta * He * t2 + t1 * Hep * om) * t3, (zeta * Hep + t1 * Hep * t2 + zeta * He * om) * t3
        ne = p + Hep + Cp
        # H2 formation, dissociation by UV and electrons
        t1 = kH2ph + kH2de * ne
        t2 = t1 + 2.0 * kH2 * nt
        t3, om = E(-dt * t2), omexp(dt * t2)
        H, H2 = ((H + 2.0 * H2 * om) * t1 + 2.0 * kH2 * H * nt * t3) / t2, \
            ((2.0 * H2 + H * om) * kH2 * nt + t1 * H2 * t3) / t2
        # H2 dissociation by H collisions
        t1 = H + 2.0 * H2
        t2 = E(-dt * t1 * kH2dH)
        t3 = 1.0 / (H + 2.0 * H2 * t2)
        H, H2 = H * t1 * t3, H2 * t1 * t2 * t3
        # CO formation
        t1, om = E(-dt * kCO * nt), omexp(dt * kCO * nt)
        CO, Cp = CO + om * Cp, t1 * Cp
        ne = p + Hep + Cp
        # CO dissociation by UV, electrons and H
        q = dt * (kCOph + kCOde * ne + kCOdH * H)
        t1 = E(-dt * (kCOph + kCOde * ne + kCOdH * H))
        om = omexp(q)
        C, CO = C + om * CO, t1 * CO
        # C recombination and ionisation by cosmic rays and UV
        t1 = kCrec * ne
        t2, t3, om = E(-dt * (kCi + t1)), 1.0 / (kCi + t1), omexp(dt * (kCi + t1))
        C, Cp = (t1 * C + kCi * C * t2 + t1 * Cp * om) * t3, (kCi * Cp + t1 * Cp * t2 + kCi * C * om) * t3
        ne = p + Hep + Cp
        # H, He, C ionisation by electrons
        H1, He1, C1 = H * E(-dt * kHie * ne), He * E(-dt * kHeie * ne), C * E(-dt * kCie * ne)
        p = omexp(dt * kHie * ne) * H + p
        Hep = omexp(dt * kHeie * ne) * He + Hep
        Cp = omexp(dt * kCie * ne) * C + Cp
        H, He, C = H1, He1, C1
        ne = p + Hep + Cp
        # H, He, C ionisation by H, H2 and p
        t1 = 1.0 / (1.0 + kHiH * dt * H)
        H, p = H * t1, p + t1 * kHiH * dt * (H * H)
        t1 = H + p + H2
        He1, C1 = He * E(-dt * kHeiH * t1), C * E(-dt * kCiH * t1)
        Hep = omexp(dt * kHeiH * t1) * He + Hep
        Cp = omexp(dt * kCiH * t1) * C + Cp
        He, C = He1, C1
        ne = p + Hep + Cp

        # H2, then CO, destroyed by He+ recombination (two branches each)
        def hep_pair(Hep, X, k):
            t1 = Hep - X
            up = t1 >= 0.0
            e_up = E(-dt * k * t1)
            r_up = 1.0 / (Hep - X * e_up)
            e_dn = E(dt * k * t1)
            r_dn = 1.0 / (Hep * e_dn - X)
            Hep_n = np.where(up, Hep * t1 * r_up, Hep * t1 * r_dn * e_dn)
            X_n = np.where(up, X * t1 * r_up * e_up, X * t1 * r_dn)
            d = np.where(up, Hep * (1.0 - t1 * r_up), Hep * (1.0 - t1 * r_dn * e_dn))
            return Hep_n, X_n, d

        Hep, H2, d = hep_pair(Hep, H2, kH2dHep)
        p, H, He = p + d, H + d, He + d
        Hep, CO, d = hep_pair(Hep, CO, kCOdHep)
        Cp, He = Cp + d, He + d
    floors = (rmin * 0.91, 1e-20, 1e-20, rmin * 0.09, 1e-20, 1e-20, 1e-20, 1e-20)
    out = [fmax2(f, v) for f, v in zip(floors, (H, p, H2, He, Hep, C, Cp, CO))]
    H, p, H2, He, Hep, C, Cp, CO = out
    ne = p + Hep + Cp
    nt = p + H + 2.0 * H2 + He + Hep
    rho = M_H * p + M_H * H + M_H2 * H2 + M_HE * He + M_HE * Hep
    return out, ne, nt, rho


def totals(sp):
    """nde and ndtot of the species (:2460-2463)."""
    return sp[1] + sp[4] + sp[6], sp[1] + sp[0] + 2.0 * sp[2] + sp[3] + sp[4]


def shield(U, sp, nde, ndtot, col, dx1, kb):
    """SHIELD (:2924-3036) for one block holding whole x lines: the C+
    optical-depth source of every interior cell from the previous tCII
    columns, then the columns of ndtot, H2, C, CO and that source along each
    x line from the left and from the right, each cell adding half its
    width before and after its own column is stored.  col holds Ntot, NH2,
    NnC, NCO, tCII, each from the left and from the right."""
    nz, ny, nx = (a - 4 for a in U[0].shape)
    K, J, I = slice(2, nz + 2), slice(2, ny + 2), slice(2, nx + 2)
    H, p, H2, He, Hep, C, Cp, CO = (a[K, J, I] for a in sp)
    b21 = fesc(col[8][K, J, I]) + fesc(col[9][K, J, I])
    T = U[4][K, J, I] / (kb * (p + H + H2 + He + Hep))
    n1, n2 = levc2(T, b21, H, H2, nde[K, J, I], Cp)
    src = 1.15563e1 * (n1 - n2) * (1.0 / DV)
    dxh = 0.5 * dx1
    vals = (ndtot[K, J, I], H2, C, CO, src)
    out = col.copy()
    for side, order in ((0, range(nx)), (1, range(nx - 1, -1, -1))):
        acc = [np.zeros((nz, ny)) for _ in range(5)]
        for i in order:
            for q in range(5):
                acc[q] = acc[q] + dxh * vals[q][:, :, i]
                out[2 * q + side][K, J, 2 + i] = acc[q]
                acc[q] = acc[q] + dxh * vals[q][:, :, i]
    return out


def source_chem(U, sp, nde, ndtot, col, st, dt, xfill=None, with_columns=False):
    """SOURCE with ifchem = 2: nde and ndtot rebuilt on the interior, SHIELD
    when ifrad = 2, the thermal branch with the species cooling, the
    network.  with_columns: return the columns too."""
    p = st.params
    K, J, I = slice(2, p.nz + 2), slice(2, p.ny + 2), slice(2, p.nx + 2)
    nde, ndtot = nde.copy(), ndtot.copy()
    e, t = totals([s[K, J, I] for s in sp])
    nde[K, J, I], ndtot[K, J, I] = e, t
    if p.ifrad == 2:
        col = shield(U, sp, nde, ndtot, col, st.dx[2], p.kb)
    cells = [s[K, J, I] for s in sp]
    cc = [c[K, J, I] for c in col]
    ne, nt = nde[K, J, I], ndtot[K, J, I]

    def cool(T, sel):
        if sel is None:
            return fcool(T, cells, ne, nt, cc)
        return fcool(T, [a[sel] for a in cells], ne[sel], nt[sel], [a[sel] for a in cc])

    U, sp, _ = source_thermal(U, sp, st, dt, xfill, cool)
    sp = sp.copy()
    U = U.copy()
    out, ne1, nt1, rho = network([s[K, J, I] for s in sp], ne, nt, U[4][K, J, I], cc, dt, p.rmin, p.kb)
    for q in range(8):
        sp[q][K, J, I] = out[q]
    nde[K, J, I], ndtot[K, J, I], U[0][K, J, I] = ne1, nt1, rho
    if with_columns:
        return U, sp, nde, ndtot, col
    return U, sp, nde, ndtot


def species_cool_at(sp, nde, ndtot, col, p):
    K, J, I = slice(2, p.nz + 2), slice(2, p.ny + 2), slice(2, p.nx + 2)
    cells = [s[K, J, I] for s in sp]
    cc = [c[K, J, I] for c in col]
    return lambda T: fcool(T, cells, nde[K, J, I], ndtot[K, J, I], cc)


# ----------------------------------------------------------------- tests

def test_fcool_and_rates_bit_for_bit():
    st = mixed_state(5)
    o = Oracle3D(st.params)
    o.upload(st)
    s = 10 + 4
    rng = np.random.default_rng(11)
    Ts = np.concatenate([10.0 ** rng.uniform(-2.0, 2.0, 60), [0.01, 15.78, 15.79, 100.0]])
    outs = []
    for T in Ts:
        i, j, k = (int(v) for v in rng.integers(2, 12, size=3))
        outs.append(o.chem_probe(T, i + s * (j + s * k)))
    outs = np.array(outs)
    sp, ne, nt, col = list(outs[:, 22:30].T), outs[:, 30], outs[:, 31], list(outs[:, 32:42].T)
    assert np.array_equal(outs[:, 0], fcool(Ts, sp, ne, nt, col))
    assert np.array_equal(outs[:, 1:22], np.array(rates(Ts, sp[2], ne, col)).T)
    assert np.any(outs[:, 32:42] > 0.0)


def test_network_bit_for_bit():
    st = mixed_state(7)
    o = Oracle3D(st.params)
    o.upload(st)
    s = 10 + 4
    rng = np.random.default_rng(13)
    outs, dts = [], []
    for q in range(120):
        i, j, k = (int(v) for v in rng.integers(2, 12, size=3))
        dt = 10.0 ** rng.uniform(-4.0, 0.0)
        outs.append(o.chem_cell_probe(i + s * (j + s * k), dt))
        dts.append(dt)
    outs, dts = np.array(outs), np.array(dts)
    sp, ne, nt, pres, col = list(outs[:, 0:8].T), outs[:, 8], outs[:, 9], outs[:, 10], list(outs[:, 11:21].T)
    out, ne1, nt1, rho = network(sp, ne, nt, pres, col, dts, st.params.rmin, st.params.kb)
    assert np.array_equal(outs[:, 21:29], np.array(out).T)
    assert np.array_equal(outs[:, 29], ne1) and np.array_equal(outs[:, 30], nt1)
    assert np.array_equal(outs[:, 31], rho)
    # both branches of each He+ stage were taken
    assert np.any(sp[4] >= sp[2]) and np.any(sp[4] < sp[2]) and np.any(sp[4] >= sp[7]) and np.any(sp[4] < sp[7])


def deck_state(n, bc, seed):
    """A random state with the chemistry on: the species of the sweep tests'
    states with molecular and CO fractions, T of 1e2-1e4 K."""
    st = make_state(n, bc, seed)
    st.params = st.params.replace(ifchem=2)
    rng = np.random.default_rng(seed + 1)
    sh = st.U[0].shape
    nH = st.U[0] / problems.MU
    fco = rng.uniform(0.0, 0.8, sh)
    st.species[7] = 1.4e-4 * nH * fco
    st.species[5] = 1.4e-4 * nH * (1.0 - fco) * rng.uniform(0.0, 0.5, sh)
    st.species[6] = 1.4e-4 * nH - st.species[7] - st.species[5]
    T = np.exp(rng.uniform(np.log(0.1), np.log(10.0), sh))
    sp = st.species
    st.U[4] = T * problems.KB * (sp[1] + sp[0] + sp[2] + sp[3] + sp[4])
    return st


@pytest.mark.parametrize("dt", [0.02, 0.002])
def test_source_with_chemistry_bit_for_bit(dt):
    st = deck_state((10, 9, 8), (1, 1, 3, 3, 3, 3), 3)
    o = Oracle3D(st.params)
    o.upload(st)
    U0, sp0, _ = o.download()
    col = np.zeros((10,) + U0[0].shape)
    nde, ndtot = np.zeros_like(U0[0]), np.zeros_like(U0[0])
    o.source(dt)
    U1, sp1, _ = o.download()
    U2, sp2, _, _ = source_chem(U0, sp0, nde, ndtot, col, st, dt)
    assert np.all(np.isfinite(U1))
    for f in range(8):
        assert np.array_equal(U1[f], U2[f]), f
    for q in range(8):
        assert np.array_equal(sp1[q], sp2[q]), q
    assert np.any(U1[0] != U0[0]) and np.any(sp1[7] != sp0[7])


def deck_step(U, sp, bcc, nde, ndtot, col, st, ifevo, xf):
    """One EVOLVE iteration with the chemistry on (SHIELD off) and the x
    exchanges of xf; returns the new state, nde, ndtot, dt and the limiter
    id (the caller advances xf.time by dt)."""
    p = st.params
    coords = (st.x, st.dx, st.y, st.dy, st.z, st.dz)
    dt, lim, _ = timestep(U, sp, bcc, st, species_cool_at(sp, nde, ndtot, col, p))
    U, sp, nde, ndtot = source_chem(U, sp, nde, ndtot, col, st, 0.5 * dt, xf)
    for d in ORDERS[ifevo - 1]:
        U, sp = sweep(d, U, sp, bcc, coords, p, dt, xf)
    U, bcc = ct(U, st, dt, xf)
    U, sp, nde, ndtot = source_chem(U, sp, nde, ndtot, col, st, 0.5 * dt, xf)
    U = U.copy()
    U[1:4] = dissip(U, (p.nx, p.ny, p.nz), dissip_fill(xf, p))
    return U, sp, bcc, nde, ndtot, dt, lim


@pytest.mark.parametrize("first", [1, 4])
def test_shipped_deck_steps_bit_for_bit(first):
    """Inflow on both x sides, the chemistry on, SHIELD off: the shipped
    deck's configuration, three whole steps."""
    st = deck_state((20, 9, 8), (4, 4, 3, 3, 3, 3), 29)
    p = st.params
    inflow, dtf = make_inflow(st, 6)
    o = Oracle3D(p)
    o.upload(st)
    o.set_inflow(inflow.vector(), dtf, 0.0)
    o.set_order(first)
    U, sp, bcc = o.download()
    col = np.zeros((10,) + U[0].shape)
    # nde and ndtot as INITIA leaves them (cells 1..n+1, :471-474)
    nde, ndtot = np.zeros_like(U[0]), np.zeros_like(U[0])
    Kp, Jp, Ip = slice(2, p.nz + 3), slice(2, p.ny + 3), slice(2, p.nx + 3)
    nde[Kp, Jp, Ip], ndtot[Kp, Jp, Ip] = totals([s[Kp, Jp, Ip] for s in sp])
    xf = InflowX(inflow, dtf, st)
    for s in range(3):
        ifevo = (first - 1 + s) % 6 + 1
        U, sp, bcc, nde, ndtot, dt, lim = deck_step(U, sp, bcc, nde, ndtot, col, st, ifevo, xf)
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
        xf.time += dt


def test_shield_and_source_with_columns_bit_for_bit():
    """INITIA's twenty SHIELD passes after the species totals of cells
    1..n+1 (:471-479), then SOURCE with SHIELD on (ifrad = 2): the columns,
    the state and the species."""
    st = deck_state((10, 9, 8), (1, 1, 3, 3, 3, 3), 41)
    st.params = st.params.replace(ifrad=2)
    p = st.params
    o = Oracle3D(p)
    o.upload(st)
    U0, sp0, _ = o.download()
    col0 = o.columns()
    nde, ndtot = np.zeros_like(U0[0]), np.zeros_like(U0[0])
    Kp, Jp, Ip = slice(2, p.nz + 3), slice(2, p.ny + 3), slice(2, p.nx + 3)
    nde[Kp, Jp, Ip], ndtot[Kp, Jp, Ip] = totals([s[Kp, Jp, Ip] for s in sp0])
    col = np.zeros((10,) + U0[0].shape)
    for _ in range(20):
        col = shield(U0, sp0, nde, ndtot, col, st.dx[2], p.kb)
    assert np.array_equal(col, col0)
    assert np.all(col[:8][:, 2:-2, 2:-2, 2:-2] > 0.0) and np.any(col[8:] != 0.0)
    dt = 0.01
    o.source(dt)
    U1, sp1, _ = o.download()
    col1 = o.columns()
    U2, sp2, _, _, col2 = source_chem(U0, sp0, nde, ndtot, col0, st, dt, with_columns=True)
    assert np.array_equal(col1, col2)
    for f in range(8):
        assert np.array_equal(U1[f], U2[f]), f
    for q in range(8):
        assert np.array_equal(sp1[q], sp2[q]), q
