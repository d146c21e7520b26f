"""A second, independent restatement of the species cooling function and
the reaction rates of the reference's chemistry (3DMHD-CfCA/
MCF3DSGincfca3.f90: Fcool :2825-2880, fesc :2882-2887, LEVC2 :2889-2895,
RATES :3037-3131, constants :28) in NumPy, term by term from the Fortran,
against the oracle's C++ (which the GPU's FP64 path matches bit for bit).
The oracle evaluates exp, log and real powers with its own deterministic
routines and NumPy with the C library's, so the two agree to a few ulps per
operation: rates to 1e-12 relative, Fcool to 1e-12 of the sum of the
magnitudes of its ten terms (it is a difference of cooling and heating).
The cells carry SHIELD's columns (ifrad = 2, INITIA's 20 iterations),
random molecular, atomic and ionised fractions and temperatures from 10 K
to 10^5 K, so every branch of fesc, ATN5 and kHrec is taken.  The network
(SOURCE's CHEM branch, :2580-2770, Omexp :3134-3140) is restated the same
way, stage by stage, and compared cell by cell after one step; changing a
stage's rate, a transfer term or an electron density that a stage reads
makes it fail."""
import numpy as np

from oracle.pyoracle import Oracle3D
from test_chem_oracle import chem_state

G0, XO, DV, TGR = 1.0, 3.2e-4, 2.0, 5.0e-3   # :28
F32_06 = float(np.float32(0.6))              # the REAL*4 literal of ATN5 (:3068)


def fsign(a, b):
    """Fortran DSIGN(a, b): |a| with the sign of b (+ for b = +0)."""
    return np.where(b >= 0.0, abs(a), -abs(a))


def fesc(tau):   # :2882-2887
    return ((0.5 + fsign(0.5, 0.1 - 1.0e-16 - tau)) * (0.5 - 0.585 * tau + 0.4563 * tau ** 2)
            + (0.5 + fsign(0.5, 11.9025 - (tau - 3.55) ** 2)) * (1.0 - np.exp(-2.34 * tau)) / (4.68 * tau + 1.0e-8)
            + (0.5 + fsign(0.5, tau - 7.0)) / (4.0 * tau * np.sqrt(np.log(max(tau * 0.56419, 4.0))) + 1.0e-8))


def levc2(T, b21, nH, nH2, ne, nCp):   # :2889-2895
    c21 = 8.854e-8 * ne / np.sqrt(T) + 9.399e-10 * T ** 0.07 * (nH + nH2)
    c12 = 2.0 * c21 * np.exp(-0.092 / T)
    a21 = 2.4e-6 * b21
    return nCp * (c21 + a21) / (c12 + c21 + a21), nCp * c12 / (c12 + c21 + a21)


def fcool_terms(T, sp, ne, nt, col):
    """The ten terms of Fcool (cooling positive, heating negative)."""
    nH, np_, nH2, nHe, nHep, nC, nCp, nCO = sp
    Ntot1, Ntot2, NH21, NH22, NnC1, NnC2, NCO1, NCO2, tC1, tC2 = col
    Av1, x1 = 1.63542e-3 * Ntot1, 6.1714e3 * NH21
    Av2, x2 = 1.63542e-3 * Ntot2, 6.1714e3 * NH22
    atn1 = (np.exp(-2.5 * Av1) + np.exp(-2.5 * Av2)) * 0.5
    atn2 = (np.exp(-3.77358 * Av1) + np.exp(-3.77358 * Av2)) * 0.5
    pha = G0 * np.sqrt(1.0e3 * T) * atn1 / ne
    laml = nH * ne * 1.44049e9 * np.exp(-1.184e2 / T) + np_ * ne * 1.48e6 * np.exp(-8.0e1 / T)
    b21 = fesc(tC1) + fesc(tC2)
    _, n2 = levc2(T, b21, nH, nH2, ne, nCp)
    lamc = 6.0157e7 * n2 * b21
    to1, to2 = 3.40057e-6 * Ntot1 / XO, 3.40057e-6 * Ntot2 / XO
    lamo = (max(nt * XO - nCO, 0.0) / XO) * (nH + 0.5 * nH2) * 1.23916e1 * T ** 0.4 * np.exp(-0.228 / T)
    lamo *= fesc(to1) + fesc(to2)
    lamd = ne * nt * 6.06236 * T ** 0.94 * pha ** (0.462628 / T ** 6.8e-2)
    ncr = 3.3e6 * T ** 0.75 / (nH + np_ + nH2 + nHe + nHep)
    tau1, tau2 = 1.33194e1 * NCO1 / (T * DV), 1.33194e1 * NCO2 / (T * DV)
    ct1 = tau1 * np.sqrt(6.283 * np.log(2.13 + (tau1 * 0.36788) ** 2))
    ct2 = tau2 * np.sqrt(6.283 * np.log(2.13 + (tau2 * 0.36788) ** 2))
    ym1, ym2 = np.log(1.0 + ct1 / (1.0 + 1.0e1 * ncr)), np.log(1.0 + ct2 / (1.0 + 1.0e1 * ncr))
    fes = ((2.0 + ym1 + 0.6 * ym1 ** 2) / (1.0 + ct1 + ncr + 1.5 * np.sqrt(ncr))
           + (2.0 + ym2 + 0.6 * ym2 ** 2) / (1.0 + ct2 + ncr + 1.5 * np.sqrt(ncr)))
    lcor = nCO * 1.91505e10 * T ** 2 * fes
    lcoh = nH * nCO * 7.96086e4 * np.sqrt(T) * np.exp(-(2.0 / T) ** 3.43) * np.exp(-3.08 / T)
    lcoh2 = nH2 * nCO * 3.60834e4 * T * np.exp(-(3.14e2 / T) ** 0.333) * np.exp(-3.08 / T)
    gampe = nt * 2.56526e3 * G0 * atn1 * (7.382e-3 * T ** 0.7 / (1.0 + 2.0e-4 * pha)
                                          + 4.9e-2 / (1.0 + 4.0e-3 * pha ** 0.73))
    gamcr = (nH + nHe + nH2) * 1.89435
    shld1 = 0.965 / (1.0 + x1 / DV) ** 2 + 0.035 / np.sqrt(1.0 + x1) * np.exp(-8.5e-4 * np.sqrt(1.0 + x1))
    shld2 = 0.965 / (1.0 + x2 / DV) ** 2 + 0.035 / np.sqrt(1.0 + x2) * np.exp(-8.5e-4 * np.sqrt(1.0 + x2))
    gampd = nH2 * 4.16362e4 * G0 * atn2 * (shld1 + shld2) * 0.5
    return [laml, lamc, lamo, lamd, lcor, lcoh, lcoh2, -gampe, -gamcr, -gampd]


def rates(T, sp, ne, col):
    """zeta, kHrec, kHerec, kH2, kH2ph, kH2dH, kH2de, kCO, kCOph, kCi, kCrec,
    kCOde, kCOdH, kHie, kHeie, kCie, kHiH, kHeiH, kCiH, kCOdHep, kH2dHep."""
    nH2 = sp[2]
    Ntot1, Ntot2, NH21, NH22, NnC1, NnC2, NCO1, NCO2, _, _ = col
    Av1, x1 = 1.63542e-3 * Ntot1, 6.1714e3 * NH21
    Av2, x2 = 1.63542e-3 * Ntot2, 6.1714e3 * NH22
    atn2 = (np.exp(-3.77358 * Av1) + np.exp(-3.77358 * Av2)) * 0.5
    atn3 = (np.exp(-2.3585 * Av1) + np.exp(-2.3585 * Av2)) * 0.5
    atn4 = 0.5 * (min(1.0, (3.0857e1 * NH21) ** -3.0e-2 * np.exp(-1.54285e-3 * NH21))
                  + min(1.0, (3.0857e1 * NH22) ** -3.0e-2 * np.exp(-1.54285e-3 * NH22)))

    def atn5_one(nco):
        return ((0.5 - fsign(0.5, nco - 1.40995e-3)) * np.exp(-1.0 * (1.02857e3 * nco) ** F32_06)
                + (0.5 + fsign(0.5, nco - 1.40995e-3))
                * min((3.75439e3 * nco + 1.0e-100) ** -0.75, (7.3469e1 * nco + 1.0e-100) ** -1.3))

    atn5 = 0.5 * (atn5_one(NCO1) + atn5_one(NCO2))
    zeta = 9.4671e-4
    khrec = ((0.5 + fsign(0.5, 15.78 - T)) * 0.45 * np.log(1.578e2 / T)
             + (0.5 - fsign(0.5, 15.78 - T)) * 0.4 * np.sqrt(1.578e2 / T))
    khrec = 2.05572e1 * T ** -0.5 * khrec
    kherec = 6.37623e1 * T ** -0.672
    kh2 = 3.4569e-3 * np.sqrt(T) / (1.0 + 1.26491 * np.sqrt(T + TGR) + 2.0 * T + 8.0 * T ** 2)
    shld1 = 0.965 / (1.0 + x1 / DV) ** 2 + 0.035 / np.sqrt(1.0 + x1) * np.exp(-8.5e-4 * np.sqrt(1.0 + x1))
    shld2 = 0.965 / (1.0 + x2 / DV) ** 2 + 0.035 / np.sqrt(1.0 + x2) * np.exp(-8.5e-4 * np.sqrt(1.0 + x2))
    kh2ph = 1.04138e3 * G0 * atn2 * (shld1 + shld2) * 0.5
    kh2dh = 1.07294e5 * np.exp(-4.39e1 / T)
    kh2de = 1.133e6 * T ** 0.35 * np.exp(-1.02e2 / T)
    kco = 1.57785e-2 / (1.0 + G0 * atn3 / (nH2 * XO))
    kcoph = 3.155e3 * G0 * atn3 * atn4 * atn5
    shlc1 = np.exp(-2.6 * Av1 - 3.0857e1 * NnC1 - 4.33743413e-4 * NH21) / (1.0 + 4.33743413e-4 * NH21)
    shlc2 = np.exp(-2.6 * Av2 - 3.0857e1 * NnC2 - 4.33743413e-4 * NH22) / (1.0 + 4.33743413e-4 * NH22)
    kci = 3.97 * zeta + 6.62697e3 * G0 * (shlc1 + shlc2) * 0.5
    kcrec = 2.69267e1 * T ** -0.62 * (1.0 + 1.0e-4 * np.sqrt(ne) / T ** 2)
    kcode = 1.4e4 * T ** -0.5 * np.exp(-1.14e2 / T)
    kcodh = 1.91858e3 * T ** -0.5 * np.exp(-7.77e1 / T)
    khie = 5.76e4 * np.sqrt(T) * np.exp(-1.58e2 / T)
    kheie = 2.76e4 * T ** 0.43 * np.exp(-2.85e2 / T)
    kcie = 1.74e5 * T ** 0.4 * np.exp(-1.31e2 / T)
    khih = 9.79 * np.sqrt(T) * np.exp(-1.58e2 / T)
    kheih = 4.57 * T ** 0.43 * np.exp(-2.85e2 / T)
    kcih = 3.01e1 * T ** 0.4 * np.exp(-1.31e2 / T)
    kh2dhep = 1.1676 * np.exp(-0.035 / T)
    kcodhep = 5.0491e4
    return [zeta, khrec, kherec, kh2, kh2ph, kh2dh, kh2de, kco, kcoph, kci, kcrec, kcode, kcodh, khie, kheie,
            kcie, khih, kheih, kcih, kcodhep, kh2dhep]


def test_fcool_and_rates_match_an_independent_restatement():
    st = mixed_state(5)
    o = Oracle3D(st.params)
    o.upload(st)
    s = 10 + 4   # padded extent
    rng = np.random.default_rng(11)
    checked = 0
    # temperatures in units of 1e3 K: 10 K .. 1e5 K, both sides of 15.78
    for T in np.concatenate([10.0 ** rng.uniform(-2.0, 2.0, 40), [0.01, 15.78, 15.79, 100.0]]):
        i, j, k = (int(v) for v in rng.integers(2, 12, size=3))   # interior cells
        out = o.chem_probe(T, i + s * (j + s * k))
        sp, ne, nt, col = out[22:30], out[30], out[31], out[32:42]
        terms = fcool_terms(T, sp, ne, nt, col)
        scale = sum(abs(x) for x in terms)
        assert abs(out[0] - sum(terms)) <= 1e-12 * scale, (T, out[0], sum(terms))
        np.testing.assert_allclose(out[1:22], rates(T, sp, ne, col), rtol=1e-12, atol=0.0)
        checked += 1
    assert checked == 44
    # the columns are not trivial: shielding is exercised
    assert np.any(out[32:42] > 0.0)


KB = 8.63359                                     # :11
M_H, M_HE, M_H2 = 1.0, 4.0, 2.0                  # :27


def omexp(eps):   # :3134-3140
    return ((0.5 + fsign(0.5, eps - 1.0e-4)) * (1.0 - np.exp(-eps))
            + (0.5 - fsign(0.5, eps - 1.0e-4))
            * (eps - 0.5 * eps ** 2 + 0.16666666666666667 * eps ** 3 - 4.16666666666666667e-2 * eps ** 4))


def chem_network(sp, ne, nt, pres, col, dt, rmin):
    """SOURCE's CHEM branch for one cell (:2580-2770), stage by stage."""
    H, p, H2, He, Hep, C, Cp, CO = (float(v) for v in sp)
    T = pres / KB / (p + H + H2 + He + Hep)
    (zeta, kHrec, kHerec, kH2, kH2ph, kH2dH, kH2de, kCO, kCOph, kCi, kCrec, kCOde, kCOdH, kHie, kHeie, kCie,
     kHiH, kHeiH, kCiH, kCOdHep, kH2dHep) = rates(T, sp, ne, col)
    # H recombination and ionization by cosmic rays
    a = kHrec * ne
    e, r, om = np.exp(-dt * (zeta + a)), 1.0 / (zeta + a), omexp(dt * (zeta + a))
    H, p = (a * H + zeta * H * e + a * p * om) * r, (zeta * p + a * p * e + zeta * H * om) * r
    ne = p + Hep + Cp
    # He recombination and ionization by cosmic rays
    a = kHerec * ne
    e, r, om = np.exp(-dt * (zeta + a)), 1.0 / (zeta + a), omexp(dt * (zeta + a))
    He, Hep = (a * He + zeta * He * e + a * Hep * om) * r, (zeta * Hep + a * Hep * e + zeta * He * om) * r
    ne = p + Hep + Cp
    # H2 formation, UV and electron dissociation
    a = kH2ph + kH2de * ne
    b = a + 2.0 * kH2 * nt
    e, om = np.exp(-dt * b), omexp(dt * b)
    H, H2 = (((H + 2.0 * H2 * om) * a + 2.0 * kH2 * H * nt * e) / b,
             ((2.0 * H2 + H * om) * kH2 * nt + a * H2 * e) / b)
    # H2 dissociation by H collisions
    a = H + 2.0 * H2
    e = np.exp(-dt * a * kH2dH)
    r = 1.0 / (H + 2.0 * H2 * e)
    H, H2 = H * a * r, H2 * a * e * r
    # CO formation
    e, om = np.exp(-dt * kCO * nt), omexp(dt * kCO * nt)
    CO, Cp = CO + om * Cp, e * Cp
    ne = p + Hep + Cp
    # CO dissociation by UV, electrons and H
    q = dt * (kCOph + kCOde * ne + kCOdH * H)
    e, om = np.exp(-q), omexp(q)
    C, CO = C + om * CO, e * CO
    # C recombination and ionization by cosmic rays and UV
    a = kCrec * ne
    e, r, om = np.exp(-dt * (kCi + a)), 1.0 / (kCi + a), omexp(dt * (kCi + a))
    C, Cp = (a * C + kCi * C * e + a * Cp * om) * r, (kCi * Cp + a * Cp * e + kCi * C * om) * r
    ne = p + Hep + Cp
    # H, He, C ionization by electrons
    H_, He_, C_ = H * np.exp(-dt * kHie * ne), He * np.exp(-dt * kHeie * ne), C * np.exp(-dt * kCie * ne)
    p, Hep, Cp = omexp(dt * kHie * ne) * H + p, omexp(dt * kHeie * ne) * He + Hep, omexp(dt * kCie * ne) * C + Cp
    H, He, C = H_, He_, C_
    ne = p + Hep + Cp
    # H, He, C ionization by H, H2 and p collisions
    r = 1.0 / (1.0 + kHiH * dt * H)
    H, p = H * r, p + r * kHiH * dt * H ** 2
    q = H + p + H2
    He_, C_ = He * np.exp(-dt * kHeiH * q), C * np.exp(-dt * kCiH * q)
    Hep, Cp = omexp(dt * kHeiH * q) * He + Hep, omexp(dt * kCiH * q) * C + Cp
    He, C = He_, C_
    ne = p + Hep + Cp
    # H2 dissociation by He+ recombination
    a = Hep - H2
    if a >= 0.0:
        e = np.exp(-dt * kH2dHep * a)
        r = 1.0 / (Hep - H2 * e)
        Hep_, H2 = Hep * a * r, H2 * a * r * e
        d = Hep * (1.0 - a * r)
    else:
        e = np.exp(dt * kH2dHep * a)
        r = 1.0 / (Hep * e - H2)
        Hep_, H2 = Hep * a * r * e, H2 * a * r
        d = Hep * (1.0 - a * r * e)
    Hep, p, H, He = Hep_, p + d, H + d, He + d
    # CO dissociation by He+ recombination
    a = Hep - CO
    if a >= 0.0:
        e = np.exp(-dt * kCOdHep * a)
        r = 1.0 / (Hep - CO * e)
        Hep_, CO = Hep * a * r, CO * a * r * e
        d = Hep * (1.0 - a * r)
    else:
        e = np.exp(dt * kCOdHep * a)
        r = 1.0 / (Hep * e - CO)
        Hep_, CO = Hep * a * r * e, CO * a * r
        d = Hep * (1.0 - a * r * e)
    Hep, Cp, He = Hep_, Cp + d, He + d
    # floors (:178-179), then nde, ndtot and rho
    floors = (0.91 * rmin, 1e-20, 1e-20, 0.09 * rmin, 1e-20, 1e-20, 1e-20, 1e-20)
    out = [max(f, v) for f, v in zip(floors, (H, p, H2, He, Hep, C, Cp, CO))]
    H, p, H2, He, Hep, C, Cp, CO = out
    ne = p + Hep + Cp
    nt = p + H + 2.0 * H2 + He + Hep
    rho = M_H * p + M_H * H + M_H2 * H2 + M_HE * He + M_HE * Hep
    return np.array(out), ne, nt, rho


def mixed_state(seed):
    """The chemistry workload with every composition the network acts on:
    in each cell random fractions of the H nuclei in H2 and of the C nuclei
    in CO and C (the rest ionised or atomic), and temperatures from cold
    molecular to warm ionised gas."""
    st = chem_state(n=10, seed=seed)
    st.params = st.params.replace(ifrad=2)
    rng = np.random.default_rng(seed + 100)
    sp = st.species
    shape = sp[0].shape
    hn, hen, cn = sp[0] + sp[1] + 2 * sp[2], sp[3] + sp[4], sp[5] + sp[6] + sp[7]
    fh2, fp = rng.uniform(0.0, 0.45, shape), 10.0 ** rng.uniform(-4.0, -0.5, shape)
    sp[2] = fh2 * hn
    sp[1] = fp * (hn - 2 * sp[2])
    sp[0] = hn - 2 * sp[2] - sp[1]
    fhep = 10.0 ** rng.uniform(-4.0, -0.5, shape)
    sp[4], sp[3] = fhep * hen, (1 - fhep) * hen
    fco, fc = rng.uniform(0.0, 0.9, shape), rng.uniform(0.0, 0.5, shape)
    sp[7] = fco * cn
    sp[5] = fc * (cn - sp[7])
    sp[6] = cn - sp[7] - sp[5]
    st.U[4] *= 10.0 ** rng.uniform(-1.5, 0.5, shape)
    return st


def test_chemistry_network_matches_an_independent_restatement():
    st = mixed_state(7)
    o = Oracle3D(st.params)
    o.upload(st)
    s = 10 + 4
    rng = np.random.default_rng(13)
    for q in range(60):
        i, j, k = (int(v) for v in rng.integers(2, 12, size=3))
        dt = 10.0 ** rng.uniform(-4.0, 0.0)
        out = o.chem_cell_probe(i + s * (j + s * k), dt)
        sp, ne, nt, pres, col = out[0:8], out[8], out[9], out[10], out[11:21]
        sp1, ne1, nt1, rho1 = chem_network(sp, ne, nt, pres, col, dt, st.params.rmin)
        # each species against its element's total: a stage moves nuclei
        # between species, so absolute agreement is relative to the element
        tot = np.array([sp[0] + sp[1] + 2 * sp[2]] * 3 + [sp[3] + sp[4]] * 2 + [sp[5] + sp[6] + sp[7]] * 3)
        np.testing.assert_allclose(out[21:29], sp1, rtol=1e-11, atol=1e-12 * tot.max())
        np.testing.assert_allclose(out[21:29] / tot, sp1 / tot, rtol=0.0, atol=1e-11)
        np.testing.assert_allclose([out[29], out[30], out[31]], [ne1, nt1, rho1], rtol=1e-11)


def shield_pass(U, sp, col_old, dx1, n):
    """SHIELD (:2924-3036) on one block holding every line whole: the C+
    optical-depth source of each interior cell from the previous tCII
    columns, then along each x line the columns from the left and from the
    right, each cell adding half its width times its value before and after
    its own column is stored.  nde and ndtot are rebuilt from the species
    first, as SOURCE does before calling SHIELD (:2460-2463)."""
    nx, ny, nz = n
    H, p, H2, He, Hep, C, Cp, CO = sp
    nde = p + Hep + Cp
    ndtot = p + H + 2.0 * H2 + He + Hep
    dxh = 0.5 * dx1
    out = np.zeros_like(col_old)
    for k in range(2, nz + 2):
        for j in range(2, ny + 2):
            src = np.zeros(nx + 4)
            for i in range(2, nx + 2):
                b21 = fesc(col_old[8][k, j, i]) + fesc(col_old[9][k, j, i])
                T = U[4][k, j, i] / (KB * (p[k, j, i] + H[k, j, i] + H2[k, j, i] + He[k, j, i] + Hep[k, j, i]))
                n1, n2 = levc2(T, b21, H[k, j, i], H2[k, j, i], nde[k, j, i], Cp[k, j, i])
                src[i] = 1.15563e1 * (n1 - n2) * (1.0 / DV)
            vals = (ndtot[k, j], H2[k, j], C[k, j], CO[k, j], src)
            for side, rng_i in ((0, range(2, nx + 2)), (1, range(nx + 1, 1, -1))):
                acc = [0.0] * 5
                for i in rng_i:
                    for q in range(5):
                        acc[q] += dxh * vals[q][i]
                        out[2 * q + side][k, j, i] = acc[q]
                        acc[q] += dxh * vals[q][i]
    return out


def test_shield_pass_matches_an_independent_restatement():
    """One SHIELD pass (the one at the start of SOURCE) against its
    restatement, from the columns INITIA's twenty passes left; the column
    order of the handle is Ntot, NH2, NnC, NCO, tCII, each from the left
    and from the right."""
    st = mixed_state(9)
    o = Oracle3D(st.params)
    o.upload(st)
    col0 = o.columns()
    U0, sp0, _ = o.download()
    o.source(1.0e-6)
    col1 = o.columns()
    n = (st.params.nx, st.params.ny, st.params.nz)
    ref = shield_pass(U0, sp0, col0, st.dx[2], n)
    inner = (slice(None), slice(2, -2), slice(2, -2), slice(2, -2))
    got, want = col1[inner], ref[inner]
    assert np.all(want[:8] > 0.0) and np.any(want[8:] != 0.0)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-300)
