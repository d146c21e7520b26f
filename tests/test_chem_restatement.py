"""A second, independent restatement of the species cooling function and
the reaction rates of the reference's chemistry (3DMHD-CfCA/
MCF3DSGincfca3.f90: Fcool :2825-2880, fesc :2882-2887, LEVC2 :2889-2895,
RATES :3037-3131, constants :28) in NumPy, term by term from the Fortran,
against the oracle's C++ (which the GPU's FP64 path matches bit for bit).
The oracle evaluates exp, log and real powers with its own deterministic
routines and NumPy with the C library's, so the two agree to a few ulps per
operation: rates to 1e-12 relative, Fcool to 1e-12 of the sum of the
magnitudes of its ten terms (it is a difference of cooling and heating).
The cells carry SHIELD's columns (ifrad = 2, INITIA's 20 iterations) and
temperatures from 10 K to 10^5 K, so every branch of fesc, ATN5 and kHrec
is taken."""
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
    st = chem_state(n=10, seed=5)
    st.params = st.params.replace(ifrad=2)
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
