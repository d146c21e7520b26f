// mhd_chem.cuh — the reference's own microphysics (ifchem = 2): the cooling
// function of its 8 species (Fcool, MCF3DSGincfca3.f90:2825-2880, with fesc
// :2882-2887 and LEVC2 :2889-2895), the reaction rates (RATES :3037-3131)
// and the chemistry network SOURCE runs after the thermal update
// (:2576-2776), including Omexp (:3134-3140).
//
// One template serves both forms: R = double uses the deterministic math of
// detmath.h and is built without contraction, so it reproduces the oracle's
// restatement bit for bit; R = float (the chosen form) uses the fast FP32
// intrinsics.  The operation order is the reference's in both.
//
// Column densities (Ntot, NH2, NnC, NCO, tCII from each x side) come from
// SHIELD (:2924-3036), which runs only with ifrad = 2; with ifrad = 0 (the
// shipped deck) they keep their INITIA value 0 (:476-477).
#pragma once

namespace mhd {

__device__ __forceinline__ double mexp(double x) { return detmath::exp(x); }
__device__ __forceinline__ float mexp(float x) { return __expf(x); }
__device__ __forceinline__ double mlog(double x) { return detmath::log(x); }
__device__ __forceinline__ float mlog(float x) { return __logf(x); }
__device__ __forceinline__ double mpow(double x, double y) { return detmath::pow(x, y); }
__device__ __forceinline__ float mpow(float x, float y) {
  if (x == 0.0f) return y > 0.0f ? 0.0f : (y < 0.0f ? __int_as_float(0x7f800000) : 1.0f);
  return __powf(x, y);
}

// w * y for a 0/1 branch weight w of the reference's arithmetic selects.
// In FP64 an unselected y is finite (its 1e-100 guard keeps pow of a zero
// column finite); in FP32 that guard rounds to 0 and y can be inf, so a
// zero weight selects 0 explicitly instead of forming 0 * inf.
__device__ __forceinline__ double wmul(double w, double y) { return w * y; }
__device__ __forceinline__ float wmul(float w, float y) { return w == 0.0f ? 0.0f : w * y; }
// the reference's 1e-100 guard: below FP32's range, so 0 in the float form
__device__ __forceinline__ double guard100(double) { return 1.e-100; }
__device__ __forceinline__ float guard100(float) { return 0.0f; }

// the species of one cell (number densities), and its nde / ndtot
// slots of the columns in CellSpecies::col and Fields::col
enum { COL_NTOT1 = 0, COL_NTOT2, COL_NH21, COL_NH22, COL_NNC1, COL_NNC2, COL_NCO1, COL_NCO2, COL_TC1, COL_TC2 };

template <class R>
struct CellSpecies {
  R H, p, H2, He, Hep, C, Cp, CO, ne, nt;
  R col[10];
};

template <class R>
__device__ __forceinline__ R fesc_t(R tau) {
  return (R(0.5) + fsgn(R(0.5), R(0.1) - R(1.e-16) - tau)) * (R(0.5) - R(0.585) * tau + R(0.4563) * (tau * tau)) +
         (R(0.5) + fsgn(R(0.5), R(11.9025) - (tau - R(3.55)) * (tau - R(3.55)))) * (R(1) - mexp(R(-2.34) * tau)) /
             (R(4.68) * tau + R(1.e-8)) +
         (R(0.5) + fsgn(R(0.5), tau - R(7))) /
             (R(4) * tau * dsq(mlog(fmx(tau * R(0.56419), R(4)))) + R(1.e-8));
}

// LEVC2 (:2889-2895): the C+ level populations n1, n2
template <class R>
__device__ __forceinline__ void levc2(R T, R b21, R ndH, R ndH2, R nde, R ndCp, R &n1, R &n2) {
  R c21 = R(8.854e-8) * nde / dsq(T) + R(9.399e-10) * mpow(T, R(0.07)) * (ndH + ndH2);
  R c12 = R(2) * c21 * mexp(R(-0.092) / T);
  R A21 = R(2.4e-6) * b21;
  n2 = ndCp * c12 / (c12 + c21 + A21);
  n1 = ndCp * (c21 + A21) / (c12 + c21 + A21);
}

// SHIELD's source term of the C+ optical depth at one cell (:2939-2944):
// 11.5563 (n1 - n2) / dv with the level populations of LEVC2 at the escape
// probabilities of the previous columns tCII
template <class R>
__device__ __forceinline__ R shield_tau_source(R pr, R kb, const CellSpecies<R> &c) {
  const R dv = R(2);
  R b21 = fesc_t(c.col[COL_TC1]) + fesc_t(c.col[COL_TC2]);
  R T = pr / (kb * (c.p + c.H + c.H2 + c.He + c.Hep));
  R n1, n2;
  levc2(T, b21, c.H, c.H2, c.ne, c.Cp, n1, n2);
  return R(1.15563e1) * (n1 - n2) * (R(1) / dv);
}

// Fcool of the species (:2825-2880): Ly-alpha, CII, OI, dust-recombination
// and CO cooling minus photo-electric, cosmic-ray and photo-destruction
// heating, T in 1e3 K
template <class R>
__device__ __forceinline__ R fcool_species(R T, const CellSpecies<R> &c, R *mag = nullptr) {
  const R G0 = R(1), xo = R(3.2e-4), dv = R(2);
  const R Ntot1 = c.col[COL_NTOT1], Ntot2 = c.col[COL_NTOT2], NH21 = c.col[COL_NH21], NH22 = c.col[COL_NH22];
  const R NCO1 = c.col[COL_NCO1], NCO2 = c.col[COL_NCO2], tC1 = c.col[COL_TC1], tC2 = c.col[COL_TC2];
  R Av1 = R(1.63542e-3) * Ntot1, x1 = R(6.1714e3) * NH21;
  R Av2 = R(1.63542e-3) * Ntot2, x2 = R(6.1714e3) * NH22;
  R ATN1 = (mexp(R(-2.5) * Av1) + mexp(R(-2.5) * Av2)) * R(0.5);
  R ATN2 = (mexp(R(-3.77358) * Av1) + mexp(R(-3.77358) * Av2)) * R(0.5);
  R pha = G0 * dsq(R(1.e3) * T) * ATN1 / c.ne;
  R Laml = c.H * c.ne * R(1.44049e9) * mexp(R(-1.184e2) / T);
  Laml = Laml + c.p * c.ne * R(1.48e6) * mexp(R(-8.e1) / T);
  R fesC1 = fesc_t(tC1), fesC2 = fesc_t(tC2);
  R b21 = fesC1 + fesC2;
  R n1, n2;
  levc2(T, b21, c.H, c.H2, c.ne, c.Cp, n1, n2);
  R Lamc = R(6.0157e7) * n2 * b21;
  R tO1 = R(3.40057e-6) * Ntot1 / xo, tO2 = R(3.40057e-6) * Ntot2 / xo;
  R fesO1 = fesc_t(tO1), fesO2 = fesc_t(tO2);
  R Lamo = (fmx(c.nt * xo - c.CO, R(0)) / xo) * (c.H + R(0.5) * c.H2) * R(1.23916e1) * mpow(T, R(0.4)) *
           mexp(R(-0.228) / T);
  Lamo = Lamo * (fesO1 + fesO2);
  R Lamd = c.ne * c.nt * R(6.06236) * mpow(T, R(0.94)) * mpow(pha, R(0.462628) / mpow(T, R(6.8e-2)));
  R ncr = R(3.3e6) * mpow(T, R(0.75)) / (c.H + c.p + c.H2 + c.He + c.Hep);
  R tau1 = R(1.33194e1) * NCO1 / (T * dv), tau2 = R(1.33194e1) * NCO2 / (T * dv);
  R q1 = tau1 * R(0.36788), q2 = tau2 * R(0.36788);
  R ct1 = tau1 * dsq(R(6.283) * mlog(R(2.13) + q1 * q1));
  R ct2 = tau2 * dsq(R(6.283) * mlog(R(2.13) + q2 * q2));
  R ym1 = mlog(R(1) + ct1 / (R(1) + R(1.e1) * ncr)), ym2 = mlog(R(1) + ct2 / (R(1) + R(1.e1) * ncr));
  R fes = (R(2) + ym1 + R(0.6) * (ym1 * ym1)) / (R(1) + ct1 + ncr + R(1.5) * dsq(ncr)) +
          (R(2) + ym2 + R(0.6) * (ym2 * ym2)) / (R(1) + ct2 + ncr + R(1.5) * dsq(ncr));
  R LCOr = c.CO * R(1.91505e10) * (T * T) * fes;
  R LCOH = c.H * c.CO * R(7.96086e4) * dsq(T) * mexp(-mpow(R(2) / T, R(3.43))) * mexp(R(-3.08) / T);
  R LCOH2 = c.H2 * c.CO * R(3.60834e4) * T * mexp(-mpow(R(3.14e2) / T, R(0.333))) * mexp(R(-3.08) / T);
  R Gampe = c.nt * R(2.56526e3) * G0 * ATN1 *
            (R(7.382e-3) * mpow(T, R(0.7)) / (R(1) + R(2.e-4) * pha) + R(4.9e-2) / (R(1) + R(4.e-3) * mpow(pha, R(0.73))));
  R Gamcr = (c.H + c.He + c.H2) * R(1.89435);
  R s1 = R(1) + x1 / dv, s2 = R(1) + x2 / dv;
  R SHLD1 = R(0.965) / (s1 * s1) + R(0.035) / dsq(R(1) + x1) * mexp(R(-8.5e-4) * dsq(R(1) + x1));
  R SHLD2 = R(0.965) / (s2 * s2) + R(0.035) / dsq(R(1) + x2) * mexp(R(-8.5e-4) * dsq(R(1) + x2));
  R Gampd = c.H2 * R(4.16362e4) * G0 * ATN2 * (SHLD1 + SHLD2) * R(0.5);
  // mag: the sum of the magnitudes of the terms, which bounds the rounding
  // error of the difference (the chosen form's time-step screen)
  if (mag) *mag = Laml + Lamc + Lamo + Lamd + LCOr + LCOH + LCOH2 + Gampe + Gamcr + Gampd;
  return Laml + Lamc + Lamo + Lamd + LCOr + LCOH + LCOH2 - Gampe - Gamcr - Gampd;
}

template <class R>
struct ChemRates {
  R zeta, kHrec, kHerec, kH2, kH2ph, kH2dH, kH2de, kCO, kCOph, kCi, kCrec, kCOde, kCOdH, kHie, kHeie, kCie, kHiH,
      kHeiH, kCiH, kCOdHep, kH2dHep;
};

template <class R>
__device__ __forceinline__ ChemRates<R> chem_rates(R T, const CellSpecies<R> &c) {
  const R G0 = R(1), xo = R(3.2e-4), dv = R(2), Tgr = R(5.e-3);
  const R ndH2 = c.H2, nde = c.ne;
  const R Ntot1 = c.col[COL_NTOT1], Ntot2 = c.col[COL_NTOT2], NH21 = c.col[COL_NH21], NH22 = c.col[COL_NH22];
  const R NCO1 = c.col[COL_NCO1], NCO2 = c.col[COL_NCO2], NnC1 = c.col[COL_NNC1], NnC2 = c.col[COL_NNC2];
  ChemRates<R> r;
  R Av1 = R(1.63542e-3) * Ntot1, x1 = R(6.1714e3) * NH21;
  R Av2 = R(1.63542e-3) * Ntot2, x2 = R(6.1714e3) * NH22;
  R ATN2 = (mexp(R(-3.77358) * Av1) + mexp(R(-3.77358) * Av2)) * R(0.5);
  R ATN3 = (mexp(R(-2.3585) * Av1) + mexp(R(-2.3585) * Av2)) * R(0.5);
  R ATN4 = fmn(R(1), mpow(R(3.0857e1) * NH21, R(-3.e-2)) * mexp(R(-1.54285e-3) * NH21)) +
           fmn(R(1), mpow(R(3.0857e1) * NH22, R(-3.e-2)) * mexp(R(-1.54285e-3) * NH22));
  ATN4 = ATN4 * R(0.5);
  const R e06 = R(0.6f);   // the literal 0.6 is REAL*4 in the reference (:3068)
  R ATN5 = (R(0.5) - fsgn(R(0.5), NCO1 - R(1.40995e-3))) * mexp(R(-1) * mpow(R(1.02857e3) * NCO1, e06)) +
           wmul(R(0.5) + fsgn(R(0.5), NCO1 - R(1.40995e-3)),
                fmn(mpow(R(3.75439e3) * NCO1 + guard100(R(0)), R(-0.75)), mpow(R(7.3469e1) * NCO1 + guard100(R(0)), R(-1.3))));
  ATN5 = ATN5 + (R(0.5) - fsgn(R(0.5), NCO2 - R(1.40995e-3))) * mexp(R(-1) * mpow(R(1.02857e3) * NCO2, e06)) +
         wmul(R(0.5) + fsgn(R(0.5), NCO2 - R(1.40995e-3)),
              fmn(mpow(R(3.75439e3) * NCO2 + guard100(R(0)), R(-0.75)), mpow(R(7.3469e1) * NCO2 + guard100(R(0)), R(-1.3))));
  ATN5 = ATN5 * R(0.5);
  r.zeta = R(9.4671e-4);
  R kh = (R(0.5) + fsgn(R(0.5), R(15.78) - T)) * R(0.45) * mlog(R(1.578e2) / T) +
         (R(0.5) - fsgn(R(0.5), R(15.78) - T)) * R(0.4) * dsq(R(1.578e2) / T);
  r.kHrec = R(2.05572e1) * mpow(T, R(-0.5)) * kh;
  r.kHerec = R(6.37623e1) * mpow(T, R(-0.672));
  r.kH2 = R(3.4569e-3) * dsq(T) / (R(1) + R(1.26491) * dsq(T + Tgr) + R(2) * T + R(8) * (T * T));
  R s1 = R(1) + x1 / dv, s2 = R(1) + x2 / dv;
  R SHLD1 = R(0.965) / (s1 * s1) + R(0.035) / dsq(R(1) + x1) * mexp(R(-8.5e-4) * dsq(R(1) + x1));
  R SHLD2 = R(0.965) / (s2 * s2) + R(0.035) / dsq(R(1) + x2) * mexp(R(-8.5e-4) * dsq(R(1) + x2));
  r.kH2ph = R(1.04138e3) * G0 * ATN2 * (SHLD1 + SHLD2) * R(0.5);
  r.kH2dH = R(1.07294e5) * mexp(R(-4.39e1) / T);
  r.kH2de = R(1.133e6) * mpow(T, R(0.35)) * mexp(R(-1.02e2) / T);
  r.kCO = R(1.57785e-2) / (R(1) + G0 * ATN3 / (ndH2 * xo));
  r.kCOph = R(3.155e3) * G0 * ATN3 * ATN4 * ATN5;
  R SHLC1 = mexp(R(-2.6) * Av1 - R(3.0857e1) * NnC1 - R(4.33743413e-4) * NH21) / (R(1) + R(4.33743413e-4) * NH21);
  R SHLC2 = mexp(R(-2.6) * Av2 - R(3.0857e1) * NnC2 - R(4.33743413e-4) * NH22) / (R(1) + R(4.33743413e-4) * NH22);
  r.kCi = R(3.97) * r.zeta + R(6.62697e3) * G0 * (SHLC1 + SHLC2) * R(0.5);
  r.kCrec = R(2.69267e1) * mpow(T, R(-0.62)) * (R(1) + R(1.e-4) * dsq(nde) / (T * T));
  r.kCOde = R(1.4e4) * mpow(T, R(-0.5)) * mexp(R(-1.14e2) / T);
  r.kCOdH = R(1.91858e3) * mpow(T, R(-0.5)) * mexp(R(-7.77e1) / T);
  r.kHie = R(5.76e4) * dsq(T) * mexp(R(-1.58e2) / T);
  r.kHeie = R(2.76e4) * mpow(T, R(0.43)) * mexp(R(-2.85e2) / T);
  r.kCie = R(1.74e5) * mpow(T, R(0.4)) * mexp(R(-1.31e2) / T);
  r.kHiH = R(9.79) * dsq(T) * mexp(R(-1.58e2) / T);
  r.kHeiH = R(4.57) * mpow(T, R(0.43)) * mexp(R(-2.85e2) / T);
  r.kCiH = R(3.01e1) * mpow(T, R(0.4)) * mexp(R(-1.31e2) / T);
  r.kH2dHep = R(1.1676) * mexp(R(-0.035) / T);
  r.kCOdHep = R(5.0491e4);
  return r;
}

// 1 - exp(-eps), its series below 1e-4 (:3134-3140)
template <class R>
__device__ __forceinline__ R omexp(R eps) {
  R e2 = eps * eps;
  return (R(0.5) + fsgn(R(0.5), eps - R(1.e-4))) * (R(1) - mexp(-eps)) +
         (R(0.5) - fsgn(R(0.5), eps - R(1.e-4))) *
             (eps - R(0.5) * e2 + R(0.16666666666666667) * (e2 * eps) - R(4.16666666666666667e-2) * (e2 * e2));
}

// the network of one cell over dt (:2580-2770); c holds the species and
// nde / ndtot on entry and on return; pr is U(:,5); floors: ndmin
template <class R>
__device__ __forceinline__ void chem_network(CellSpecies<R> &c, R pr, R kb, R dt, const R (&ndmin)[8]) {
  R pold = c.p, Hold = c.H, H2old = c.H2, Heold = c.He, Hepold = c.Hep, Cold = c.C, Cpold = c.Cp, COold = c.CO;
  R T = pr / kb / (pold + Hold + H2old + Heold + Hepold);
  const ChemRates<R> k = chem_rates(T, c);
  R t1, t2, t3, om;
  R &H = c.H, &p = c.p, &H2 = c.H2, &He = c.He, &Hep = c.Hep, &C = c.C, &Cp = c.Cp, &CO = c.CO, &ne = c.ne,
    &nt = c.nt;
  // H recombination & ionization by CR
  t1 = k.kHrec * ne;
  t2 = mexp(-dt * (k.zeta + t1));
  t3 = R(1) / (k.zeta + t1);
  om = omexp(dt * (k.zeta + t1));
  H = (t1 * Hold + k.zeta * Hold * t2 + t1 * pold * om) * t3;
  p = (k.zeta * pold + t1 * pold * t2 + k.zeta * Hold * om) * t3;
  Hold = H; pold = p; ne = p + Hep + Cp;
  // He recombination & ionization by CR
  t1 = k.kHerec * ne;
  t2 = mexp(-dt * (k.zeta + t1));
  t3 = R(1) / (k.zeta + t1);
  om = omexp(dt * (k.zeta + t1));
  He = (t1 * Heold + k.zeta * Heold * t2 + t1 * Hepold * om) * t3;
  Hep = (k.zeta * Hepold + t1 * Hepold * t2 + k.zeta * Heold * om) * t3;
  Heold = He; Hepold = Hep; ne = p + Hep + Cp;
  // H2 formation & dissociation by UV & electron collision
  t1 = k.kH2ph + k.kH2de * ne;
  t2 = t1 + R(2) * k.kH2 * nt;
  t3 = mexp(-dt * t2);
  om = omexp(dt * t2);
  H = (Hold + R(2) * H2old * om) * t1 + R(2) * k.kH2 * Hold * nt * t3;
  H = H / t2;
  H2 = (R(2) * H2old + Hold * om) * k.kH2 * nt + t1 * H2old * t3;
  H2 = H2 / t2;
  Hold = H; H2old = H2;
  // H2 dissociation by H collision
  t1 = Hold + R(2) * H2old;
  t2 = mexp(-dt * t1 * k.kH2dH);
  t3 = R(1) / (Hold + R(2) * H2old * t2);
  H = Hold * t1 * t3;
  H2 = H2old * t1 * t2 * t3;
  Hold = H; H2old = H2;
  // CO formation
  t1 = mexp(-dt * k.kCO * nt);
  om = omexp(dt * k.kCO * nt);
  CO = COold + om * Cpold;
  Cp = t1 * Cpold;
  COold = CO; Cpold = Cp; ne = p + Hep + Cp;
  // CO dissociation by UV & electron collision & H collision
  t1 = mexp(-dt * (k.kCOph + k.kCOde * ne + k.kCOdH * Hold));
  om = omexp(dt * (k.kCOph + k.kCOde * ne + k.kCOdH * Hold));
  C = Cold + om * COold;
  CO = t1 * COold;
  Cold = C; COold = CO;
  // C recombination & ionization by CR & UV
  t1 = k.kCrec * ne;
  t2 = mexp(-dt * (k.kCi + t1));
  t3 = R(1) / (k.kCi + t1);
  om = omexp(dt * (k.kCi + t1));
  C = (t1 * Cold + k.kCi * Cold * t2 + t1 * Cpold * om) * t3;
  Cp = (k.kCi * Cpold + t1 * Cpold * t2 + k.kCi * Cold * om) * t3;
  Cold = C; Cpold = Cp; ne = p + Hep + Cp;
  // H, He, C ionization by e collision
  H = Hold * mexp(-dt * k.kHie * ne);
  He = Heold * mexp(-dt * k.kHeie * ne);
  C = Cold * mexp(-dt * k.kCie * ne);
  om = omexp(dt * k.kHie * ne); p = om * Hold + pold;
  om = omexp(dt * k.kHeie * ne); Hep = om * Heold + Hepold;
  om = omexp(dt * k.kCie * ne); Cp = om * Cold + Cpold;
  Hold = H; Heold = He; Cold = C;
  pold = p; Hepold = Hep; Cpold = Cp;
  ne = p + Hep + Cp;
  // H, He, C ionization by H or H2 or p collision
  t1 = R(1) / (R(1) + k.kHiH * dt * Hold);
  H = Hold * t1;
  p = pold + t1 * k.kHiH * dt * (Hold * Hold);
  t1 = H + p + H2old;
  He = Heold * mexp(-dt * k.kHeiH * t1);
  C = Cold * mexp(-dt * k.kCiH * t1);
  om = omexp(dt * k.kHeiH * t1); Hep = om * Heold + Hepold;
  om = omexp(dt * k.kCiH * t1); Cp = om * Cold + Cpold;
  Hold = H; Heold = He; Cold = C;
  pold = p; Hepold = Hep; Cpold = Cp;
  ne = p + Hep + Cp;
  // H2 dissociation by He+ recombination
  t1 = Hepold - H2old;
  if (t1 >= R(0)) {
    t3 = mexp(-dt * k.kH2dHep * t1);
    t2 = R(1) / (Hepold - H2old * t3);
    Hep = Hepold * t1 * t2;
    H2 = H2old * t1 * t2 * t3;
    t3 = Hepold * (R(1) - t1 * t2);
  } else {
    t3 = mexp(dt * k.kH2dHep * t1);
    t2 = R(1) / (Hepold * t3 - H2old);
    Hep = Hepold * t1 * t2 * t3;
    H2 = H2old * t1 * t2;
    t3 = Hepold * (R(1) - t1 * t2 * t3);
  }
  p = pold + t3;
  H = Hold + t3;
  He = Heold + t3;
  Hold = H; pold = p; H2old = H2;
  Heold = He; Hepold = Hep;
  // CO dissociation by He+ recombination
  t1 = Hepold - COold;
  if (t1 >= R(0)) {
    t3 = mexp(-dt * k.kCOdHep * t1);
    t2 = R(1) / (Hepold - COold * t3);
    Hep = Hepold * t1 * t2;
    CO = COold * t1 * t2 * t3;
    t3 = Hepold * (R(1) - t1 * t2);
  } else {
    t3 = mexp(dt * k.kCOdHep * t1);
    t2 = R(1) / (Hepold * t3 - COold);
    Hep = Hepold * t1 * t2 * t3;
    CO = COold * t1 * t2;
    t3 = Hepold * (R(1) - t1 * t2 * t3);
  }
  Cp = Cpold + t3;
  He = Heold + t3;
  H = fmx(ndmin[0], H);
  p = fmx(ndmin[1], p);
  H2 = fmx(ndmin[2], H2);
  He = fmx(ndmin[3], He);
  Hep = fmx(ndmin[4], Hep);
  C = fmx(ndmin[5], C);
  Cp = fmx(ndmin[6], Cp);
  CO = fmx(ndmin[7], CO);
  ne = p + Hep + Cp;
  nt = p + H + R(2) * H2 + He + Hep;
}

}  // namespace mhd
