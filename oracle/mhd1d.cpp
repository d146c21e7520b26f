// oracle/mhd1d.cpp — TEST INFRASTRUCTURE ONLY (the oracle; never shipped,
// never on the product path).
//
// CPU restatement of the reference's 1D Lagrange + remap MHD driver with
// Koyama–Inutsuka heating/cooling, the program that produced the golden
// files KIcool/cooling.dat, KIcool/bw051.dat and KIcool/time.DAT:
//   KIcool/1DMHDwCC3.f90            (KI deck, ifthrm=2, free boundaries)
//   1DMHDmany/1DMHDwCC3bw.f90       (Brio–Wu: gamma forced to 2 in the
//                                    sound speed and the CFL, no source)
// Every routine keeps the reference's loop bounds and operation order so
// that, compiled with -ffp-contract=off, it reproduces the Fortran
// arithmetic; each function cites the lines it follows.  exp/log10/10**x go
// through detmath.h (the product's deterministic math, shared on purpose so
// the GPU and this restatement use the same transcendental bits).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../code_tohoku_gb300/csrc/detmath.h"

namespace {

using detmath::fmax2;
using detmath::fmin2;
using detmath::fsign;

constexpr double kb = 8.63359, Kcond = 1.6384e-2;   // 1DMHDwCC3.f90:18

struct Mhd1D {
  // deck (1DMHDwCC3.f90:57-79)
  int Np1x = 512, Np2x = 512;
  double ql1x = 10, ql2x = 10;
  double dinit1 = 1, dinit2 = 1, vinitx1 = 0, vinitx2 = 0, vinity1 = 0, vinity2 = 0;
  double vinitz1 = 0, vinitz2 = 0, pinit1 = 1, pinit2 = 1;
  double binitx1 = 0, binitx2 = 0, binity1 = 0, binity2 = 0, binitz1 = 0, binitz2 = 0;
  double Hini1 = 1, Hini2 = 1, pini1 = 0, pini2 = 0, H2ini1 = 0, H2ini2 = 0;
  double Heini1 = 0, Heini2 = 0, Hepini1 = 0, Hepini2 = 0, Cini1 = 0, Cini2 = 0;
  double COini1 = 0, COini2 = 0, Cpini1 = 0, Cpini2 = 0;
  double CFL = 0.49, facdep = 1.0, tfinal = 40.0;
  int BCx1 = 1, BCx2 = 1, iflag = 0, ifthrm = 2;
  int brio_wu = 0;   // 1DMHDwCC3bw.f90: gamma=2 in RHS sound speed + Couran, SOURCE off
  // RHS's RIEMAN iterations: 5 in the 1D codes (1DMHDwCC3.f90, itrn = 5);
  // the 3D code unrolls 4 (MCF3DSGincfca3.f90:1500-1546, its loop
  // commented out), which a test sets here to compare the two schemes
  int itrn = 5;

  // state
  int Ncell = 0, nd = 0;
  double gamma = 0, gammi1 = 0, gammi2 = 0, gammi3 = 0, gampl1 = 0, gampl2 = 0, gampl3 = 0;
  double pmin = 1e-20, pmax = 1e20, rmin = 1e-20, rmax = 1e20;
  double ndHmin = 0, ndpmin = 0, ndH2min = 0, ndHemin = 0, ndHepmin = 0, ndCmin = 0, ndCpmin = 0,
         ndCOmin = 0;
  double time = 0;
  std::vector<double> x, dx, Va, Uv;
  std::vector<double> ndp, ndH, ndH2, ndHe, ndHep, ndC, ndCp, ndCO;

  // index helpers: Fortran arrays (-1:nd) are stored at [i+1]
  double &X(int i) { return x[i + 1]; }
  double &DX(int i) { return dx[i + 1]; }
  double &VA(int i) { return Va[i + 1]; }
  double &U(int i, int f) { return Uv[(size_t)(f - 1) * (nd + 2) + (i + 1)]; }
  static double &A(std::vector<double> &a, int i) { return a[i + 1]; }

  // BC (1DMHDwCC3.f90:355-378) on a column Q(-1:Ncell+2)
  void BC(double *Q /* points at Q(-1) */) {
    auto q = [&](int i) -> double & { return Q[i + 1]; };
    if (BCx1 == 1) { q(0) = q(1); q(-1) = q(1); }
    if (BCx2 == 1) { q(Ncell + 1) = q(Ncell); q(Ncell + 2) = q(Ncell); }
    if (BCx1 == 3) { q(0) = q(Ncell); q(-1) = q(Ncell - 1); }
    if (BCx2 == 3) { q(Ncell + 1) = q(1); q(Ncell + 2) = q(2); }
  }
  double *col(int f) { return &U(-1, f); }
  static double *colv(std::vector<double> &a) { return a.data(); }

  // INITIA (1DMHDwCC3.f90:44-225)
  void initia() {
    Ncell = Np1x + Np2x;
    nd = Ncell + 2;
    x.assign(nd + 2, 0);
    dx.assign(nd + 2, 0);
    Va.assign(nd + 2, 0);
    Uv.assign((size_t)8 * (nd + 2), 0);
    for (auto *v : {&ndp, &ndH, &ndH2, &ndHe, &ndHep, &ndC, &ndCp, &ndCO}) v->assign(nd + 2, 0);
    gamma = (5.0 * (Hini1 + pini1 + Heini1 + Hepini1) + 7.0 * H2ini1) /
            (3.0 * (Hini1 + pini1 + Heini1 + Hepini1) + 5.0 * H2ini1);
    if (brio_wu) gamma = 2.0;   // 1DMHDwCC3bw.f90:95
    gammi1 = gamma - 1.0; gammi2 = gamma - 2.0; gammi3 = gamma - 3.0;
    gampl1 = gamma + 1.0; gampl2 = gamma + 2.0; gampl3 = gamma + 3.0;
    pmin = 1e-20; pmax = 1e20; rmin = 1e-20; rmax = 1e20;
    ndHmin = rmin * 0.91; ndpmin = 1e-20; ndH2min = 1e-20; ndHemin = rmin * 0.09;
    ndHepmin = 1e-20; ndCpmin = 1e-20; ndCmin = 1e-20; ndCOmin = 1e-20;
    for (int i = -1; i <= Ncell + 2; i++) {
      bool left = (i <= Np1x);
      U(i, 1) = left ? dinit1 : dinit2;
      U(i, 2) = left ? vinitx1 : vinitx2;
      U(i, 3) = left ? vinity1 : vinity2;
      U(i, 4) = left ? vinitz1 : vinitz2;
      U(i, 5) = left ? pinit1 : pinit2;
      U(i, 6) = left ? binitx1 : binitx2;
      U(i, 7) = left ? binity1 : binity2;
      U(i, 8) = left ? binitz1 : binitz2;
      A(ndH, i) = left ? Hini1 : Hini2;
      A(ndp, i) = left ? pini1 : pini2;
      A(ndH2, i) = left ? H2ini1 : H2ini2;
      A(ndHe, i) = left ? Heini1 : Heini2;
      A(ndHep, i) = left ? Hepini1 : Hepini2;
      A(ndC, i) = left ? Cini1 : Cini2;
      A(ndCO, i) = left ? COini1 : COini2;
      A(ndCp, i) = left ? Cpini1 : Cpini2;
    }
    for (int i = -1; i <= Ncell + 2; i++) DX(i) = ql1x / (double)Np1x;   // :180-182
    X(-1) = -DX(0);
    for (int i = 0; i <= Ncell + 2; i++) X(i) = X(i - 1) + DX(i);
    time = 0.0;
  }

  // VLIMIT (1DMHDwCC3.f90:713-731), i = 0 .. Ncell+1
  void VLIMIT(double *Uc, double *grd, double *dxx) {
    const double eps = 1e-10;
    for (int i = 0; i <= Ncell + 1; i++) {
      double delp = Uc[i + 2] - Uc[i + 1];
      double delm = Uc[i + 1] - Uc[i];
      double flmt = fmax2(0.0, (2.0 * delp * delm + eps) / (delp * delp + delm * delm + eps));
      grd[i + 1] = flmt * (Uc[i + 2] - Uc[i]) / (dxx[i + 1] + 0.5 * dxx[i] + 0.5 * dxx[i + 2]);
    }
  }

  // RIEMAN (1DMHDwCC3.f90:566-610): itrn fixed-point iterations
  void RIEMAN(double uLi1, double uLi2, double uLi3, double uLi4, double uRi1, double uRi2,
              double uRi3, double uRi4, double &Pai, double &Vai, int itrn) {
    double D1i = uLi1, V1i = uLi2, P1i = uLi3, B1i = 0.5 * uLi4;
    double D2i = uRi1, V2i = uRi2, P2i = uRi3, B2i = 0.5 * uRi4;
    P1i = P1i + B1i;
    P2i = P2i + B2i;
    double GP1i = gammi1 * P1i, GP2i = gammi1 * P2i;
    double GP1B1i = gammi3 * P1i - gammi2 * B1i * 2.0;
    double GP2B2i = gammi3 * P2i - gammi2 * B2i * 2.0;
    Pai = (P1i + P2i) * 0.5;
    double qM1i = 0, qM2i = 0;
    for (int loop = 1; loop <= itrn; loop++) {
      double pp1i = gampl3 * Pai + GP1B1i;
      double qM1sqi = pp1i + std::sqrt(pp1i * pp1i - 8.0 * (Pai - P1i) * (gampl1 * Pai + GP1i));
      qM1i = std::sqrt(qM1sqi * D1i) * 0.5;
      double pp2i = gampl3 * Pai + GP2B2i;
      double qM2sqi = pp2i + std::sqrt(pp2i * pp2i - 8.0 * (Pai - P2i) * (gampl1 * Pai + GP2i));
      qM2i = std::sqrt(qM2sqi * D2i) * 0.5;
      double PaOLDi = Pai;
      Pai = qM2i * P1i + qM1i * P2i + qM2i * qM1i * (V1i - V2i);
      Pai = Pai / (qM2i + qM1i);
      if (Pai <= 0.0) Pai = 0.1 * PaOLDi;
    }
    Vai = qM1i * V1i + qM2i * V2i + P1i - P2i;
    Vai = Vai / (qM2i + qM1i);
  }

  static double gam_of(double H, double p, double He, double Hep, double H2) {
    double g = 3.0 * (H + p + He + Hep) + 5.0 * H2;
    return (5.0 * (H + p + He + Hep) + 7.0 * H2) / g;
  }
  static double gmi1_of(double H, double p, double He, double Hep, double H2) {
    double g = 3.0 * (H + p + He + Hep) + 5.0 * H2;
    return (2.0 * (H + p + He + Hep) + 2.0 * H2) / g;
  }
  static double posmask(double q, double fallback) {
    // (0.5-dsign(0.5,-q))*q + (0.5+dsign(0.5,-q))*fallback
    return (0.5 - fsign(0.5, -q)) * q + (0.5 + fsign(0.5, -q)) * fallback;
  }

  // RHS (1DMHDwCC3.f90:460-559)
  void RHS(double dt, std::vector<double> &xlag) {
    std::vector<double> grd1(nd + 2), grd2(nd + 2), grd5(nd + 2), grd7(nd + 2), grd8(nd + 2);
    std::vector<double> Pa(nd + 2), dm(nd + 2);
    BC(col(1)); VLIMIT(col(1), grd1.data(), dx.data());
    BC(col(2)); VLIMIT(col(2), grd2.data(), dx.data());
    BC(col(5)); VLIMIT(col(5), grd5.data(), dx.data());
    BC(col(7)); VLIMIT(col(7), grd7.data(), dx.data());
    BC(col(8)); VLIMIT(col(8), grd8.data(), dx.data());
    BC(colv(ndH)); BC(colv(ndp)); BC(colv(ndH2)); BC(colv(ndHe)); BC(colv(ndHep));
    auto g = [&](std::vector<double> &a, int i) { return a[i + 1]; };
    for (int i = 0; i <= Ncell; i++) {
      int ix = i, ixp = i + 1;
      double gam = gam_of(A(ndH, ix), A(ndp, ix), A(ndHe, ix), A(ndHep, ix), A(ndH2, ix));
      if (brio_wu) gam = 2.0;   // 1DMHDwCC3bw.f90:489-491
      double cm = std::sqrt((gam * U(ix, 5) + U(ix, 7) * U(ix, 7) + U(ix, 8) * U(ix, 8)) / U(ix, 1));
      double depend1 = 0.5 * (DX(i) - cm * dt) * facdep;
      depend1 = fmax2(0.0, depend1);
      gam = gam_of(A(ndH, ixp), A(ndp, ixp), A(ndHe, ixp), A(ndHep, ixp), A(ndH2, ixp));
      if (brio_wu) gam = 2.0;   // 1DMHDwCC3bw.f90:497-499
      cm = std::sqrt((gam * U(ixp, 5) + U(ixp, 7) * U(ixp, 7) + U(ixp, 8) * U(ixp, 8)) / U(ixp, 1));
      double depend2 = 0.5 * (DX(i + 1) - cm * dt) * facdep;
      depend2 = fmax2(0.0, depend2);

      double QL1 = U(ix, 1) + depend1 * g(grd1, i);
      QL1 = posmask(QL1, U(ix, 1));
      double QR1 = U(ixp, 1) - depend2 * g(grd1, i + 1);
      QR1 = posmask(QR1, U(ixp, 1));
      double QL2 = U(ix, 2) + depend1 * g(grd2, i);
      double QR2 = U(ixp, 2) - depend2 * g(grd2, i + 1);
      double QL3 = U(ix, 5) + depend1 * g(grd5, i);
      QL3 = posmask(QL3, U(ix, 5));
      double QR3 = U(ixp, 5) - depend2 * g(grd5, i + 1);
      QR3 = posmask(QR3, U(ixp, 5));
      double a7 = U(ix, 7) + depend1 * g(grd7, i), a8 = U(ix, 8) + depend1 * g(grd8, i);
      double QL4 = a7 * a7 + a8 * a8;
      double b7 = U(ixp, 7) - depend2 * g(grd7, i + 1), b8 = U(ixp, 8) - depend2 * g(grd8, i + 1);
      double QR4 = b7 * b7 + b8 * b8;

      double ndHm = 0.5 * (A(ndH, ix) + A(ndH, ixp)), ndpm = 0.5 * (A(ndp, ix) + A(ndp, ixp));
      double ndHem = 0.5 * (A(ndHe, ix) + A(ndHe, ixp)), ndHepm = 0.5 * (A(ndHep, ix) + A(ndHep, ixp));
      double ndH2m = 0.5 * (A(ndH2, ix) + A(ndH2, ixp));
      gamma = (5.0 * (ndHm + ndpm + ndHem + ndHepm) + 7.0 * ndH2m) /
              (3.0 * (ndHm + ndpm + ndHem + ndHepm) + 5.0 * ndH2m);
      gammi1 = gamma - 1.0; gammi2 = gamma - 2.0; gammi3 = gamma - 3.0;
      gampl1 = gamma + 1.0; gampl2 = gamma + 2.0; gampl3 = gamma + 3.0;
      RIEMAN(QL1, QL2, QL3, QL4, QR1, QR2, QR3, QR4, Pa[i + 1], VA(i), itrn);
    }
    for (int i = 0; i <= Ncell; i++) {
      dm[i + 1] = DX(i) * U(i, 1);
      xlag[i + 1] = xlag[i + 1] + VA(i) * dt;
    }
    for (int i = 1; i <= Ncell; i++) {
      int ix = i, ixm = i - 1;
      gammi1 = gmi1_of(A(ndH, ix), A(ndp, ix), A(ndHe, ix), A(ndHep, ix), A(ndH2, ix));
      U(ix, 5) = U(ix, 5) / (U(ix, 1) * gammi1) +
                 0.5 * (U(ix, 2) * U(ix, 2) + U(ix, 3) * U(ix, 3) + U(ix, 4) * U(ix, 4)) +
                 0.5 * (U(ix, 6) * U(ix, 6) + U(ix, 7) * U(ix, 7) + U(ix, 8) * U(ix, 8)) / U(ix, 1);
      double dxl = xlag[ix + 1] - xlag[ixm + 1];
      U(ix, 1) = dm[i + 1] / dxl;
      U(ix, 2) = U(ix, 2) - dt / dm[i + 1] * (Pa[i + 1] - Pa[i]);
      U(ix, 5) = U(ix, 5) - dt / dm[i + 1] * (Pa[i + 1] * VA(i) - Pa[i] * VA(i - 1));
      U(ix, 7) = U(ix, 7) * DX(i) / dxl;
      U(ix, 8) = U(ix, 8) * DX(i) / dxl;
      for (auto *sp : {&ndH, &ndp, &ndH2, &ndHe, &ndHep, &ndC, &ndCp, &ndCO})
        A(*sp, ix) = DX(i) * A(*sp, ix) / dxl;
    }
  }

  // CHAREQ (1DMHDwCC3.f90:831-841)
  static void CHAREQ(double QL1, double QL2, double QL3, double QR1, double QR2, double QR3,
                     double &Bay, double &Vay) {
    double vyp = QL1, vym = QR1, Byp = QL2, Bym = QR2;
    double sqdyp = std::sqrt(QL3), sqdym = std::sqrt(QR3);
    Vay = (sqdyp * vyp + sqdym * vym + Bym - Byp) / (sqdyp + sqdym);
    Bay = (sqdyp * sqdym * (vym - vyp) + sqdyp * Bym + sqdym * Byp) / (sqdyp + sqdym);
  }

  // MOC (1DMHDwCC3.f90:759-828)
  void MOC(double dt, std::vector<double> &xlag) {
    std::vector<double> g1(nd + 2), g3(nd + 2), g4(nd + 2), g7(nd + 2), g8(nd + 2), dxlag(nd + 2);
    std::vector<double> Vay(nd + 2), Bay(nd + 2), Vaz(nd + 2), Baz(nd + 2);
    for (int i = 1; i <= Ncell; i++) dxlag[i + 1] = xlag[i + 1] - xlag[i];
    BC(dxlag.data());
    BC(col(1)); VLIMIT(col(1), g1.data(), dxlag.data());
    BC(col(3)); VLIMIT(col(3), g3.data(), dxlag.data());
    BC(col(4)); VLIMIT(col(4), g4.data(), dxlag.data());
    BC(col(7)); VLIMIT(col(7), g7.data(), dxlag.data());
    BC(col(8)); VLIMIT(col(8), g8.data(), dxlag.data());
    BC(col(6));
    auto D = [&](int i) { return dxlag[i + 1]; };
    for (int i = 0; i <= Ncell; i++) {
      int ix = i, ixp = i + 1;
      double Bnap = U(i, 6);
      double deni = std::sqrt((D(i) + D(i + 1)) / (D(i) * U(ixp, 1) + D(i + 1) * U(ix, 1)));
      double ca = std::fabs(Bnap * deni) * 0.5 * dt;
      ca = fmin2(D(i), ca);
      double depend1 = (0.5 * D(i) - ca) * facdep;
      ca = std::fabs(Bnap * deni) * 0.5 * dt;
      ca = fmin2(D(i + 1), ca);
      double depend2 = (0.5 * D(i + 1) - ca) * facdep;
      double QL11 = U(ix, 3) + depend1 * g3[i + 1];
      double QR11 = U(ixp, 3) - depend2 * g3[i + 2];
      double QL12 = U(ix, 7) + depend1 * g7[i + 1];
      double QR12 = U(ixp, 7) - depend2 * g7[i + 2];
      double QL13 = U(ix, 1) + depend1 * g1[i + 1];
      QL13 = posmask(QL13, U(ix, 1));
      double QR13 = U(ixp, 1) - depend2 * g1[i + 2];
      QR13 = posmask(QR13, U(ixp, 1));
      double QL21 = U(ix, 4) + depend1 * g4[i + 1];
      double QR21 = U(ixp, 4) - depend2 * g4[i + 2];
      double QL22 = U(ix, 8) + depend1 * g8[i + 1];
      double QR22 = U(ixp, 8) - depend2 * g8[i + 2];
      CHAREQ(QL11, QL12, QL13, QR11, QR12, QR13, Bay[i + 1], Vay[i + 1]);
      CHAREQ(QL21, QL22, QL13, QR21, QR22, QR13, Baz[i + 1], Vaz[i + 1]);
    }
    for (int i = 1; i <= Ncell; i++) {
      int ix = i;
      double B6 = U(i, 6);
      U(ix, 3) = U(ix, 3) + dt / U(ix, 1) / D(i) * (Bay[i + 1] - Bay[i]) * B6;
      U(ix, 4) = U(ix, 4) + dt / U(ix, 1) / D(i) * (Baz[i + 1] - Baz[i]) * B6;
      U(ix, 5) = U(ix, 5) + dt / U(ix, 1) / D(i) *
                 ((0.5 * B6 * VA(i) + Bay[i + 1] * Vay[i + 1] + Baz[i + 1] * Vaz[i + 1]) * B6 -
                  (0.5 * B6 * VA(i - 1) + Bay[i] * Vay[i] + Baz[i] * Vaz[i]) * B6);
      U(ix, 7) = U(ix, 7) + dt / D(i) * (Vay[i + 1] - Vay[i]) * B6;
      U(ix, 8) = U(ix, 8) + dt / D(i) * (Vaz[i + 1] - Vaz[i]) * B6;
    }
  }

  // REMAP (1DMHDwCC3.f90:615-707)
  void REMAP(double dt, std::vector<double> &xlag) {
    std::vector<double> dxlag(nd + 2);
    for (int i = 1; i <= Ncell; i++) dxlag[i + 1] = xlag[i + 1] - xlag[i];
    BC(dxlag.data());
    // the 7 MHD columns and the 8 species, each limited then fluxed
    int ucols[7] = {1, 2, 3, 4, 5, 7, 8};
    std::vector<double> *spc[8] = {&ndH, &ndp, &ndH2, &ndHe, &ndHep, &ndC, &ndCp, &ndCO};
    std::vector<std::vector<double>> grd(15, std::vector<double>(nd + 2));
    std::vector<std::vector<double>> F(15, std::vector<double>(nd + 2));
    double *qs[15];
    for (int c = 0; c < 7; c++) qs[c] = col(ucols[c]);
    for (int c = 0; c < 8; c++) qs[7 + c] = spc[c]->data();
    for (int c = 0; c < 15; c++) { BC(qs[c]); VLIMIT(qs[c], grd[c].data(), dxlag.data()); }
    for (int i = 0; i <= Ncell; i++) {
      double vadt = VA(i) * dt;
      if (vadt <= 0.0) {
        double depend = 0.5 * (dxlag[i + 2] + vadt) * facdep;
        for (int c = 0; c < 15; c++) F[c][i + 1] = -vadt * (qs[c][i + 2] - depend * grd[c][i + 2]);
      } else {
        double depend = 0.5 * (dxlag[i + 1] - vadt) * facdep;
        for (int c = 0; c < 15; c++) F[c][i + 1] = -vadt * (qs[c][i + 1] + depend * grd[c][i + 1]);
      }
    }
    for (int i = 1; i <= Ncell; i++) {
      double dxi = 1.0 / (X(i) - X(i - 1));
      for (int c = 0; c < 15; c++)
        qs[c][i + 1] = (qs[c][i + 1] * dxlag[i + 1] + F[c][i + 1] - F[c][i]) * dxi;
    }
  }

  // MHD (1DMHDwCC3.f90:396-454)
  void MHD(double dt) {
    std::vector<double> xlag(nd + 2);
    for (int i = -1; i <= Ncell + 2; i++) xlag[i + 1] = X(i);
    RHS(dt, xlag);
    MOC(dt, xlag);
    for (int i = 1; i <= Ncell; i++) {
      U(i, 2) = U(i, 2) * U(i, 1); U(i, 3) = U(i, 3) * U(i, 1);
      U(i, 4) = U(i, 4) * U(i, 1); U(i, 5) = U(i, 5) * U(i, 1);
    }
    REMAP(dt, xlag);   // iflag = 0 in every deck used here
    for (int i = 1; i <= Ncell; i++) {
      U(i, 1) = fmax2(1.27 * rmin, U(i, 1));
      double invd = 1.0 / U(i, 1);
      U(i, 2) = U(i, 2) * invd;
      U(i, 3) = U(i, 3) * invd;
      U(i, 4) = U(i, 4) * invd;
      gammi1 = gmi1_of(A(ndH, i), A(ndp, i), A(ndHe, i), A(ndHep, i), A(ndH2, i));
      double ekin = 0.5 * (U(i, 2) * U(i, 2) + U(i, 3) * U(i, 3) + U(i, 4) * U(i, 4)) * U(i, 1);
      double emag = 0.5 * (U(i, 6) * U(i, 6) + U(i, 7) * U(i, 7) + U(i, 8) * U(i, 8));
      U(i, 5) = (U(i, 5) - ekin - emag) * gammi1;
      U(i, 5) = fmax2(pmin, U(i, 5));
      U(i, 5) = fmin2(pmax, U(i, 5));
      A(ndH, i) = fmax2(rmin, A(ndH, i));
      A(ndp, i) = fmax2(ndpmin, A(ndp, i));
      A(ndH2, i) = fmax2(ndH2min, A(ndH2, i));
      A(ndHe, i) = fmax2(rmin * 0.09, A(ndHe, i));
      A(ndHep, i) = fmax2(ndHepmin, A(ndHep, i));
      A(ndC, i) = fmax2(ndCmin, A(ndC, i));
      A(ndCp, i) = fmax2(ndCpmin, A(ndCp, i));
      A(ndCO, i) = fmax2(ndCOmin, A(ndCO, i));
    }
  }

  // Couran (1DMHDwCC3.f90:737-750)
  double Couran() {
    double tCFL = tfinal;
    for (int i = 1; i <= Ncell; i++) {
      double gam = gam_of(A(ndH, i), A(ndp, i), A(ndHe, i), A(ndHep, i), A(ndH2, i));
      if (brio_wu) gam = 2.0;   // 1DMHDwCC3bw.f90:751-752
      double c2 = (gam * U(i, 5) + U(i, 6) * U(i, 6) + U(i, 7) * U(i, 7) + U(i, 8) * U(i, 8)) / U(i, 1);
      tCFL = fmin2(tCFL, DX(i) / (std::sqrt(c2) + std::fabs(U(i, 2))));
    }
    return tCFL;
  }

  // Fcool, KI form (1DMHDwCC3.f90:1148-1173): NN = U(i,1)/1.27
  double Fcool(double T, int i) {
    double NN = U(i, 1) / 1.27;
    double AbsL = 3.94656e1, T0 = 1.0e3;
    double Laml = 1.0e7 * detmath::exp(-1.184e5 / (T * T0 + 1.0e3));
    Laml = fmin2(Laml, 5.e3);
    double Lamc = 1.4e-2 * std::sqrt(T * T0) * detmath::exp(-9.2e1 / (T * T0));
    return (NN * NN * (Laml + Lamc) - NN) * AbsL;
  }

  // Stblty (1DMHDwCC3.f90:1086-1111)
  double Stblty() {
    double tLMT = tfinal;
    for (int i = 1; i <= Ncell; i++) {
      double Nn = A(ndH, i) + A(ndp, i) + A(ndH2, i) + A(ndHe, i) + A(ndHep, i);
      double Tn = U(i, 5) / (kb * Nn);
      gammi1 = gmi1_of(A(ndH, i), A(ndp, i), A(ndHe, i), A(ndHep, i), A(ndH2, i));
      double alpha = gammi1 * Kcond * std::sqrt(Tn);
      alpha = Nn * kb * (DX(i) * DX(i)) / alpha;
      double CooL = Fcool(Tn, i);
      double tauC = U(i, 5) / gammi1 / std::fabs(CooL);
      tLMT = fmin2(tLMT, alpha);
      tLMT = fmin2(tLMT, tauC);
    }
    return tLMT;
  }

  // IMC (1DMHDwCC3.f90:1114-1137): log-space bisection, <= 30 iterations
  void IMC(double &P, double n, double dt, int i) {
    double Pu = 1.e10, Pd = 1.e-10, Pm = 1.e1, Pmold = -1.0;
    double nkbi = 1.0 / (kb * n);
    for (int kkk = 1; kkk <= 30; kkk++) {
      double T = Pm * nkbi;
      double CooL = Fcool(T, i);
      double fev = Pm + CooL * dt * gammi1 - P;
      double iud = fsign(1.0, fev);
      Pd = fmax2(-iud * Pm, Pd);
      Pu = fmin2(2.0 * Pm / (iud + 1.0 + 1.e-10), Pu);
      Pm = detmath::exp10(0.5 * (detmath::log10(Pu) + detmath::log10(Pd)));
      if (std::fabs(Pm - Pmold) < 1.e-5) break;
      Pmold = Pm;
    }
    P = Pm;
  }

  // SOURCE, thermal branch ifthrm=2 (1DMHDwCC3.f90:844-926)
  void SOURCE(double dt) {
    if (ifthrm != 2) return;
    std::vector<double> Tn(nd + 2), Pn(nd + 2), Qx(nd + 2);
    BC(col(1)); BC(col(5));
    BC(colv(ndH)); BC(colv(ndp)); BC(colv(ndH2)); BC(colv(ndHe)); BC(colv(ndHep));
    auto T_ = [&](int i) -> double & { return Tn[i + 1]; };
    auto P_ = [&](int i) -> double & { return Pn[i + 1]; };
    auto Q_ = [&](int i) -> double & { return Qx[i + 1]; };
    auto ntot = [&](int i) {
      return A(ndp, i) + A(ndH, i) + A(ndH2, i) + A(ndHe, i) + A(ndHep, i);
    };
    for (int i = 0; i <= Ncell + 1; i++) {
      T_(i) = U(i, 5) / (kb * ntot(i));
      P_(i) = U(i, 5);
    }
    for (int i = 0; i <= Ncell; i++) {
      double rtTx = std::sqrt((DX(i) * T_(i + 1) + DX(i + 1) * T_(i)) / (DX(i) + DX(i + 1)));
      Q_(i) = Kcond * rtTx * (T_(i + 1) - T_(i)) * 2.0 / (DX(i) + DX(i + 1));
    }
    for (int i = 1; i <= Ncell; i++) {
      double CooL = Fcool(T_(i), i);
      gammi1 = gmi1_of(A(ndH, i), A(ndp, i), A(ndHe, i), A(ndHep, i), A(ndH2, i));
      if (dt <= 0.2 * P_(i) / (gammi1 * std::fabs(CooL))) {
        U(i, 5) = U(i, 5) - gammi1 * CooL * dt * 0.5;
      } else {
        IMC(U(i, 5), A(ndH, i) + A(ndp, i) + A(ndHe, i) + A(ndHep, i) + A(ndH2, i), dt * 0.5, i);
      }
      U(i, 5) = U(i, 5) + gammi1 * dt * 0.5 * (Q_(i) - Q_(i - 1)) / DX(i);
      U(i, 5) = fmax2(U(i, 5), pmin);
      U(i, 5) = fmin2(U(i, 5), pmax);
    }
    BC(col(5));
    for (int i = 0; i <= Ncell + 1; i++) T_(i) = U(i, 5) / (kb * ntot(i));
    for (int i = 0; i <= Ncell; i++) {
      double rtTx = std::sqrt((DX(i) * T_(i + 1) + DX(i + 1) * T_(i)) / (DX(i) + DX(i + 1)));
      Q_(i) = Kcond * rtTx * (T_(i + 1) - T_(i)) * 2.0 / (DX(i) + DX(i + 1));
    }
    for (int i = 1; i <= Ncell; i++) {
      double CooL = Fcool(T_(i), i);
      gammi1 = gmi1_of(A(ndH, i), A(ndp, i), A(ndHe, i), A(ndHep, i), A(ndH2, i));
      if (dt <= 0.2 * P_(i) / (gammi1 * std::fabs(CooL))) {
        U(i, 5) = P_(i) - gammi1 * CooL * dt;
      } else {
        IMC(P_(i), A(ndH, i) + A(ndp, i) + A(ndHe, i) + A(ndHep, i) + A(ndH2, i), dt, i);
        U(i, 5) = P_(i);
      }
      U(i, 5) = U(i, 5) + gammi1 * dt * (Q_(i) - Q_(i - 1)) / DX(i);
      U(i, 5) = fmax2(U(i, 5), pmin);
      U(i, 5) = fmin2(U(i, 5), pmax);
    }
  }

  // one in20 iteration of EVOLVE (1DMHDwCC3.f90:254-277); returns dt.
  // dt_given > 0 replaces the Couran/Stblty limit (a test drives this code
  // with the 3D code's steps, whose Stblty differs)
  double step(double dt_given = -1.0) {
    double dt = tfinal;
    if (dt_given > 0.0) {
      dt = dt_given;
    } else {
      double tLMT = Couran();
      dt = fmin2(dt, CFL * tLMT);
      if (ifthrm == 2) {
        tLMT = Stblty();
        dt = fmin2(dt, 0.2 * tLMT);
      }
    }
    if (time + dt > tfinal) dt = tfinal - time;
    if (!brio_wu) SOURCE(dt * 0.5);
    MHD(dt);
    if (!brio_wu) SOURCE(dt * 0.5);
    time = time + dt;
    return dt;
  }
};

}  // namespace

extern "C" {

// Deck values in the order of INPUT.DAT (1DMHDwCC3.f90:57-79):
//  [0..1] Np1x,Np2x  [2..3] ql1x,ql2x  [4..5] d  [6..7] vx  [8..9] vy
//  [10..11] vz  [12..13] p  [14..15] Bx  [16..17] By  [18..19] Bz
//  [20..35] H,p,H2,He,Hep,C,Cp,CO pairs (deck order; CO/Cp follow the
//  reader at 1DMHDwCC3.f90:73-75)  [36..37] CFL,facdep  [38..39] nitera-unused,tfinal
//  [40..41] BCx1,BCx2  [42] ifthrm  [43] brio_wu  [44] p override (<0: none)
void *o1d_create(const double *d) {
  Mhd1D *m = new Mhd1D();
  m->Np1x = (int)d[0]; m->Np2x = (int)d[1];
  m->ql1x = d[2]; m->ql2x = d[3];
  m->dinit1 = d[4]; m->dinit2 = d[5];
  m->vinitx1 = d[6]; m->vinitx2 = d[7];
  m->vinity1 = d[8]; m->vinity2 = d[9];
  m->vinitz1 = d[10]; m->vinitz2 = d[11];
  m->pinit1 = d[12]; m->pinit2 = d[13];
  m->binitx1 = d[14]; m->binitx2 = d[15];
  m->binity1 = d[16]; m->binity2 = d[17];
  m->binitz1 = d[18]; m->binitz2 = d[19];
  m->Hini1 = d[20]; m->Hini2 = d[21];
  m->pini1 = d[22]; m->pini2 = d[23];
  m->H2ini1 = d[24]; m->H2ini2 = d[25];
  m->Heini1 = d[26]; m->Heini2 = d[27];
  m->Hepini1 = d[28]; m->Hepini2 = d[29];
  m->Cini1 = d[30]; m->Cini2 = d[31];
  m->COini1 = d[32]; m->COini2 = d[33];
  m->Cpini1 = d[34]; m->Cpini2 = d[35];
  m->CFL = d[36]; m->facdep = d[37];
  m->tfinal = d[39];
  m->BCx1 = (int)d[40]; m->BCx2 = (int)d[41];
  m->ifthrm = (int)d[42];
  m->brio_wu = (int)d[43];
  if (d[44] >= 0) { m->pinit1 = d[44]; m->pinit2 = d[44]; }   // 1DMHDwCC3.f90:82-83
  m->initia();
  return m;
}

int o1d_ncell(void *h) { return static_cast<Mhd1D *>(h)->Ncell; }
double o1d_time(void *h) { return static_cast<Mhd1D *>(h)->time; }
double o1d_step(void *h) { return static_cast<Mhd1D *>(h)->step(); }
void o1d_set_riemann_iterations(void *h, int n) { static_cast<Mhd1D *>(h)->itrn = n; }
double o1d_step_dt(void *h, double dt) { return static_cast<Mhd1D *>(h)->step(dt); }

// Runs nsteps iterations and records the cooling.dat row after each:
// time, U(512,1)/1.27, U(512,5)*1.52/1.38*100, U(510,7)  (1DMHDwCC3.f90:277)
void o1d_run_trace(void *h, int nsteps, int probe_n, int probe_b, double *trace) {
  Mhd1D *m = static_cast<Mhd1D *>(h);
  for (int s = 0; s < nsteps; s++) {
    if (m->time >= m->tfinal) break;
    m->step();
    trace[4 * s + 0] = m->time;
    trace[4 * s + 1] = m->U(probe_n, 1) / 1.27;
    trace[4 * s + 2] = m->U(probe_n, 5) * 1.52 / 1.38 * 1.e2;
    trace[4 * s + 3] = m->U(probe_b, 7);
  }
}

// State in the bw###.dat column order (1DMHDwCC3.f90:303-304):
// x-centre, U1..U8, ndH, ndp, ndH2, ndHe, ndHep, ndC, ndCO, ndCp; Ncell rows
void o1d_state(void *h, double *out) {
  Mhd1D *m = static_cast<Mhd1D *>(h);
  for (int i = 1; i <= m->Ncell; i++) {
    double *r = out + (size_t)17 * (i - 1);
    r[0] = 0.5 * (m->X(i) + m->X(i - 1));
    for (int f = 1; f <= 8; f++) r[f] = m->U(i, f);
    r[9] = m->A(m->ndH, i); r[10] = m->A(m->ndp, i); r[11] = m->A(m->ndH2, i);
    r[12] = m->A(m->ndHe, i); r[13] = m->A(m->ndHep, i); r[14] = m->A(m->ndC, i);
    r[15] = m->A(m->ndCO, i); r[16] = m->A(m->ndCp, i);
  }
}

void o1d_destroy(void *h) { delete static_cast<Mhd1D *>(h); }

}  // extern "C"
