// mhd_kernels.cuh — the GB300 kernels of the MHD + KI-cooling step.
//
// Included by two translation units: mhd_fp64.cu (plain form, built with
// --fmad=false so every a*b+c rounds twice, as the reference Fortran does)
// and mhd_fp32.cu (chosen form: FP32 reconstruction and flux arithmetic,
// FP64 accumulation, fused multiply-add allowed).  Kernels are templated on
// the reconstruction type R.
//
// Memory layout: every field is one FP64 array of (nx+4)(ny+4)(nz+4) cells
// with two ghost layers, x unit-stride — the reference's
// U(-1:ndx,-1:ndy,-1:ndz,k) column.  The whole grid is resident in HBM; the
// reference's MPI halo exchanges become the ghost copies below (periodic
// wrap or the free-boundary copy), done either in global memory
// (ghost_fill_all_kernel) or inside the fused sweep kernel on its pencils.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "detmath.h"

namespace mhd {

// error word bits (read by the host after each call)
enum : int {
  ERRB_NONFINITE = 1,
  ERRB_DT = 2,
  ERRB_IMC = 4,
  ERRB_TC = 8,            // a tensor-core completion wait timed out (the network was switched off)
  ERRB_TMA = 16,          // a sweep's wait for its TMA-staged inputs timed out
};

struct Grid {
  int n[3];                 // interior cells per direction
  int s[3];                 // padded extents n+4
  long long st[3];          // strides: 1, sx, sx*sy
  long long ncell;          // sx*sy*sz
  int bcl[3], bcr[3];       // 1 = free boundary, otherwise periodic
  const double *x[3];       // coordinates x(-1..n+2) per direction
  const double *dx[3];      // spacings dx(-1..n+2)
  const double *rdx[3];     // 1/(x(i)-x(i-1)), i = -1..n+2 (chosen form)
  const double *rdxc[3];    // 1/dx(i) (chosen form)
  const float *dxf[3];      // dx(i) in FP32 (chosen form)
};

// BC=4 inflow in x (BC_MPI :814-890, BC_MPI_OT :948-1080, INITIA
// :182-200): the values a ghost cell on an inflow side receives.  Side 0 is
// x = 0, side 1 the far end; an inflow side has no periodic neighbour.
struct InflowDev {
  int on[2];               // BC=4 on the left / right side of x
  double rho_ref;          // BBRV(1,*,*)
  double v[2][3];          // BBRV(2..4,1,side)
  double p[2];             // BBRV(5,1,side)
  double b[2][3];          // BBRV(6..8,1,side)
  double cm[8];            // BBRV_cm, species order H,p,H2,He,He+,C,C+,CO
  const float *dtf;        // DTF reservoir, REAL*4, padded layout of U
  double time;             // time of the step (the reference's module time)
};

struct Phys {
  double facdep, pmin, pmax, rmin, kb, kcond, cfl, tfinal;
  int ifthrm;
  int ifchem;              // 2: species cooling + chemistry network; 0: KI cooling
  int ifrad;               // 2: SHIELD column densities; 0: columns stay 0
  double ndmin[8];
  float ndminf[8];         // the floors rounded to FP32 (chosen form)
  InflowDev in;
};

// what a ghost cell on an inflow side receives at one exchange (the
// reference's rule for that field and exchange mode); IN_KEEP leaves it
enum : int {
  IN_KEEP = 0,
  IN_RHO,               // the DTF reservoir advected at the inflow speed (:818-826, :855-862)
  IN_V1, IN_V2, IN_V3,  // inflow velocity components (primitive exchanges)
  IN_M1,                // rho(ghost) vx_in (conserved exchange, :839-843)
  IN_M2, IN_M3,         // rho_ref vy_in, rho_ref vz_in
  IN_P,                 // inflow pressure
  IN_E,                 // 1.5 p_in + 0.5 (rho vx_in^2 + Bcc1^2 + Blg1^2 + Blg2^2) (:833-837)
  IN_BXF,               // face Bx: ghost faces copy face 1, or face n+1 into n+2 (:827-831)
  IN_B2, IN_B3,         // inflow By, Bz (U7, U8, Bcc 2-3, Blg)
  IN_DXLAG,             // dxlagM = dx(0) or dx(n+1) (:951-962)
  IN_BCC1,              // Bcc x copies cell 1 or cell n (:971-988)
  IN_VFC,               // Vfc copies cell 1 or cell n (:1018-1036)
  IN_SPEC,              // + s: BBRV_cm(s) rho(ghost), interior y,z rows only (:1052-1080)
};

struct Fields {
  double *U[8];
  double *sp[8];
  double *bcc[3];
  double *nde, *ndtot;     // electron / particle densities of the chemistry (ifchem = 2)
  // SHIELD's columns from the two x sides (ifrad = 2; else null and 0):
  // Ntot(1,2), NH2(1,2), NnC(1,2), NCO(1,2), tCII(1,2)
  double *col[10];
};

__host__ __device__ inline long long gidx(const Grid &g, int i, int j, int k) {
  return (long long)(i + 1) + g.st[1] * (long long)(j + 1) + g.st[2] * (long long)(k + 1);
}

// The 0-based (i, j, k) of a linear index t over an nx x ny box of
// positions, in 32-bit unsigned arithmetic: every linear index here is
// below 2^31 (mhd_create refuses larger grids), and the 32-bit division is
// a short multiply sequence where a 64-bit one is a long library routine.
__host__ __device__ __forceinline__ void split3(long long t, int nx, int ny, int &i, int &j, int &k) {
  const unsigned u = (unsigned)t, q = u / (unsigned)nx, r = q / (unsigned)ny;
  i = (int)(u - q * (unsigned)nx);
  j = (int)(q - r * (unsigned)ny);
  k = (int)r;
}
// the padded index of interior cell t of the n[0] x n[1] x n[2] block
__host__ __device__ __forceinline__ long long gidx_lin(const Grid &g, long long t, int nx, int ny) {
  int i, j, k;
  split3(t, nx, ny, i, j, k);
  return gidx(g, 1 + i, 1 + j, 1 + k);
}

// density of inflow ghost cell gi of row (j,k): DTF at the upstream position
// x - time vx_in, wrapped into the box (BC_MPI :821-825, :857-861).  The
// operation order is the reference's; the index is clamped into the padded
// reservoir (DTF(-1..n+2)).
__device__ __forceinline__ double inflow_rho(const Grid &g, const InflowDev &in, int side, int gi, int j, int k) {
  const double *xe = g.x[0], *dxe = g.dx[0];   // x(i) at xe[i+1], dx(i) at dxe[i+1]
  const double dx0 = dxe[1];
  const double L = dx0 * g.n[0] * 1;            // dx(0)*Ncellx*NSPLTx
  double xp;
  if (side == 0) {
    xp = xe[1] - 0.5 * dx0 + gi * dx0 - in.time * in.v[0][0];
    int nn = (int)(fabs(xp) / L) + 1;
    xp = xp + L * nn;
  } else {
    xp = 0.5 * (xe[gi] + xe[gi + 1]) - in.time * in.v[1][0];
    int nn = (int)(fabs(xp) / L);
    xp = xp - L * nn;
  }
  int II = (int)(xp / dx0) + 1;
  II = II < -1 ? -1 : (II > g.n[0] + 2 ? g.n[0] + 2 : II);
  return (double)in.dtf[gidx(g, II, j, k)];
}

// the value of rule r for inflow ghost cell gi of row (j,k); bccx is Bcc_x
// at that cell (IN_E), self1 / selfn the array's own cell-1 / cell-n (or
// face n+1) value for the copy rules
__device__ __forceinline__ double inflow_value(const Grid &g, const InflowDev &in, int r, int side, int gi, int j,
                                               int k, double bccx, double self1, double selfn) {
  const double *v = in.v[side];
  switch (r) {
    case IN_RHO: return inflow_rho(g, in, side, gi, j, k);
    case IN_V1: return v[0];
    case IN_V2: return v[1];
    case IN_V3: return v[2];
    case IN_M1: return inflow_rho(g, in, side, gi, j, k) * v[0];
    case IN_M2: return in.rho_ref * v[1];
    case IN_M3: return in.rho_ref * v[2];
    case IN_P: return in.p[side];
    case IN_E: {
      const double rho = inflow_rho(g, in, side, gi, j, k);
      const double b1 = in.b[side][1], b2 = in.b[side][2];
      return in.p[side] * 1.5 + 0.5 * (rho * (v[0] * v[0]) + bccx * bccx + b1 * b1 + b2 * b2);
    }
    case IN_B2: return in.b[side][1];
    case IN_B3: return in.b[side][2];
    case IN_DXLAG: return side == 0 ? g.dx[0][1] : g.dx[0][g.n[0] + 2];
    case IN_BXF:
    case IN_BCC1:
    case IN_VFC: return side == 0 ? self1 : selfn;
    default: return in.cm[r - IN_SPEC] * inflow_rho(g, in, side, gi, j, k);
  }
}

// ---------------------------------------------------------------- scalars
// Fortran SIGN/MAX/MIN with the semantics of detmath.h (shared with the
// CPU restatement so both agree on signed zeros).
__device__ __forceinline__ double fsgn(double a, double b) { return detmath::fsign(a, b); }
__device__ __forceinline__ float fsgn(float a, float b) { return copysignf(fabsf(a), b); }
template <class T> __device__ __forceinline__ T fmx(T a, T b) { return (b > a) ? b : a; }
template <class T> __device__ __forceinline__ T fmn(T a, T b) { return (b < a) ? b : a; }
__device__ __forceinline__ double dsq(double a) { return sqrt(a); }
__device__ __forceinline__ float dsq(float a) { return sqrtf(a); }
__device__ __forceinline__ double dab(double a) { return fabs(a); }
__device__ __forceinline__ float dab(float a) { return fabsf(a); }

// (0.5-sign(0.5,-q))*q + (0.5+sign(0.5,-q))*fallback : keep q if q > 0
template <class T> __device__ __forceinline__ T posmask(T q, T fallback) {
  T s = fsgn(T(0.5), -q);
  return (T(0.5) - s) * q + (T(0.5) + s) * fallback;
}

// VLIMIT body (MCF3DSGincfca3.f90:1716-1724): van Albada slope when s < 0,
// minmod when s > 0, where s = sign(0.5, T-3) is passed in.
template <class R>
__device__ __forceinline__ R vlim(R qm, R q0, R qp, R dxm, R dx0, R dxp, R s) {
  const R eps = R(1e-10);
  R delp = qp - q0;
  R delm = q0 - qm;
  R flmt = fmx(R(0), (R(2) * delp * delm + eps) / (delp * delp + delm * delm + eps));
  R g = flmt * (qp - qm) / (dx0 + R(0.5) * dxm + R(0.5) * dxp);
  delp = R(2) * delp / (dx0 + dxp);
  delm = R(2) * delm / (dx0 + dxm);
  R gmm = (R(0.5) + fsgn(R(0.5), delp * delm)) * fsgn(R(1), delp) * fmn(dab(delp), dab(delm));
  return g * (R(0.5) - s) + gmm * (R(0.5) + s);
}

// The same value as vlim(...) evaluating only the branch the switch keeps.
// vlim returns g*(0.5-s) + gmm*(0.5+s) with s = +-0.5: one term is exactly
// the selected slope and the other is a zero whose sign is known without
// computing it (sign(g) = sign(qp-qm) since flmt >= +0 and the width sum is
// positive; sign(gmm) = sign(delp)), so IEEE addition gives the selected
// slope unless it is zero, and then -0 only when both zeros are -0.  This
// saves the two divisions of the branch not taken; inputs beyond 1e150 take
// the full formula (where the skipped branch could overflow to Inf/NaN).
__device__ __forceinline__ double vlim_sel(double qm, double q0, double qp, double dxm, double dx0, double dxp,
                                           double s) {
  const double eps = 1e-10;
  double delp = qp - q0;
  double delm = q0 - qm;
  if (!(fabs(delp) < 1e150 && fabs(delm) < 1e150)) return vlim<double>(qm, q0, qp, dxm, dx0, dxp, s);
  double r;
  bool zneg;   // sign of the discarded zero term
  if (s > 0.0) {
    // minmod kept
    double dp = 2.0 * delp / (dx0 + dxp);
    double dm = 2.0 * delm / (dx0 + dxm);
    r = (0.5 + fsgn(0.5, dp * dm)) * fsgn(1.0, dp) * fmn(fabs(dp), fabs(dm));
    zneg = signbit(qp - qm);
  } else {
    // van Albada kept
    double flmt = fmx(0.0, (2.0 * delp * delm + eps) / (delp * delp + delm * delm + eps));
    r = flmt * (qp - qm) / (dx0 + 0.5 * dxm + 0.5 * dxp);
    zneg = signbit(delp);
  }
  if (r == 0.0) return (signbit(r) && zneg) ? -0.0 : 0.0;
  return r;
}
__device__ __forceinline__ float vlim_sel(float qm, float q0, float qp, float dxm, float dx0, float dxp, float s) {
  if (s > 0.0f) {
    float dp = 2.0f * (qp - q0) / (dx0 + dxp);
    float dm = 2.0f * (q0 - qm) / (dx0 + dxm);
    return (dp * dm > 0.0f) ? copysignf(fminf(fabsf(dp), fabsf(dm)), dp) : 0.0f;
  }
  float delp = qp - q0, delm = q0 - qm;
  float flmt = fmaxf(0.0f, __fdividef(2.0f * delp * delm + 1e-10f, delp * delp + delm * delm + 1e-10f));
  return __fdividef(flmt * (qp - qm), dx0 + 0.5f * dxm + 0.5f * dxp);
}

// VLIMIT (vlim_sel) with the cell widths' divisors formed once per cell and
// shared by every field limited there (the chosen form's sweeps and EMFs):
// minmod's 2 dq / (dx0 + dx+-) as dq * (2 / (dx0 + dx+-)), van Albada's
// slope as a product with 1 / (dx0 + dx-/2 + dx+/2); only the branch the
// switch s keeps is formed.
struct LimW {
  float rp, rm, ra, s;
};
__device__ __forceinline__ LimW lim_w(float dxm, float dx0, float dxp, float s) {
  LimW w;
  w.s = s;
  w.rp = w.rm = w.ra = 0.0f;
  if (s > 0.0f) {
    w.rp = __fdividef(2.0f, dx0 + dxp);
    w.rm = __fdividef(2.0f, dx0 + dxm);
  } else {
    w.ra = __fdividef(1.0f, dx0 + 0.5f * dxm + 0.5f * dxp);
  }
  return w;
}
__device__ __forceinline__ float vlim_w(float qm, float q0, float qp, const LimW &w) {
  if (w.s > 0.0f) {
    const float dp = (qp - q0) * w.rp, dm = (q0 - qm) * w.rm;
    return (dp * dm > 0.0f) ? copysignf(fminf(fabsf(dp), fabsf(dm)), dp) : 0.0f;
  }
  const float delp = qp - q0, delm = q0 - qm;
  const float flmt = fmaxf(0.0f, __fdividef(2.0f * delp * delm + 1e-10f, delp * delp + delm * delm + 1e-10f));
  return flmt * (qp - qm) * w.ra;
}

template <class R>
__device__ __forceinline__ R tswitch(double e5, double rho, double kb) {
  // T = 1.27*U(:,5)/(kb*U(:,1)); s = sign(0.5, T-3)
  R T = R(1.27) * R(e5) / (R(kb) * R(rho));
  return fsgn(R(0.5), T - R(3));
}

// RIEMAN (MCF3DSGincfca3.f90:1474-1551): four fixed-point iterations of the
// two-shock Lagrangian solver with total pressure P + Bt^2/2.
template <class R>
__device__ __forceinline__ void riemann(R g1, R g2, R g3, R p1, R p3, R uL1, R uL2, R uL3, R uL4,
                                        R uR1, R uR2, R uR3, R uR4, R &Pai, R &Vai) {
  R D1i = uL1, V1i = uL2, P1i = uL3, B1i = R(0.5) * uL4;
  R D2i = uR1, V2i = uR2, P2i = uR3, B2i = R(0.5) * uR4;
  P1i = P1i + B1i;
  P2i = P2i + B2i;
  R GP1i = g1 * P1i, GP2i = g1 * P2i;
  R GP1B1i = g3 * P1i - g2 * B1i * R(2);
  R GP2B2i = g3 * P2i - g2 * B2i * R(2);
  Pai = (P1i + P2i) * R(0.5);
  R qM1i = 0, qM2i = 0;
#pragma unroll
  for (int loop = 0; loop < 4; loop++) {
    R pp1i = p3 * Pai + GP1B1i;
    R qM1sqi = pp1i + dsq(pp1i * pp1i - R(8) * (Pai - P1i) * (p1 * Pai + GP1i));
    qM1i = dsq(qM1sqi * D1i) * R(0.5);
    R pp2i = p3 * Pai + GP2B2i;
    R qM2sqi = pp2i + dsq(pp2i * pp2i - R(8) * (Pai - P2i) * (p1 * Pai + GP2i));
    qM2i = dsq(qM2sqi * D2i) * R(0.5);
    R PaOLDi = Pai;
    Pai = qM2i * P1i + qM1i * P2i + qM2i * qM1i * (V1i - V2i);
    Pai = Pai / (qM2i + qM1i);
    if (Pai <= R(0)) Pai = R(0.1) * PaOLDi;
  }
  Vai = qM1i * V1i + qM2i * V2i + P1i - P2i;
  Vai = Vai / (qM2i + qM1i);
}

// CHAREQ (MCF3DSGincfca3.f90:2101-2111)
template <class R>
__device__ __forceinline__ void chareq(R QL1, R QL2, R QL3, R QR1, R QR2, R QR3, R &Bay, R &Vay) {
  R sqdyp = dsq(QL3), sqdym = dsq(QR3);
  Vay = (sqdyp * QL1 + sqdym * QR1 + QR2 - QL2) / (sqdyp + sqdym);
  Bay = (sqdyp * sqdym * (QR1 - QL1) + sqdyp * QR2 + sqdym * QL2) / (sqdyp + sqdym);
}

__device__ __forceinline__ double gam_of(double H, double p, double He, double Hep, double H2) {
  double gg = 3.0 * (H + p + He + Hep) + 5.0 * H2;
  return (5.0 * (H + p + He + Hep) + 7.0 * H2) / gg;
}
__device__ __forceinline__ double gmi1_of(double H, double p, double He, double Hep, double H2) {
  double gg = 3.0 * (H + p + He + Hep) + 5.0 * H2;
  return (2.0 * (H + p + He + Hep) + 2.0 * H2) / gg;
}

__device__ __forceinline__ void flag(int *err, int bit) { atomicOr(err, bit); }

}  // namespace mhd
#include "mhd_chem.cuh"
namespace mhd {

template <class R, class Load>
__device__ __forceinline__ CellSpecies<R> cell_species(const Fields &f, long long a, Load &&ld) {
  CellSpecies<R> c;
  c.H = ld(f.sp[0][a]); c.p = ld(f.sp[1][a]); c.H2 = ld(f.sp[2][a]); c.He = ld(f.sp[3][a]);
  c.Hep = ld(f.sp[4][a]); c.C = ld(f.sp[5][a]); c.Cp = ld(f.sp[6][a]); c.CO = ld(f.sp[7][a]);
  c.ne = ld(f.nde[a]); c.nt = ld(f.ndtot[a]);
  if (f.col[0]) {
#pragma unroll
    for (int q = 0; q < 10; q++) c.col[q] = ld(f.col[q][a]);
  } else {
#pragma unroll
    for (int q = 0; q < 10; q++) c.col[q] = R(0);
  }
  return c;
}

// SHIELD (:2924-3036), one block: the C+ optical-depth source term of every
// interior cell into tau (R = double: the oracle's arithmetic; float: the
// chosen form) ...
template <class R, class Load, class Store>
__device__ __forceinline__ void shield_tau_cell(const Grid &g, const Phys &ph, const Fields &f, double *tau,
                                                long long t, Load &&ld, Store &&st) {
  const int nx = g.n[0], ny = g.n[1];
  const long long a = gidx_lin(g, t, nx, ny);
  const CellSpecies<R> c = cell_species<R>(f, a, ld);
  tau[a] = st(shield_tau_source<R>(ld(f.U[4][a]), ld(ph.kb), c));
}

// ============================================================ ghost fill
// One direction of one BC_MPI / BC_MPI_OT exchange for up to 8 arrays.
// Thread = one line along direction d (all transverse indices, ghosts
// included, like the MPI vector types).  Periodic wrap first, then the
// free-boundary copy; species restrict the copy to interior transverse
// indices (…-feedback.f90:1057).
struct FillArgs {
  double *f[8];
  int nf;
  int rule[8];          // BC=4 rule per array (IN_KEEP where x has no inflow rule)
  unsigned spmask;      // bit q: array q is a species array (interior transverse lines only)
  InflowDev in;
};

#ifdef MHD_COMMON_KERNELS
// One BC_MPI / BC_MPI_OT exchange of up to 8 arrays, all its directions in
// one launch.  The exchange is a pass per direction x, y, z (those in
// dirs), each over every line along its direction with all transverse
// indices, ghosts included (like the MPI vector types): the periodic wrap,
// then the free-boundary copy on a free side (species arrays: on lines with
// interior transverse indices only, ...-feedback.f90:1057), or on an x side
// with inflow (BC=4) the inflow value of the array's rule.  Those passes are
// pure gathers except the inflow rule, so the value a ghost cell holds after
// them is the pre-exchange value of one source cell, found here by walking
// the passes backwards from the cell: at each pass whose ghost layers hold
// the current coordinate, move it to where that pass copied from, with the
// rule the pass applies to the current line (its transverse coordinates
// decide the species restriction), or end at the inflow value it computes.
// Sources are never written (every pass reads interior cells only, and a
// cell the passes leave alone maps to itself and is skipped), so the launch
// is free of races and equals the passes run one after another (checked
// against them on the CPU for every direction set, 1 and 2 layers, species
// and free / periodic sides).
struct FillAll {
  long long nreg[3];   // threads per array in the x, y and z shells
  // rdim >= 0: only the ghost cells whose padded index along rdim lies in
  // [rlo, rhi) (a slab of the grid), or outside it when rout is set
  int rdim, rlo, rhi, rout;
};
__device__ __forceinline__ int fill_layer(int f, int nol, int N) {   // f-th filled ghost index
  return f < nol ? 1 - nol + f : N + 1 + (f - nol);
}
__device__ __forceinline__ int fill_other(int u, bool masked, int nol, int N) {   // u-th index outside them
  if (!masked) return u - 1;
  if (nol == 2) return u + 1;
  return u == 0 ? -1 : (u <= N ? u : N + 2);
}
__global__ void ghost_fill_all_kernel(Grid g, FillArgs a, int dirs, int nol, FillAll r) {
  const long long per = r.nreg[0] + r.nreg[1] + r.nreg[2];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= per * a.nf) return;
  const int fi = (int)(t / per);
  long long u = t - (long long)fi * per;
  const bool mk[3] = {(dirs & 1) != 0, (dirs & 2) != 0, (dirs & 4) != 0};
  const int N[3] = {g.n[0], g.n[1], g.n[2]};
  int c[3];
  // the shell: x ghosts; else y ghosts; else z ghosts (disjoint)
  int reg = 0;
  while (u >= r.nreg[reg]) u -= r.nreg[reg++];
  {
    int ext[3];
    for (int d = 0; d < 3; d++) ext[d] = d < reg ? (g.s[d] - (mk[d] ? 2 * nol : 0)) : (d == reg ? 2 * nol : g.s[d]);
    int e0, e1, e2;
    split3(u, ext[0], ext[1], e0, e1, e2);
    const int e[3] = {e0, e1, e2};
    for (int d = 0; d < 3; d++)
      c[d] = d == reg ? fill_layer(e[d], nol, N[d]) : (d < reg ? fill_other(e[d], mk[d], nol, N[d]) : e[d] - 1);
  }
  if (r.rdim >= 0 && ((c[r.rdim] + 1 >= r.rlo && c[r.rdim] + 1 < r.rhi) == (r.rout != 0))) return;
  double *F = a.f[fi];
  const bool species = (a.spmask >> fi) & 1u;
  const int rule = a.rule[fi];
  int cur[3] = {c[0], c[1], c[2]};
  for (int d = 2; d >= 0; d--) {
    if (!mk[d]) continue;
    const int q = cur[d];
    const bool left = q <= 0 && q >= 1 - nol, right = q >= N[d] + 1 && q <= N[d] + nol;
    if (!left && !right) continue;
    const int o1 = (d + 1) % 3, o2 = (d + 2) % 3;
    const bool tr_in = cur[o1] >= 1 && cur[o1] <= N[o1] && cur[o2] >= 1 && cur[o2] <= N[o2];
    const bool infl = d == 0 && a.in.on[left ? 0 : 1];
    if (infl) {
      if (rule != IN_KEEP && (!species || tr_in)) {
        // the inflow value (x is the first pass: it reads the pre-exchange state)
        const double f1 = F[gidx(g, 1, cur[1], cur[2])], fN = F[gidx(g, N[0], cur[1], cur[2])];
        F[gidx(g, c[0], c[1], c[2])] = inflow_value(g, a.in, rule, left ? 0 : 1, q, cur[1], cur[2], 0.0, f1, fN);
        return;
      }
      continue;   // kept: this pass leaves the cell alone
    }
    const bool freeb = (left ? g.bcl[d] : g.bcr[d]) == 1 && (!species || tr_in);
    cur[d] = freeb ? (left ? 1 : N[d]) : (left ? q + N[d] : q - N[d]);
  }
  if (cur[0] == c[0] && cur[1] == c[1] && cur[2] == c[2]) return;
  F[gidx(g, c[0], c[1], c[2])] = F[gidx(g, cur[0], cur[1], cur[2])];
}

// dst = src on the ghost shell of layer lay (1: every cell with an index 0
// or n+1 in some direction, the cells a one-layer exchange of all three
// directions writes; 2: every cell with an index -1 or n+2): thread per cell
// of the six planes, each plane spanning the padded extents of the other
// two directions (a cell on two planes is copied twice, with one value).
// Indices are the reference's, -1..n+2.
__global__ void __launch_bounds__(256) shell_copy_kernel(Grid g, const double *src, double *dst, int lay) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long a01 = (long long)g.s[1] * g.s[2], a02 = (long long)g.s[0] * g.s[2],
                  a03 = (long long)g.s[0] * g.s[1];
  const long long per[3] = {a01, a02, a03};
  long long r = t;
  int d = 0;
  while (d < 3 && r >= 2 * per[d]) {
    r -= 2 * per[d];
    d++;
  }
  if (d == 3) return;
  const int side = (int)(r / per[d]);
  const long long q = r % per[d];
  const int o1 = (d + 1) % 3, o2 = (d + 2) % 3;
  const int lo = (o1 < o2) ? o1 : o2, hi = (o1 < o2) ? o2 : o1;
  int c[3];
  // index along d: 1 - lay or n + lay
  c[d] = side == 0 ? 1 - lay : g.n[d] + lay;
  c[lo] = (int)(q % g.s[lo]) - 1;
  c[hi] = (int)(q / g.s[lo]) - 1;
  const long long a = gidx(g, c[0], c[1], c[2]);
  dst[a] = src[a];
}

#endif  // MHD_COMMON_KERNELS

// ============================================================ the sweep
// Fused MHD(xelr,dxelr,dt) for direction DIR: RHS (Lagrangian step with the
// Riemann solver), MOC (Alfvén characteristics), REMAP (upwind MUSCL back to
// the Euler grid) and the conversion to primitives with floors
// (MCF3DSGincfca3.f90:1264-2098).  A CTA owns P neighbouring pencils; each
// whole pencil (n+4 positions) lives in shared memory, so the reference's
// per-stage halo exchanges along the sweep become copies inside the
// pencil, and every field is read from and written to HBM once.  For the
// y and z sweeps the P pencils are adjacent in x, so every global access
// touches P*8 contiguous bytes.
//
// Shared buffers (each L*P entries, L = n+4, index (i+1)*P + p):
enum {
  B_RHO = 0, B_V0, B_V1, B_V2, B_E, B_T1, B_T2, B_XL, B_VA, B_PA,
  B_G0, B_G1, B_G2, B_G3, B_G4, B_S0, B_S1, B_S2, B_S3, B_S4, B_BNA, B_COUNT
};
// B_T1/B_T2 hold Bcc transverse then Blg; B_PA holds Pa then dxlag;
// B_S0..4 hold species (RHS), then Bn, Bay, Vay, Baz, Vaz (MOC), then the
// remapped species (REMAP); B_G* hold slopes, the T switch and fluxes;
// B_XL holds the per-cell gamma during the RHS slopes, then xlag; B_BNA
// holds the face-normal B interpolated to each Lagrangian interface.

struct SweepArgs {
  Grid g;
  Phys ph;
  Fields f;
  double dt;
  int *err;
  // the chosen-form sweep may run over the pencil groups of blockIdx.y in
  // [by0, by1) only (by1 = 0: all of them); the plain form runs them all
  int by0, by1;
};

template <int DIR, int P>
struct Pencil {
  long long base[P];
  long long sd;
  __device__ Pencil(const Grid &g) {
    sd = g.st[DIR];
    for (int p = 0; p < P; p++) {
      int i, j, k;
      if (DIR == 0) { j = blockIdx.x * P + p + 1; k = blockIdx.y + 1; i = -1; }
      else if (DIR == 1) { i = blockIdx.x * P + p + 1; k = blockIdx.y + 1; j = -1; }
      else { i = blockIdx.x * P + p + 1; j = blockIdx.y + 1; k = -1; }
      base[p] = gidx(g, i, j, k);
    }
  }
  // global offset of sweep position i (-1..n+2) on pencil p
  __device__ __forceinline__ long long at(int p, int i) const { return base[p] + (long long)(i + 1) * sd; }
};

template <int DIR, int P, class R>
__global__ void __launch_bounds__(256) sweep_kernel(SweepArgs A) {
  extern __shared__ double sm[];
  const Grid &g = A.g;
  const int N = g.n[DIR];
  const int L = N + 4;
  const int LP = L * P;
  const double dt = A.dt;
  const double facdep = A.ph.facdep;
  const double kb = A.ph.kb;
  const int tid = threadIdx.x, nth = blockDim.x;
  const double *xe = g.x[DIR];   // xelr(i) at xe[i+1]
  const double *dxe = g.dx[DIR];
  Pencil<DIR, P> pc(g);
  constexpr int C1 = (DIR + 1) % 3, C2 = (DIR + 2) % 3;   // transverse components
  auto B = [&](int b, int i, int p) -> double & { return sm[b * LP + (i + 1) * P + p]; };
  auto VB = [](int c) { return B_V0 + c; };   // velocity buffer of component c
  const bool perL = g.bcl[DIR] != 1, perR = g.bcr[DIR] != 1;
  // BC=4 inflow sides of the x sweep (the other sweeps never exchange in x)
  const bool inL = DIR == 0 && A.ph.in.on[0], inR = DIR == 0 && A.ph.in.on[1];
  // in-pencil ghost fill of the listed buffers: periodic wrap or free copy,
  // or on an inflow side the reference's BC=4 value of that buffer's field
  auto fill = [&](const int *bl, const int *rules, int nb) {
    for (int t = tid; t < 4 * P * nb; t += nth) {
      int bq = t / (4 * P);
      int b = bl[bq];
      int r = t % (4 * P);
      int q = r / P, p = r % P;
      int i = (q < 2) ? (q - 1) : (N + q - 1);   // -1, 0, N+1, N+2
      const int side = i <= 0 ? 0 : 1;
      if (side == 0 ? inL : inR) {
        const int rule = rules[bq];
        if (rule == IN_KEEP || (rule == IN_BXF && i == N + 1)) continue;
        // DIR == 0 here: pencil p is row (j, k) = (blockIdx.x*P+p+1, blockIdx.y+1)
        const double bccx = (rule == IN_E) ? A.f.bcc[0][pc.at(p, i)] : 0.0;
        // the face copy reads face 1 or face n+1, which this fill never writes
        const double f1 = (rule == IN_BXF) ? B(b, 1, p) : 0.0, fn = (rule == IN_BXF) ? B(b, N + 1, p) : 0.0;
        B(b, i, p) = inflow_value(g, A.ph.in, rule, side, i, blockIdx.x * P + p + 1, blockIdx.y + 1, bccx, f1, fn);
        continue;
      }
      int src;
      if (i <= 0) src = perL ? i + N : 1;
      else src = perR ? i - N : N;
      B(b, i, p) = B(b, src, p);
    }
  };

  // ---------------------------------------------------------------- load
  for (int t = tid; t < N * P; t += nth) {
    int i = 1 + t / P, p = t % P;
    long long a = pc.at(p, i);
    B(B_RHO, i, p) = A.f.U[0][a];
    B(B_V0, i, p) = A.f.U[1][a];
    B(B_V1, i, p) = A.f.U[2][a];
    B(B_V2, i, p) = A.f.U[3][a];
    B(B_E, i, p) = A.f.U[4][a];
#pragma unroll
    for (int s = 0; s < 5; s++) B(B_S0 + s, i, p) = A.f.sp[s][a];
  }
  for (int t = tid; t < L * P; t += nth) {
    int i = t / P - 1, p = t % P;
    long long a = pc.at(p, i);
    B(B_T1, i, p) = A.f.bcc[C1][a];
    B(B_T2, i, p) = A.f.bcc[C2][a];
  }
  __syncthreads();
  {
    // E1 (RHS :1355,:1357): rho, vn, p, species; E2 (:1960): vt1, vt2
    const int bl[10] = {B_RHO, B_V0, B_V1, B_V2, B_E, B_S0, B_S1, B_S2, B_S3, B_S4};
    const int rl[10] = {IN_RHO, IN_V1, IN_V2, IN_V3, IN_P, IN_SPEC, IN_SPEC + 1, IN_SPEC + 2, IN_SPEC + 3, IN_SPEC + 4};
    fill(bl, rl, 10);
  }
  __syncthreads();

  // ------------------------------------------------------------ RHS
  // slopes of rho, vn, p, Bt1, Bt2 at i = 0..N+1 (:1362-1366)
  for (int t = tid; t < (N + 2) * P; t += nth) {
    int i = t / P, p = t % P;
    R dm = R(dxe[i]), d0 = R(dxe[i + 1]), dp = R(dxe[i + 2]);
    R s = tswitch<R>(B(B_E, i, p), B(B_RHO, i, p), kb);
    B(B_XL, i, p) = gam_of(B(B_S0, i, p), B(B_S1, i, p), B(B_S3, i, p), B(B_S4, i, p), B(B_S2, i, p));
    const int src[5] = {B_RHO, VB(DIR), B_E, B_T1, B_T2};
#pragma unroll
    for (int q = 0; q < 5; q++)
      B(B_G0 + q, i, p) = (double)vlim_sel(R(B(src[q], i - 1, p)), R(B(src[q], i, p)),
                                           R(B(src[q], i + 1, p)), dm, d0, dp, s);
  }
  __syncthreads();
  // Riemann problem at every interface i = 0..N (:1368-1415)
  for (int t = tid; t < (N + 1) * P; t += nth) {
    int i = t / P, p = t % P;
    double rhoA = B(B_RHO, i, p), rhoB = B(B_RHO, i + 1, p);
    double pA = B(B_E, i, p), pB = B(B_E, i + 1, p);
    double t1A = B(B_T1, i, p), t2A = B(B_T2, i, p), t1B = B(B_T1, i + 1, p), t2B = B(B_T2, i + 1, p);
    double HA = B(B_S0, i, p), prA = B(B_S1, i, p), H2A = B(B_S2, i, p), HeA = B(B_S3, i, p), HepA = B(B_S4, i, p);
    double HB = B(B_S0, i + 1, p), prB = B(B_S1, i + 1, p), H2B = B(B_S2, i + 1, p), HeB = B(B_S3, i + 1, p),
           HepB = B(B_S4, i + 1, p);
    R gamA = R(B(B_XL, i, p));
    R cm = dsq((gamA * R(pA) + R(t1A) * R(t1A) + R(t2A) * R(t2A)) / R(rhoA));
    R depend1 = R(0.5) * (R(dxe[i + 1]) - cm * R(dt)) * R(facdep);
    depend1 = fmx(R(0), depend1);
    R gamB = R(B(B_XL, i + 1, p));
    cm = dsq((gamB * R(pB) + R(t1B) * R(t1B) + R(t2B) * R(t2B)) / R(rhoB));
    R depend2 = R(0.5) * (R(dxe[i + 2]) - cm * R(dt)) * R(facdep);
    depend2 = fmx(R(0), depend2);
    R QL1 = R(rhoA) + depend1 * R(B(B_G0, i, p));
    QL1 = posmask(QL1, R(rhoA));
    R QR1 = R(rhoB) - depend2 * R(B(B_G0, i + 1, p));
    QR1 = posmask(QR1, R(rhoB));
    R QL2 = R(B(VB(DIR), i, p)) + depend1 * R(B(B_G1, i, p));
    R QR2 = R(B(VB(DIR), i + 1, p)) - depend2 * R(B(B_G1, i + 1, p));
    R QL3 = R(pA) + depend1 * R(B(B_G2, i, p));
    QL3 = posmask(QL3, R(pA));
    R QR3 = R(pB) - depend2 * R(B(B_G2, i + 1, p));
    QR3 = posmask(QR3, R(pB));
    R l1 = R(t1A) + depend1 * R(B(B_G3, i, p)), l2 = R(t2A) + depend1 * R(B(B_G4, i, p));
    R QL4 = l1 * l1 + l2 * l2;
    R r1 = R(t1B) - depend2 * R(B(B_G3, i + 1, p)), r2 = R(t2B) - depend2 * R(B(B_G4, i + 1, p));
    R QR4 = r1 * r1 + r2 * r2;
    double ndHm = 0.5 * (HA + HB), ndpm = 0.5 * (prA + prB);
    double ndHem = 0.5 * (HeA + HeB), ndHepm = 0.5 * (HepA + HepB);
    double ndH2m = 0.5 * (H2A + H2B);
    double gamma = (5.0 * (ndHm + ndpm + ndHem + ndHepm) + 7.0 * ndH2m) /
                   (3.0 * (ndHm + ndpm + ndHem + ndHepm) + 5.0 * ndH2m);
    R Pa, Va;
    riemann<R>(R(gamma - 1.0), R(gamma - 2.0), R(gamma - 3.0), R(gamma + 1.0), R(gamma + 3.0), QL1, QL2,
               QL3, QL4, QR1, QR2, QR3, QR4, Pa, Va);
    B(B_PA, i, p) = (double)Pa;
    B(B_VA, i, p) = (double)Va;
  }
  __syncthreads();
  // Lagrangian interface positions (:1418-1424); xlag = xelr elsewhere
  for (int t = tid; t < L * P; t += nth) {
    int i = t / P - 1, p = t % P;
    double xl = xe[i + 1];
    if (i >= 0 && i <= N) xl = xl + B(B_VA, i, p) * dt;
    B(B_XL, i, p) = xl;
  }
  __syncthreads();
  // conservation laws in Lagrangian form (:1427-1454)
  for (int t = tid; t < N * P; t += nth) {
    int i = 1 + t / P, p = t % P;
    long long a = pc.at(p, i);
    double rho = B(B_RHO, i, p);
    double dm = dxe[i + 1] * rho;
    double g1c = gmi1_of(B(B_S0, i, p), B(B_S1, i, p), B(B_S3, i, p), B(B_S4, i, p), B(B_S2, i, p));
    double vx = B(B_V0, i, p), vy = B(B_V1, i, p), vz = B(B_V2, i, p);
    double bx = A.f.bcc[0][a], by = A.f.bcc[1][a], bz = A.f.bcc[2][a];
    double e = B(B_E, i, p) / (rho * g1c) + 0.5 * (vx * vx + vy * vy + vz * vz) +
               0.5 * (bx * bx + by * by + bz * bz) / rho;
    double dxl = B(B_XL, i, p) - B(B_XL, i - 1, p);
    B(B_RHO, i, p) = dm / dxl;
    B(VB(DIR), i, p) = B(VB(DIR), i, p) - dt / dm * (B(B_PA, i, p) - B(B_PA, i - 1, p));
    B(B_E, i, p) = e - dt / dm * (B(B_PA, i, p) * B(B_VA, i, p) - B(B_PA, i - 1, p) * B(B_VA, i - 1, p));
    B(B_T1, i, p) = B(B_T1, i, p) * dxe[i + 1] / dxl;
    B(B_T2, i, p) = B(B_T2, i, p) * dxe[i + 1] / dxl;
  }
  __syncthreads();

  // ------------------------------------------------------------ MOC
  // dxlagM (:1962-1970) into B_PA, face-normal B into B_S0
  for (int t = tid; t < N * P; t += nth) {
    int i = 1 + t / P, p = t % P;
    B(B_PA, i, p) = B(B_XL, i, p) - B(B_XL, i - 1, p);
    B(B_S0, i, p) = A.f.U[5 + DIR][pc.at(p, i)];
    // an inflow side's exchange leaves face n+1 as it is (:862-866)
    if (inR && i == N) B(B_S0, N + 1, p) = A.f.U[5 + DIR][pc.at(p, N + 1)];
  }
  __syncthreads();
  {
    // E2 rho (:1960), E3 dxlagM + Blg (:1974), and the face-normal B
    const int bl[5] = {B_RHO, B_PA, B_T1, B_T2, B_S0};
    const int rl[5] = {IN_RHO, IN_DXLAG, IN_B2, IN_B3, IN_BXF};
    fill(bl, rl, 5);
  }
  __syncthreads();
  // the reference's exchange of the face field also rewrites its ghost
  // faces in global memory (including face n+1); do the same
  for (int t = tid; t < 4 * P; t += nth) {
    int q = t / P, p = t % P;
    int i = (q < 2) ? (q - 1) : (N + q - 1);
    A.f.U[5 + DIR][pc.at(p, i)] = B(B_S0, i, p);
  }
  // slopes of rho, vt1, vt2, Blg1, Blg2 with the Lagrangian spacing
  // (:1989-1993); T uses U(:,5) = e inside, p in the ghosts
  for (int t = tid; t < (N + 2) * P; t += nth) {
    int i = t / P, p = t % P;
    R dm = R(B(B_PA, i - 1, p)), d0 = R(B(B_PA, i, p)), dp = R(B(B_PA, i + 1, p));
    R s = tswitch<R>(B(B_E, i, p), B(B_RHO, i, p), kb);
    const int src[5] = {B_RHO, VB(C1), VB(C2), B_T1, B_T2};
#pragma unroll
    for (int q = 0; q < 5; q++)
      B(B_G0 + q, i, p) = (double)vlim_sel(R(B(src[q], i - 1, p)), R(B(src[q], i, p)),
                                           R(B(src[q], i + 1, p)), dm, d0, dp, s);
  }
  __syncthreads();
  // characteristics at every interface (:1996-2057)
  for (int t = tid; t < (N + 1) * P; t += nth) {
    int i = t / P, p = t % P;
    double Bnap = B(B_S0, i + 1, p) + (B(B_XL, i, p) - xe[i + 1]) * (B(B_S0, i + 2, p) - B(B_S0, i, p)) /
                                          (xe[i + 2] - xe[i]);
    B(B_BNA, i, p) = Bnap;
    double D0 = B(B_PA, i, p), D1 = B(B_PA, i + 1, p);
    double rA = B(B_RHO, i, p), rB = B(B_RHO, i + 1, p);
    R deni = dsq(R(D0 + D1) / (R(D0) * R(rB) + R(D1) * R(rA)));
    R QL11, QR11, QL12, QR12, QL13, QR13, QL21, QR21, QL22, QR22;
    const int bT1 = VB(C1), bT2 = VB(C2);
    if (Bnap > 0.0) {
      R ca = dab(R(Bnap) * deni) * R(0.5) * R(dt);
      ca = fmn(R(D0), ca);
      R depend1 = (R(0.5) * R(D0) - ca) * R(facdep);
      ca = dab(R(Bnap) * deni) * R(0.5) * R(dt);
      ca = fmn(R(D1), ca);
      R depend2 = (R(0.5) * R(D1) - ca) * R(facdep);
      QL11 = R(B(bT1, i, p)) + depend1 * R(B(B_G1, i, p));
      QR11 = R(B(bT1, i + 1, p)) - depend2 * R(B(B_G1, i + 1, p));
      QL12 = R(B(B_T1, i, p)) + depend1 * R(B(B_G3, i, p));
      QR12 = R(B(B_T1, i + 1, p)) - depend2 * R(B(B_G3, i + 1, p));
      QL13 = R(rA) + depend1 * R(B(B_G0, i, p));
      QL13 = posmask(QL13, R(rA));
      QR13 = R(rB) - depend2 * R(B(B_G0, i + 1, p));
      QR13 = posmask(QR13, R(rB));
      QL21 = R(B(bT2, i, p)) + depend1 * R(B(B_G2, i, p));
      QR21 = R(B(bT2, i + 1, p)) - depend2 * R(B(B_G2, i + 1, p));
      QL22 = R(B(B_T2, i, p)) + depend1 * R(B(B_G4, i, p));
      QR22 = R(B(B_T2, i + 1, p)) - depend2 * R(B(B_G4, i + 1, p));
    } else {
      R ca = dab(R(Bnap) * deni) * R(0.5) * R(dt);
      ca = fmn(R(D1), ca);
      R depend1 = (R(0.5) * R(D1) - ca) * R(facdep);
      ca = dab(R(Bnap) * deni) * R(0.5) * R(dt);
      ca = fmn(R(D0), ca);
      R depend2 = (R(0.5) * R(D0) - ca) * R(facdep);
      QL11 = R(B(bT1, i + 1, p)) - depend1 * R(B(B_G1, i + 1, p));
      QR11 = R(B(bT1, i, p)) + depend2 * R(B(B_G1, i, p));
      QL12 = R(B(B_T1, i + 1, p)) - depend1 * R(B(B_G3, i + 1, p));
      QR12 = R(B(B_T1, i, p)) + depend2 * R(B(B_G3, i, p));
      QL13 = R(rB) - depend1 * R(B(B_G0, i + 1, p));
      QL13 = posmask(QL13, R(rB));
      QR13 = R(rA) + depend2 * R(B(B_G0, i, p));
      QR13 = posmask(QR13, R(rA));
      QL21 = R(B(bT2, i + 1, p)) - depend1 * R(B(B_G2, i + 1, p));
      QR21 = R(B(bT2, i, p)) + depend2 * R(B(B_G2, i, p));
      QL22 = R(B(B_T2, i + 1, p)) - depend1 * R(B(B_G4, i + 1, p));
      QR22 = R(B(B_T2, i, p)) + depend2 * R(B(B_G4, i, p));
    }
    R Bay, Vay, Baz, Vaz;
    chareq<R>(QL11, QL12, QL13, QR11, QR12, QR13, Bay, Vay);
    chareq<R>(QL21, QL22, QL13, QR21, QR22, QR13, Baz, Vaz);
    B(B_S1, i, p) = (double)Bay;
    B(B_S2, i, p) = (double)Vay;
    B(B_S3, i, p) = (double)Baz;
    B(B_S4, i, p) = (double)Vaz;
  }
  __syncthreads();
  // Lorentz force and induction, v -> rho v, e -> E (:2059-2093)
  for (int t = tid; t < N * P; t += nth) {
    int i = 1 + t / P, p = t % P;
    // Bnam at cell i is Bnap at interface i-1: the same expression
    double Bnap = B(B_BNA, i, p), Bnam = B(B_BNA, i - 1, p);
    double Vnap = B(B_VA, i, p), Vnam = B(B_VA, i - 1, p);
    double rho = B(B_RHO, i, p), DL = B(B_PA, i, p);
    double Bay1 = B(B_S1, i, p), Bay0 = B(B_S1, i - 1, p), Vay1 = B(B_S2, i, p), Vay0 = B(B_S2, i - 1, p);
    double Baz1 = B(B_S3, i, p), Baz0 = B(B_S3, i - 1, p), Vaz1 = B(B_S4, i, p), Vaz0 = B(B_S4, i - 1, p);
    B(VB(DIR), i, p) = B(VB(DIR), i, p) * rho + dt / DL * 0.5 * (Bnap * Bnap - Bnam * Bnam);
    B(VB(C1), i, p) = B(VB(C1), i, p) * rho + dt / DL * (Bnap * Bay1 - Bnam * Bay0);
    B(VB(C2), i, p) = B(VB(C2), i, p) * rho + dt / DL * (Bnap * Baz1 - Bnam * Baz0);
    B(B_E, i, p) = B(B_E, i, p) * rho + dt / DL *
                   ((0.5 * Bnap * Vnap + Bay1 * Vay1 + Baz1 * Vaz1) * Bnap -
                    (0.5 * Bnam * Vnam + Bay0 * Vay0 + Baz0 * Vaz0) * Bnam);
    B(B_T1, i, p) = B(B_T1, i, p) + dt / DL * (Bnap * Vay1 - Bnam * Vay0);
    B(B_T2, i, p) = B(B_T2, i, p) + dt / DL * (Bnap * Vaz1 - Bnam * Vaz0);
  }
  __syncthreads();

  // ------------------------------------------------------------ REMAP
  {
    // E4 (:1572, :1581): Blg and U(1..5) in conserved form
    const int bl[7] = {B_RHO, B_V0, B_V1, B_V2, B_E, B_T1, B_T2};
    const int rl[7] = {IN_RHO, IN_M1, IN_M2, IN_M3, IN_E, IN_B2, IN_B3};
    fill(bl, rl, 7);
  }
  __syncthreads();
  // T switch of every limiter in REMAP, from the state before remapping
  for (int t = tid; t < (N + 2) * P; t += nth) {
    int i = t / P, p = t % P;
    B(B_G0, i, p) = (double)tswitch<R>(B(B_E, i, p), B(B_RHO, i, p), kb);
  }
  __syncthreads();
  // one remapped column: slope (i=0..N+1) -> upwind flux (i=0..N) -> update
  auto remap_column = [&](int b) {
    for (int t = tid; t < (N + 2) * P; t += nth) {
      int i = t / P, p = t % P;
      B(B_G1, i, p) = (double)vlim_sel(R(B(b, i - 1, p)), R(B(b, i, p)), R(B(b, i + 1, p)),
                                       R(B(B_PA, i - 1, p)), R(B(B_PA, i, p)), R(B(B_PA, i + 1, p)),
                                       R(B(B_G0, i, p)));
    }
    __syncthreads();
    for (int t = tid; t < (N + 1) * P; t += nth) {
      int i = t / P, p = t % P;
      double vadt = B(B_VA, i, p) * dt;
      double F;
      if (vadt <= 0.0) {
        double depend = 0.5 * (B(B_PA, i + 1, p) + vadt) * facdep;
        F = -vadt * (B(b, i + 1, p) - (double)(R(depend) * R(B(B_G1, i + 1, p))));
      } else {
        double depend = 0.5 * (B(B_PA, i, p) - vadt) * facdep;
        F = -vadt * (B(b, i, p) + (double)(R(depend) * R(B(B_G1, i, p))));
      }
      B(B_G2, i, p) = F;
    }
    __syncthreads();
    for (int t = tid; t < N * P; t += nth) {
      int i = 1 + t / P, p = t % P;
      B(b, i, p) = (B(b, i, p) * B(B_PA, i, p) + B(B_G2, i, p) - B(B_G2, i - 1, p)) / (xe[i + 1] - xe[i]);
    }
    __syncthreads();
  };
  // species: compressed by the Lagrangian step (:1446-1453), ghosts
  // exchanged (:1594), remapped; the first five are kept for gamma
  for (int s = 0; s < 8; s++) {
    int b = (s < 5) ? (B_S0 + s) : B_G3;
    for (int t = tid; t < N * P; t += nth) {
      int i = 1 + t / P, p = t % P;
      B(b, i, p) = dxe[i + 1] * A.f.sp[s][pc.at(p, i)] / B(B_PA, i, p);   // dxlag = xlag(i)-xlag(i-1)
    }
    __syncthreads();
    const int bl[1] = {b};
    const int rl[1] = {IN_SPEC + s};
    fill(bl, rl, 1);
    __syncthreads();
    remap_column(b);
    const double mn = A.ph.ndmin[s];
    for (int t = tid; t < N * P; t += nth) {
      int i = 1 + t / P, p = t % P;
      A.f.sp[s][pc.at(p, i)] = fmx(mn, B(b, i, p));
    }
  }
  {
    const int cols[7] = {B_RHO, B_V0, B_V1, B_V2, B_E, B_T1, B_T2};
    for (int c = 0; c < 7; c++) remap_column(cols[c]);
  }

  // -------------------------------------------- primitives and floors
  // (:1293-1314)
  const double rfloor = 1.27 * A.ph.rmin;
  for (int t = tid; t < N * P; t += nth) {
    int i = 1 + t / P, p = t % P;
    long long a = pc.at(p, i);
    double rho = fmx(rfloor, B(B_RHO, i, p));
    double invd = 1.0 / rho;
    double vx = B(B_V0, i, p) * invd, vy = B(B_V1, i, p) * invd, vz = B(B_V2, i, p) * invd;
    double g1c = gmi1_of(B(B_S0, i, p), B(B_S1, i, p), B(B_S3, i, p), B(B_S4, i, p), B(B_S2, i, p));
    double ekin = 0.5 * (vx * vx + vy * vy + vz * vz) * rho;
    double bn = A.f.bcc[DIR][a], l1 = B(B_T1, i, p), l2 = B(B_T2, i, p);
    double emag = 0.5 * (bn * bn + l1 * l1 + l2 * l2);
    double pr = (B(B_E, i, p) - ekin - emag) * g1c;
    pr = fmx(A.ph.pmin, pr);
    pr = fmn(A.ph.pmax, pr);
    A.f.U[0][a] = rho;
    A.f.U[1][a] = vx;
    A.f.U[2][a] = vy;
    A.f.U[3][a] = vz;
    A.f.U[4][a] = pr;
    if (!(pr == pr) || !(vx == vx) || !(vy == vy) || !(vz == vz) || !(rho < 1e300)) flag(A.err, ERRB_NONFINITE);
  }
}

// ============================================================ CT
#ifdef MHD_COMMON_KERNELS
// CC(1) face velocities (:2126-2134)
__global__ void face_velocity_kernel(Grid g, Fields f, double *vf0, double *vf1, double *vf2) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int nx1 = g.n[0] + 1, ny1 = g.n[1] + 1, nz1 = g.n[2] + 1;
  if (t >= (long long)nx1 * ny1 * nz1) return;
  int i, j, k;
  split3(t, nx1, ny1, i, j, k);
  i += 1; j += 1; k += 1;
  long long a = gidx(g, i, j, k);
  const double *dx = g.dx[0], *dy = g.dx[1], *dz = g.dx[2];
  if (j <= g.n[1] && k <= g.n[2])
    vf0[a] = (dx[i] * f.U[1][a] + dx[i + 1] * f.U[1][a - 1]) / (dx[i] + dx[i + 1]);
  if (i <= g.n[0] && k <= g.n[2])
    vf1[a] = (dy[j] * f.U[2][a] + dy[j + 1] * f.U[2][a - g.st[1]]) / (dy[j] + dy[j + 1]);
  if (i <= g.n[0] && j <= g.n[1])
    vf2[a] = (dz[k] * f.U[3][a] + dz[k + 1] * f.U[3][a - g.st[2]]) / (dz[k] + dz[k + 1]);
}

#endif  // MHD_COMMON_KERNELS

struct CTArgs {
  Grid g;
  Phys ph;
  Fields f;
  const double *vf[3];
  double *emf[3];
  double dt;
};

// VLIMIT of a face array along direction d at cell position c (T from the
// cell with the same index), :1778-1801 / :1704-1726
template <class R>
__device__ __forceinline__ R face_slope(const Grid &g, const CTArgs &A, const double *q, long long c, int d,
                                        int pos) {
  long long sd = g.st[d];
  const double *dxx = g.dx[d];
  R s = tswitch<R>(A.f.U[4][c], A.f.U[0][c], A.ph.kb);
  return vlim_sel(R(q[c - sd]), R(q[c]), R(q[c + sd]), R(dxx[pos]), R(dxx[pos + 1]), R(dxx[pos + 2]), s);
}

// CC(2) + CCT for the edge direction E (0: Ez on x/y, 1: Ex on y/z,
// 2: Ey on z/x), one thread per edge (:2140-2157, :2186-2445).  The four
// limited slopes each edge needs are evaluated here from the face arrays
// instead of being stored in a dQ scratch array.
template <int E, class R>
__global__ void __launch_bounds__(128) emf_kernel(CTArgs A) {
  const Grid &g = A.g;
  constexpr int da = E, db = (E + 1) % 3, dc = (E + 2) % 3;
  int Na = g.n[da], Nb = g.n[db], Nc = g.n[dc];
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long na1 = Na + 1, nb1 = Nb + 1;
  if (t >= na1 * nb1 * Nc) return;
  int aa = 1 + (int)(t % na1);
  int bb = 1 + (int)((t / na1) % nb1);
  int cc = 1 + (int)(t / (na1 * nb1));
  int c3[3];
  c3[da] = aa; c3[db] = bb; c3[dc] = cc;
  long long p0 = gidx(g, c3[0], c3[1], c3[2]);
  long long sa = g.st[da], sb = g.st[db];
  const double *U1 = A.f.U[0];
  // edge density (:2143-2155)
  double dncv;
  if (E == 0) dncv = 0.25 * (U1[p0] + U1[p0 - sa] + U1[p0 - sb] + U1[p0 - sa - sb]);
  else if (E == 1) dncv = 0.25 * (U1[p0] + U1[p0 - sa] + U1[p0 - sb] + U1[p0 - sa - sb]);
  else dncv = 0.25 * (U1[p0] + U1[p0 - sb] + U1[p0 - sa] + U1[p0 - sa - sb]);
  const double *Vx = A.vf[da], *Vy = A.vf[db];
  const double *Bxf = A.f.U[5 + da], *Byf = A.f.U[5 + db];
  R dsqinv = R(1.0 / sqrt(dncv));
  R facm = R(A.ph.facdep * 0.5);
  R dt = R(A.dt);
  const double *dxe = g.dx[da], *dye = g.dx[db];
  R dxm = R(dxe[aa]), dx0 = R(dxe[aa + 1]), dym = R(dye[bb]), dy0 = R(dye[bb + 1]);
  // characteristic variables at the two x-faces (along b) and y-faces
  // (along a) that meet at this edge
  auto load1 = [&](long long p, int bpos, R &a1p, R &a1m, R &da1p, R &da1m) {
    R v = R(Vx[p]), b = R(Bxf[p]);
    R q1 = face_slope<R>(g, A, Vx, p, db, bpos);
    R q3 = face_slope<R>(g, A, Bxf, p, db, bpos);
    a1p = v + b * dsqinv;
    da1p = (q1 + q3 * dsqinv) * facm;
    a1m = v - b * dsqinv;
    da1m = (q1 - q3 * dsqinv) * facm;
  };
  auto load2 = [&](long long p, int apos, R &a2m, R &a2p, R &da2m, R &da2p) {
    R v = R(Vy[p]), b = R(Byf[p]);
    R q2 = face_slope<R>(g, A, Vy, p, da, apos);
    R q4 = face_slope<R>(g, A, Byf, p, da, apos);
    a2m = v - b * dsqinv;
    da2m = (q2 - q4 * dsqinv) * facm;
    a2p = v + b * dsqinv;
    da2p = (q2 + q4 * dsqinv) * facm;
  };
  R a1pL, a1mL, da1pL, da1mL, a1pR, a1mR, da1pR, da1mR;
  R a2mL, a2pL, da2mL, da2pL, a2mR, a2pR, da2mR, da2pR;
  load1(p0 - sb, bb - 1, a1pL, a1mL, da1pL, da1mL);   // (a, b-1)
  load1(p0, bb, a1pR, a1mR, da1pR, da1mR);            // (a, b)
  load2(p0 - sa, aa - 1, a2mL, a2pL, da2mL, da2pL);   // (a-1, b)
  load2(p0, aa, a2mR, a2pR, da2mR, da2pR);            // (a, b)

  auto cand = [&](R a1p, R da1p, R a1m, R da1m, R a2m, R da2m, R a2p, R da2p, R dyv, R dxv, R S1, R S2,
                  R &C1p, R &C2m, R &C1m, R &C2p) {
    C1p = a1p + da1p * dyv * S1 - da1p * (a2m + da2m * dxv * S2) * dt;
    C1p = C1p / (R(1) - da1p * da2m * dt * dt);
    C2m = a2m + da2m * dxv * S2 - da2m * (a1p + da1p * dyv * S1) * dt;
    C2m = C2m / (R(1) - da1p * da2m * dt * dt);
    C1m = a1m + da1m * dyv * S1 - da1m * (a2p + da2p * dxv * S2) * dt;
    C1m = C1m / (R(1) - da1m * da2p * dt * dt);
    C2p = a2p + da2p * dxv * S2 - da2p * (a1m + da1m * dyv * S1) * dt;
    C2p = C2p / (R(1) - da1m * da2p * dt * dt);
  };
  R C1pLL, C2mLL, C1mLL, C2pLL, C1pRL, C2mRL, C1mRL, C2pRL;
  R C1pLR, C2mLR, C1mLR, C2pLR, C1pRR, C2mRR, C1mRR, C2pRR;
  cand(a1pL, da1pL, a1mL, da1mL, a2mL, da2mL, a2pL, da2pL, dym, dxm, R(1), R(1), C1pLL, C2mLL, C1mLL, C2pLL);
  cand(a1pR, da1pR, a1mR, da1mR, a2mL, da2mL, a2pL, da2pL, dy0, dxm, R(-1), R(1), C1pRL, C2mRL, C1mRL, C2pRL);
  cand(a1pL, da1pL, a1mL, da1mL, a2mR, da2mR, a2pR, da2pR, dym, dx0, R(1), R(-1), C1pLR, C2mLR, C1mLR, C2pLR);
  cand(a1pR, da1pR, a1mR, da1mR, a2mR, da2mR, a2pR, da2pR, dy0, dx0, R(-1), R(-1), C1pRR, C2mRR, C1mRR, C2pRR);

  int w11 = (C1pLL > R(0) && C2mLL > R(0)), w12 = (C1mLL > R(0) && C2pLL > R(0));
  int w21 = (C1pRL > R(0) && C2mRL < R(0)), w22 = (C1mRL > R(0) && C2pRL < R(0));
  int w31 = (C1pLR < R(0) && C2mLR > R(0)), w32 = (C1mLR < R(0) && C2pLR > R(0));
  int w41 = (C1pRR < R(0) && C2mRR < R(0)), w42 = (C1mRR < R(0) && C2pRR < R(0));
  auto boost = [](int x1, int x2) { return R((double)(int)(0.51 * (double)x1 + 0.51 * (double)x2)); };
  const R big = R(1.e13 - 1.0);
  R W11 = R(w11) + big * boost(w11, w12), W12 = R(w12) + big * boost(w11, w12);
  R W21 = R(w21) + big * boost(w21, w22), W22 = R(w22) + big * boost(w21, w22);
  R W31 = R(w31) + big * boost(w31, w32), W32 = R(w32) + big * boost(w31, w32);
  R W41 = R(w41) + big * boost(w41, w42), W42 = R(w42) + big * boost(w41, w42);
  R C1p = 0, C2m = 0, C1m = 0, C2p = 0;
  if (w11 + w21 + w31 + w41 != 0) {
    C1p = W11 * dab(C2mLL) * C1pLL + W21 * dab(C2mRL) * C1pRL + W31 * dab(C2mLR) * C1pLR + W41 * dab(C2mRR) * C1pRR;
    C1p = C1p / (W11 * dab(C2mLL) + W21 * dab(C2mRL) + W31 * dab(C2mLR) + W41 * dab(C2mRR));
    C2m = W11 * dab(C1pLL) * C2mLL + W21 * dab(C1pRL) * C2mRL + W31 * dab(C1pLR) * C2mLR + W41 * dab(C1pRR) * C2mRR;
    C2m = C2m / (W11 * dab(C1pLL) + W21 * dab(C1pRL) + W31 * dab(C1pLR) + W41 * dab(C1pRR));
  }
  if (w12 + w22 + w32 + w42 != 0) {
    C1m = W12 * dab(C2pLL) * C1mLL + W22 * dab(C2pRL) * C1mRL + W32 * dab(C2pLR) * C1mLR + W42 * dab(C2pRR) * C1mRR;
    C1m = C1m / (W12 * dab(C2pLL) + W22 * dab(C2pRL) + W32 * dab(C2pLR) + W42 * dab(C2pRR));
    C2p = W12 * dab(C1mLL) * C2pLL + W22 * dab(C1mRL) * C2pRL + W32 * dab(C1mLR) * C2pLR + W42 * dab(C1mRR) * C2pRR;
    C2p = C2p / (W12 * dab(C1mLL) + W22 * dab(C1mRL) + W32 * dab(C1mLR) + W42 * dab(C1mRR));
  }
  R v1a = C1p + C1m, v2a = C2p + C2m, B1a = C1p - C1m, B2a = C2p - C2m;
  A.emf[E][p0] = (double)(R(0.25) * (v1a * B2a - v2a * B1a)) * sqrt(dncv);
}

#ifdef MHD_COMMON_KERNELS
// CC(3): face B from the EMF curl (:2159-2169); emf[0]=Ez, [1]=Ex, [2]=Ey
__global__ void face_b_kernel(Grid g, Fields f, const double *Ez, const double *Ex, const double *Ey, double dt) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int nx1 = g.n[0] + 1, ny1 = g.n[1] + 1, nz1 = g.n[2] + 1;
  if (t >= (long long)nx1 * ny1 * nz1) return;
  int i, j, k;
  split3(t, nx1, ny1, i, j, k);
  i += 1; j += 1; k += 1;
  long long a = gidx(g, i, j, k);
  long long sx = 1, sy = g.st[1], sz = g.st[2];
  const double *dx = g.dx[0], *dy = g.dx[1], *dz = g.dx[2];
  if (j <= g.n[1] && k <= g.n[2])
    f.U[5][a] = f.U[5][a] + dt / dy[j + 1] * (Ez[a + sy] - Ez[a]) - dt / dz[k + 1] * (Ey[a + sz] - Ey[a]);
  if (i <= g.n[0] && k <= g.n[2])
    f.U[6][a] = f.U[6][a] + dt / dz[k + 1] * (Ex[a + sz] - Ex[a]) - dt / dx[i + 1] * (Ez[a + sx] - Ez[a]);
  if (i <= g.n[0] && j <= g.n[1])
    f.U[7][a] = f.U[7][a] + dt / dx[i + 1] * (Ey[a + sx] - Ey[a]) - dt / dy[j + 1] * (Ex[a + sy] - Ex[a]);
}

// CC(4): cell-centred B (:2171-2177)
// 0.5 x, bit for bit the FP64 product: for a normal x whose half is normal
// the exponent field drops by one (an integer subtraction, off GB300's
// narrow FP64 pipe); zeros, subnormals, Inf and NaN take the multiply.
__device__ __forceinline__ double half_exact(double x) {
  const int hi = __double2hiint(x);
  const int e = (hi >> 20) & 0x7ff;
  if (e > 1 && e < 0x7ff) return __hiloint2double(hi - 0x00100000, __double2loint(x));
  return 0.5 * x;
}

// two cells per thread, blockDim apart (every warp access stays coalesced),
// the six loads of both issued before either is used; interior cells of
// linear index [c0, c1)
__global__ void __launch_bounds__(256) cell_b_kernel(Grid g, Fields f, long long c0, long long c1) {
  const long long n = c1;
  const long long t0 = c0 + (long long)blockIdx.x * (2 * blockDim.x) + threadIdx.x;
  double v[2][6];
  long long aa[2];
#pragma unroll
  for (int u = 0; u < 2; u++) {
    const long long t = t0 + u * blockDim.x;
    aa[u] = -1;
    if (t < n) {
      const long long a = gidx_lin(g, t, g.n[0], g.n[1]);
      aa[u] = a;
      v[u][0] = f.U[5][a]; v[u][1] = f.U[5][a + 1];
      v[u][2] = f.U[6][a]; v[u][3] = f.U[6][a + g.st[1]];
      v[u][4] = f.U[7][a]; v[u][5] = f.U[7][a + g.st[2]];
    }
  }
#pragma unroll
  for (int u = 0; u < 2; u++) {
    const long long a = aa[u];
    if (a < 0) continue;
    f.bcc[0][a] = half_exact(v[u][0] + v[u][1]);
    f.bcc[1][a] = half_exact(v[u][2] + v[u][3]);
    f.bcc[2][a] = half_exact(v[u][4] + v[u][5]);
  }
}

#endif  // MHD_COMMON_KERNELS

// ============================================================ source
// KI cooling function, KIcool/1DMHDwCC3.f90:1166-1173 (NN = rho/1.27).
__device__ __forceinline__ double fcool_ki(double T, double NN) {
  const double AbsL = 3.94656e1, T0 = 1.0e3;
  double Laml = 1.0e7 * detmath::exp(-1.184e5 / (T * T0 + 1.0e3));
  Laml = fmn(Laml, 5.e3);
  double Lamc = 1.4e-2 * sqrt(T * T0) * detmath::exp(-9.2e1 / (T * T0));
  return (NN * NN * (Laml + Lamc) - NN) * AbsL;
}
__device__ __forceinline__ float fcool_ki(float T, float NN) {
  float Laml = 1.0e7f * __expf(-1.184e5f / (T * 1.0e3f + 1.0e3f));
  Laml = fmn(Laml, 5.e3f);
  float Lamc = 1.4e-2f * sqrtf(T * 1.0e3f) * __expf(-9.2e1f / (T * 1.0e3f));
  return (NN * NN * (Laml + Lamc) - NN) * 3.94656e1f;
}

// the KI form in FP32 with the sum of the magnitudes of its cooling and
// heating terms (mag), which bounds the rounding error of their difference
__device__ __forceinline__ float fcool_ki_mag(float T, float NN, float &mag) {
  float Laml = 1.0e7f * __expf(-1.184e5f / (T * 1.0e3f + 1.0e3f));
  Laml = fmn(Laml, 5.e3f);
  float Lamc = 1.4e-2f * sqrtf(T * 1.0e3f) * __expf(-9.2e1f / (T * 1.0e3f));
  const float A = NN * NN * (Laml + Lamc);
  mag = (A + NN) * 3.94656e1f;
  return (A - NN) * 3.94656e1f;
}

// the cooling function of the run at temperature T of cell a: the KI form
// (NN = rho/1.27) or, with ifchem = 2, the species form
__device__ __forceinline__ double cool_of(const Phys &ph, const Fields &f, long long a, double T) {
  if (ph.ifchem == 2) return fcool_species<double>(T, cell_species<double>(f, a, [](double v) { return v; }));
  return fcool_ki(T, f.U[0][a] / 1.27);
}

// IMC, log-space bisection for P + Lambda(P) dt (gamma-1) = P_old, at most
// 30 iterations (:2898-2921).  The loop bound is the reference's.
template <class Cool>
__device__ __forceinline__ double imc_f(double Pold, double n, double dt, double g1c, double kb, Cool &&cool) {
  double Pu = 1.e10, Pd = 1.e-10, Pm = 1.e1, Pmold = -1.0;
  double nkbi = 1.0 / (kb * n);
  for (int kkk = 1; kkk <= 30; kkk++) {
    double T = Pm * nkbi;
    double CooL = cool(T);
    double fev = Pm + CooL * dt * g1c - Pold;
    double iud = fsgn(1.0, fev);
    Pd = fmx(-iud * Pm, Pd);
    Pu = fmn(2.0 * Pm / (iud + 1.0 + 1.e-10), Pu);
    Pm = detmath::exp10(0.5 * (detmath::log10(Pu) + detmath::log10(Pd)));
    if (fabs(Pm - Pmold) < 1.e-5) break;
    Pmold = Pm;
  }
  return Pm;
}
__device__ __forceinline__ double imc(double Pold, double n, double dt, double g1c, double NN, double kb) {
  return imc_f(Pold, n, dt, g1c, kb, [&](double T) { return fcool_ki(T, NN); });
}

struct SourceArgs {
  Grid g;
  Phys ph;
  Fields f;
  const double *pin;    // pressure the temperatures are formed from
  const double *pold;   // Pn: pressure at the start of SOURCE
  double *pout;
  double dt;
  int pass;             // 0 predictor (half of dt), 1 corrector
  int *err;
  unsigned long long *imc_count;
  const unsigned char *skip;   // cells already solved (surrogate), or null
};

__device__ __forceinline__ double ntot_T(const Fields &f, long long a) {
  // ndp+ndH+ndH2+ndHe+ndHep (:2489)
  return f.sp[1][a] + f.sp[0][a] + f.sp[2][a] + f.sp[3][a] + f.sp[4][a];
}
__device__ __forceinline__ double ntot_imc(const Fields &f, long long a) {
  // ndH+ndp+ndHe+ndHep+ndH2 (:2512)
  return f.sp[0][a] + f.sp[1][a] + f.sp[3][a] + f.sp[4][a] + f.sp[2][a];
}

// Couran (:1912-1930) and Stblty (:2784-2822) limits of interior cell t
// (linear index over nx*ny*nz); c_min/s_min come in as tfinal.  dt_kernel
// and the allocation-free variant in mhd_noalloc.cu both call it.
__device__ __forceinline__ void cell_dt_limits(const Grid &g, const Phys &ph, const Fields &f, long long t,
                                               double &c_min, double &s_min) {
  int nx = g.n[0], ny = g.n[1];
  int i, j, k;
  split3(t, nx, ny, i, j, k);
  i += 1; j += 1; k += 1;
  long long a = gidx(g, i, j, k);
  double H = f.sp[0][a], pr = f.sp[1][a], H2 = f.sp[2][a], He = f.sp[3][a], Hep = f.sp[4][a];
  double gam = gam_of(H, pr, He, Hep, H2);
  double bx = f.bcc[0][a], by = f.bcc[1][a], bz = f.bcc[2][a];
  double rho = f.U[0][a], p5 = f.U[4][a];
  double c2 = (gam * p5 + bx * bx + by * by + bz * bz) / rho;
  double cs = sqrt(c2);
  double dxi = g.dx[0][i + 1], dyj = g.dx[1][j + 1], dzk = g.dx[2][k + 1];
  c_min = fmn(c_min, dxi / (cs + fabs(f.U[1][a])));
  c_min = fmn(c_min, dyj / (cs + fabs(f.U[2][a])));
  c_min = fmn(c_min, dzk / (cs + fabs(f.U[3][a])));
  if (ph.ifthrm == 2) {
    double Nn = pr + H + H2 + He + Hep;
    double Tn = p5 / (ph.kb * Nn);
    double dl = fmn(fmn(dxi, dyj), dzk);
    double g1c = gmi1_of(H, pr, He, Hep, H2);
    double alpha = g1c * ph.kcond * sqrt(fmn(Tn, 15.0));
    alpha = 0.4 * Nn * ph.kb / alpha * (dl * dl);
    double CooL = cool_of(ph, f, a, Tn);
    double tauC = p5 / g1c / fabs(CooL);
    tauC = fmx(0.2 * tauC, 2.5e-4);
    s_min = fmn(s_min, tauC);
    s_min = fmn(s_min, alpha);
  }
}

#ifdef MHD_COMMON_KERNELS
// One pass of the thermal SOURCE (:2488-2522 for pass 0, :2530-2568 for
// pass 1) for one cell: T of the cell and its six neighbours, capped
// Spitzer-like conduction fluxes on the six faces, cooling (explicit when
// dt <= 0.2 p/((gamma-1)|Lambda|), else IMC) and the conduction update.
__global__ void source_kernel(SourceArgs A) {
  const Grid &g = A.g;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  if (t >= (long long)nx * ny * nz) return;
  int i, j, k;
  split3(t, nx, ny, i, j, k);
  i += 1; j += 1; k += 1;
  long long a = gidx(g, i, j, k);
  const double kb = A.ph.kb, Kc = A.ph.kcond, dt = A.dt;
  const double *pin = A.pin;
  auto Tn = [&](long long c) { return pin[c] / (kb * ntot_T(A.f, c)); };
  const double *dx = g.dx[0], *dy = g.dx[1], *dz = g.dx[2];
  double T0 = Tn(a);
  long long sx = 1, sy = g.st[1], sz = g.st[2];
  // face flux between lower cell (position q in direction d) and upper
  auto flux = [&](double Tl, double Tu, double dl, double du) {
    double rt = sqrt((dl * Tu + du * Tl) / (dl + du));
    return Kc * fmn(rt, 3.873) * (Tu - Tl) * 2.0 / (dl + du);
  };
  double Qxp = flux(T0, Tn(a + sx), dx[i + 1], dx[i + 2]);
  double Qxm = flux(Tn(a - sx), T0, dx[i], dx[i + 1]);
  double Qyp = flux(T0, Tn(a + sy), dy[j + 1], dy[j + 2]);
  double Qym = flux(Tn(a - sy), T0, dy[j], dy[j + 1]);
  double Qzp = flux(T0, Tn(a + sz), dz[k + 1], dz[k + 2]);
  double Qzm = flux(Tn(a - sz), T0, dz[k], dz[k + 1]);
  const Fields &f = A.f;
  double g1c = gmi1_of(f.sp[0][a], f.sp[1][a], f.sp[3][a], f.sp[4][a], f.sp[2][a]);
  double CooL = cool_of(A.ph, f, a, T0);
  auto cool = [&](double T) { return cool_of(A.ph, f, a, T); };
  double Pn = A.pold[a];
  double pnew;
  bool skip = A.skip && A.skip[a];
  if (A.pass == 0) {
    if (skip) pnew = A.pout[a];
    else if (dt <= 0.2 * Pn / (g1c * fabs(CooL))) pnew = pin[a] - g1c * CooL * dt * 0.5;
    else {
      pnew = imc_f(pin[a], ntot_imc(f, a), dt * 0.5, g1c, kb, cool);
      atomicAdd(A.imc_count, 1ull);
    }
  } else {
    if (skip) pnew = A.pout[a];
    else if (dt <= 0.2 * Pn / (g1c * fabs(CooL))) pnew = Pn - g1c * CooL * dt;
    else {
      pnew = imc_f(Pn, ntot_imc(f, a), dt, g1c, kb, cool);
      atomicAdd(A.imc_count, 1ull);
    }
  }
  double tcd = g1c * Kc * sqrt(T0);
  tcd = 0.49 * ntot_imc(f, a) * kb / tcd * (dx[i + 1] * dx[i + 1]);
  tcd = fsgn(0.5, tcd - dt);
  double div = (Qxp - Qxm) / dx[i + 1] + (Qyp - Qym) / dy[j + 1] + (Qzp - Qzm) / dz[k + 1];
  if (A.pass == 0) pnew = pnew + (tcd + 0.5) * g1c * dt * 0.5 * div;
  else pnew = pnew + (tcd + 0.5) * g1c * dt * div;
  pnew = fmx(pnew, A.ph.pmin);
  pnew = fmn(pnew, A.ph.pmax);
  A.pout[a] = pnew;
  if (!(pnew == pnew)) flag(A.err, ERRB_NONFINITE);
}

// the chemistry network of every interior cell after the thermal update
// (ifchem = 2, :2576-2776): species, nde, ndtot, and rho = sum m n
__global__ void chem_kernel(Grid g, Phys ph, Fields f, double dt, int *err) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  if (t >= (long long)nx * ny * nz) return;
  long long a = gidx_lin(g, t, nx, ny);
  CellSpecies<double> c = cell_species<double>(f, a, [](double v) { return v; });
  const double (&mn)[8] = ph.ndmin;
  chem_network<double>(c, f.U[4][a], ph.kb, dt, mn);
  f.sp[0][a] = c.H; f.sp[1][a] = c.p; f.sp[2][a] = c.H2; f.sp[3][a] = c.He;
  f.sp[4][a] = c.Hep; f.sp[5][a] = c.C; f.sp[6][a] = c.Cp; f.sp[7][a] = c.CO;
  f.nde[a] = c.ne;
  f.ndtot[a] = c.nt;
  double rho = 1.0 * c.p + 1.0 * c.H + 2.0 * c.H2 + 4.0 * c.He + 4.0 * c.Hep;   // mH, mH2, mHe
  f.U[0][a] = rho;
  if (!(rho == rho)) flag(err, ERRB_NONFINITE);
}

// nde and ndtot from the species of cells 1..n+plus: plus = 1 at INITIA
// (:471-474), plus = 0 at the start of every SOURCE (:2460-2463)
__global__ void shield_tau_kernel(Grid g, Phys ph, Fields f, double *tau) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)g.n[0] * g.n[1] * g.n[2]) return;
  shield_tau_cell<double>(g, ph, f, tau, t, [](double v) { return v; }, [](double v) { return v; });
}

// ... and the columns from each x side of every (j, k) line (:2946-2985):
// thread per line, the reference's sequential sums (each cell adds half its
// width before and half after its own value is stored), so the columns are
// bit for bit the oracle's
__global__ void shield_scan_kernel(Grid g, Fields f, const double *tau, double dxh) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int ny = g.n[1];
  if (t >= (long long)ny * g.n[2]) return;
  const int j = 1 + (int)(t % ny), k = 1 + (int)(t / ny);
  const double *src[5] = {f.ndtot, f.sp[2], f.sp[5], f.sp[7], tau};   // ndtot, H2, C, CO, tau
  for (int side = 0; side < 2; side++) {
    double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int s = 1; s <= g.n[0]; s++) {
      const int i = side == 0 ? s : g.n[0] + 1 - s;
      const long long a = gidx(g, i, j, k);
#pragma unroll
      for (int q = 0; q < 5; q++) {
        const double v = src[q][a];
        acc[q] = acc[q] + dxh * v;
        f.col[2 * q + side][a] = acc[q];
        acc[q] = acc[q] + dxh * v;
      }
    }
  }
}

__global__ void chem_totals_kernel(Grid g, Fields f, int plus) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int nx = g.n[0] + plus, ny = g.n[1] + plus, nz = g.n[2] + plus;
  if (t >= (long long)nx * ny * nz) return;
  long long a = gidx_lin(g, t, nx, ny);
  f.nde[a] = f.sp[1][a] + f.sp[4][a] + f.sp[6][a];
  f.ndtot[a] = f.sp[1][a] + f.sp[0][a] + 2.0 * f.sp[2][a] + f.sp[3][a] + f.sp[4][a];
}

// ============================================================ dt
// Couran (:1912-1930) and Stblty (:2784-2822) per cell, then a warp-shuffle
// + block + grid min.  Positive doubles order like their bit patterns, so
// the grid-wide min is an atomicMin on the 64-bit pattern: the result does
// not depend on thread order.
__device__ __forceinline__ unsigned long long dbits(double v) { return (unsigned long long)__double_as_longlong(v); }

__global__ void dt_kernel(Grid g, Phys ph, Fields f, unsigned long long *out /* [0]=tCFL [1]=tLMT */, int *err) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double c_min = ph.tfinal, s_min = ph.tfinal;
  if (t < (long long)g.n[0] * g.n[1] * g.n[2]) {
    cell_dt_limits(g, ph, f, t, c_min, s_min);
    if (!(c_min > 0.0) || !(s_min > 0.0)) flag(err, ERRB_DT);
  }
  // reduce as bit patterns (values are positive)
  unsigned long long cb = dbits(c_min > 0.0 ? c_min : 0.0), sb = dbits(s_min > 0.0 ? s_min : 0.0);
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long c2 = __shfl_xor_sync(0xffffffffu, cb, o);
    unsigned long long s2 = __shfl_xor_sync(0xffffffffu, sb, o);
    cb = c2 < cb ? c2 : cb;
    sb = s2 < sb ? s2 : sb;
  }
  __shared__ unsigned long long wc[32], ws[32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { wc[w] = cb; ws[w] = sb; }
  __syncthreads();
  if (w == 0) {
    int nw = (blockDim.x + 31) >> 5;
    cb = lane < nw ? wc[lane] : ~0ull;
    sb = lane < nw ? ws[lane] : ~0ull;
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long c2 = __shfl_xor_sync(0xffffffffu, cb, o);
      unsigned long long s2 = __shfl_xor_sync(0xffffffffu, sb, o);
      cb = c2 < cb ? c2 : cb;
      sb = s2 < sb ? s2 : sb;
    }
    if (lane == 0) {
      atomicMin(&out[0], cb);
      atomicMin(&out[1], sb);
    }
  }
}

// The chosen form's time step, second kernel: the warps whose FP32 interval
// (dt32_screen_kernel) reaches the smallest upper end of a limit recompute
// their cells with cell_dt_limits -- dt_kernel's FP64 arithmetic -- and
// reduce like dt_kernel.  Every other cell's FP64 limits are surely larger
// than some cell's, so the result is dt_kernel's bit for bit.  lo: [3][nwarps]
// lower ends (c, tau, alpha); words[0..2]: smallest upper ends as float bits,
// words[3]: some cooling time is at its floor, whose FP64 value the host adds.
// A capped grid: each lane of a warp checks one of the screen's warps
// (coalesced, independent loads of the three lower ends), the warp ballots
// the candidates and recomputes their cells together; at 256^3 a thread per
// screened cell, or a warp walking the screen's warps one at a time, spent
// 0.2-0.3 ms on the checks alone.
__global__ void __launch_bounds__(256) dt_refine_kernel(Grid g, Phys ph, Fields f, const float *lo,
                                                        const unsigned *words, int nwarps,
                                                        unsigned long long *out /* [0]=tCFL [1]=tLMT */) {
  const float mc = __uint_as_float(words[0]), mt = __uint_as_float(words[1]), ma = __uint_as_float(words[2]);
  const bool thermal = ph.ifthrm == 2, floored = words[3] != 0;
  const long long ncells = (long long)g.n[0] * g.n[1] * g.n[2];
  const int lane = threadIdx.x & 31;
  const long long nw_grid = ((long long)gridDim.x * blockDim.x) >> 5;
  unsigned long long cb = ~0ull, sb = ~0ull;
  const long long first = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
  for (long long wb = first; wb < nwarps; wb += 32 * nw_grid) {
    const long long w = wb + lane;
    bool cand = false;
    if (w < nwarps) {
      const float l0 = lo[w], l1 = lo[(long long)nwarps + w], l2 = lo[2 * (long long)nwarps + w];
      cand = l0 <= mc || (thermal && (l2 <= ma || (!floored && l1 <= mt)));
    }
    unsigned m = __ballot_sync(0xffffffffu, cand);
    while (m) {                // the same on every lane
      const int b = __ffs(m) - 1;
      m &= m - 1;
      const long long t = 32 * (wb + b) + lane;
      double c_min = ph.tfinal, s_min = ph.tfinal;
      if (t < ncells) cell_dt_limits(g, ph, f, t, c_min, s_min);
      const unsigned long long c1 = dbits(c_min > 0.0 ? c_min : 0.0), s1 = dbits(s_min > 0.0 ? s_min : 0.0);
      cb = c1 < cb ? c1 : cb;
      sb = s1 < sb ? s1 : sb;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long c2 = __shfl_xor_sync(0xffffffffu, cb, o);
    unsigned long long s2 = __shfl_xor_sync(0xffffffffu, sb, o);
    cb = c2 < cb ? c2 : cb;
    sb = s2 < sb ? s2 : sb;
  }
  if (lane == 0 && cb != ~0ull) {
    atomicMin(&out[0], cb);
    atomicMin(&out[1], sb);
  }
}

// ============================================================ DISSIP
// (:3143-3173) divv on the two x-edge slabs (i = 0..11 from each edge)
__global__ void divv_kernel(Grid g, Fields f, double *divv) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int ny2 = g.n[1] + 2, nz2 = g.n[2] + 2;
  if (t >= 2LL * 12 * ny2 * nz2) return;
  int i = (int)(t % 12);
  int j = (int)((t / 12) % ny2);
  int k = (int)((t / (12LL * ny2)) % nz2);
  int e = (int)(t / (12LL * ny2 * nz2));
  int ix = i + (e == 0 ? 0 : g.n[0] - 10);
  long long a = gidx(g, ix, j, k);
  long long sy = g.st[1], sz = g.st[2];
  divv[t] = (f.U[1][a + 1] - f.U[1][a - 1] + f.U[2][a + sy] - f.U[2][a - sy] + f.U[3][a + sz] - f.U[3][a - sz]) * 0.25;
}
__global__ void dissip_kernel(Grid g, Fields f, const double *divv, int e) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int ny = g.n[1], nz = g.n[2];
  if (t >= 10LL * ny * nz) return;
  int i = 1 + (int)(t % 10);
  int j = 1 + (int)((t / 10) % ny);
  int k = 1 + (int)(t / (10LL * ny));
  int ny2 = ny + 2, nz2 = nz + 2;
  auto dv = [&](int ii, int jj, int kk) {
    return divv[(long long)ii + 12LL * ((long long)jj + (long long)ny2 * ((long long)kk + (long long)nz2 * e))];
  };
  long long a = gidx(g, i + (e == 0 ? 0 : g.n[0] - 10), j, k);
  f.U[1][a] = f.U[1][a] + 0.1 * (dv(i + 1, j, k) - dv(i - 1, j, k));
  f.U[2][a] = f.U[2][a] + 0.1 * (dv(i, j + 1, k) - dv(i, j - 1, k));
  f.U[3][a] = f.U[3][a] + 0.1 * (dv(i, j, k + 1) - dv(i, j, k - 1));
}

// ============================================================ diagnostics
// per-block partial sums (mass, momentum, total energy with face-averaged
// B) and max |div B|; the host adds the block partials in a fixed order.
__global__ void diag_kernel(Grid g, Phys ph, Fields f, double *part /* 6 per block */) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  double v[6] = {0, 0, 0, 0, 0, 0};
  if (t < (long long)nx * ny * nz) {
    int i, j, k;
    split3(t, nx, ny, i, j, k);
    i += 1; j += 1; k += 1;
    long long a = gidx(g, i, j, k);
    double dV = g.dx[0][i + 1] * g.dx[1][j + 1] * g.dx[2][k + 1];
    double rho = f.U[0][a];
    double H = f.sp[0][a], pr = f.sp[1][a], H2 = f.sp[2][a], He = f.sp[3][a], Hep = f.sp[4][a];
    double g1c = gmi1_of(H, pr, He, Hep, H2);
    double vx = f.U[1][a], vy = f.U[2][a], vz = f.U[3][a];
    double bx = f.bcc[0][a], by = f.bcc[1][a], bz = f.bcc[2][a];
    v[0] = rho * dV;
    v[1] = rho * vx * dV;
    v[2] = rho * vy * dV;
    v[3] = rho * vz * dV;
    v[4] = (f.U[4][a] / g1c + 0.5 * rho * (vx * vx + vy * vy + vz * vz) + 0.5 * (bx * bx + by * by + bz * bz)) * dV;
    double div = (f.U[5][a + 1] - f.U[5][a]) / g.dx[0][i + 1] + (f.U[6][a + g.st[1]] - f.U[6][a]) / g.dx[1][j + 1] +
                 (f.U[7][a + g.st[2]] - f.U[7][a]) / g.dx[2][k + 1];
    v[5] = fabs(div);
  }
  __shared__ double red[6][256];
  for (int q = 0; q < 6; q++) red[q][threadIdx.x] = v[q];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int q = 0; q < 6; q++) {
        if (q < 5) red[q][threadIdx.x] += red[q][threadIdx.x + s];
        else red[q][threadIdx.x] = fmx(red[q][threadIdx.x], red[q][threadIdx.x + s]);
      }
    __syncthreads();
  }
  if (threadIdx.x < 6) part[blockIdx.x * 6 + threadIdx.x] = red[threadIdx.x][0];
}

#endif  // MHD_COMMON_KERNELS

}  // namespace mhd
