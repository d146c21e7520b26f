// mhd_sweep32.cuh — the chosen-form sweep: the same Lagrange + MOC + remap
// scheme as sweep_kernel (MCF3DSGincfca3.f90:1264-2098) with every
// reconstruction, limiter, Riemann and characteristic solve and division in
// FP32, and FP64 used only where the resident FP64 state is updated:
//
//   rho_new = rho + rdx * ((double)F_i - (double)F_{i-1})     FP64 flux difference
//   v_new   = v   + (double)dv,  dv = (dM - drho v) / rho_new  (dM, drho in FP32)
//   n_new   = n   + (double)dn                                 species
//   p_new   = (double)p(E, rho_new, v_new, B)                  FP32 energy
//
// dM is the reference's Lagrangian pressure and MOC Lorentz increments plus
// the remap flux difference, i.e. M_new dx = (rho v dx + dM dx): the update
// of the momentum content multiplied through by the cell width, written as
// an increment so its FP32 rounding scales with the change, not the state.
// The mass update differences the FP32 fluxes in FP64, so the total mass of
// a periodic grid is conserved to FP64 round-off.  The energy follows the
// reference's own structure — E is rebuilt from the pressure every sweep
// and turned back into a pressure at the end — and runs in FP32.
//
// On GB300 the FP64 pipe runs at ~1/64 of the FP32 rate and also executes
// the hardware double<->float conversions, so this kernel converts with
// integer instructions (mhd_conv.cuh) and keeps 13 FP64 operations per cell
// (the additions above).  All pencil buffers are FP32: 22 of them, L*P floats
// each (L = n+4), plus FP32 copies of the coordinate widths.  Ghost entries
// of a buffer are written by the thread that computes their source cell
// (periodic wrap or free copy), so the in-pencil halo exchanges cost no
// extra barrier: the sweep has 10 barriers, one after each of its 11
// phases but the last (the eight species share one reconstruction, one
// flux and one finishing phase).
//
// VLIMIT's T switch keeps the reference's meaning at every stage: p for
// RHS, e inside and p in the ghosts for MOC, E for the remap.
#pragma once

#include <cuda.h>

#include "mhd_conv.cuh"
#include "mhd_kernels.cuh"
#include "mhd_tc.cuh"

namespace mhd {

// Pencil buffers and their successive contents.  The first ten are unused
// until the Lagrangian step, so the TMA load phase stages the FP64 inputs
// there (two buffers per FP64 field).
enum {
  F_DXL = 0, // Lagrangian width
  F_VA,      // Va at interface i+1/2
  F_PA,      // Pa -> Bay -> flux E -> species flux 4
  F_GAM,     // gamma -> Vay -> flux B1 -> species flux 5
  F_G0,      // slope; then IM1 -> species q 0
  F_G1,      // slope; then IM2 -> species q 1
  F_G2,      // slope; then flux rho -> species flux 0
  F_G3,      // slope; then flux mn -> species flux 1
  F_G4,      // slope; then flux m1 -> species flux 2
  F_IMN,     // momentum increment along the sweep -> species q 2
  F_R,       // rho -> rho_lag (= q_rho)
  F_VN,      // v_n -> q_mn -> species q 4
  F_VT1,     // v_t1 -> q_m1 -> species q 5
  F_VT2,     // v_t2 -> q_m2 -> species q 6
  F_P,       // p -> Bnap (MOC) -> flux m2 -> species flux 3
  F_B1,      // Bcc_t1 -> Blg1 -> q_B1 -> species q 7
  F_B2,      // Bcc_t2 -> Blg2 -> q_B2 -> species flux 7
  F_BN,      // face-normal B -> cell-centred normal B (from the MOC update on)
  F_S,       // sum H+p+He+He+ -> Baz -> flux B2 -> species flux 6
  F_H2,      // H2 -> Vaz -> species q 3
  F_T,       // T-switch variable (p ghosts, e inside) -> q_E -> E_new - ekin - emag
  F_SW,      // cell-centred normal B -> remap T switch (+-0.5) of cells 0..n+1
  F_COUNT
};
enum { C_DX = 0, C_RDX, C_X2, C_COUNT };
// FP64 staging slots of the TMA load phase: buffers 0..9, free until the
// Lagrangian step, two per slot; the 14 inputs come in three rounds.  (Two
// rounds of seven, with two more slots after the coordinate rows, measured
// slower at 256^3: y 2.28 against 1.99 ms, z 2.51 against 2.36; the larger
// shared-memory carve-out leaves less L1 for the finishing phases' loads.)
constexpr int kStageSlots = 5;
// inflow rules of this kernel's derived buffers (beside the IN_* of the
// shared header): the species sum H+p+He+He+ and the remap's T switch
enum : int { IN_SSUM = 100, IN_SW = 101 };   // FP32 dx(i), 1/(x(i)-x(i-1)), x(i+1)-x(i-1)

// Shared memory of one CTA: the buffers hold LS >= n+4 positions each (LS =
// n+4 when the stride is a run-time value).
__host__ __device__ inline size_t sweep32_smem_bytes(int n, int P, int LS = 0) {
  size_t L = LS > 0 ? (size_t)LS : (size_t)n + 4;
  return (L * P * F_COUNT + L * C_COUNT) * sizeof(float);
}

__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }


// Work loop of a phase: items t = threadIdx.x + k*NT < cnt.  Groups of UNR
// items that are all in range run as one unrolled block, so the loads of
// the group can be in flight together; the rest run one by one.
template <int NT, int UNR, class F>
__device__ __forceinline__ void unrolled(int cnt, F &&f) {
  int t0 = threadIdx.x;
  for (; t0 + (UNR - 1) * NT < cnt; t0 += UNR * NT) {
#pragma unroll
    for (int k = 0; k < UNR; k++) f(t0 + k * NT);
  }
  for (int t = t0; t < cnt; t += NT) f(t);
}

// Unroll depth of the phases that only touch shared memory.  Their loads
// have short latency and deeper unrolling raises register pressure: with
// depth 2 or 4 the 256^3 sweeps run 15-40 % slower on GB300 than with 1.
#ifndef MHD_SWEEP_SMEM_UNROLL
#define MHD_SWEEP_SMEM_UNROLL 1
#endif
constexpr int kSmemUnroll = MHD_SWEEP_SMEM_UNROLL;
// Unroll depth of the phases that load from global memory.  With 384 or
// more threads, a phase over 4 pencils of 256 cells (1024 items) never
// fills a group of 4 trips, yet the group's code sets the kernel's
// register count: depth 4 needs 96 registers, depth 1 fits in 56 at 576
// threads without spills and depth 2 measured no faster.
#ifndef MHD_SWEEP_GLOBAL_UNROLL
#define MHD_SWEEP_GLOBAL_UNROLL 1
#endif
constexpr int kGlobalUnroll = MHD_SWEEP_GLOBAL_UNROLL;
// Bit d set: the load phase of the direction-d sweep issues all loads of a
// position in one pass, in kernels with at least 64 registers a thread
// (NT * MINB <= 1024; the one pass holds 14 FP64 values) and a compile-time
// buffer stride; clear, or otherwise: one pass per field group.  The z sweep with 768 threads and
// one CTA per SM: 2.21 -> 2.17 ms at 256^3 with the one pass; the 512^3 y
// sweep (768 threads, one CTA per SM) 19.46 -> 19.29 ms.
#ifndef MHD_SWEEP_MERGE_LOADS
#define MHD_SWEEP_MERGE_LOADS 7
#endif
constexpr int kMergeLoads = MHD_SWEEP_MERGE_LOADS;
// Bit d set: the finishing phases of the direction-d sweep load every FP64
// value of a position before using any; clear: each value where it is used.
// Measured at 256^3 (ms, x / y / z): hoisted 2.16 / 2.41 / 2.61, in place
// 2.23 / 2.47 / 2.68 (the z sweep with eight columns per CTA; with four and
// two CTAs per SM it was the other way round, 3.21 hoisted against 3.01);
// with the current shapes x / y hoisted 1.65 / 1.94, in place 1.70 / 2.14.
// (Merging the load pass did not help the z sweep of 1024 threads and 64
// registers: 2.69.)
#ifndef MHD_SWEEP_HOIST_LOADS
#define MHD_SWEEP_HOIST_LOADS 7
#endif
constexpr int kHoistLoads = MHD_SWEEP_HOIST_LOADS;
// Bit d set: the field-finish phase of the direction-d sweep also loads its
// eight species with rho and v (with the register and stride conditions of
// kMergeLoads); clear: in one batch after the field finish
// (the x sweep runs at 64 registers, where twelve FP64 values held at once
// spill; the z sweep and the 512^3 y sweep, one 768-thread CTA per SM, have
// the room).
#ifndef MHD_SWEEP_HOIST_SPECIES
#define MHD_SWEEP_HOIST_SPECIES 6
#endif
constexpr int kHoistSpecies = MHD_SWEEP_HOIST_SPECIES;

// The P pencils of a CTA, addressed without a per-pencil table: pencil p
// starts p transverse strides after pencil 0 (adjacent y rows for the x
// sweep, adjacent x columns for the y and z sweeps).  For the y and z
// sweeps a group starts at padded x index P*blockIdx.x, so the P words a
// row of the group reads fill whole 32-byte sectors for P = 4 or 8 (the
// padded row length n+4 is a multiple of 4 for n divisible by 4); the group may then contain
// ghost columns (x < 1 or x > n), which are computed along but never
// stored.  Columns beyond the padded grid read the last column.
template <int DIR, int P>
struct PencilRun {
  int b0, sp, sd;   // 32-bit cell offsets: the padded grid has fewer than 2^31 cells
  unsigned act;   // bit p: pencil p is an interior pencil
  int plast;      // last pencil inside the padded grid
  // by: the CTA's transverse block index (blockIdx.y plus the launch's offset)
  __device__ PencilRun(const Grid &g, int by) {
    sd = (int)g.st[DIR];
    act = (1u << P) - 1;
    plast = P - 1;
    if (DIR == 0) {
      b0 = (int)gidx(g, -1, blockIdx.x * P + 1, by + 1);
      sp = (int)g.st[1];
    } else {
      const int x0 = (int)blockIdx.x * P - 1;
      b0 = (int)((DIR == 1) ? gidx(g, x0, -1, by + 1) : gidx(g, x0, by + 1, -1));
      sp = 1;
      act = 0;
      for (int p = 0; p < P; p++)
        if (x0 + p >= 1 && x0 + p <= g.n[0]) act |= 1u << p;
      plast = min(P - 1, g.n[0] + 2 - x0);
    }
  }
  __device__ __forceinline__ bool active(int p) const { return (act >> p) & 1u; }
  // global offset of sweep position i (-1..n+2) on pencil p
  __device__ __forceinline__ int at(int p, int i) const {
    return b0 + min(p, plast) * sp + (i + 1) * sd;
  }
};

// The TMA load phase of the sweeps.  The handle's FP64 arrays are one
// allocation of equal-sized arrays, seen by the tensor map as a 4-D tensor
// (x, y, z, array); a box is kStageRows positions along the sweep of P
// pencils of one array (x sweep {R, P, 1, 1}, y sweep {P, R, 1, 1}, z sweep
// {P, 1, R, 1}).  fld holds the array index of each input,
// in the order of the stage rounds (SF_*).
constexpr int kStageRows = 132;   // positions per box: two boxes cover a 256-cell pencil and its ghosts
enum {
  SF_BT1 = 0, SF_BT2, SF_RHO, SF_VN,  SF_VT1,   // round 0: transverse field, rho, v_n, v_t1
  SF_VT2, SF_P, SF_S0, SF_S1, SF_S2,            // round 1: v_t2, p, species 0-2
  SF_S3, SF_S4, SF_BN, SF_BNC,                  // round 2: species 3-4, face and cell-centred normal field
  SF_COUNT
};
struct SweepTma {
  CUtensorMap map;
  int fld[SF_COUNT];
  int nbox;   // boxes per pencil group: ceil((n+4) / kStageRows)
};

// LS > 0: every pencil buffer is LS positions long, a compile-time stride,
// so each shared-memory access is one load or store at a constant offset
// from a per-item base address; LS = 0: the stride is n+4, computed at run
// time (any length).  TM: the sweep stages its FP64 inputs with TMA box
// loads (LS = 2 kStageRows, the staged positions of a pencil group).
template <int DIR, int P, int NT, int MINB, int LS, bool TM = false>
__global__ void __launch_bounds__(NT, MINB) sweep32_kernel(SweepArgs A, const __grid_constant__ SweepTma T) {
  static_assert(!TM || (LS == 2 * kStageRows && P % 2 == 0), "TMA staging: staged stride, 16-byte rows");
  extern __shared__ __align__(128) float smf[];
  // the x and y sweeps convert with the branching form (mhd_conv.cuh)
  constexpr bool kBranchConv = DIR != 2;
  auto d2f = [](double v) { return d2f_t<kBranchConv>(v); };
  auto f2d = [](float v) { return f2d_t<kBranchConv>(v); };
  const Grid &g = A.g;
  const int N = g.n[DIR];
  const int L = N + 4;
  const int LB = LS > 0 ? LS : L;   // buffer stride
  const int LP = LB * P;
  float *cf = smf + (size_t)F_COUNT * LP;
  const float dt = (float)A.dt;
  const float facdep = (float)A.ph.facdep;
  const float kb = (float)A.ph.kb;
  const int tid = threadIdx.x;
  const double *rdx = g.rdx[DIR];
  const int by = (int)blockIdx.y + A.by0;   // transverse block index (a launch may cover a slab)
  PencilRun<DIR, P> pc(g, by);
  constexpr int C1 = (DIR + 1) % 3, C2 = (DIR + 2) % 3;
  auto Fb = [&](int b, int i, int p) -> float & { return smf[b * LP + (i + 1) * P + p]; };
  auto cx = [&](int c, int i) -> float { return cf[c * LB + i + 1]; };
  const bool perL = g.bcl[DIR] != 1, perR = g.bcr[DIR] != 1;
  // BC=4 inflow sides of the x sweep (the other sweeps never exchange in x)
  const bool inL = DIR == 0 && A.ph.in.on[0], inR = DIR == 0 && A.ph.in.on[1];
  // ghost positions whose value is a copy of interior cell i
  auto for_ghosts = [&](int i, auto &&fn) {
    if (!inL && (perL ? i == N - 1 : i == 1)) fn(-1);
    if (!inL && (perL ? i == N : i == 1)) fn(0);
    if (!inR && (perR ? i == 1 : i == N)) fn(N + 1);
    if (!inR && (perR ? i == 2 : i == N)) fn(N + 2);
  };
  // value of an inflow ghost cell gi of pencil p under rule r (DIR == 0:
  // pencil p is row (blockIdx.x*P+p+1, by+1)); two rules of this
  // kernel's derived buffers: the species sum of gamma and the remap switch
  auto inflow32 = [&](int r, int side, int gi, int p) -> float {
    const int j = blockIdx.x * P + p + 1, k = by + 1;
    if (r == IN_SSUM) {
      const double rho = inflow_rho(g, A.ph.in, side, gi, j, k);
      const double *cm = A.ph.in.cm;
      return d2f(cm[0] * rho) + d2f(cm[1] * rho) + d2f(cm[3] * rho) + d2f(cm[4] * rho);
    }
    const double bccx = (r == IN_E || r == IN_SW) ? __ldg(A.f.bcc[0] + pc.at(p, gi)) : 0.0;
    if (r == IN_SW) {
      const float e = d2f(inflow_value(g, A.ph.in, IN_E, side, gi, j, k, bccx, 0.0, 0.0));
      const float rho = d2f(inflow_rho(g, A.ph.in, side, gi, j, k));
      return (1.27f * e >= 3.0f * kb * rho) ? 0.5f : -0.5f;
    }
    return d2f(inflow_value(g, A.ph.in, r, side, gi, j, k, bccx, 0.0, 0.0));
  };
  // the ghosts cell i feeds (copies); on an inflow side only the face copy
  // of face 1 is fed here, the other rules by inflow_fill
  auto put_ghosts = [&](int b, int i, int p, float v, int rule) {
    for_ghosts(i, [&](int gi) { Fb(b, gi, p) = v; });
    if (rule == IN_BXF && inL && i == 1) {
      Fb(b, -1, p) = v;
      Fb(b, 0, p) = v;
    }
  };
  // Only cells 1, 2, n-1 and n feed ghosts.  A phase stores its interior
  // values first and copies them into the ghosts in one block for those
  // cells (copy_ghosts: the ghosts of buffer b take its entry i), so the
  // other items skip the ghost tests with one branch.
  auto edge = [&](int i) { return i <= 2 || i >= N - 1; };
  auto copy_ghosts = [&](int b, int i, int p) {
    const float v = Fb(b, i, p);
    for_ghosts(i, [&](int gi) { Fb(b, gi, p) = v; });
  };
  // the inflow ghosts of listed buffers (values that depend on no interior
  // cell); run by the phase that writes those buffers, before its barrier
  auto inflow_fill = [&](const int *bl, const int *rl, int nb) {
    for (int t = tid; t < 4 * P * nb; t += NT) {
      const int bq = t / (4 * P), r = t % (4 * P), q = r / P, p = r % P;
      const int gi = (q < 2) ? (q - 1) : (N + q - 1);
      const int side = gi <= 0 ? 0 : 1;
      if (side == 0 ? inL : inR) Fb(bl[bq], gi, p) = inflow32(rl[bq], side, gi, p);
    }
  };
  auto vlw = [&](int b, int i, int p, const LimW &w) {
    return vlim_w(Fb(b, i - 1, p), Fb(b, i, p), Fb(b, i + 1, p), w);
  };
  auto tsw = [&](float e5, float rho) { return (1.27f * e5 >= 3.0f * kb * rho) ? 0.5f : -0.5f; };
  // Upwind MUSCL fluxes through interface i: the upwind cell c, its
  // Lagrangian widths and switch are read once per interface (upwind) and
  // shared by the fields (flux), whose values a phase stores only after all
  // are formed, so no store separates the shared loads from their uses.
  struct Upwind {
    int c;
    bool left;   // vadt <= 0: the upwind cell is i+1
    float vadt, dm, d0, dp, s, w;
    LimW lw;   // the limiter's width divisors of cell c
  };
  auto upwind = [&](int i, int p, float vadt) {
    Upwind u;
    u.vadt = vadt;
    u.left = vadt <= 0.0f;
    u.c = u.left ? i + 1 : i;
    u.dm = Fb(F_DXL, u.c - 1, p);
    u.d0 = Fb(F_DXL, u.c, p);
    u.dp = Fb(F_DXL, u.c + 1, p);
    u.s = Fb(F_SW, u.c, p);
    u.w = u.left ? (0.5f * (u.d0 + vadt) * facdep) : (0.5f * (u.d0 - vadt) * facdep);
    u.lw = lim_w(u.dm, u.d0, u.dp, u.s);
    return u;
  };
  auto flux = [&](int qb, const Upwind &u, int p) {
    const float gs = vlw(qb, u.c, p, u.lw);
    const float q = Fb(qb, u.c, p);
    return u.left ? -u.vadt * (q - u.w * gs) : -u.vadt * (q + u.w * gs);
  };

  // ------------------------------------------------ A: load (+ ghosts)
  for (int t = tid; t < L; t += NT) {
    const double *xe = g.x[DIR];
    cf[C_DX * LB + t] = d2f(g.dx[DIR][t]);
    cf[C_RDX * LB + t] = d2f(rdx[t]);
    cf[C_X2 * LB + t] = (t >= 1 && t + 1 < L) ? d2f(xe[t + 1] - xe[t - 1]) : 1.0f;
  }
  // the interior state of position i: flow variables ...
  auto load_flow = [&](int i, int p, double u0, double un, double u1, double u2, double u4) {
    Fb(F_R, i, p) = d2f(u0);
    Fb(F_VN, i, p) = d2f(un);
    Fb(F_VT1, i, p) = d2f(u1);
    Fb(F_VT2, i, p) = d2f(u2);
    Fb(F_P, i, p) = d2f(u4);
  };
  // ... species sums, the face-normal field and the cell-centred normal
  // field (held in F_SW until the MOC update moves it to F_BN, for the
  // Lagrangian step and the pressure at the end) ...
  auto load_species_face = [&](int i, int p, double s0, double s1, double s2, double s3, double s4, double bn,
                               double bnc) {
    Fb(F_S, i, p) = d2f(s0) + d2f(s1) + d2f(s3) + d2f(s4);
    Fb(F_H2, i, p) = d2f(s2);
    Fb(F_BN, i, p) = d2f(bn);
    Fb(F_SW, i, p) = d2f(bnc);
  };
  // ... and the ghosts they feed (the face-field exchange rewrites the ghost
  // faces, incl. face n+1; an inflow side copies face 1 into faces -1, 0
  // and face n+1 into n+2)
  auto load_ghosts = [&](int i, int p, double bn) {
    copy_ghosts(F_R, i, p);
    copy_ghosts(F_VN, i, p);
    copy_ghosts(F_VT1, i, p);
    copy_ghosts(F_VT2, i, p);
    copy_ghosts(F_P, i, p);
    const float pr = Fb(F_P, i, p);
    for_ghosts(i, [&](int gi) { Fb(F_T, gi, p) = pr; });
    copy_ghosts(F_S, i, p);
    copy_ghosts(F_H2, i, p);
    put_ghosts(F_BN, i, p, Fb(F_BN, i, p), IN_BXF);
    if (pc.active(p)) for_ghosts(i, [&](int gi) { A.f.U[5 + DIR][pc.at(p, gi)] = bn; });
    if (inL && i == 1)
      for (int gi = -1; gi <= 0; gi++) A.f.U[5 + DIR][pc.at(p, gi)] = bn;
    if (inR && i == N) {
      const double bn1 = __ldg(A.f.U[5 + DIR] + pc.at(p, N + 1));
      Fb(F_BN, N + 1, p) = d2f(bn1);
      Fb(F_BN, N + 2, p) = d2f(bn1);
      A.f.U[5 + DIR][pc.at(p, N + 2)] = bn1;
    }
  };
  // The transverse cell-centred field is needed at positions -1..n+2.  In
  // the merged pass the threads of cells 1 and n also load the two
  // positions beyond them, so the pass has n*P items (no extra trip for the
  // four ghost positions: x sweep at 256^3 1.87 -> 1.83 ms); the y and z
  // sweeps keep a separate pass over all n+4 positions (2.34 / 2.42 ms
  // folded against 2.32 / 2.42).
  auto load_transverse = [&](int i, int p, int a) {
    const double c1 = __ldg(A.f.bcc[C1] + a), c2 = __ldg(A.f.bcc[C2] + a);
    double l1a = 0.0, l1b = 0.0, l2a = 0.0, l2b = 0.0, r1a = 0.0, r1b = 0.0, r2a = 0.0, r2b = 0.0;
    if (i == 1) {
      const int g0 = pc.at(p, -1), g1 = pc.at(p, 0);
      l1a = __ldg(A.f.bcc[C1] + g0); l1b = __ldg(A.f.bcc[C1] + g1);
      l2a = __ldg(A.f.bcc[C2] + g0); l2b = __ldg(A.f.bcc[C2] + g1);
    }
    if (i == N) {
      const int g0 = pc.at(p, N + 1), g1 = pc.at(p, N + 2);
      r1a = __ldg(A.f.bcc[C1] + g0); r1b = __ldg(A.f.bcc[C1] + g1);
      r2a = __ldg(A.f.bcc[C2] + g0); r2b = __ldg(A.f.bcc[C2] + g1);
    }
    Fb(F_B1, i, p) = d2f(c1);
    Fb(F_B2, i, p) = d2f(c2);
    if (i == 1) {
      Fb(F_B1, -1, p) = d2f(l1a); Fb(F_B1, 0, p) = d2f(l1b);
      Fb(F_B2, -1, p) = d2f(l2a); Fb(F_B2, 0, p) = d2f(l2b);
    }
    if (i == N) {
      Fb(F_B1, N + 1, p) = d2f(r1a); Fb(F_B1, N + 2, p) = d2f(r1b);
      Fb(F_B2, N + 1, p) = d2f(r2a); Fb(F_B2, N + 2, p) = d2f(r2b);
    }
  };
  if constexpr (TM) {
    // TMA staging: three rounds of at most five FP64 arrays, each staged in
    // one slot (two free buffers), waited for on an mbarrier and converted
    // into the FP32 buffers; the next round's boxes are issued once every
    // thread has read the slots (barrier).  The values are the ones the
    // load passes below read, so the sweep's results are the same.
    __shared__ __align__(8) uint64_t tbar;
    const uint32_t sbase = tc::smem_u32(smf);
    const int slot_doubles = LB * P;   // one slot: LB positions x P pencils of FP64
    const double *stg = reinterpret_cast<const double *>(smf);
    // staged layout: y and z sweeps [position][pencil] (the box's columns
    // are the pencils); x sweep [box][pencil][position in the box] (the
    // box's rows are the pencils)
    auto st = [&](int slot, int i, int p) -> double {
      if constexpr (DIR == 0) {
        const int r = i + 1, b = r / kStageRows;
        return stg[slot * slot_doubles + (b * P + p) * kStageRows + (r - b * kStageRows)];
      } else {
        return stg[slot * slot_doubles + (i + 1) * P + p];
      }
    };
    if (tid == 0) {
      tc::mbar_init(&tbar, 1);
      tc::fence_mbar_init();
    }
    __syncthreads();
    // y and z sweeps: padded x of the group's first column; x sweep: padded
    // y of its first row
    const int cx0 = DIR == 0 ? P * (int)blockIdx.x + 2 : P * (int)blockIdx.x;
    const int ct = by + 2;                 // padded index of the other transverse coordinate
    bool ok = (sbase & 127u) == 0;         // TMA writes 128-byte aligned boxes
    if (!ok && tid == 0) flag(A.err, ERRB_TMA);
    auto round = [&](int r, int f0, int nf) {
      if (tid == 0 && ok) {
        tc::fence_async_smem();   // the slots' reads of the last round before the boxes overwrite them
        tc::mbar_arrive_expect_tx(&tbar, (uint32_t)(nf * T.nbox * kStageRows * P * 8));
        for (int q = 0; q < nf; q++)
          for (int b = 0; b < T.nbox; b++) {
            const uint32_t dst = sbase + (uint32_t)((q * slot_doubles + b * kStageRows * P) * 8);
            if (DIR == 0) tc::tma_load_4d(dst, &T.map, b * kStageRows, cx0, ct, T.fld[f0 + q], &tbar);
            else if (DIR == 1) tc::tma_load_4d(dst, &T.map, cx0, b * kStageRows, ct, T.fld[f0 + q], &tbar);
            else tc::tma_load_4d(dst, &T.map, cx0, ct, b * kStageRows, T.fld[f0 + q], &tbar);
          }
      }
      if (ok && !tc::mbar_wait(&tbar, (uint32_t)(r & 1))) {
        // a bounded second wait for the copies still in flight, then the
        // error bit; the state this launch writes is then not used (the
        // host reports the error)
        tc::mbar_wait(&tbar, (uint32_t)(r & 1));
        flag(A.err, ERRB_TMA);
        ok = false;
      }
    };
    static_assert(SF_VT2 == kStageSlots && SF_S3 == 2 * kStageSlots && SF_COUNT <= 3 * kStageSlots,
                  "three rounds of at most kStageSlots staged arrays");
    // round 0: transverse field at every position; rho, v_n, v_t1 inside
    round(0, SF_BT1, 5);
    for (int t = tid; t < L * P; t += NT) {
      const int i = t / P - 1, p = t % P;
      Fb(F_B1, i, p) = d2f(st(0, i, p));
      Fb(F_B2, i, p) = d2f(st(1, i, p));
    }
    for (int t = tid; t < N * P; t += NT) {
      const int i = 1 + t / P, p = t % P;
      Fb(F_R, i, p) = d2f(st(2, i, p));
      Fb(F_VN, i, p) = d2f(st(3, i, p));
      Fb(F_VT1, i, p) = d2f(st(4, i, p));
    }
    __syncthreads();
    // round 1: v_t2, p, species 0-2 (the sum H+p+He+He+ in the order of
    // load_species_face: ((s0 + s1) + s3) + s4)
    round(1, SF_VT2, 5);
    for (int t = tid; t < N * P; t += NT) {
      const int i = 1 + t / P, p = t % P;
      Fb(F_VT2, i, p) = d2f(st(0, i, p));
      Fb(F_P, i, p) = d2f(st(1, i, p));
      Fb(F_S, i, p) = d2f(st(2, i, p)) + d2f(st(3, i, p));
      Fb(F_H2, i, p) = d2f(st(4, i, p));
    }
    __syncthreads();
    // round 2: species 3-4 and the normal field; then the ghosts of every
    // buffer fed by cells 1, 2, n-1, n
    round(2, SF_S3, 4);
    for (int t = tid; t < N * P; t += NT) {
      const int i = 1 + t / P, p = t % P;
      Fb(F_S, i, p) = Fb(F_S, i, p) + d2f(st(0, i, p)) + d2f(st(1, i, p));
      const double bn = st(2, i, p);
      Fb(F_BN, i, p) = d2f(bn);
      Fb(F_SW, i, p) = d2f(st(3, i, p));
      if (edge(i)) load_ghosts(i, p, bn);
    }
  } else if constexpr (((kMergeLoads >> DIR) & 1) != 0 && NT * MINB <= 1024 && LS > 0) {
    // one pass over the interior cells: the transverse field and the state,
    // all loads of a position issued together so that a thread waits for
    // memory once per position rather than once per field group
    unrolled<NT, kGlobalUnroll>(N * P, [&](int t) {
      const int i = 1 + t / P, p = t % P;
      const int a = pc.at(p, i);
      const double u0 = __ldg(A.f.U[0] + a), un = __ldg(A.f.U[1 + DIR] + a), u1 = __ldg(A.f.U[1 + C1] + a),
                   u2 = __ldg(A.f.U[1 + C2] + a), u4 = __ldg(A.f.U[4] + a);
      const double s0 = __ldg(A.f.sp[0] + a), s1 = __ldg(A.f.sp[1] + a), s2 = __ldg(A.f.sp[2] + a),
                   s3 = __ldg(A.f.sp[3] + a), s4 = __ldg(A.f.sp[4] + a), bn = __ldg(A.f.U[5 + DIR] + a),
                   bnc = __ldg(A.f.bcc[DIR] + a);
      load_transverse(i, p, a);
      load_flow(i, p, u0, un, u1, u2, u4);
      load_species_face(i, p, s0, s1, s2, s3, s4, bn, bnc);
      if (edge(i)) load_ghosts(i, p, bn);
    });
  } else {
    // three passes: transverse field (-1..n+2), flow state, species + face field
    unrolled<NT, kGlobalUnroll>(L * P, [&](int t) {
      const int i = t / P - 1, p = t % P;
      const int a = pc.at(p, i);
      Fb(F_B1, i, p) = d2f(__ldg(A.f.bcc[C1] + a));
      Fb(F_B2, i, p) = d2f(__ldg(A.f.bcc[C2] + a));
    });
    unrolled<NT, kGlobalUnroll>(N * P, [&](int t) {
      const int i = 1 + t / P, p = t % P;
      const int a = pc.at(p, i);
      const double u0 = __ldg(A.f.U[0] + a), un = __ldg(A.f.U[1 + DIR] + a), u1 = __ldg(A.f.U[1 + C1] + a),
                   u2 = __ldg(A.f.U[1 + C2] + a), u4 = __ldg(A.f.U[4] + a);
      load_flow(i, p, u0, un, u1, u2, u4);
    });
    unrolled<NT, kGlobalUnroll>(N * P, [&](int t) {
      const int i = 1 + t / P, p = t % P;
      const int a = pc.at(p, i);
      const double s0 = __ldg(A.f.sp[0] + a), s1 = __ldg(A.f.sp[1] + a), s2 = __ldg(A.f.sp[2] + a),
                   s3 = __ldg(A.f.sp[3] + a), s4 = __ldg(A.f.sp[4] + a), bn = __ldg(A.f.U[5 + DIR] + a),
                   bnc = __ldg(A.f.bcc[DIR] + a);
      load_species_face(i, p, s0, s1, s2, s3, s4, bn, bnc);
      if (edge(i)) load_ghosts(i, p, bn);
    });
  }
  if (inL || inR) {
    const int bl[8] = {F_R, F_VN, F_VT1, F_VT2, F_P, F_T, F_S, F_H2};
    const int rl[8] = {IN_RHO, IN_V1, IN_V2, IN_V3, IN_P, IN_P, IN_SSUM, IN_SPEC + 2};
    inflow_fill(bl, rl, 8);
  }
  __syncthreads();
  // ------------------------------------------------ B: gamma, RHS slopes
  unrolled<NT, kSmemUnroll>((N + 2) * P, [&](int t) {
    int i = t / P, p = t % P;
    float S = Fb(F_S, i, p), H2 = Fb(F_H2, i, p);
    Fb(F_GAM, i, p) = fdiv(5.0f * S + 7.0f * H2, 3.0f * S + 5.0f * H2);
    float dm = cx(C_DX, i - 1), d0 = cx(C_DX, i), dp = cx(C_DX, i + 1);
    float s = tsw(Fb(F_P, i, p), Fb(F_R, i, p));
    const LimW w = lim_w(dm, d0, dp, s);
    Fb(F_G0, i, p) = vlw(F_R, i, p, w);
    Fb(F_G1, i, p) = vlw(F_VN, i, p, w);
    Fb(F_G2, i, p) = vlw(F_P, i, p, w);
    Fb(F_G3, i, p) = vlw(F_B1, i, p, w);
    Fb(F_G4, i, p) = vlw(F_B2, i, p, w);
  });
  __syncthreads();
  // ------------------------------------------------ C: Riemann (RHS)
  unrolled<NT, kSmemUnroll>((N + 1) * P, [&](int t) {
    int i = t / P, p = t % P;
    float rA = Fb(F_R, i, p), rB = Fb(F_R, i + 1, p), pA = Fb(F_P, i, p), pB = Fb(F_P, i + 1, p);
    float t1A = Fb(F_B1, i, p), t2A = Fb(F_B2, i, p), t1B = Fb(F_B1, i + 1, p), t2B = Fb(F_B2, i + 1, p);
    float cm = sqrtf(fdiv(Fb(F_GAM, i, p) * pA + t1A * t1A + t2A * t2A, rA));
    float depend1 = fmx(0.0f, 0.5f * (cx(C_DX, i) - cm * dt) * facdep);
    cm = sqrtf(fdiv(Fb(F_GAM, i + 1, p) * pB + t1B * t1B + t2B * t2B, rB));
    float depend2 = fmx(0.0f, 0.5f * (cx(C_DX, i + 1) - cm * dt) * facdep);
    float QL1 = posmask(rA + depend1 * Fb(F_G0, i, p), rA);
    float QR1 = posmask(rB - depend2 * Fb(F_G0, i + 1, p), rB);
    float QL2 = Fb(F_VN, i, p) + depend1 * Fb(F_G1, i, p);
    float QR2 = Fb(F_VN, i + 1, p) - depend2 * Fb(F_G1, i + 1, p);
    float QL3 = posmask(pA + depend1 * Fb(F_G2, i, p), pA);
    float QR3 = posmask(pB - depend2 * Fb(F_G2, i + 1, p), pB);
    float l1 = t1A + depend1 * Fb(F_G3, i, p), l2 = t2A + depend1 * Fb(F_G4, i, p);
    float r1 = t1B - depend2 * Fb(F_G3, i + 1, p), r2 = t2B - depend2 * Fb(F_G4, i + 1, p);
    float Sm = 0.5f * (Fb(F_S, i, p) + Fb(F_S, i + 1, p)), Hm = 0.5f * (Fb(F_H2, i, p) + Fb(F_H2, i + 1, p));
    float gamma = fdiv(5.0f * Sm + 7.0f * Hm, 3.0f * Sm + 5.0f * Hm);
    float Pa, Va;
    riemann<float>(gamma - 1.0f, gamma - 2.0f, gamma - 3.0f, gamma + 1.0f, gamma + 3.0f, QL1, QL2, QL3,
                   l1 * l1 + l2 * l2, QR1, QR2, QR3, r1 * r1 + r2 * r2, Pa, Va);
    Fb(F_PA, i, p) = Pa;
    Fb(F_VA, i, p) = Va;
  });
  __syncthreads();
  // ------------------------------------------------ D: Lagrangian step
  unrolled<NT, kSmemUnroll>(N * P, [&](int t) {
    int i = 1 + t / P, p = t % P;
    float dx0 = cx(C_DX, i);
    float Va1 = Fb(F_VA, i, p), Va0 = Fb(F_VA, i - 1, p), Pa1 = Fb(F_PA, i, p), Pa0 = Fb(F_PA, i - 1, p);
    float dxl = (dx0 + Va1 * dt) - Va0 * dt;
    float rho = Fb(F_R, i, p);
    float dm = dx0 * rho;
    float S = Fb(F_S, i, p), H2 = Fb(F_H2, i, p);
    float g1 = fdiv(2.0f * S + 2.0f * H2, 3.0f * S + 5.0f * H2);
    float vn = Fb(F_VN, i, p), v1 = Fb(F_VT1, i, p), v2 = Fb(F_VT2, i, p);
    float bn = Fb(F_SW, i, p), b1 = Fb(F_B1, i, p), b2 = Fb(F_B2, i, p);
    float e = fdiv(Fb(F_P, i, p), rho * g1) + 0.5f * (vn * vn + v1 * v1 + v2 * v2) +
              fdiv(0.5f * (bn * bn + b1 * b1 + b2 * b2), rho);
    float EL = e * dm - dt * (Pa1 * Va1 - Pa0 * Va0);
    Fb(F_IMN, i, p) = -dt * (Pa1 - Pa0);
    float inv = fdiv(1.0f, dxl);
    Fb(F_T, i, p) = fdiv(EL, dm);   // e after RHS: MOC's T switch inside
    Fb(F_DXL, i, p) = dxl;
    Fb(F_R, i, p) = dm * inv;
    Fb(F_B1, i, p) = b1 * dx0 * inv;
    Fb(F_B2, i, p) = b2 * dx0 * inv;
    if (edge(i)) {
      copy_ghosts(F_DXL, i, p);
      copy_ghosts(F_R, i, p);
      copy_ghosts(F_B1, i, p);
      copy_ghosts(F_B2, i, p);
    }
  });
  if (inL || inR) {
    const int bl[4] = {F_DXL, F_R, F_B1, F_B2};
    const int rl[4] = {IN_DXLAG, IN_RHO, IN_B2, IN_B3};
    inflow_fill(bl, rl, 4);
  }
  __syncthreads();
  // ------------------------------------------------ E: MOC slopes
  unrolled<NT, kSmemUnroll>((N + 2) * P, [&](int t) {
    int i = t / P, p = t % P;
    float dm = Fb(F_DXL, i - 1, p), d0 = Fb(F_DXL, i, p), dp = Fb(F_DXL, i + 1, p);
    float s = tsw(Fb(F_T, i, p), Fb(F_R, i, p));
    const LimW w = lim_w(dm, d0, dp, s);
    Fb(F_G0, i, p) = vlw(F_R, i, p, w);
    Fb(F_G1, i, p) = vlw(F_VT1, i, p, w);
    Fb(F_G2, i, p) = vlw(F_VT2, i, p, w);
    Fb(F_G3, i, p) = vlw(F_B1, i, p, w);
    Fb(F_G4, i, p) = vlw(F_B2, i, p, w);
  });
  __syncthreads();
  // ------------------------------------------------ F: characteristics
  unrolled<NT, kSmemUnroll>((N + 1) * P, [&](int t) {
    int i = t / P, p = t % P;
    float Bnap = Fb(F_BN, i + 1, p) + Fb(F_VA, i, p) * dt * fdiv(Fb(F_BN, i + 2, p) - Fb(F_BN, i, p), cx(C_X2, i));
    float D0 = Fb(F_DXL, i, p), D1 = Fb(F_DXL, i + 1, p);
    float rA = Fb(F_R, i, p), rB = Fb(F_R, i + 1, p);
    float deni = sqrtf(fdiv(D0 + D1, D0 * rB + D1 * rA));
    float ca0 = fabsf(Bnap * deni) * 0.5f * dt;
    bool up = Bnap > 0.0f;
    float dA = up ? D0 : D1, dB = up ? D1 : D0;   // upstream-first widths
    float depend1 = (0.5f * dA - fmn(dA, ca0)) * facdep;
    float depend2 = (0.5f * dB - fmn(dB, ca0)) * facdep;
    int iL = up ? i : i + 1, iR = up ? i + 1 : i;
    float sL = up ? 1.0f : -1.0f;   // + slope from the left cell, - from the right
    float QL11 = Fb(F_VT1, iL, p) + sL * depend1 * Fb(F_G1, iL, p);
    float QR11 = Fb(F_VT1, iR, p) - sL * depend2 * Fb(F_G1, iR, p);
    float QL12 = Fb(F_B1, iL, p) + sL * depend1 * Fb(F_G3, iL, p);
    float QR12 = Fb(F_B1, iR, p) - sL * depend2 * Fb(F_G3, iR, p);
    float QL13 = posmask(Fb(F_R, iL, p) + sL * depend1 * Fb(F_G0, iL, p), Fb(F_R, iL, p));
    float QR13 = posmask(Fb(F_R, iR, p) - sL * depend2 * Fb(F_G0, iR, p), Fb(F_R, iR, p));
    float QL21 = Fb(F_VT2, iL, p) + sL * depend1 * Fb(F_G2, iL, p);
    float QR21 = Fb(F_VT2, iR, p) - sL * depend2 * Fb(F_G2, iR, p);
    float QL22 = Fb(F_B2, iL, p) + sL * depend1 * Fb(F_G4, iL, p);
    float QR22 = Fb(F_B2, iR, p) - sL * depend2 * Fb(F_G4, iR, p);
    float Bay, Vay, Baz, Vaz;
    chareq<float>(QL11, QL12, QL13, QR11, QR12, QR13, Bay, Vay);
    chareq<float>(QL21, QL22, QL13, QR21, QR22, QR13, Baz, Vaz);
    Fb(F_P, i, p) = Bnap;
    Fb(F_PA, i, p) = Bay;
    Fb(F_GAM, i, p) = Vay;
    Fb(F_S, i, p) = Baz;
    Fb(F_H2, i, p) = Vaz;
  });
  __syncthreads();
  // ------------------------------ G: MOC update and remap reconstruction
  unrolled<NT, kGlobalUnroll>(N * P, [&](int t) {
    int i = 1 + t / P, p = t % P;
    float Bnap = Fb(F_P, i, p), Bnam = Fb(F_P, i - 1, p);
    float Vnap = Fb(F_VA, i, p), Vnam = Fb(F_VA, i - 1, p);
    float Bay1 = Fb(F_PA, i, p), Bay0 = Fb(F_PA, i - 1, p), Vay1 = Fb(F_GAM, i, p), Vay0 = Fb(F_GAM, i - 1, p);
    float Baz1 = Fb(F_S, i, p), Baz0 = Fb(F_S, i - 1, p), Vaz1 = Fb(F_H2, i, p), Vaz0 = Fb(F_H2, i - 1, p);
    float dxl = Fb(F_DXL, i, p), inv = fdiv(1.0f, dxl);
    float rl = Fb(F_R, i, p), dm = rl * dxl;
    float imn = Fb(F_IMN, i, p) + dt * (0.5f * (Bnap * Bnap - Bnam * Bnam));
    float im1 = dt * (Bnap * Bay1 - Bnam * Bay0);
    float im2 = dt * (Bnap * Baz1 - Bnam * Baz0);
    Fb(F_IMN, i, p) = imn;
    Fb(F_G0, i, p) = im1;
    Fb(F_G1, i, p) = im2;
    float EL = Fb(F_T, i, p) * dm + dt * ((0.5f * Bnap * Vnap + Bay1 * Vay1 + Baz1 * Vaz1) * Bnap -
                                          (0.5f * Bnam * Vnam + Bay0 * Vay0 + Baz0 * Vaz0) * Bnam);
    const float qE = EL * inv;
    Fb(F_BN, i, p) = Fb(F_SW, i, p);   // cell-centred normal field, kept for the pressure
    Fb(F_T, i, p) = qE;
    Fb(F_SW, i, p) = tsw(qE, rl);   // the remap's T switch, from E and rho
    Fb(F_B1, i, p) = Fb(F_B1, i, p) + dt * (Bnap * Vay1 - Bnam * Vay0) * inv;
    Fb(F_B2, i, p) = Fb(F_B2, i, p) + dt * (Bnap * Vaz1 - Bnam * Vaz0) * inv;
    Fb(F_VN, i, p) = Fb(F_VN, i, p) * rl + imn * inv;
    Fb(F_VT1, i, p) = Fb(F_VT1, i, p) * rl + im1 * inv;
    Fb(F_VT2, i, p) = Fb(F_VT2, i, p) * rl + im2 * inv;
    if (edge(i)) {
      copy_ghosts(F_T, i, p);
      copy_ghosts(F_SW, i, p);
      copy_ghosts(F_B1, i, p);
      copy_ghosts(F_B2, i, p);
      copy_ghosts(F_VN, i, p);
      copy_ghosts(F_VT1, i, p);
      copy_ghosts(F_VT2, i, p);
    }
  });
  if (inL || inR) {
    const int bl[7] = {F_T, F_SW, F_B1, F_B2, F_VN, F_VT1, F_VT2};
    const int rl[7] = {IN_E, IN_SW, IN_B2, IN_B3, IN_M1, IN_M2, IN_M3};
    inflow_fill(bl, rl, 7);
  }
  __syncthreads();
  // ------------------------------------------------ H: field fluxes
  unrolled<NT, kSmemUnroll>((N + 1) * P, [&](int t) {
    int i = t / P, p = t % P;
    const Upwind u = upwind(i, p, Fb(F_VA, i, p) * dt);
    const float fr = flux(F_R, u, p), fn = flux(F_VN, u, p), f1 = flux(F_VT1, u, p), f2 = flux(F_VT2, u, p),
                fe = flux(F_T, u, p), fb1 = flux(F_B1, u, p), fb2 = flux(F_B2, u, p);
    Fb(F_G2, i, p) = fr;
    Fb(F_G3, i, p) = fn;
    Fb(F_G4, i, p) = f1;
    Fb(F_P, i, p) = f2;
    Fb(F_PA, i, p) = fe;
    Fb(F_GAM, i, p) = fb1;
    Fb(F_S, i, p) = fb2;
  });
  __syncthreads();
  // --------- I: field finish, internal energy, species 0-7 reconstruction
  // The species' remap runs in one flux phase for all eight: their
  // reconstructions go to kRec, their fluxes (phase J) to kFlx.  Phase I
  // reads the kRec buffers, if at all, only at its own position before it
  // overwrites them, and reads the field fluxes of the other buffers at i-1.
  // It leaves the pressure's other inputs as one number per cell, the
  // internal energy E - ekin - emag (in F_T), so the velocity and field
  // buffers are free for the species.
  constexpr int kRec[8] = {F_G0, F_G1, F_IMN, F_H2, F_VN, F_VT1, F_VT2, F_B1};
  constexpr int kFlx[8] = {F_G2, F_G3, F_G4, F_P, F_PA, F_GAM, F_S, F_B2};
  const double rfloor = 1.27 * A.ph.rmin;
  const float rfloor_f = d2f(rfloor);
  unrolled<NT, kGlobalUnroll>(N * P, [&](int t) {
    int i = 1 + t / P, p = t % P;
    const bool act = pc.active(p);
    const int a = pc.at(p, i);
    // FP64 inputs of the position: rho and v loaded here together (hoisted)
    // or by get() where they are used; the species with them (kHoistSpecies)
    // or in one batch after the field finish
    const double *src[12] = {A.f.U[0],  A.f.U[1 + DIR], A.f.U[1 + C1], A.f.U[1 + C2],
                             A.f.sp[0], A.f.sp[1],      A.f.sp[2],     A.f.sp[3],
                             A.f.sp[4], A.f.sp[5],      A.f.sp[6],     A.f.sp[7]};
    constexpr bool hoist = ((kHoistLoads >> DIR) & 1) != 0;
    constexpr bool hoist_sp = ((kHoistSpecies >> DIR) & 1) != 0 && NT * MINB <= 1024 && LS > 0;
    double pre[12];
    if constexpr (hoist) {
#pragma unroll
      for (int q = 0; q < (hoist_sp ? 12 : 4); q++) pre[q] = __ldg(src[q] + a);
    }
    auto get = [&](int q) -> double {
      if constexpr (hoist) return pre[q];
      else return __ldg(src[q] + a);
    };
    const double r0 = get(0), rdxi = rdx[i + 1];
    const float rw = cx(C_RDX, i), dxl = Fb(F_DXL, i, p);
    double r1 = r0 + rdxi * (f2d(Fb(F_G2, i, p)) - f2d(Fb(F_G2, i - 1, p)));
    float rf = d2f(r1);
    float drho = (Fb(F_G2, i, p) - Fb(F_G2, i - 1, p)) * rw;
    if (!(rf > rfloor_f)) {   // density floor (:1293-1296)
      r1 = rfloor;
      rf = rfloor_f;
      drho = rfloor_f - d2f(r0);
    }
    if (act) A.f.U[0][a] = r1;
    const float irf = fdiv(1.0f, rf);
    auto mom = [&](int comp, double v0, int fb, float inc) {
      float v0f = d2f(v0);
      float dM = (inc + Fb(fb, i, p) - Fb(fb, i - 1, p)) * rw;
      float dv = (dM - drho * v0f) * irf;
      if (act) A.f.U[1 + comp][a] = v0 + f2d(dv);
      return v0f + dv;
    };
    const float vn = mom(DIR, get(1), F_G3, Fb(F_IMN, i, p));
    const float v1 = mom(C1, get(2), F_G4, Fb(F_G0, i, p));
    const float v2 = mom(C2, get(3), F_P, Fb(F_G1, i, p));
    const float E = (Fb(F_T, i, p) * dxl + Fb(F_PA, i, p) - Fb(F_PA, i - 1, p)) * rw;
    const float l1 = (Fb(F_B1, i, p) * dxl + Fb(F_GAM, i, p) - Fb(F_GAM, i - 1, p)) * rw;
    const float l2 = (Fb(F_B2, i, p) * dxl + Fb(F_S, i, p) - Fb(F_S, i - 1, p)) * rw;
    if (act && (!(vn == vn) || !(v1 == v1) || !(v2 == v2) || !(rf < 3e38f))) flag(A.err, ERRB_NONFINITE);
    const float ekin = 0.5f * (vn * vn + v1 * v1 + v2 * v2) * rf;
    const float bn = Fb(F_BN, i, p);
    const float emag = 0.5f * (bn * bn + l1 * l1 + l2 * l2);
    Fb(F_T, i, p) = E - ekin - emag;
    // species: content n dx is unchanged by the Lagrangian step
    const float w = cx(C_DX, i) * fdiv(1.0f, dxl);
    double ns[8];
#pragma unroll
    for (int s = 0; s < 8; s++) ns[s] = (hoist && hoist_sp) ? pre[4 + s] : __ldg(src[4 + s] + a);
#pragma unroll
    for (int s = 0; s < 8; s++) Fb(kRec[s], i, p) = d2f(ns[s]) * w;
    if (edge(i)) {
#pragma unroll
      for (int s = 0; s < 8; s++) copy_ghosts(kRec[s], i, p);
    }
  });
  if (inL || inR) {
    const int rl[8] = {IN_SPEC + 0, IN_SPEC + 1, IN_SPEC + 2, IN_SPEC + 3,
                       IN_SPEC + 4, IN_SPEC + 5, IN_SPEC + 6, IN_SPEC + 7};
    inflow_fill(kRec, rl, 8);
  }
  __syncthreads();
  // ------------------------------------------------ J: species fluxes
  unrolled<NT, kSmemUnroll>((N + 1) * P, [&](int t) {
    int i = t / P, p = t % P;
    const Upwind u = upwind(i, p, Fb(F_VA, i, p) * dt);
    float f[8];
#pragma unroll
    for (int s = 0; s < 8; s++) f[s] = flux(kRec[s], u, p);
#pragma unroll
    for (int s = 0; s < 8; s++) Fb(kFlx[s], i, p) = f[s];
  });
  __syncthreads();
  // ------------------------------- K: species finish, pressure + floors
  auto species_new = [&](int s, double n0, int a, int i, int p, bool act) {
    const float rw = cx(C_RDX, i);
    float dn = (Fb(kFlx[s], i, p) - Fb(kFlx[s], i - 1, p)) * rw;
    float nf = d2f(n0) + dn;   // remapped value, before the floor
    if (act) A.f.sp[s][a] = (nf > A.ph.ndminf[s]) ? n0 + f2d(dn) : A.ph.ndmin[s];
    return nf;
  };
  const float pmin = d2f(A.ph.pmin), pmax = d2f(A.ph.pmax);
  unrolled<NT, kGlobalUnroll>(N * P, [&](int t) {
    int i = 1 + t / P, p = t % P;
    const bool act = pc.active(p);
    const int a = pc.at(p, i);
    double pre[8];
    if constexpr (((kHoistLoads >> DIR) & 1) != 0) {
#pragma unroll
      for (int q = 0; q < 8; q++) pre[q] = __ldg(A.f.sp[q] + a);
    }
    auto get = [&](int q) -> double {
      if constexpr (((kHoistLoads >> DIR) & 1) != 0) return pre[q];
      else return __ldg(A.f.sp[q] + a);
    };
    const float n0 = species_new(0, get(0), a, i, p, act), n1 = species_new(1, get(1), a, i, p, act);
    const float n3 = species_new(3, get(3), a, i, p, act);
    const float S = n0 + n1 + n3 + species_new(4, get(4), a, i, p, act);
    const float H2 = species_new(2, get(2), a, i, p, act);
    species_new(5, get(5), a, i, p, act);
    species_new(6, get(6), a, i, p, act);
    species_new(7, get(7), a, i, p, act);
    float g1 = fdiv(2.0f * S + 2.0f * H2, 3.0f * S + 5.0f * H2);
    float pr = Fb(F_T, i, p) * g1;
    pr = fminf(pmax, fmaxf(pmin, pr));
    if (act) A.f.U[4][a] = f2d(pr);
  });
}

}  // namespace mhd
