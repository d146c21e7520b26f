// mhd_source32.cuh — chosen-form thermal SOURCE: the predictor/corrector of
// MCF3DSGincfca3.f90:2477-2572 with temperatures, conduction fluxes, the KI
// cooling function and the implicit solve in FP32, and the pressure
// accumulated in FP64 (p_new = p + dp).  The implicit solve is the same
// log-space bisection as IMC (:2898-2921); its midpoint
// 10^((log10 Pu + log10 Pd)/2) is evaluated as sqrt(Pu*Pd), which is the
// same number.  When a surrogate is attached (mhd_surrogate.cu) stiff cells
// first take the network's answer and fall back to the bisection when they
// are outside the training box or their implicit residual exceeds the
// tolerance.
#pragma once

#include "mhd_conv.cuh"
#include "mhd_kernels.cuh"
#include "mhd_surrogate_net.cuh"

namespace mhd {

// KI cooling and its temperature derivative (FP32), for the Newton polish
__device__ __forceinline__ void fcool_ki_d(float T, float NN, float &L, float &dL) {
  float Tk = T * 1.0e3f;
  float el = __expf(-1.184e5f / (Tk + 1.0e3f));
  float Laml = 1.0e7f * el;
  float dLaml = 0.0f;
  if (Laml > 5.e3f) Laml = 5.e3f;
  else dLaml = Laml * 1.184e5f * 1.0e3f / ((Tk + 1.0e3f) * (Tk + 1.0e3f));
  float Lamc = 1.4e-2f * sqrtf(Tk) * __expf(-9.2e1f / Tk);
  float dLamc = Lamc * (0.5f / T + 9.2e1f / (T * Tk));
  L = (NN * NN * (Laml + Lamc) - NN) * 3.94656e1f;
  dL = NN * NN * (dLaml + dLamc) * 3.94656e1f;
}

template <class Cool>
__device__ __forceinline__ float imc32(float Pold, float nkbi, float c /* dt*g1 */, Cool &&cool) {
  float Pu = 1.e10f, Pd = 1.e-10f, Pm = 1.e1f, Pmold = -1.0f;
  for (int k = 0; k < 30; k++) {
    float CooL = cool(Pm * nkbi);
    float fev = Pm + CooL * c - Pold;
    float iud = fev >= 0.0f ? 1.0f : -1.0f;
    Pd = fmx(-iud * Pm, Pd);
    Pu = fmn(2.0f * Pm / (iud + 1.0f + 1.e-10f), Pu);
    Pm = sqrtf(Pu * Pd);
    if (fabsf(Pm - Pmold) < 1.e-5f) break;
    Pmold = Pm;
  }
  return Pm;
}

struct Source32Args {
  Grid g;
  Phys ph;
  Fields f;
  const double *pin;
  const double *pold;
  double *pout;
  const float *T;                  // FP32 temperature of every cell (temp32_kernel)
  double dt;
  int pass;
  int *err;
  unsigned long long *imc_count;
  unsigned long long *sur_count;   // surrogate accepted
  unsigned long long *fb_count;    // surrogate rejected -> bisection
  const SurNet *W;                 // surrogate network (null: none)
  float tol;                       // residual tolerance for accepting a polished guess
  const float *sh2;                // S = H+p+He+He+ and H2 of every cell (temp32), or null
  int *stiff_list;                 // guess-and-polish modes: the stiff cells left to the second kernel
  unsigned long long *stiff_count; // their number (zeroed before each pass)
};

// How a stiff cell's implicit solve starts when it does not go straight to
// the bisection (KI cooling only): from the network's answer, or -- the
// same solver without the network, for comparison -- from the frozen-rate
// implicit update P_b / (1 + c Lambda_b / P_b) (the explicit update when
// Lambda_b heats).
enum : int { STIFF_NETWORK = 1, STIFF_NEWTON = 2 };
// the FP32 time-step screen: threads per block and cells per block (two per
// thread)
constexpr int kDtScreenThreads = 256, kDtScreenCells = 2 * kDtScreenThreads;
constexpr int kFusedTiles = 2;                  // 128-cell tiles per CTA of the stiff-cell kernel
constexpr int kFusedThreads = 128 * kFusedTiles;
// block size of the explicit pass that lists the stiff cells (one list
// append per block)
constexpr int kSourceDeferThreads = 512;

}  // namespace mhd

namespace mhd {

#ifdef MHD_FP32_KERNELS
// T = p / (kb (H + p + He + He+ + H2)) of every padded cell in FP32: the
// conduction stencil of SOURCE reads the temperatures of six neighbours,
// so they are formed once per pass instead of once per neighbour.  The
// predictor pass also stores S = H + p + He + He+ and H2 (sh2[t], sh2[ncell
// + t]), which both passes of the KI source read instead of the five
// species (they do not change within a SOURCE call); the host keeps them
// while the species stay unchanged, for the next time step and the next
// SOURCE, whose predictor pass then takes the <false> form too.
// The species pass handles two cells per thread (block-strided, loads of
// both issued first) to keep more loads in flight.
template <bool FROM_SPECIES>
__global__ void __launch_bounds__(256) temp32_kernel(long long ncell, Fields f, const double *pin, float kb,
                                                     float *T, float *sh2) {
  if constexpr (FROM_SPECIES) {
    const long long t0 = (long long)blockIdx.x * (2 * blockDim.x) + threadIdx.x;
    double v[2][6];
#pragma unroll
    for (int u = 0; u < 2; u++) {
      const long long t = t0 + u * blockDim.x;
      if (t < ncell) {
#pragma unroll
        for (int q = 0; q < 5; q++) v[u][q] = __ldg(f.sp[q] + t);
        v[u][5] = __ldg(pin + t);
      }
    }
#pragma unroll
    for (int u = 0; u < 2; u++) {
      const long long t = t0 + u * blockDim.x;
      if (t >= ncell) continue;
      const float S = d2f(v[u][0]) + d2f(v[u][1]) + d2f(v[u][3]) + d2f(v[u][4]), H2 = d2f(v[u][2]);
      sh2[t] = S;
      sh2[ncell + t] = H2;
      T[t] = __fdividef(d2f(v[u][5]), kb * (S + H2));
    }
  } else {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncell) return;
    T[t] = __fdividef(d2f(pin[t]), kb * (sh2[t] + sh2[ncell + t]));
  }
}

// One pass of the chosen-form SOURCE for one cell: the quantities of the
// cell (source32_prep) and the pressure update from the cooling increment
// (source32_finish).  The only FP64 operation is p_new = base + dp;
// conversions are integer ones.
template <bool CHEM>
struct Cell32 {
  int a;   // 32-bit cell offset (the padded grid has fewer than 2^31 cells)
  float T0, div, g1, NN, nimc, nkbi, dts, basef, CooL, dx0;
  double base;
  bool stiff;
  CellSpecies<float> cs;
};

template <bool CHEM>
__device__ __forceinline__ Cell32<CHEM> source32_prep(const Source32Args &A, long long t) {
  const Grid &g = A.g;
  const int nx = g.n[0], ny = g.n[1];
  int i, j, k;
  split3(t, nx, ny, i, j, k);
  i += 1; j += 1; k += 1;
  Cell32<CHEM> c;
  const int a = (int)gidx(g, i, j, k);
  c.a = a;
  const float kb = d2f(A.ph.kb), Kc = d2f(A.ph.kcond);
  const float dt = d2f(A.dt);
  const Fields &f = A.f;
  const float *T = A.T;
  const float *dx = g.dxf[0], *dy = g.dxf[1], *dz = g.dxf[2];
  const int sy = (int)g.st[1], sz = (int)g.st[2];
  const float T0 = T[a];
  auto flux = [&](float Tl, float Tu, float dl, float du) {
    float rdu = __fdividef(1.0f, dl + du);
    float rt = sqrtf((dl * Tu + du * Tl) * rdu);
    return Kc * fminf(rt, 3.873f) * (Tu - Tl) * 2.0f * rdu;
  };
  const float dxm = dx[i], dx0 = dx[i + 1], dxp = dx[i + 2];
  const float dym = dy[j], dy0 = dy[j + 1], dyp = dy[j + 2];
  const float dzm = dz[k], dz0 = dz[k + 1], dzp = dz[k + 2];
  c.div = __fdividef(flux(T0, T[a + 1], dx0, dxp) - flux(T[a - 1], T0, dxm, dx0), dx0) +
          __fdividef(flux(T0, T[a + sy], dy0, dyp) - flux(T[a - sy], T0, dym, dy0), dy0) +
          __fdividef(flux(T0, T[a + sz], dz0, dzp) - flux(T[a - sz], T0, dzm, dz0), dz0);
  float S, H2;
  if (!CHEM && A.sh2) {
    S = A.sh2[a];
    H2 = A.sh2[(int)g.ncell + a];
  } else {
    S = d2f(f.sp[0][a]) + d2f(f.sp[1][a]) + d2f(f.sp[3][a]) + d2f(f.sp[4][a]);
    H2 = d2f(f.sp[2][a]);
  }
  c.g1 = __fdividef(2.0f * S + 2.0f * H2, 3.0f * S + 5.0f * H2);
  c.NN = d2f(f.U[0][a]) * (1.0f / 1.27f);
  // the cooling function of the run: KI, or the species form (ifchem = 2)
  if constexpr (CHEM) {
    c.cs = cell_species<float>(f, a, [](double v) { return d2f(v); });
    c.CooL = fcool_species<float>(T0, c.cs);
  } else {
    c.CooL = fcool_ki(T0, c.NN);
  }
  const double Pn = A.pold[a];
  const float Pnf = d2f(Pn);
  c.dts = dt * ((A.pass == 0) ? 0.5f : 1.0f);      // predictor: half of dt
  c.base = (A.pass == 0) ? A.pin[a] : Pn;          // p the cooling acts on
  c.basef = (A.pass == 0) ? d2f(c.base) : Pnf;
  c.stiff = !(dt <= 0.2f * Pnf / (c.g1 * fabsf(c.CooL)));
  c.nimc = S + H2;
  c.nkbi = __fdividef(1.0f, kb * c.nimc);
  c.T0 = T0;
  c.dx0 = dx0;
  return c;
}

template <bool CHEM>
__device__ __forceinline__ void source32_finish(const Source32Args &A, const Cell32<CHEM> &c, float dp_cool) {
  const float kb = d2f(A.ph.kb), Kc = d2f(A.ph.kcond), dt = d2f(A.dt);
  float tcd = c.g1 * Kc * sqrtf(c.T0);
  tcd = __fdividef(0.49f * c.nimc * kb, tcd) * (c.dx0 * c.dx0);
  const float w = (tcd - dt >= 0.0f) ? 1.0f : 0.0f;      // (sign(0.5, tcd-dt) + 0.5)
  const float dp = dp_cool + w * c.g1 * c.dts * c.div;
  double pnew = c.base + f2d(dp);
  const float pf = c.basef + dp;
  // floors max(pnew, pmin), min(pnew, pmax); a NaN passes and is reported
  if (pf < d2f(A.ph.pmin)) pnew = A.ph.pmin;
  if (pf > d2f(A.ph.pmax)) pnew = A.ph.pmax;
  A.pout[c.a] = pnew;
  if (!(pf == pf)) flag(A.err, ERRB_NONFINITE);
}

// The implicit solve of a stiff cell (IMC bisection), kept out of line: few
// cells take it.
template <bool CHEM>
__device__ __noinline__ float imc32_cell(const Cell32<CHEM> &c) {
  const float cc = c.dts * c.g1;
  if constexpr (CHEM) return imc32(c.basef, c.nkbi, cc, [&](float T) { return fcool_species<float>(T, c.cs); });
  else return imc32(c.basef, c.nkbi, cc, [&](float T) { return fcool_ki(T, c.NN); });
}

// Thread per cell.  CHEM: the species cooling function (ifchem = 2) instead
// of the KI one.  DEFER (a guess-and-polish mode): stiff cells are appended
// to A.stiff_list and left to source32_stiff_kernel, so this pass keeps the
// registers and occupancy of the explicit update; otherwise they are
// solved here by the bisection.
template <bool CHEM, bool DEFER>
__global__ void __launch_bounds__(DEFER ? kSourceDeferThreads : 128) source32_kernel(Source32Args A) {
  const Grid &g = A.g;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = t < (long long)g.n[0] * g.n[1] * g.n[2];
  const Cell32<CHEM> c = source32_prep<CHEM>(A, valid ? t : 0);
  const bool stiff = valid && c.stiff;
  if constexpr (DEFER) {
    // block-aggregated append of the stiff cells' indices: one atomic per
    // block on the shared counter; a block without stiff cells passes one
    // barrier only
    if (__syncthreads_or(stiff)) {
      __shared__ unsigned wcnt[kSourceDeferThreads / 32];
      __shared__ unsigned long long bbase;
      const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
      const unsigned m = __ballot_sync(0xffffffffu, stiff);
      if (lane == 0) wcnt[w] = __popc(m);
      __syncthreads();
      if (threadIdx.x == 0) {
        unsigned tot = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) tot += wcnt[q];
        bbase = atomicAdd(A.stiff_count, (unsigned long long)tot);
      }
      __syncthreads();
      if (stiff) {
        unsigned long long pos = bbase;
        for (int q = 0; q < w; q++) pos += wcnt[q];
        A.stiff_list[pos + __popc(m & ((1u << lane) - 1u))] = (int)t;
      }
    }
    if (!valid || stiff) return;
  }
  if (!valid) return;
  float dp_cool;
  if (!stiff) {
    dp_cool = -(c.g1 * c.CooL * c.dts);
  } else {
    dp_cool = imc32_cell<CHEM>(c) - c.basef;
    atomicAdd(A.imc_count, 1ull);
  }
  source32_finish<CHEM>(A, c, dp_cool);
}

// Two Newton steps on f(P) = P + c Lambda(P) - P_b (c = dt (gamma-1)) from
// P, then the implicit residual |P + Lambda(P) c - P_b| / P_b of
// IMC's equation (MCF3DSGincfca3.f90:2911) as the acceptance test.
__device__ __forceinline__ bool polish_accept(const Source32Args &A, const Cell32<false> &c, float P, float *dp) {
  const float cc = c.dts * c.g1;
  for (int it = 0; it < 2; it++) {
    float L, dL;
    fcool_ki_d(P * c.nkbi, c.NN, L, dL);
    const float fv = P + cc * L - c.basef;
    const float fp = 1.0f + cc * dL * c.nkbi;
    if (fp > 0.0f) P = fmaxf(P - fv / fp, 0.1f * P);
  }
  const float res = fabsf(P + fcool_ki(P * c.nkbi, c.NN) * cc - c.basef) / c.basef;
  if (!(res <= A.tol)) return false;
  *dp = P - c.basef;
  return true;
}

// The stiff cells listed by source32_kernel<false, true> (KI cooling), in
// dense blocks of 256 list entries (thread per cell, two 128-cell tiles):
// each thread forms its cell's guess -- MODE STIFF_NETWORK: the surrogate
// network on the tensor cores for the whole block (sur_tile_forward; the
// weights are staged and TMEM allocated once per CTA, and a CTA without
// list entries returns before either), inputs outside the training box
// going straight to the bisection -- then polishes and tests it, and the
// rejected cells take the bisection.  A persistent grid strides over the
// list.  Counters: sur_count accepted guesses, fb_count rejected ones,
// imc_count every bisection.
template <int MODE>
__global__ void __launch_bounds__(kFusedThreads, 3) source32_stiff_kernel(Source32Args A) {
  extern __shared__ __align__(128) unsigned char stiff_smem[];
  using Tile = SurTileSmem<kFusedTiles>;
  Tile *s = reinterpret_cast<Tile *>(stiff_smem);
  const long long cnt = (long long)*A.stiff_count;
  if ((long long)blockIdx.x * kFusedThreads >= cnt) return;   // the whole CTA: no list entry for it
  if constexpr (MODE == STIFF_NETWORK) sur_tile_setup<kFusedTiles>(A.W, s);
  const int lane = threadIdx.x & 31;
  uint32_t phase = 0;
  for (long long e0 = (long long)blockIdx.x * kFusedThreads; e0 < cnt; e0 += (long long)gridDim.x * kFusedThreads) {
    const long long e = e0 + threadIdx.x;
    const bool on = e < cnt;
    const Cell32<false> c = source32_prep<false>(A, A.stiff_list[on ? e : e0]);
    const float Tb = c.basef * c.nkbi;   // temperature the implicit solve starts from
    const float Lb = fcool_ki(Tb, c.NN);
    const float cc = c.dts * c.g1;
    bool use = on;
    float P;
    if constexpr (MODE == STIFF_NETWORK) {
      const float rr = cc * fabsf(Lb) / c.basef;
      const float x0 = log10f(c.NN), x1 = log10f(Tb), x2 = log10f(fmaxf(rr, 1e-30f));
      const bool inbox = on && x0 >= -2.0f && x0 <= 5.0f && x1 >= -2.0f && x1 <= 1.30103f && x2 >= -3.0f &&
                         x2 <= 3.0f;
      float y0 = 0.0f, y1 = 0.0f;
      const bool ok = sur_tile_forward<kFusedTiles>(s, inbox ? (x0 - SUR_C0) / SUR_S0 : 0.0f,
                                                    inbox ? (x1 - SUR_C1) / SUR_S1 : 0.0f,
                                                    inbox ? (x2 - SUR_C2) / SUR_S2 : 0.0f, phase, y0, y1);
      if (!ok && threadIdx.x == 0) flag(A.err, ERRB_TC);
      use = inbox && ok;
      P = (Tb * exp10f(y0)) / c.nkbi;
    } else {
      P = Lb > 0.0f ? c.basef / (1.0f + cc * Lb / c.basef) : c.basef - cc * Lb;
    }
    float dp_cool = 0.0f;
    const bool acc = use && polish_accept(A, c, P, &dp_cool);
    const unsigned mu = __ballot_sync(0xffffffffu, use), ma = __ballot_sync(0xffffffffu, acc);
    const unsigned mb = __ballot_sync(0xffffffffu, on && !acc);
    if (lane == 0) {
      if (ma) atomicAdd(A.sur_count, (unsigned long long)__popc(ma));
      if (mu & ~ma) atomicAdd(A.fb_count, (unsigned long long)__popc(mu & ~ma));
      if (mb) atomicAdd(A.imc_count, (unsigned long long)__popc(mb));
    }
    if (!on) continue;
    if (!acc) dp_cool = imc32_cell<false>(c) - c.basef;
    source32_finish<false>(A, c, dp_cool);
  }
  if constexpr (MODE == STIFF_NETWORK) sur_tile_teardown<kFusedTiles>(s, phase);
}

// dt for the chosen form, first of two kernels: an FP32 screen of every
// cell.  The chosen form takes the same time step as the plain FP64 form
// (the CFL minimum stays FP64): this kernel computes the Courant limit
// (:1912-1930) and the two thermal limits of Stblty (:2784-2822) of each
// cell in FP32 together with an interval that surely holds the FP64 value,
// [v (1 - eta), v (1 + eta)] (eta below, far wider than the FP32 rounding
// of these products, sums and quotients of positive terms); the cooling
// time divides by |Lambda|, a difference of cooling and heating, so its
// interval widens |Lambda| by a fraction of the sum of the terms'
// magnitudes (and is unbounded above where that covers 0).  The floor 2.5e-4 of the
// cooling time is exact: a cell whose interval lies below it has the floor
// as its FP64 value.  Each warp stores the lower ends of its three limits;
// the block minima of the upper ends go to words[0..2] (non-negative floats
// order like their bit patterns) and words[3] records a floored cell.
// dt_refine_kernel then recomputes in FP64 only the warps whose lower ends
// reach the smallest upper end -- the only cells that can hold the minimum.
struct DtScreen {
  float *lo;          // [3][nwarps]: per warp, the smallest lower end of c, tau, alpha
  unsigned *words;    // [0..2] smallest upper ends (float bits), [3] a cooling time at the floor
  int nwarps;
  int boff;           // block index of the launch's first block (a slab of the grid)
};
// The FP32 rounding of these quantities stays below ~1e-6 relative (inputs
// rounded once, IEEE quotients, the approximate square root): eta = 2^-14
// is 60 times that.  The KI cooling terms carry the exponential's
// argument error (|arg| x a few ulp, up to ~1e-5 where the term matters):
// 2^-12 of their magnitude sum; the species function's powers and
// logarithms: 2^-8.
constexpr float kDtEta = 1.0f / 16384.0f;
constexpr float kDtEtaCoolKI = 1.0f / 4096.0f;
constexpr float kDtEtaCoolSpecies = 1.0f / 256.0f;

// Two cells per thread, 256 apart (block-strided, so every warp access
// stays coalesced), the loads of both issued before either is used: the
// screen moves ~72 bytes a cell and one cell per thread left it waiting on
// memory.  The per-warp lower ends stay per 32 consecutive cells (the unit
// the refine kernel walks).
__global__ void __launch_bounds__(kDtScreenThreads) dt32_screen_kernel(Grid g, Phys ph, Fields f, const float *sh2,
                                                                       DtScreen sc, int *err) {
  const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const long long ncells = (long long)nx * ny * nz;
  const long long base = ((long long)blockIdx.x + sc.boff) * kDtScreenCells + threadIdx.x;
  const float INF = __int_as_float(0x7f800000);
  const float dn = 1.0f - kDtEta, up = 1.0f + kDtEta;
  // the inputs of both cells first: rho, v1..v3, p, Bcc1..3 (and S, H2)
  double raw[2][8];
  float sr[2][2];
  int ijk[2][3];
  long long aa[2];
#pragma unroll
  for (int u = 0; u < 2; u++) {
    const long long t = base + u * kDtScreenThreads;
    aa[u] = -1;
    if (t < ncells) {
      split3(t, nx, ny, ijk[u][0], ijk[u][1], ijk[u][2]);
      ijk[u][0] += 1; ijk[u][1] += 1; ijk[u][2] += 1;
      const long long a = gidx(g, ijk[u][0], ijk[u][1], ijk[u][2]);
      aa[u] = a;
      raw[u][0] = __ldg(f.U[0] + a); raw[u][1] = __ldg(f.U[1] + a); raw[u][2] = __ldg(f.U[2] + a);
      raw[u][3] = __ldg(f.U[3] + a); raw[u][4] = __ldg(f.U[4] + a);
      raw[u][5] = __ldg(f.bcc[0] + a); raw[u][6] = __ldg(f.bcc[1] + a); raw[u][7] = __ldg(f.bcc[2] + a);
      if (sh2) {
        sr[u][0] = __ldg(sh2 + a);
        sr[u][1] = __ldg(sh2 + g.ncell + a);
      }
    }
  }
  float lo[2][3], hi[3] = {INF, INF, INF};   // c, tau, alpha
  bool floored = false;
#pragma unroll
  for (int u = 0; u < 2; u++) {
    lo[u][0] = lo[u][1] = lo[u][2] = INF;
    if (aa[u] < 0) continue;
    const long long a = aa[u];
    const int i = ijk[u][0], j = ijk[u][1], k = ijk[u][2];
    // S = H+p+He+He+ and H2: SOURCE's floats when current (the same sums)
    float S, H2;
    if (sh2) {
      S = sr[u][0];
      H2 = sr[u][1];
    } else {
      S = d2f(f.sp[0][a]) + d2f(f.sp[1][a]) + d2f(f.sp[3][a]) + d2f(f.sp[4][a]);
      H2 = d2f(f.sp[2][a]);
    }
    float rg = __fdiv_rn(1.0f, 3.0f * S + 5.0f * H2);
    float gam = (5.0f * S + 7.0f * H2) * rg;
    float bx = d2f(raw[u][5]), by = d2f(raw[u][6]), bz = d2f(raw[u][7]);
    float rho = d2f(raw[u][0]), p5 = d2f(raw[u][4]);
    float cs = sqrtf(__fdiv_rn(gam * p5 + bx * bx + by * by + bz * bz, rho));
    float dxi = g.dxf[0][i + 1], dyj = g.dxf[1][j + 1], dzk = g.dxf[2][k + 1];
    float c = fminf(fminf(__fdiv_rn(dxi, cs + fabsf(d2f(raw[u][1]))), __fdiv_rn(dyj, cs + fabsf(d2f(raw[u][2])))),
                    __fdiv_rn(dzk, cs + fabsf(d2f(raw[u][3]))));
    lo[u][0] = c * dn;
    hi[0] = fminf(hi[0], c * up);
    bool bad = !(c > 0.0f);
    if (ph.ifthrm == 2) {
      float Nn = S + H2;
      const float kb = d2f(ph.kb);
      float Tn = __fdiv_rn(p5, kb * Nn);
      float dl = fminf(fminf(dxi, dyj), dzk);
      float g1c = (2.0f * S + 2.0f * H2) * rg;
      float alpha = __fdiv_rn(0.4f * Nn * kb, g1c * d2f(ph.kcond) * sqrtf(fminf(Tn, 15.0f))) * (dl * dl);
      lo[u][2] = alpha * dn;
      hi[2] = fminf(hi[2], alpha * up);
      float mag;
      float CooL = (ph.ifchem == 2)
                       ? fcool_species<float>(Tn, cell_species<float>(f, a, [](double v) { return d2f(v); }), &mag)
                       : fcool_ki_mag(Tn, rho * (1.0f / 1.27f), mag);
      const float ac = fabsf(CooL), num = 0.2f * p5;
      const float e = (ph.ifchem == 2 ? kDtEtaCoolSpecies : kDtEtaCoolKI) * mag;
      const float tlo = __fdiv_rn(num, g1c * (ac + e)) * dn;
      const float thi = ac > e ? __fdiv_rn(num, g1c * (ac - e)) * up : INF;
      // the floor of the cooling time, bracketed in FP32
      const float flo = 2.5e-4f * (1.0f - 1e-6f), fhi = 2.5e-4f * (1.0f + 1e-6f);
      floored = floored || thi <= flo;
      lo[u][1] = fmaxf(tlo, flo);
      hi[1] = fminf(hi[1], fmaxf(thi, fhi));
      bad = bad || !(alpha > 0.0f) || !(lo[u][1] > 0.0f);
    }
    if (bad) flag(err, ERRB_DT);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < 3; q++) {
      lo[0][q] = fminf(lo[0][q], __shfl_xor_sync(0xffffffffu, lo[0][q], o));
      lo[1][q] = fminf(lo[1][q], __shfl_xor_sync(0xffffffffu, lo[1][q], o));
      hi[q] = fminf(hi[q], __shfl_xor_sync(0xffffffffu, hi[q], o));
    }
  floored = __any_sync(0xffffffffu, floored);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int u = 0; u < 2; u++) {
      const long long gw = (base + u * kDtScreenThreads) >> 5;   // the 32 consecutive cells of this warp's half
      if (gw < sc.nwarps) {
        sc.lo[gw] = lo[u][0];
        sc.lo[sc.nwarps + gw] = lo[u][1];
        sc.lo[2 * sc.nwarps + gw] = lo[u][2];
      }
    }
  }
  __shared__ float wh[3][kDtScreenThreads / 32];
  if (lane == 0)
    for (int q = 0; q < 3; q++) wh[q][w] = hi[q];
  if (lane == 0 && floored) atomicOr(&sc.words[3], 1u);
  __syncthreads();
  if (threadIdx.x < 3) {
    float m = wh[threadIdx.x][0];
    for (int q = 1; q < (int)(blockDim.x >> 5); q++) m = fminf(m, wh[threadIdx.x][q]);
    atomicMin(&sc.words[threadIdx.x], __float_as_uint(m));
  }
}

// the chemistry network in FP32 (ifchem = 2, :2576-2776); the species,
// nde and ndtot are stored back as FP64, rho = sum m n is formed in FP64
__global__ void __launch_bounds__(128) chem32_kernel(Grid g, Phys ph, Fields f, float dt, int *err) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  if (t >= (long long)nx * ny * nz) return;
  long long a = gidx_lin(g, t, nx, ny);
  CellSpecies<float> c = cell_species<float>(f, a, [](double v) { return d2f(v); });
  float mn[8];
  for (int q = 0; q < 8; q++) mn[q] = d2f(ph.ndmin[q]);
  chem_network<float>(c, d2f(f.U[4][a]), d2f(ph.kb), dt, mn);
  const double H = f2d(c.H), p = f2d(c.p), H2 = f2d(c.H2), He = f2d(c.He), Hep = f2d(c.Hep);
  f.sp[0][a] = H; f.sp[1][a] = p; f.sp[2][a] = H2; f.sp[3][a] = He;
  f.sp[4][a] = Hep; f.sp[5][a] = f2d(c.C); f.sp[6][a] = f2d(c.Cp); f.sp[7][a] = f2d(c.CO);
  f.nde[a] = f2d(c.ne);
  f.ndtot[a] = f2d(c.nt);
  f.U[0][a] = p + H + 2.0 * H2 + 4.0 * He + 4.0 * Hep;
  if (!(c.H == c.H) || !(c.p == c.p)) flag(err, ERRB_NONFINITE);
}

#endif  // MHD_FP32_KERNELS

}  // namespace mhd
