// mhd_fp32.cu — chosen form: reconstruction, Riemann solver, characteristic
// and EMF arithmetic in FP32; accumulation into the FP64 state.  Built with
// the default contraction (FMA) enabled.
#include <cudaTypedefs.h>

#include <algorithm>
#define MHD_FP32_KERNELS
#include "mhd_sweep32.cuh"
#include "mhd_ct32.cuh"
#include "mhd_source32.cuh"
#include "mhd_sweep_impl.cuh"

namespace mhd {
// Sweep launch shapes.  The default: two CTAs per SM (the pencil buffers
// of P = 4 pencils of 256 cells take 92 KB), 512 threads for the x sweep
// (64 registers; at 256^3 1.69 -> 1.65 ms against 384 threads with 80
// registers, 1.88 with 448) and 576 for the y sweep (56 registers; 544 and
// 512 threads measured the same or slower); the z sweep and pencils longer
// than 256 cells take the shapes chosen in launch32_d below.  First
// measured at 256^3 on GB300 with P = 4 and two CTAs per SM (ms per sweep x
// / y / z): 288 threads 2.91 / 3.57 / 3.70; 384: 2.36 / 2.96 / 3.17; 576:
// 2.42 / 2.68 / 3.13 (before the compile-time stride and the load changes
// of the kernel).  More warps per SM hide the shared-memory and global-load
// latency of the phases.  The register budget this leaves (64 / 56 per
// thread) holds the kernel without spills because the global-load phases
// are not unrolled (see MHD_SWEEP_GLOBAL_UNROLL).  The thread counts can be
// overridden at build time for experiments.
#ifndef MHD_SWEEP_THREADS_X
#define MHD_SWEEP_THREADS_X 512
#endif
#ifndef MHD_SWEEP_THREADS_YZ
#define MHD_SWEEP_THREADS_YZ 576
#endif
#ifndef MHD_SWEEP_MIN_BLOCKS
#define MHD_SWEEP_MIN_BLOCKS 2
#endif
#ifndef MHD_SWEEP_MAX_PENCILS
#define MHD_SWEEP_MAX_PENCILS 4
#endif
template <int DIR>
constexpr int sweep_threads() { return DIR == 0 ? MHD_SWEEP_THREADS_X : MHD_SWEEP_THREADS_YZ; }
constexpr int kSweepMinBlocks = MHD_SWEEP_MIN_BLOCKS;
constexpr size_t kSweepSmemPerCta = (227 * 1024) / MHD_SWEEP_MIN_BLOCKS - 1024;

// Pencils of up to kSweepFixedStride - 4 cells with P = 4 use the kernel
// with a compile-time buffer stride (256^3: sweeps 4-8 % faster than with
// the run-time stride); other lengths use the run-time stride.
#ifndef MHD_SWEEP_FIXED_STRIDE
#define MHD_SWEEP_FIXED_STRIDE 260
#endif
constexpr int kSweepFixedStride = MHD_SWEEP_FIXED_STRIDE;

// Pencils of 257..512 cells (the 512^3 grid): a second compile-time stride
// (516), with the shape measured best per direction at 512^3 (ms per sweep
// x / y / z): the x sweep two pencils per CTA and two CTAs per SM (17.0 /
// 34.3 / 43.2 for all three that way), the y and z sweeps four pencils per
// CTA -- full 32-byte rows -- and one 768-thread CTA per SM (19.0 / 22.1 /
// 30.5); the run-time stride with two pencils gave 18.5 / 34.5 / 43.4.
#ifndef MHD_SWEEP_LONG_STRIDE
#define MHD_SWEEP_LONG_STRIDE 516
#endif
#ifndef MHD_SWEEP_LONG_THREADS
#define MHD_SWEEP_LONG_THREADS 768
#endif
constexpr int kSweepLongStride = MHD_SWEEP_LONG_STRIDE;
// 768 threads (three rounds of the 2048-2064 items of a phase; up to 85
// registers, so the field-finish phase loads its species with rho and v):
// 2.28 -> 2.21 ms at 256^3 against 1024 threads (two rounds and a third
// of 8-16 items for the phases over n+1 or n+2 positions)
#ifndef MHD_SWEEP_Z_THREADS
#define MHD_SWEEP_Z_THREADS 768
#endif
constexpr int kSweepZThreads = MHD_SWEEP_Z_THREADS;
#ifndef MHD_SWEEP_Z_PENCILS
#define MHD_SWEEP_Z_PENCILS 8
#endif
constexpr int kSweepZPencils = MHD_SWEEP_Z_PENCILS;
#ifndef MHD_SWEEP_Z_MINB
#define MHD_SWEEP_Z_MINB 1
#endif

// Bit d of MHD_SWEEP_TMA set: the direction-d sweep (y or z) stages its
// FP64 inputs with TMA box loads (see SweepTma) when the grid allows it:
// pencils of up to 2 kStageRows - 4 cells, an even padded row (row strides a
// multiple of 16 bytes) and every input array inside the state allocation.
// Measured at 256^3 (ms, per-thread loads -> TMA): y 2.07 -> 1.99 with two
// CTAs per SM, whose load and compute phases overlap; z 2.26 -> 2.36 with
// its one CTA per SM, where the three staging rounds are exposed; x 1.65 ->
// 1.80 (its one-pass loads of contiguous rows already hit L1 for 46 % of
// their sectors).  So the y sweep only, by default.
#ifndef MHD_SWEEP_TMA
#define MHD_SWEEP_TMA 2
#endif
constexpr int kSweepTmaStride = 2 * kStageRows;

// the CUDA driver API's tensor-map encoder, resolved once (null when
// unavailable)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// the tensor map and array indices of the direction-DIR sweep's staged
// inputs, pencil groups of P columns; false when the grid or the arrays do
// not meet the TMA rules
template <int DIR, int P>
static bool sweep_tma_map(const SweepArgs &a, const double *block, int narr, SweepTma &T) {
  const Grid &g = a.g;
  const int L = g.n[DIR] + 4;
  if (!block || g.s[0] % 2 != 0 || L > kSweepTmaStride || (P * 8) % 16 != 0) return false;
  T = SweepTma{};
  T.nbox = (L + kStageRows - 1) / kStageRows;
  constexpr int C1 = (DIR + 1) % 3, C2 = (DIR + 2) % 3;
  const Fields &f = a.f;
  const double *in[SF_COUNT] = {f.bcc[C1], f.bcc[C2], f.U[0], f.U[1 + DIR], f.U[1 + C1], f.U[1 + C2], f.U[4],
                                f.sp[0],   f.sp[1],   f.sp[2], f.sp[3],     f.sp[4],     f.U[5 + DIR], f.bcc[DIR]};
  const long long nc = g.ncell;
  for (int q = 0; q < SF_COUNT; q++) {
    const long long d = (long long)(in[q] - block);
    if (d < 0 || d % nc != 0 || d / nc >= narr) return false;
    T.fld[q] = (int)(d / nc);
  }
  auto enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)g.s[0], (cuuint64_t)g.s[1], (cuuint64_t)g.s[2], (cuuint64_t)narr};
  const cuuint64_t strides[3] = {(cuuint64_t)g.s[0] * 8, (cuuint64_t)g.s[0] * g.s[1] * 8, (cuuint64_t)nc * 8};
  const cuuint32_t box[4] = {DIR == 0 ? (cuuint32_t)kStageRows : (cuuint32_t)P,
                             DIR == 0 ? (cuuint32_t)P : DIR == 1 ? (cuuint32_t)kStageRows : 1u,
                             DIR == 2 ? (cuuint32_t)kStageRows : 1u, 1u};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return enc(&T.map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, const_cast<double *>(block), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int DIR, int P, int LS, int NT, int MINB, bool TM = false>
static cudaError_t launch32(const SweepArgs &a, cudaStream_t s, const SweepTma &T = SweepTma{}) {
  const Grid &g = a.g;
  size_t smem = sweep32_smem_bytes(g.n[DIR], P, LS);
  auto k = sweep32_kernel<DIR, P, NT, MINB, LS, TM>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // x sweep: P adjacent y rows per CTA; y and z sweeps: P adjacent x columns
  // starting at padded x = P*blockIdx.x, which covers x = -1 .. n+2
  const unsigned xgroups = (unsigned)((g.n[0] + 2 + P - 1) / P);
  dim3 grid;
  const int nby = (DIR == 2) ? g.n[1] : g.n[2];   // transverse block index: z for x and y, y for z
  const int by0 = a.by1 > 0 ? a.by0 : 0, by1 = a.by1 > 0 ? a.by1 : nby;
  if (by0 < 0 || by1 > nby || by0 >= by1) return cudaErrorInvalidValue;
  if (DIR == 0) grid = dim3(g.n[1] / P, by1 - by0);
  else grid = dim3(xgroups, by1 - by0);
  SweepArgs ar = a;
  ar.by0 = by0;
  k<<<grid, NT, smem, s>>>(ar, T);
  return cudaGetLastError();
}

template <int DIR>
static cudaError_t launch32_d(const SweepArgs &a, const double *block, int narr, cudaStream_t s) {
  constexpr int NT = sweep_threads<DIR>(), MB = kSweepMinBlocks;
  // the x sweep needs P to divide ny; the y and z sweeps pad their groups
  const int nb = (DIR == 0) ? a.g.n[1] : 4;
  const int L = a.g.n[DIR] + 4;
  // the z sweep: eight x columns per CTA, one CTA per SM (kSweepZThreads).  Its
  // pencils cross a 2 MB page every four cells, and wider groups spread the
  // CTAs running at once over fewer pages: 2.68 ms at 256^3 against 2.99
  // with four columns and two CTAs per SM (the y sweep, whose pencils stay
  // within a page or two, is faster with four: 2.41 against 2.52, and the x
  // sweep with four rows and two CTAs: 2.16 against 2.58)
  if constexpr (DIR == 2) {
    if (((MHD_SWEEP_TMA >> 2) & 1) && L <= kSweepTmaStride &&
        sweep32_smem_bytes(a.g.n[DIR], kSweepZPencils, kSweepTmaStride) <=
            (MHD_SWEEP_Z_MINB > 1 ? kSweepSmemPerCta : 226 * 1024)) {
      SweepTma T;
      if (sweep_tma_map<DIR, kSweepZPencils>(a, block, narr, T))
        return launch32<DIR, kSweepZPencils, kSweepTmaStride, kSweepZThreads, MHD_SWEEP_Z_MINB, true>(a, s, T);
    }
    if (L <= kSweepFixedStride && sweep32_smem_bytes(a.g.n[DIR], kSweepZPencils, kSweepFixedStride) <= 226 * 1024)
      return launch32<DIR, kSweepZPencils, kSweepFixedStride, kSweepZThreads, 1>(a, s);
  }
  if constexpr (DIR == 0) {
    if ((MHD_SWEEP_TMA & 1) && nb % 4 == 0 && L <= kSweepTmaStride &&
        sweep32_smem_bytes(a.g.n[DIR], 4, kSweepTmaStride) <= kSweepSmemPerCta) {
      SweepTma T;
      if (sweep_tma_map<DIR, 4>(a, block, narr, T)) return launch32<DIR, 4, kSweepTmaStride, NT, MB, true>(a, s, T);
    }
  }
  if constexpr (DIR == 1) {
    if (((MHD_SWEEP_TMA >> 1) & 1) && L <= kSweepTmaStride &&
        sweep32_smem_bytes(a.g.n[DIR], 4, kSweepTmaStride) <= kSweepSmemPerCta) {
      SweepTma T;
      if (sweep_tma_map<DIR, 4>(a, block, narr, T)) return launch32<DIR, 4, kSweepTmaStride, NT, MB, true>(a, s, T);
    }
  }
  if (MHD_SWEEP_MAX_PENCILS >= 4 && nb % 4 == 0 && L <= kSweepFixedStride &&
      sweep32_smem_bytes(a.g.n[DIR], 4, kSweepFixedStride) <= kSweepSmemPerCta)
    return launch32<DIR, 4, kSweepFixedStride, NT, MB>(a, s);
  if (L > kSweepFixedStride && L <= kSweepLongStride) {
    if constexpr (DIR != 0) {
      if (sweep32_smem_bytes(a.g.n[DIR], 4, kSweepLongStride) <= 226 * 1024)
        return launch32<DIR, 4, kSweepLongStride, MHD_SWEEP_LONG_THREADS, 1>(a, s);
    } else {
      if (nb % 2 == 0 && sweep32_smem_bytes(a.g.n[DIR], 2, kSweepLongStride) <= kSweepSmemPerCta)
        return launch32<DIR, 2, kSweepLongStride, NT, MB>(a, s);
    }
  }
  if (MHD_SWEEP_MAX_PENCILS >= 4 && nb % 4 == 0 && sweep32_smem_bytes(a.g.n[DIR], 4) <= kSweepSmemPerCta)
    return launch32<DIR, 4, 0, NT, MB>(a, s);
  if (nb % 2 == 0 && sweep32_smem_bytes(a.g.n[DIR], 2) <= kSweepSmemPerCta) return launch32<DIR, 2, 0, NT, MB>(a, s);
  if (sweep32_smem_bytes(a.g.n[DIR], 1) > 227 * 1024) return cudaErrorInvalidValue;
  return launch32<DIR, 1, 0, NT, MB>(a, s);
}

cudaError_t sweep_fp32(int dir, const SweepArgs &a, const double *block, int narr, cudaStream_t s) {
  if (dir == 0) return launch32_d<0>(a, block, narr, s);
  if (dir == 1) return launch32_d<1>(a, block, narr, s);
  return launch32_d<2>(a, block, narr, s);
}
int dt_screen_warps(const Grid &g) {
  const long long n = (long long)g.n[0] * g.n[1] * g.n[2];
  return (int)((n + 31) / 32);
}
cudaError_t dt_screen_fp32(const Grid &g, const Phys &ph, const Fields &f, const float *sh2, float *lo,
                           unsigned *words, int *err, cudaStream_t s) {
  long long n = (long long)g.n[0] * g.n[1] * g.n[2];
  // two cells per thread (a capped grid of 4864 blocks, ~13 cells per
  // thread and 50x fewer atomics, took 385 us at 256^3 against 333-358 for
  // one cell per thread)
  return dt_screen_fp32_range(g, ph, f, sh2, lo, words, err, 0, n, s);
}
cudaError_t dt_screen_fp32_range(const Grid &g, const Phys &ph, const Fields &f, const float *sh2, float *lo,
                                 unsigned *words, int *err, long long c0, long long c1, cudaStream_t s) {
  if (c0 % kDtScreenCells != 0) return cudaErrorInvalidValue;
  if (c1 <= c0) return cudaSuccess;
  DtScreen sc{lo, words, dt_screen_warps(g), (int)(c0 / kDtScreenCells)};
  dt32_screen_kernel<<<(unsigned)((c1 - c0 + kDtScreenCells - 1) / kDtScreenCells), kDtScreenThreads, 0, s>>>(
      g, ph, f, sh2, sc, err);
  return cudaGetLastError();
}

static unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

cudaError_t temp_fp32(const Grid &g, const Fields &f, const double *pin, double kb, float *T, float *sh2,
                      bool from_species, cudaStream_t s) {
  if (from_species) temp32_kernel<true><<<blocks_for(g.ncell, 512), 256, 0, s>>>(g.ncell, f, pin, d2f(kb), T, sh2);
  else temp32_kernel<false><<<blocks_for(g.ncell, 256), 256, 0, s>>>(g.ncell, f, pin, d2f(kb), T, sh2);
  return cudaGetLastError();
}

cudaError_t face_velocity_fp32(const Grid &g, const Fields &f, double *v0, double *v1, double *v2, cudaStream_t s) {
  long long n = (long long)(g.n[0] + 1) * (g.n[1] + 1) * (g.n[2] + 1);
  face_velocity32_kernel<<<blocks_for(n, 512), 256, 0, s>>>(g, f, v0, v1, v2);
  return cudaGetLastError();
}

cudaError_t ct_prep_fp32(const Grid &g, const Fields &f, double *const vf[3], double kb, const CT32Args &a,
                         cudaStream_t s) {
  ct_prep32_kernel<<<blocks_for(g.ncell, 512), 256, 0, s>>>(g.ncell, f, vf[0], vf[1], vf[2], d2f(kb), a);
  return cudaGetLastError();
}

template <int E>
static cudaError_t emf32_e(const CT32Args &a, cudaStream_t s) {
  const Grid &g = a.g;
  constexpr int da = E, db = (E + 1) % 3, dc = (E + 2) % 3;
  long long n = (long long)(g.n[da] + 1) * (g.n[db] + 1) * g.n[dc];
  // packed pairs: CT 2.09 -> 1.92 ms at 256^3 against the scalar kernel
  emf32x2_kernel<E><<<blocks_for(n, 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t emf32(int e, const CT32Args &a, cudaStream_t s) {
  if (e == 0) return emf32_e<0>(a, s);
  if (e == 1) return emf32_e<1>(a, s);
  return emf32_e<2>(a, s);
}

cudaError_t face_b_fp32(const Grid &g, const Fields &f, float *const emf[3], double dt, double *coef,
                        cudaStream_t s) {
  const int nc = g.s[0] + g.s[1] + g.s[2];
  ct_coef32_kernel<<<(nc + 255) / 256, 256, 0, s>>>(g, dt, coef);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  long long n = (long long)(g.n[0] + 1) * (g.n[1] + 1) * (g.n[2] + 1);
  face_b32_kernel<<<blocks_for(n, 256), 256, 0, s>>>(g, f, emf[0], emf[1], emf[2], coef);
  return cudaGetLastError();
}

cudaError_t chem_step_fp32(const Grid &g, const Phys &ph, const Fields &f, double dt, int *err, cudaStream_t s) {
  long long n = (long long)g.n[0] * g.n[1] * g.n[2];
  chem32_kernel<<<blocks_for(n, 128), 128, 0, s>>>(g, ph, f, d2f(dt), err);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(128) shield_tau32_kernel(Grid g, Phys ph, Fields f, double *tau) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)g.n[0] * g.n[1] * g.n[2]) return;
  shield_tau_cell<float>(g, ph, f, tau, t, [](double v) { return d2f(v); }, [](float v) { return f2d(v); });
}

cudaError_t shield_fp32(const Grid &g, const Phys &ph, const Fields &f, double *tau, double dxh, cudaStream_t s) {
  long long n = (long long)g.n[0] * g.n[1] * g.n[2];
  shield_tau32_kernel<<<blocks_for(n, 128), 128, 0, s>>>(g, ph, f, tau);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return shield_scan(g, f, tau, dxh, s);
}

cudaError_t source_fp32(const Source32Args &a, int stiff_mode, cudaStream_t s) {
  long long n = (long long)a.g.n[0] * a.g.n[1] * a.g.n[2];
  const unsigned nb = (unsigned)((n + 127) / 128);
  // the species cooling (ifchem = 2) runs with the bisection only (the
  // network and the Newton start model the KI function; mhd_create refuses
  // the combinations)
  if (a.ph.ifchem == 2) {
    source32_kernel<true, false><<<nb, 128, 0, s>>>(a);
    return cudaGetLastError();
  }
  if (stiff_mode == 0) {
    source32_kernel<false, false><<<nb, 128, 0, s>>>(a);
    return cudaGetLastError();
  }
  // guess and polish: the explicit cells in a full-occupancy pass that lists
  // the stiff ones, then the stiff cells in dense tiles
  if (!a.stiff_list || !a.stiff_count || (stiff_mode == STIFF_NETWORK && !a.W)) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(a.stiff_count, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  source32_kernel<false, true><<<(unsigned)((n + kSourceDeferThreads - 1) / kSourceDeferThreads),
                                 kSourceDeferThreads, 0, s>>>(a);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // a persistent grid over the list, at most three 256-cell CTAs per SM (the
  // launch bounds; with the network their TMEM, 128 columns each, fits in
  // the SM's 512); CTAs beyond the list's length return at once
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned grid = (unsigned)std::min<long long>((n + kFusedThreads - 1) / kFusedThreads, 3LL * sms);
  if (stiff_mode == STIFF_NETWORK)
    source32_stiff_kernel<STIFF_NETWORK><<<grid, kFusedThreads, sizeof(SurTileSmem<kFusedTiles>), s>>>(a);
  else
    source32_stiff_kernel<STIFF_NEWTON><<<grid, kFusedThreads, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace mhd
