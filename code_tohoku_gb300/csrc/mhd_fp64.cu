// mhd_fp64.cu — plain form: every operation in FP64.  This unit is built
// with --fmad=false so each a*b+c is two IEEE roundings, the arithmetic of
// the reference Fortran and of the CPU restatement; with the shared
// detmath.h transcendentals the GPU result is bit-identical to the CPU.
// It also holds the precision-independent kernels (ghosts, CT face update,
// source, dt, DISSIP, diagnostics).
#include <algorithm>
#define MHD_COMMON_KERNELS
#include "mhd_sweep_impl.cuh"

namespace mhd {

int sweep_batch(const Grid &g, int dir) {
  int nb = (dir == 0) ? g.n[1] : g.n[0];
  int maxP = (dir == 0) ? 2 : 4;
  for (int P = maxP; P > 1; P >>= 1)
    if (nb % P == 0 && sweep_smem_bytes(g, dir, P) <= 227 * 1024) return P;
  return 1;
}

size_t sweep_smem_bytes(const Grid &g, int dir, int P) {
  return (size_t)B_COUNT * (size_t)(g.n[dir] + 4) * (size_t)P * sizeof(double);
}

cudaError_t sweep_fp64(int dir, const SweepArgs &a, cudaStream_t s) { return launch_sweep<double>(dir, a, s); }
cudaError_t emf_fp64(int e, const CTArgs &a, cudaStream_t s) { return launch_emf<double>(e, a, s); }

static unsigned nblk(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

cudaError_t ghost_fill_all(const Grid &g, const FillArgs &f, int dirs, int nol, cudaStream_t s) {
  return ghost_fill_slab(g, f, dirs, nol, -1, 0, 0, false, s);
}

cudaError_t ghost_fill_slab(const Grid &g, const FillArgs &f, int dirs, int nol, int rdim, int rlo, int rhi,
                            bool outside, cudaStream_t s) {
  FillAll r{};
  r.rdim = rdim;
  r.rlo = rlo;
  r.rhi = rhi;
  r.rout = outside ? 1 : 0;
  const bool mk[3] = {(dirs & 1) != 0, (dirs & 2) != 0, (dirs & 4) != 0};
  for (int reg = 0; reg < 3; reg++) {
    if (!mk[reg]) continue;
    long long n = 1;
    for (int d = 0; d < 3; d++)
      n *= d < reg ? (g.s[d] - (mk[d] ? 2 * nol : 0)) : (d == reg ? 2 * nol : g.s[d]);
    r.nreg[reg] = n;
  }
  const long long n = (r.nreg[0] + r.nreg[1] + r.nreg[2]) * f.nf;
  if (n == 0) return cudaSuccess;
  ghost_fill_all_kernel<<<nblk(n, 256), 256, 0, s>>>(g, f, dirs, nol, r);
  return cudaGetLastError();
}


cudaError_t face_velocity(const Grid &g, const Fields &f, double *v0, double *v1, double *v2, cudaStream_t s) {
  long long n = (long long)(g.n[0] + 1) * (g.n[1] + 1) * (g.n[2] + 1);
  face_velocity_kernel<<<nblk(n, 256), 256, 0, s>>>(g, f, v0, v1, v2);
  return cudaGetLastError();
}

cudaError_t face_b(const Grid &g, const Fields &f, const double *ez, const double *ex, const double *ey, double dt,
                   cudaStream_t s) {
  long long n = (long long)(g.n[0] + 1) * (g.n[1] + 1) * (g.n[2] + 1);
  face_b_kernel<<<nblk(n, 256), 256, 0, s>>>(g, f, ez, ex, ey, dt);
  return cudaGetLastError();
}

cudaError_t cell_b(const Grid &g, const Fields &f, cudaStream_t s) {
  return cell_b_range(g, f, 0, (long long)g.n[0] * g.n[1] * g.n[2], s);
}

cudaError_t shell_copy(const Grid &g, const double *src, double *dst, int lay, cudaStream_t s) {
  if (lay != 1 && lay != 2) return cudaErrorInvalidValue;
  const long long n = 2 * ((long long)g.s[1] * g.s[2] + (long long)g.s[0] * g.s[2] + (long long)g.s[0] * g.s[1]);
  shell_copy_kernel<<<nblk(n, 256), 256, 0, s>>>(g, src, dst, lay);
  return cudaGetLastError();
}

cudaError_t cell_b_range(const Grid &g, const Fields &f, long long c0, long long c1, cudaStream_t s) {
  if (c1 <= c0) return cudaSuccess;
  cell_b_kernel<<<nblk(c1 - c0, 512), 256, 0, s>>>(g, f, c0, c1);
  return cudaGetLastError();
}

cudaError_t source_pass(const SourceArgs &a, cudaStream_t s) {
  long long n = (long long)a.g.n[0] * a.g.n[1] * a.g.n[2];
  source_kernel<<<nblk(n, 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t chem_step(const Grid &g, const Phys &ph, const Fields &f, double dt, int *err, cudaStream_t s) {
  long long n = (long long)g.n[0] * g.n[1] * g.n[2];
  chem_kernel<<<nblk(n, 128), 128, 0, s>>>(g, ph, f, dt, err);
  return cudaGetLastError();
}

cudaError_t shield(const Grid &g, const Phys &ph, const Fields &f, double *tau, double dxh, cudaStream_t s) {
  long long n = (long long)g.n[0] * g.n[1] * g.n[2];
  shield_tau_kernel<<<nblk(n, 128), 128, 0, s>>>(g, ph, f, tau);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return shield_scan(g, f, tau, dxh, s);
}

cudaError_t shield_scan(const Grid &g, const Fields &f, const double *tau, double dxh, cudaStream_t s) {
  long long n = (long long)g.n[1] * g.n[2];
  shield_scan_kernel<<<nblk(n, 128), 128, 0, s>>>(g, f, tau, dxh);
  return cudaGetLastError();
}

cudaError_t chem_totals(const Grid &g, const Fields &f, int plus, cudaStream_t s) {
  long long n = (long long)(g.n[0] + plus) * (g.n[1] + plus) * (g.n[2] + plus);
  chem_totals_kernel<<<nblk(n, 256), 256, 0, s>>>(g, f, plus);
  return cudaGetLastError();
}

cudaError_t dt_reduce(const Grid &g, const Phys &ph, const Fields &f, unsigned long long *out, int *err,
                      cudaStream_t s) {
  long long n = (long long)g.n[0] * g.n[1] * g.n[2];
  dt_kernel<<<nblk(n, 256), 256, 0, s>>>(g, ph, f, out, err);
  return cudaGetLastError();
}

cudaError_t dt_refine(const Grid &g, const Phys &ph, const Fields &f, const float *lo, const unsigned *words,
                      unsigned long long *out, cudaStream_t s) {
  long long n = (long long)g.n[0] * g.n[1] * g.n[2];
  const int nwarps = (int)((n + 31) / 32);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // a warp checks 32 of the screen's warps per trip: two 256-thread blocks
  // per SM at most, fewer for small grids
  const unsigned blocks = (unsigned)std::min<long long>((nwarps + 255) / 256, 2LL * (sms > 0 ? sms : 1));
  dt_refine_kernel<<<blocks, 256, 0, s>>>(g, ph, f, lo, words, nwarps, out);
  return cudaGetLastError();
}

cudaError_t divv(const Grid &g, const Fields &f, double *d, cudaStream_t s) {
  long long n = 2LL * 12 * (g.n[1] + 2) * (g.n[2] + 2);
  divv_kernel<<<nblk(n, 256), 256, 0, s>>>(g, f, d);
  return cudaGetLastError();
}

cudaError_t dissip(const Grid &g, const Fields &f, const double *d, int e, cudaStream_t s) {
  long long n = 10LL * g.n[1] * g.n[2];
  dissip_kernel<<<nblk(n, 256), 256, 0, s>>>(g, f, d, e);
  return cudaGetLastError();
}

cudaError_t diag(const Grid &g, const Phys &ph, const Fields &f, double *part, int *nblocks, cudaStream_t s) {
  long long n = (long long)g.n[0] * g.n[1] * g.n[2];
  *nblocks = (int)nblk(n, 256);
  diag_kernel<<<*nblocks, 256, 0, s>>>(g, ph, f, part);
  return cudaGetLastError();
}

}  // namespace mhd
