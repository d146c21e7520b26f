// mhd_fp32.cu — chosen form: reconstruction, Riemann solver, characteristic
// and EMF arithmetic in FP32; accumulation into the FP64 state.  Built with
// the default contraction (FMA) enabled.
#define MHD_FP32_KERNELS
#include "mhd_sweep32.cuh"
#include "mhd_source32.cuh"
#include "mhd_sweep_impl.cuh"

namespace mhd {
template <int DIR, int P>
static cudaError_t launch32(const SweepArgs &a, cudaStream_t s) {
  const Grid &g = a.g;
  size_t smem = sweep32_smem_bytes(g.n[DIR], P);
  auto k = sweep32_kernel<DIR, P, 512>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid;
  if (DIR == 0) grid = dim3(g.n[1] / P, g.n[2]);
  else if (DIR == 1) grid = dim3(g.n[0] / P, g.n[2]);
  else grid = dim3(g.n[0] / P, g.n[1]);
  k<<<grid, 512, smem, s>>>(a);
  return cudaGetLastError();
}

template <int DIR>
static cudaError_t launch32_d(const SweepArgs &a, cudaStream_t s) {
  int nb = (DIR == 0) ? a.g.n[1] : a.g.n[0];
  size_t lim = 227 * 1024;
  if (nb % 4 == 0 && sweep32_smem_bytes(a.g.n[DIR], 4) <= lim) return launch32<DIR, 4>(a, s);
  if (nb % 2 == 0 && sweep32_smem_bytes(a.g.n[DIR], 2) <= lim) return launch32<DIR, 2>(a, s);
  return launch32<DIR, 1>(a, s);
}

cudaError_t sweep_fp32(int dir, const SweepArgs &a, cudaStream_t s) {
  if (dir == 0) return launch32_d<0>(a, s);
  if (dir == 1) return launch32_d<1>(a, s);
  return launch32_d<2>(a, s);
}
cudaError_t emf_fp32(int e, const CTArgs &a, cudaStream_t s) { return launch_emf<float>(e, a, s); }
cudaError_t source_fp32(const Source32Args &a, cudaStream_t s) {
  long long n = (long long)a.g.n[0] * a.g.n[1] * a.g.n[2];
  source32_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace mhd
