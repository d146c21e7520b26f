// mhd_sweep_impl.cuh — launch helpers instantiated once per precision unit.
#pragma once
#include "mhd_launch.h"

namespace mhd {

template <int DIR, int P, class R>
static cudaError_t launch_sweep_dp(const SweepArgs &a, cudaStream_t s) {
  const Grid &g = a.g;
  size_t smem = sweep_smem_bytes(g, DIR, P);
  auto k = sweep_kernel<DIR, P, R>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid;
  if (DIR == 0) grid = dim3(g.n[1] / P, g.n[2]);
  else if (DIR == 1) grid = dim3(g.n[0] / P, g.n[2]);
  else grid = dim3(g.n[0] / P, g.n[1]);
  k<<<grid, 256, smem, s>>>(a);
  return cudaGetLastError();
}

template <int DIR, class R>
static cudaError_t launch_sweep_d(const SweepArgs &a, cudaStream_t s) {
  int P = sweep_batch(a.g, DIR);
  if (P == 4) return launch_sweep_dp<DIR, 4, R>(a, s);
  if (P == 2) return launch_sweep_dp<DIR, 2, R>(a, s);
  return launch_sweep_dp<DIR, 1, R>(a, s);
}

template <class R>
static cudaError_t launch_sweep(int dir, const SweepArgs &a, cudaStream_t s) {
  if (dir == 0) return launch_sweep_d<0, R>(a, s);
  if (dir == 1) return launch_sweep_d<1, R>(a, s);
  return launch_sweep_d<2, R>(a, s);
}

template <int E, class R>
static cudaError_t launch_emf_e(const CTArgs &a, cudaStream_t s) {
  const Grid &g = a.g;
  int da = E, db = (E + 1) % 3, dc = (E + 2) % 3;
  long long n = (long long)(g.n[da] + 1) * (g.n[db] + 1) * g.n[dc];
  int bs = 128;
  emf_kernel<E, R><<<(unsigned)((n + bs - 1) / bs), bs, 0, s>>>(a);
  return cudaGetLastError();
}

template <class R>
static cudaError_t launch_emf(int e, const CTArgs &a, cudaStream_t s) {
  if (e == 0) return launch_emf_e<0, R>(a, s);
  if (e == 1) return launch_emf_e<1, R>(a, s);
  return launch_emf_e<2, R>(a, s);
}

}  // namespace mhd
