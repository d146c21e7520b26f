// mhd_noalloc.cu — the time-step limits without any device allocation.
//
// mhd_timestep works on a handle, and a handle allocates the resident state
// and its scratch with cudaMalloc.  Some callers cannot do that: a Fortran
// or C++ code that already owns every device array through its own memory
// pool (an arena carved out once at start-up, or memory handed to it by a
// host framework), or a caller that is inside a region where new device
// allocations are not allowed.  mhd_timestep_noalloc serves them: the
// caller passes device pointers to arrays it already has, and the kernel's
// scratch (per-block partial minima, the error word and the two results)
// lives in the file-scope array below, which every GPU that loads this
// library holds until the process exits.  Nothing here calls cudaMalloc,
// cudaFree or any allocating library routine.
//
// The arithmetic per cell is cell_dt_limits, the device function dt_kernel
// uses, and this unit is built with --fmad=false like the FP64 kernels, so
// the result equals mhd_timestep's bit for bit.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "../../include/mhd_gb300.h"
#include "mhd_kernels.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = MHD_NOALLOC_MAX_CELLS / kThreads;
// layout: [0, kMaxBlocks) tCFL partials, [kMaxBlocks, 2 kMaxBlocks) tLMT
// partials, then the error word and the two reduced results
constexpr int kErrWord = 2 * kMaxBlocks;
constexpr int kResult = 2 * kMaxBlocks + 1;
static __device__ __align__(256) unsigned long long g_dt_scratch[2 * kMaxBlocks + 4];

constexpr int kMaxDevices = 64;
unsigned long long *g_scratch_addr[kMaxDevices];
std::once_flag g_scratch_once[kMaxDevices];
cudaError_t g_scratch_status[kMaxDevices];

__device__ __forceinline__ unsigned long long bits_of(double v) {
  return (unsigned long long)__double_as_longlong(v > 0.0 ? v : 0.0);
}

__device__ __forceinline__ void block_min2(unsigned long long &a, unsigned long long &b) {
  __shared__ unsigned long long wa[32], wb[32];
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long x = __shfl_xor_sync(0xffffffffu, a, o), y = __shfl_xor_sync(0xffffffffu, b, o);
    a = x < a ? x : a;
    b = y < b ? y : b;
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { wa[w] = a; wb[w] = b; }
  __syncthreads();
  if (w == 0) {
    int nw = (blockDim.x + 31) >> 5;
    a = lane < nw ? wa[lane] : ~0ull;
    b = lane < nw ? wb[lane] : ~0ull;
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long x = __shfl_xor_sync(0xffffffffu, a, o), y = __shfl_xor_sync(0xffffffffu, b, o);
      a = x < a ? x : a;
      b = y < b ? y : b;
    }
  }
}

// stage 1: one partial (tCFL, tLMT) per block, written (not accumulated)
__global__ void __launch_bounds__(kThreads) dt_partial_kernel(mhd::Grid g, mhd::Phys ph, mhd::Fields f,
                                                              unsigned long long *scratch) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double c_min = ph.tfinal, s_min = ph.tfinal;
  if (t < (long long)g.n[0] * g.n[1] * g.n[2]) {
    mhd::cell_dt_limits(g, ph, f, t, c_min, s_min);
    if (!(c_min > 0.0) || !(s_min > 0.0)) atomicOr(&scratch[kErrWord], (unsigned long long)mhd::ERRB_DT);
  }
  unsigned long long a = bits_of(c_min), b = bits_of(s_min);
  block_min2(a, b);
  if (threadIdx.x == 0) {
    scratch[blockIdx.x] = a;
    scratch[kMaxBlocks + blockIdx.x] = b;
  }
}

// stage 2: one block folds the partials of this call
__global__ void __launch_bounds__(1024) dt_final_kernel(unsigned long long *scratch, int nblocks) {
  unsigned long long a = ~0ull, b = ~0ull;
  for (int q = threadIdx.x; q < nblocks; q += blockDim.x) {
    unsigned long long x = scratch[q], y = scratch[kMaxBlocks + q];
    a = x < a ? x : a;
    b = y < b ? y : b;
  }
  block_min2(a, b);
  if (threadIdx.x == 0) {
    scratch[kResult] = a;
    scratch[kResult + 1] = b;
  }
}

// Set-up, once per device with that device current: the device address of
// g_dt_scratch.  In host code the symbol's name is only a host-side stand-in,
// so kernels get this address instead.
cudaError_t scratch_address(int device, unsigned long long **out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::call_once(g_scratch_once[device], [device]() {
    void *p = nullptr;
    g_scratch_status[device] = cudaGetSymbolAddress(&p, g_dt_scratch);
    g_scratch_addr[device] = static_cast<unsigned long long *>(p);
  });
  *out = g_scratch_addr[device];
  return g_scratch_status[device];
}

}  // namespace

extern "C" int mhd_timestep_noalloc(const mhd_params *p, const mhd_device_state *s, double *dt, int *st,
                                    void *stream) {
  if (!p || !s || !dt || !st || !s->U || !s->species || !s->bcc || !s->dx || !s->dy || !s->dz)
    return MHD_ERR_ARG;
  if (p->nx < 1 || p->ny < 1 || p->nz < 1) return MHD_ERR_ARG;
  if (p->precision != MHD_PREC_FP64 && p->precision != MHD_PREC_FP32) return MHD_ERR_ARG;
  if (p->ifchem != 0 && p->ifchem != 2) return MHD_ERR_ARG;
  if (p->ifrad != 0 && p->ifrad != 2) return MHD_ERR_ARG;
  // the species cooling reads the chemistry's electron and particle
  // densities, and with ifrad = 2 SHIELD's columns too
  if (p->ifchem == 2 && (!s->nde || !s->ndtot)) return MHD_ERR_ARG;
  if (p->ifchem == 2 && p->ifrad == 2 && !s->columns) return MHD_ERR_ARG;
  long long ncells = (long long)p->nx * p->ny * p->nz;
  if (ncells > MHD_NOALLOC_MAX_CELLS) return MHD_ERR_TOO_LARGE;
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(p->device) != cudaSuccess) {
    cudaGetLastError();
    return MHD_ERR_NO_DEVICE;
  }
  int rc = MHD_OK;
  cudaStream_t sm = static_cast<cudaStream_t>(stream);
  unsigned long long *scratch = nullptr;
  do {
    if (scratch_address(p->device, &scratch) != cudaSuccess || !scratch) { rc = MHD_ERR_CUDA; break; }
    mhd::Grid g{};
    g.n[0] = p->nx; g.n[1] = p->ny; g.n[2] = p->nz;
    for (int d = 0; d < 3; d++) g.s[d] = g.n[d] + 4;
    g.st[0] = 1; g.st[1] = g.s[0]; g.st[2] = (long long)g.s[0] * g.s[1];
    g.ncell = (long long)g.s[0] * g.s[1] * g.s[2];
    g.dx[0] = s->dx; g.dx[1] = s->dy; g.dx[2] = s->dz;
    mhd::Phys ph{};
    ph.kb = p->kb; ph.kcond = p->kcond; ph.tfinal = p->tfinal; ph.ifthrm = p->ifthrm;
    ph.ifchem = p->ifchem; ph.ifrad = p->ifrad;
    mhd::Fields f{};
    for (int q = 0; q < 8; q++) {
      f.U[q] = const_cast<double *>(s->U) + q * g.ncell;
      f.sp[q] = const_cast<double *>(s->species) + q * g.ncell;
    }
    for (int c = 0; c < 3; c++) f.bcc[c] = const_cast<double *>(s->bcc) + c * g.ncell;
    if (p->ifchem == 2) {
      f.nde = const_cast<double *>(s->nde);
      f.ndtot = const_cast<double *>(s->ndtot);
      if (p->ifrad == 2)
        for (int q = 0; q < 10; q++) f.col[q] = const_cast<double *>(s->columns) + q * g.ncell;
    }
    // the error word must start at zero; partials and results are overwritten
    if (cudaMemsetAsync(scratch + kErrWord, 0, sizeof(unsigned long long), sm) != cudaSuccess) { rc = MHD_ERR_CUDA; break; }
    int nblocks = (int)((ncells + kThreads - 1) / kThreads);
    dt_partial_kernel<<<nblocks, kThreads, 0, sm>>>(g, ph, f, scratch);
    dt_final_kernel<<<1, 1024, 0, sm>>>(scratch, nblocks);
    if (cudaGetLastError() != cudaSuccess) { rc = MHD_ERR_CUDA; break; }
    unsigned long long out[3];
    if (cudaMemcpyAsync(out, scratch + kErrWord, sizeof out, cudaMemcpyDeviceToHost, sm) != cudaSuccess ||
        cudaStreamSynchronize(sm) != cudaSuccess) { rc = MHD_ERR_CUDA; break; }
    if (out[0] & mhd::ERRB_DT) { rc = MHD_ERR_DT; break; }
    double tcfl, tlmt;
    memcpy(&tcfl, &out[1], sizeof tcfl);
    memcpy(&tlmt, &out[2], sizeof tlmt);
    // EVOLVE:569-596 with one rank, as in mhd_timestep
    double d = p->tfinal;
    double c = p->cfl * tcfl;
    d = (c < d) ? c : d;
    int lim = 1;
    if (p->ifthrm == 2) {
      double stt = d;
      d = (tlmt < d) ? tlmt : d;
      if (d < stt) lim = 2;
    }
    d = (d < p->tfinal) ? d : p->tfinal;
    if (!(d > 0.0)) { rc = MHD_ERR_DT; break; }
    *dt = d;
    *st = lim;
  } while (0);
  cudaSetDevice(prev);
  return rc;
}
