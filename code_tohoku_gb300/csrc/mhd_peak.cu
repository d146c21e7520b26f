// mhd_peak.cu — measured FP64 throughput of the device: the denominator of
// the plain FP64 path's roofline.  GB300's FP64 rate is a small fraction of
// its FP32 rate, so the plain form is bound by the FP64 pipe rather than by
// HBM; these kernels measure that pipe instead of quoting a datasheet.
//
// Each thread runs eight independent dependent chains (enough to hide the
// pipe's latency at eight warps per SM); the chains stay bounded, and their
// sum is stored only if it equals a value it cannot reach, which keeps the
// compiler from removing the loop.  Timed with CUDA events on a private
// stream after one warm-up launch; the best of three launches is returned.
#include <cuda_runtime.h>

#include "../../include/mhd_gb300.h"

namespace {

constexpr int kChains = 8;

__global__ void fma_chain_kernel(double *sink, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = 1.0 + 1e-3 * (threadIdx.x + c);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  if (s == -1.0) sink[blockIdx.x] = s;
}

__global__ void div_chain_kernel(double *sink, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = 1.0 + 1e-3 * (threadIdx.x + c);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = a / (x[c] + b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  if (s == -1.0) sink[blockIdx.x] = s;
}

__global__ void sqrt_chain_kernel(double *sink, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = 1.0 + 1e-3 * (threadIdx.x + c);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = sqrt(a * x[c] + b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  if (s == -1.0) sink[blockIdx.x] = s;
}

template <class K>
cudaError_t best_ms(K kernel, int blocks, int threads, int iters, double a, double b, double *sink,
                    cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1, float *out) {
  kernel<<<blocks, threads, 0, s>>>(sink, iters, a, b);   // warm-up
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  float best = 1e30f;
  for (int r = 0; r < 3; r++) {
    cudaEventRecord(e0, s);
    kernel<<<blocks, threads, 0, s>>>(sink, iters, a, b);
    cudaEventRecord(e1, s);
    if ((e = cudaEventSynchronize(e1)) != cudaSuccess) return e;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  *out = best;
  return cudaGetLastError();
}

}  // namespace

extern "C" int mhd_fp64_peak(int device, double *fma_gflops, double *div_gps, double *sqrt_gps) {
  if (!fma_gflops || !div_gps || !sqrt_gps) return MHD_ERR_ARG;
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return MHD_ERR_NO_DEVICE;
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int threads = 256, blocks = 4 * (sms > 0 ? sms : 1);   // eight warps per SM
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double *sink = nullptr;
  int rc = MHD_OK;
  float ms_fma = 0.f, ms_div = 0.f, ms_sqrt = 0.f;
  const int it_fma = 4096, it_div = 256, it_sqrt = 256;
  do {
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess || cudaMalloc(&sink, blocks * sizeof(double)) != cudaSuccess) {
      rc = MHD_ERR_CUDA;
      break;
    }
    if (best_ms(fma_chain_kernel, blocks, threads, it_fma, 0.9999999, 1e-7, sink, s, e0, e1, &ms_fma) != cudaSuccess ||
        best_ms(div_chain_kernel, blocks, threads, it_div, 1.5, 0.25, sink, s, e0, e1, &ms_div) != cudaSuccess ||
        best_ms(sqrt_chain_kernel, blocks, threads, it_sqrt, 0.5, 0.75, sink, s, e0, e1, &ms_sqrt) != cudaSuccess) {
      rc = MHD_ERR_CUDA;
      break;
    }
    const double ops = (double)blocks * threads * kChains;
    *fma_gflops = 2.0 * ops * it_fma / (ms_fma * 1e-3) / 1e9;
    *div_gps = ops * it_div / (ms_div * 1e-3) / 1e9;
    *sqrt_gps = ops * it_sqrt / (ms_sqrt * 1e-3) / 1e9;
  } while (0);
  if (sink) cudaFree(sink);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  cudaSetDevice(prev);
  return rc;
}
