// mhd_surrogate_net.cuh — the KI-cooling surrogate network on tensor cores.
//
// The stiff branch of SOURCE solves P + Lambda(P) dt (gamma-1) = P_old by a
// 30-step log-space bisection (IMC, MCF3DSGincfca3.f90:2898-2921).  Written
// in temperature, the solution depends only on
//   x0 = log10 N      (N = rho/1.27, the KI cooling density)
//   x1 = log10 T      (T in 1e3 K at the start of the solve)
//   x2 = log10(dt/t_cool),  t_cool = P/((gamma-1)|Lambda|)
// and the network maps (x0,x1,x2) -> (log10(T_new/T), c), where c is a
// learned estimate of log10 of its own error.  Layers 3->64->64->2 with SiLU;
// the 64-wide layers run on the fifth-generation tensor cores (tcgen05.mma
// kind::f16, BF16 operands in shared memory, FP32 accumulators in tensor
// memory), layer 1 and the biases in FP32 on the CUDA cores.  Inference
// (below) and the training gradients (mhd_surrogate.cu) use the same
// operand layout and rounding points.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "mhd_tc.cuh"

namespace mhd {

constexpr int SUR_H = 64;           // hidden width
constexpr int SUR_NPARAM = 64 * 3 + 64 + 64 * 64 + 64 + 2 * 64 + 2;   // FP32 master parameters
// offsets in the FP32 master vector: W1[64][3], b1, W2[64][64], b2, W3[2][64], b3
constexpr int SUR_OW1 = 0, SUR_OB1 = 192, SUR_OW2 = 256, SUR_OB2 = 256 + 4096, SUR_OW3 = SUR_OB2 + 64,
              SUR_OB3 = SUR_OW3 + 128;

// input normalisation: box [-2,5] x [-2, log10 20] x [-3,3] -> [-1,1]^3
constexpr float SUR_C0 = 1.5f, SUR_S0 = 3.5f;
constexpr float SUR_C1 = -0.3494850f, SUR_S1 = 1.6505150f;
constexpr float SUR_C2 = 0.0f, SUR_S2 = 3.0f;

// packed device copy used by the kernels
struct SurNet {
  __nv_bfloat16 W1[64 * 16];    // [out][in padded to 16]
  __nv_bfloat16 W2[64 * 64];    // [out][in]
  __nv_bfloat16 W3[8 * 64];     // [out padded to 8][in]
  float b1[64], b2[64], b3[8];
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
__device__ __forceinline__ float dsilu(float z) {
  float s = sigm(z);
  return s * (1.0f + z * (1.0f - s));
}

// SiLU of two accumulator entries, packed as the BF16 pair of the next A
// fragment: s = z/2 rounded to BF16, then s + s tanh(s) on the BF16 pair
// (one tanh approximation for both entries).
__device__ __forceinline__ uint32_t silu2_bf16(float z0, float z1) {
  const uint32_t h = pack_bf16(0.5f * z0, 0.5f * z1);
  uint32_t th, r;
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(th) : "r"(h));
  asm("fma.rn.bf16x2 %0, %1, %2, %1;" : "=r"(r) : "r"(h), "r"(th));
  return r;
}

// ---------------------------------------------------------------------
// Inference on the fifth-generation tensor cores (tcgen05), for SOURCE's
// stiff cells: a CTA of 128 * NT threads holds NT tiles of 128 cells, one
// cell per thread (row r = threadIdx.x % 128 of tile threadIdx.x / 128).
// Layer 1 (3 inputs) runs on the CUDA cores in FP32 and writes SiLU(z1) as
// the BF16 A operand of layer 2 into shared memory; one thread issues the
// 64 x 64 layer of every tile (M = 128, N = 64, K = 4 x 16) and the 64 -> 2
// output layer (N padded to 16) as tcgen05.mma with the FP32 accumulators
// in tensor memory (64 columns per tile, reused by the output layer);
// every thread reads its row back with tcgen05.ld, adds the bias and applies
// SiLU for the next layer: silu2_bf16 above.

template <int NT>
struct SurTileSmem {
  __nv_bfloat16 A[NT][128 * 64];   // activations, K-major core-matrix layout (16 KB per tile)
  __nv_bfloat16 W2[64 * 64];       // [out][in], the same layout
  __nv_bfloat16 W3[16 * 64];       // [out padded to 16][in]
  float4 w1[64];                   // (w0, w1, w2, b1) of hidden unit n
  float b2[64], b3[16];
  uint64_t bar;                    // MMA completion
  uint32_t tmem;                   // TMEM base address (64 columns per tile)
  int broken;                      // a wait timed out: the network is off for the rest of the kernel
};

constexpr uint32_t kSurTmemCols = 64;

// stage the weights (all threads), initialise the mbarrier and allocate
// TMEM (warp 0); ends with a barrier
template <int NT>
__device__ __forceinline__ void sur_tile_setup(const SurNet *net, SurTileSmem<NT> *s) {
  char *w2 = reinterpret_cast<char *>(s->W2), *w3 = reinterpret_cast<char *>(s->W3);
  for (int q = threadIdx.x; q < 64 * 64; q += blockDim.x) {
    const int n = q >> 6, k = q & 63;
    *reinterpret_cast<__nv_bfloat16 *>(w2 + tc::kmajor_off(n, k, 64)) = net->W2[q];
  }
  for (int q = threadIdx.x; q < 16 * 64; q += blockDim.x) {
    const int n = q >> 6, k = q & 63;
    *reinterpret_cast<__nv_bfloat16 *>(w3 + tc::kmajor_off(n, k, 64)) =
        n < 8 ? net->W3[q] : __float2bfloat16_rn(0.0f);
  }
  for (int q = threadIdx.x; q < 64; q += blockDim.x) {
    const __nv_bfloat16 *w = net->W1 + q * 16;
    s->w1[q] = make_float4(__bfloat162float(w[0]), __bfloat162float(w[1]), __bfloat162float(w[2]), net->b1[q]);
    s->b2[q] = net->b2[q];
  }
  for (int q = threadIdx.x; q < 16; q += blockDim.x) s->b3[q] = q < 8 ? net->b3[q] : 0.0f;
  if (threadIdx.x == 0) {
    tc::mbar_init(&s->bar, 1);
    s->broken = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) tc::tmem_alloc(&s->tmem, NT * kSurTmemCols);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

// free TMEM (warp 0) once no tensor-core work of this CTA is in flight:
// phase is the parity of the next (or, after a timed-out wait, the still
// outstanding) completion, which gets one more bounded wait first
template <int NT>
__device__ __forceinline__ void sur_tile_teardown(SurTileSmem<NT> *s, uint32_t phase) {
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (s->broken && threadIdx.x == 0) tc::mbar_wait(&s->bar, phase);
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_free(s->tmem, NT * kSurTmemCols);
  if (threadIdx.x == 0) tc::mbar_inval(&s->bar);
}

// one thread: the 4 K-steps of a layer for every tile, then one commit
template <int NT>
__device__ __forceinline__ void sur_tile_issue(SurTileSmem<NT> *s, const __nv_bfloat16 *B, int N) {
  tc::fence_after_sync();
  const uint32_t idesc = tc::idesc_bf16_f32(128, N);
  const uint32_t bbase = tc::smem_u32(B);
#pragma unroll
  for (int tl = 0; tl < NT; tl++) {
    const uint32_t abase = tc::smem_u32(s->A[tl]);
#pragma unroll
    for (int kk = 0; kk < 4; kk++)
      tc::mma_bf16(s->tmem + tl * kSurTmemCols, tc::smem_desc(abase + 256 * kk, 128, 1024),
                   tc::smem_desc(bbase + 256 * kk, 128, 1024), idesc, kk > 0);
  }
  tc::mma_commit(&s->bar);
}

// Forward pass of every tile of the CTA; all threads call.  n0..n2: this
// thread's normalised inputs (any finite values on rows without a cell).
// Returns false (on every thread) when a wait timed out; y0, y1 are then
// not set.
template <int NT>
__device__ __forceinline__ bool sur_tile_forward(SurTileSmem<NT> *s, float n0, float n1, float n2, uint32_t &phase,
                                                 float &y0, float &y1) {
  const int r = threadIdx.x & 127, tl = threadIdx.x >> 7, w = (threadIdx.x >> 5) & 3;
  char *arow = reinterpret_cast<char *>(s->A[tl]);
  // layer 1 on the CUDA cores: 8 chunks of 8 hidden units, one 16-byte store each
#pragma unroll
  for (int kc = 0; kc < 8; kc++) {
    uint32_t p[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const float4 a = s->w1[8 * kc + 2 * q], b = s->w1[8 * kc + 2 * q + 1];
      // explicit FMAs: the same bits in every translation unit, whatever its contraction flag
      p[q] = silu2_bf16(__fmaf_rn(a.z, n2, __fmaf_rn(a.y, n1, __fmaf_rn(a.x, n0, a.w))),
                        __fmaf_rn(b.z, n2, __fmaf_rn(b.y, n1, __fmaf_rn(b.x, n0, b.w))));
    }
    *reinterpret_cast<uint4 *>(arow + tc::kmajor_off(r, 8 * kc, 64)) = make_uint4(p[0], p[1], p[2], p[3]);
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x == 0 && !s->broken) sur_tile_issue(s, s->W2, 64);
  bool ok = !s->broken && tc::mbar_wait(&s->bar, phase);
  if (!__syncthreads_and(ok)) {
    if (threadIdx.x == 0) s->broken = 1;
    return false;
  }
  phase ^= 1u;
  tc::fence_after_sync();
  // layer 2: accumulators back, bias, SiLU, BF16 A operand of the output layer
  const uint32_t taddr = s->tmem + tl * kSurTmemCols + ((uint32_t)(w * 32) << 16);
  // 16 columns at a time keeps 16 accumulator registers live, not 64
#pragma unroll
  for (int cc = 0; cc < 4; cc++) {
    float v[16];
    tc::tmem_ld16(taddr + 16 * cc, v);
    tc::tmem_wait_ld();
#pragma unroll
    for (int hlf = 0; hlf < 2; hlf++) {
      uint32_t p[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int k = 16 * cc + 8 * hlf + 2 * q;
        p[q] = silu2_bf16(v[8 * hlf + 2 * q] + s->b2[k], v[8 * hlf + 2 * q + 1] + s->b2[k + 1]);
      }
      *reinterpret_cast<uint4 *>(arow + tc::kmajor_off(r, 16 * cc + 8 * hlf, 64)) = make_uint4(p[0], p[1], p[2], p[3]);
    }
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  // output layer into the same TMEM columns (their values are read)
  if (threadIdx.x == 0) sur_tile_issue(s, s->W3, 16);
  ok = tc::mbar_wait(&s->bar, phase);
  if (!__syncthreads_and(ok)) {
    if (threadIdx.x == 0) s->broken = 1;
    return false;
  }
  phase ^= 1u;
  tc::fence_after_sync();
  tc::tmem_ld2(taddr, y0, y1);
  tc::tmem_wait_ld();
  y0 += s->b3[0];
  y1 += s->b3[1];
  tc::fence_before_sync();
  return true;
}

}  // namespace mhd
