// mhd_surrogate.cu — training data, training and evaluation of the KI
// cooling surrogate on the GPU with the project's own kernels:
//   sur_label_kernel  labels from the plain integrator (FP64 IMC bisection,
//                     the same device code as the FP64 SOURCE)
//   sur_pack_kernel   FP32 master parameters -> BF16 packed SurNet
//   sur_grad_kernel   forward + backward on tcgen05 tensor-core tiles (BF16
//                     operands, FP32 accumulators in tensor memory), gradients
//                     of the mean squared error summed into an FP32 vector
//   sur_adam_kernel   Adam update of the FP32 master parameters
//   sur_eval_kernel   batch inference (tcgen05 tiles: the fused SOURCE's network code)
// and the extern "C" entry points that expose them.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/mhd_gb300.h"
#include "mhd_launch.h"

namespace mhd {

// counter-based uniform random numbers (splitmix64 finaliser)
__device__ __forceinline__ double u01(unsigned long long seed, unsigned long long idx) {
  unsigned long long z = seed + 0x9e3779b97f4a7c15ull * (idx + 1);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  z = z ^ (z >> 31);
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// box of the training inputs (log10 N, log10 T[1e3 K], log10 dt/t_cool)
__constant__ double kLo[3] = {-2.0, -2.0, -3.0};
__constant__ double kHi[3] = {5.0, 1.3010299956639813, 3.0};

// Label of one input point by the plain integrator.  With N the KI density
// and n = N the particle density, P = kb n T, c = dt (gamma-1) chosen so
// that c |Lambda(N,T)| / P = 10^x2; the FP64 IMC bisection gives P_new.
__device__ double label_of(double x0, double x1, double x2, double kb) {
  double N = detmath::exp10(x0), T = detmath::exp10(x1), r = detmath::exp10(x2);
  double L = fcool_ki(T, N);
  if (L == 0.0) return 0.0;
  double P = kb * N * T;
  double c = r * P / fabs(L);
  double Pn = imc(P, N, c, 1.0, N, kb);
  return detmath::log10((Pn / (kb * N)) / T);
}

__global__ void sur_label_kernel(const float *x, float *y, long long n, double kb) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  y[i] = (float)label_of(x[3 * i], x[3 * i + 1], x[3 * i + 2], kb);
}

__global__ void sur_sample_kernel(float *x, float *y, long long n, unsigned long long seed, double kb) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v[3];
  for (int q = 0; q < 3; q++) {
    v[q] = kLo[q] + (kHi[q] - kLo[q]) * u01(seed, 3 * (unsigned long long)i + q);
    x[3 * i + q] = (float)v[q];
  }
  y[i] = (float)label_of(v[0], v[1], v[2], kb);
}

__global__ void sur_pack_kernel(const float *m, SurNet *net) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 64 * 16) {
    int o = t / 16, k = t % 16;
    net->W1[t] = __float2bfloat16_rn(k < 3 ? m[SUR_OW1 + o * 3 + k] : 0.0f);
  }
  if (t < 64 * 64) {
    net->W2[t] = __float2bfloat16_rn(m[SUR_OW2 + t]);
  }
  if (t < 8 * 64) {
    int o = t / 64, k = t % 64;
    net->W3[t] = __float2bfloat16_rn(o < 2 ? m[SUR_OW3 + o * 64 + k] : 0.0f);
  }
  if (t < 64) {
    net->b1[t] = m[SUR_OB1 + t];
    net->b2[t] = m[SUR_OB2 + t];
  }
  if (t < 8) net->b3[t] = t < 2 ? m[SUR_OB3 + t] : 0.0f;
}

// Batch inference with the fused SOURCE's network code: tcgen05 tiles of
// 128 samples, two per 256-thread CTA, the weights staged once per CTA.
__global__ void __launch_bounds__(kFusedThreads) sur_eval_kernel(const SurNet *net, const float *x, float *out,
                                                                 long long n, int *err) {
  extern __shared__ __align__(128) unsigned char eval_smem[];
  auto *s = reinterpret_cast<SurTileSmem<kFusedTiles> *>(eval_smem);
  sur_tile_setup<kFusedTiles>(net, s);
  uint32_t phase = 0;
  for (long long i0 = (long long)blockIdx.x * kFusedThreads; i0 < n; i0 += (long long)gridDim.x * kFusedThreads) {
    const long long i = i0 + threadIdx.x;
    const bool act = i < n;
    const float n0 = act ? (x[3 * i] - SUR_C0) / SUR_S0 : 0.0f;
    const float n1 = act ? (x[3 * i + 1] - SUR_C1) / SUR_S1 : 0.0f;
    const float n2 = act ? (x[3 * i + 2] - SUR_C2) / SUR_S2 : 0.0f;
    float y0 = 0.0f, y1 = 0.0f;
    if (!sur_tile_forward<kFusedTiles>(s, n0, n1, n2, phase, y0, y1)) {
      if (threadIdx.x == 0) atomicOr(err, ERRB_TC);
      break;   // the same on every thread
    }
    if (act) {
      out[2 * i] = y0;
      out[2 * i + 1] = y1;
    }
  }
  sur_tile_teardown<kFusedTiles>(s, phase);
}

// Loss per sample: (o0 - y)^2 + w_c (o1 - log10(|o0 - y| + 1e-4))^2, the
// second term with the error treated as a constant (the confidence head
// learns the log of the first head's error).
constexpr float kConfWeight = 0.1f;

// Forward + backward of one batch on the fifth-generation tensor cores.  A
// CTA of 128 threads takes tiles of 128 samples (thread r = sample row r),
// one CTA per SM striding over the batch's tiles.  Per tile:
//   layer 1 on the CUDA cores in FP32: h1 = bf16(SiLU(z1));
//   Z2 = h1 W2^T                       tcgen05 (M 128, N 64, K 64)
//   h2 = bf16(SiLU(Z2 + b2)),  Y = h2 W3^T   (N 16, the 2 outputs padded)
//   output gradients d = (d0, d1) of the loss per sample (CUDA cores),
//   dz2 = (d W3) SiLU'(z2) in FP32, rounded to BF16 for the products;
//   dh1 = dz2 W2                       tcgen05 (B = W2^T, K-major)
//   and, accumulated in tensor memory over all the CTA's tiles:
//   [dW2 | gb2]  = dz2^T [h1 | 1]      (M 64 padded to 128, N 80, K 128)
//   [gW3 | gb3]^T = [h2 | 1]^T d      (M 65 padded to 128, N 16, K 128)
//   [gW1 | gb1]  = dz1^T [x | 1]       (dz1 = dh1 SiLU'(z1); N 16, K 128)
// with the BF16 rounding points of oracle/surrogate_ref.py.  The
// transposed operands are written transposed into shared memory by the
// threads; the ones columns and zero rows are set once.  Gradients are summed
// over the batch (divided by the batch size) into g (FP32).
struct SurGradSmem {
  __nv_bfloat16 W2[64 * 64];       // B of Z2: [out][in], K-major
  __nv_bfloat16 W2T[64 * 64];      // B of dh1: [in][out], K-major
  __nv_bfloat16 W3[16 * 64];       // B of Y: [out padded to 16][in]
  __nv_bfloat16 A[128 * 64];       // h1, then h2, then dz2: [sample][feature]
  __nv_bfloat16 dz2T[128 * 128];   // [feature n (64, rest 0)][sample]: A of dW2, then dz1^T, A of gW1
  __nv_bfloat16 h2T[128 * 128];    // [feature k (64), row 64 ones, rest 0][sample]: A of gW3
  __nv_bfloat16 h1T[80 * 128];     // [feature k (64), row 64 ones, rest 0][sample]: B of dW2
  __nv_bfloat16 dT[16 * 128];      // [d0, d1, rest 0][sample]: B of gW3
  __nv_bfloat16 xT[16 * 128];      // [x0, x1, x2, 1, rest 0][sample]: B of gW1
  float4 w1[64];                   // (w0, w1, w2, b1)
  float b2[64], b3[2], w3[2][64];  // BF16-rounded W3 for dh2 on the CUDA cores
  uint64_t bar;
  uint32_t tmem;
  int broken;
};
// TMEM columns: Z2 0-63, Y 64-79, dh1 80-143, [dW2|gb2] 144-223, [gW3|gb3] 224-239, [gW1|gb1] 240-255
constexpr uint32_t kGZ2 = 0, kGY = 64, kGDH1 = 80, kGDW2 = 144, kGW3 = 224, kGW1 = 240, kGCols = 256;

__device__ __forceinline__ void gstore(__nv_bfloat16 *buf, int row, int col, int K, float v) {
  *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<char *>(buf) + tc::kmajor_off(row, col, K)) =
      __float2bfloat16_rn(v);
}
__device__ __forceinline__ void gstore8(__nv_bfloat16 *buf, int row, int col8, int K, const float (&v)[8]) {
  const uint4 q = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                             pack_bf16(v[6], v[7]));
  *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(buf) + tc::kmajor_off(row, col8, K)) = q;
}
// one thread issues nk K-steps of 16 (A: K-major with K = 16 nk... columns)
__device__ __forceinline__ void gmma(uint32_t d, const __nv_bfloat16 *Am, int KA, const __nv_bfloat16 *Bm, int KB,
                                     int N, int nk, bool acc_first) {
  const uint32_t idesc = tc::idesc_bf16_f32(128, N), ab = tc::smem_u32(Am), bb = tc::smem_u32(Bm);
  for (int kk = 0; kk < nk; kk++)
    tc::mma_bf16(d, tc::smem_desc(ab + 256 * kk, 128, 16 * KA), tc::smem_desc(bb + 256 * kk, 128, 16 * KB), idesc,
                 acc_first || kk > 0);
}
// the commit of the MMAs issued so far and the CTA-wide wait for it; false
// on every thread when the wait timed out
__device__ __forceinline__ bool gsync(SurGradSmem *s, uint32_t &phase, bool issued) {
  if (threadIdx.x == 0 && issued) tc::mma_commit(&s->bar);
  const bool ok = !s->broken && tc::mbar_wait(&s->bar, phase);
  if (!__syncthreads_and(ok)) {
    if (threadIdx.x == 0) s->broken = 1;
    return false;
  }
  phase ^= 1u;
  tc::fence_after_sync();
  return true;
}
__device__ __forceinline__ void gbarrier() {
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

__global__ void __launch_bounds__(128, 1) sur_grad_kernel(const SurNet *net, const float *x, const float *y,
                                                          long long n, float inv_batch, float *gout, float *loss,
                                                          int *err) {
  extern __shared__ __align__(128) unsigned char grad_smem[];
  SurGradSmem *s = reinterpret_cast<SurGradSmem *>(grad_smem);
  const int r = threadIdx.x, w = r >> 5;
  // set-up: weights in the operand layouts, the constant rows, TMEM
  for (int q = r; q < 64 * 64; q += 128) {
    const int o = q >> 6, i = q & 63;
    *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<char *>(s->W2) + tc::kmajor_off(o, i, 64)) = net->W2[q];
    *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<char *>(s->W2T) + tc::kmajor_off(i, o, 64)) = net->W2[q];
  }
  for (int q = r; q < 16 * 64; q += 128) {
    const int o = q >> 6, i = q & 63;
    *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<char *>(s->W3) + tc::kmajor_off(o, i, 64)) =
        o < 2 ? net->W3[q] : __float2bfloat16_rn(0.0f);
  }
  for (int q = r; q < 64; q += 128) {
    const __nv_bfloat16 *wv = net->W1 + q * 16;
    s->w1[q] = make_float4(__bfloat162float(wv[0]), __bfloat162float(wv[1]), __bfloat162float(wv[2]), net->b1[q]);
    s->b2[q] = net->b2[q];
    s->w3[0][q] = __bfloat162float(net->W3[q]);
    s->w3[1][q] = __bfloat162float(net->W3[64 + q]);
  }
  if (r < 2) s->b3[r] = net->b3[r];
  // column r (sample r) of the transposed operands: zero rows, the ones rows
  for (int row = 64; row < 128; row++) {
    gstore(s->dz2T, row, r, 128, 0.0f);
    gstore(s->h2T, row, r, 128, row == 64 ? 1.0f : 0.0f);
  }
  for (int row = 64; row < 80; row++) gstore(s->h1T, row, r, 128, row == 64 ? 1.0f : 0.0f);
  for (int row = 2; row < 16; row++) gstore(s->dT, row, r, 128, 0.0f);
  for (int row = 3; row < 16; row++) gstore(s->xT, row, r, 128, row == 3 ? 1.0f : 0.0f);
  if (r == 0) {
    tc::mbar_init(&s->bar, 1);
    s->broken = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (r < 32) tc::tmem_alloc(&s->tmem, kGCols);
  gbarrier();
  const uint32_t tm = s->tmem, lane_off = (uint32_t)(w * 32) << 16;
  uint32_t phase = 0;
  bool first = true, ok = true;
  float lacc = 0.0f;
  const long long ntile = (n + 127) / 128;
  for (long long tile = blockIdx.x; tile < ntile && ok; tile += gridDim.x) {
    const long long smp = tile * 128 + r;
    const bool act = smp < n;
    const float n0 = act ? (x[3 * smp] - SUR_C0) / SUR_S0 : 0.0f;
    const float n1 = act ? (x[3 * smp + 1] - SUR_C1) / SUR_S1 : 0.0f;
    const float n2 = act ? (x[3 * smp + 2] - SUR_C2) / SUR_S2 : 0.0f;
    // layer 1 (FP32), h1 into A and, transposed, into h1T
    for (int kc = 0; kc < 8; kc++) {
      float hv[8];
      for (int q = 0; q < 8; q++) {
        const float4 c = s->w1[8 * kc + q];
        hv[q] = bf16_round(silu(c.w + c.x * n0 + c.y * n1 + c.z * n2));
        gstore(s->h1T, 8 * kc + q, r, 128, act ? hv[q] : 0.0f);
      }
      gstore8(s->A, r, 8 * kc, 64, hv);
    }
    gstore(s->xT, 0, r, 128, n0);
    gstore(s->xT, 1, r, 128, n1);
    gstore(s->xT, 2, r, 128, n2);
    gbarrier();
    if (r == 0) gmma(tm + kGZ2, s->A, 64, s->W2, 64, 64, 4, false);
    if (!(ok = gsync(s, phase, true))) break;
    // h2 = bf16(SiLU(Z2 + b2)) into A and h2T
    for (int cc = 0; cc < 4; cc++) {
      float v[16];
      tc::tmem_ld16(tm + lane_off + kGZ2 + 16 * cc, v);
      tc::tmem_wait_ld();
      for (int hf = 0; hf < 2; hf++) {
        float hv[8];
        for (int q = 0; q < 8; q++) {
          const int k = 16 * cc + 8 * hf + q;
          hv[q] = bf16_round(silu(v[8 * hf + q] + s->b2[k]));
          gstore(s->h2T, k, r, 128, act ? hv[q] : 0.0f);
        }
        gstore8(s->A, r, 16 * cc + 8 * hf, 64, hv);
      }
    }
    gbarrier();
    if (r == 0) gmma(tm + kGY, s->A, 64, s->W3, 64, 16, 4, false);
    if (!(ok = gsync(s, phase, true))) break;
    float o0, o1;
    tc::tmem_ld2(tm + lane_off + kGY, o0, o1);
    tc::tmem_wait_ld();
    o0 += s->b3[0];
    o1 += s->b3[1];
    float d0 = 0.0f, d1 = 0.0f;
    if (act) {
      const float e = o0 - y[smp];
      const float tcf = log10f(fabsf(e) + 1e-4f);
      d0 = 2.0f * e * inv_batch;
      d1 = kConfWeight * 2.0f * (o1 - tcf) * inv_batch;
      lacc += e * e;
    }
    gstore(s->dT, 0, r, 128, d0);
    gstore(s->dT, 1, r, 128, d1);
    // dz2 = (d W3) SiLU'(Z2 + b2): into A (K-major) and dz2T
    for (int cc = 0; cc < 4; cc++) {
      float v[16];
      tc::tmem_ld16(tm + lane_off + kGZ2 + 16 * cc, v);
      tc::tmem_wait_ld();
      for (int hf = 0; hf < 2; hf++) {
        float dv[8];
        for (int q = 0; q < 8; q++) {
          const int k = 16 * cc + 8 * hf + q;
          dv[q] = (d0 * s->w3[0][k] + d1 * s->w3[1][k]) * dsilu(v[8 * hf + q] + s->b2[k]);
          gstore(s->dz2T, k, r, 128, dv[q]);
        }
        gstore8(s->A, r, 16 * cc + 8 * hf, 64, dv);
      }
    }
    gbarrier();
    if (r == 0) {
      gmma(tm + kGDH1, s->A, 64, s->W2T, 64, 64, 4, false);
      gmma(tm + kGDW2, s->dz2T, 128, s->h1T, 128, 80, 8, !first);
      gmma(tm + kGW3, s->h2T, 128, s->dT, 128, 16, 8, !first);
    }
    if (!(ok = gsync(s, phase, true))) break;
    // dz1 = dh1 SiLU'(z1) into dz2T (its products are done), then [gW1 | gb1]
    for (int cc = 0; cc < 4; cc++) {
      float v[16];
      tc::tmem_ld16(tm + lane_off + kGDH1 + 16 * cc, v);
      tc::tmem_wait_ld();
      for (int q = 0; q < 16; q++) {
        const int k = 16 * cc + q;
        const float4 c = s->w1[k];
        const float z1 = c.w + c.x * n0 + c.y * n1 + c.z * n2;
        gstore(s->dz2T, k, r, 128, act ? v[q] * dsilu(z1) : 0.0f);
      }
    }
    gbarrier();
    if (r == 0) gmma(tm + kGW1, s->dz2T, 128, s->xT, 128, 16, 8, !first);
    if (!(ok = gsync(s, phase, true))) break;
    first = false;
  }
  // the accumulators out: lane n of [dW2 | gb2] and [gW1 | gb1] (n < 64), lane
  // k of [gW3 | gb3] (k <= 64); every warp takes part in the loads
  if (ok && !first) {
    float v[16];
    for (int cc = 0; cc < 5; cc++) {
      tc::tmem_ld16(tm + lane_off + kGDW2 + 16 * cc, v);
      tc::tmem_wait_ld();
      if (r < 64)
        for (int q = 0; q < 16; q++) {
          const int k = 16 * cc + q;
          if (k < 64) atomicAdd(&gout[SUR_OW2 + r * 64 + k], v[q]);
          else if (k == 64) atomicAdd(&gout[SUR_OB2 + r], v[q]);
        }
    }
    tc::tmem_ld16(tm + lane_off + kGW3, v);
    tc::tmem_wait_ld();
    if (r < 64) {
      atomicAdd(&gout[SUR_OW3 + r], v[0]);
      atomicAdd(&gout[SUR_OW3 + 64 + r], v[1]);
    } else if (r == 64) {
      atomicAdd(&gout[SUR_OB3], v[0]);
      atomicAdd(&gout[SUR_OB3 + 1], v[1]);
    }
    tc::tmem_ld16(tm + lane_off + kGW1, v);
    tc::tmem_wait_ld();
    if (r < 64) {
      for (int c = 0; c < 3; c++) atomicAdd(&gout[SUR_OW1 + 3 * r + c], v[c]);
      atomicAdd(&gout[SUR_OB1 + r], v[3]);
    }
  }
  if (!ok && r == 0) atomicOr(err, ERRB_TC);
  for (int o = 16; o > 0; o >>= 1) lacc += __shfl_xor_sync(0xffffffffu, lacc, o);
  if ((r & 31) == 0) atomicAdd(loss, lacc);
  // TMEM free once nothing of this CTA is in flight (a timed-out wait: one more bounded wait)
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (s->broken && r == 0) tc::mbar_wait(&s->bar, phase);
  __syncthreads();
  if (r < 32) tc::tmem_free(tm, kGCols);
  if (r == 0) tc::mbar_inval(&s->bar);
}

__global__ void sur_adam_kernel(float *m, float *mom1, float *mom2, float *grad, float lr, float b1, float b2,
                                float eps, float c1, float c2) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= SUR_NPARAM) return;
  float gq = grad[q];
  float a = b1 * mom1[q] + (1.0f - b1) * gq;
  float v = b2 * mom2[q] + (1.0f - b2) * gq * gq;
  mom1[q] = a;
  mom2[q] = v;
  m[q] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
  grad[q] = 0.0f;
}

// one 128-thread CTA per SM (the kernel's 131 KB of operands), striding
// over the batch's 128-sample tiles
cudaError_t sur_grad_launch(const SurNet *net, const float *x, const float *y, long long n, float *g, float *loss,
                            int *err, cudaStream_t st) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int smem = (int)sizeof(SurGradSmem);
  cudaError_t e = cudaFuncSetAttribute(sur_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const long long tiles = (n + 127) / 128;
  const unsigned grid = (unsigned)(tiles < (long long)sms ? tiles : (long long)sms);
  sur_grad_kernel<<<grid, 128, smem, st>>>(net, x, y, n, 1.0f / (float)n, g, loss, err);
  return cudaGetLastError();
}

cudaError_t surrogate_pack(const float *master, SurNet *net, cudaStream_t s) {
  sur_pack_kernel<<<16, 256, 0, s>>>(master, net);
  return cudaGetLastError();
}

}  // namespace mhd

using namespace mhd;

namespace {

struct DevBuf {
  void *p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
  template <class T> T *as() { return static_cast<T *>(p); }
};

#define SCK(call)                                 \
  do {                                            \
    if ((call) != cudaSuccess) {                  \
      cudaGetLastError();                         \
      return MHD_ERR_CUDA;                        \
    }                                             \
  } while (0)

int sur_device(int device) {
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd <= device) {
    cudaGetLastError();
    return MHD_ERR_NO_DEVICE;
  }
  return cudaSetDevice(device) == cudaSuccess ? MHD_OK : MHD_ERR_NO_DEVICE;
}

unsigned nb(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

extern "C" {

int mhd_surrogate_nparams(void) { return SUR_NPARAM; }

int mhd_surrogate_label(const float *x, float *y, long long n, double kb, int device) {
  if (!x || !y || n <= 0) return MHD_ERR_ARG;
  int r = sur_device(device);
  if (r) return r;
  DevBuf dx, dy;
  SCK(cudaMalloc(&dx.p, n * 3 * sizeof(float)));
  SCK(cudaMalloc(&dy.p, n * sizeof(float)));
  SCK(cudaMemcpy(dx.p, x, n * 3 * sizeof(float), cudaMemcpyHostToDevice));
  sur_label_kernel<<<nb(n, 128), 128>>>(dx.as<float>(), dy.as<float>(), n, kb);
  SCK(cudaGetLastError());
  SCK(cudaMemcpy(y, dy.p, n * sizeof(float), cudaMemcpyDeviceToHost));
  return MHD_OK;
}

int mhd_surrogate_eval(const float *params, const float *x, float *out, long long n, int device) {
  if (!params || !x || !out || n <= 0) return MHD_ERR_ARG;
  int r = sur_device(device);
  if (r) return r;
  DevBuf dm, dnet, dx, dout, derr;
  SCK(cudaMalloc(&dm.p, SUR_NPARAM * sizeof(float)));
  SCK(cudaMalloc(&dnet.p, sizeof(SurNet)));
  SCK(cudaMalloc(&dx.p, n * 3 * sizeof(float)));
  SCK(cudaMalloc(&dout.p, n * 2 * sizeof(float)));
  SCK(cudaMalloc(&derr.p, sizeof(int)));
  SCK(cudaMemset(derr.p, 0, sizeof(int)));
  SCK(cudaMemcpy(dm.p, params, SUR_NPARAM * sizeof(float), cudaMemcpyHostToDevice));
  SCK(cudaMemcpy(dx.p, x, n * 3 * sizeof(float), cudaMemcpyHostToDevice));
  sur_pack_kernel<<<16, 256>>>(dm.as<float>(), dnet.as<SurNet>());
  // a persistent grid, at most four CTAs per SM (128 TMEM columns each)
  int sms = 0, per_sm = 0;
  SCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const size_t smem = sizeof(SurTileSmem<kFusedTiles>);
  SCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sur_eval_kernel, kFusedThreads, smem));
  per_sm = per_sm < 1 ? 1 : (per_sm > 4 ? 4 : per_sm);
  const long long tiles = (n + kFusedThreads - 1) / kFusedThreads;
  const unsigned grid = (unsigned)(tiles < (long long)per_sm * sms ? tiles : (long long)per_sm * sms);
  sur_eval_kernel<<<grid, kFusedThreads, smem>>>(dnet.as<SurNet>(), dx.as<float>(), dout.as<float>(), n,
                                                  derr.as<int>());
  SCK(cudaGetLastError());
  SCK(cudaMemcpy(out, dout.p, n * 2 * sizeof(float), cudaMemcpyDeviceToHost));
  int e = 0;
  SCK(cudaMemcpy(&e, derr.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) return MHD_ERR_CUDA;
  return MHD_OK;
}

// Gradient of the batch loss (mean over n samples) at params; for checks.
int mhd_surrogate_grad(const float *params, const float *x, const float *y, long long n, float *grad,
                       float *loss, int device) {
  if (!params || !x || !y || !grad || n <= 0) return MHD_ERR_ARG;
  int r = sur_device(device);
  if (r) return r;
  DevBuf dm, dnet, dx, dy, dg, dl, derr;
  SCK(cudaMalloc(&dm.p, SUR_NPARAM * sizeof(float)));
  SCK(cudaMalloc(&dnet.p, sizeof(SurNet)));
  SCK(cudaMalloc(&dx.p, n * 3 * sizeof(float)));
  SCK(cudaMalloc(&dy.p, n * sizeof(float)));
  SCK(cudaMalloc(&dg.p, SUR_NPARAM * sizeof(float)));
  SCK(cudaMalloc(&dl.p, sizeof(float)));
  SCK(cudaMemcpy(dm.p, params, SUR_NPARAM * sizeof(float), cudaMemcpyHostToDevice));
  SCK(cudaMemcpy(dx.p, x, n * 3 * sizeof(float), cudaMemcpyHostToDevice));
  SCK(cudaMemcpy(dy.p, y, n * sizeof(float), cudaMemcpyHostToDevice));
  SCK(cudaMemset(dg.p, 0, SUR_NPARAM * sizeof(float)));
  SCK(cudaMemset(dl.p, 0, sizeof(float)));
  sur_pack_kernel<<<16, 256>>>(dm.as<float>(), dnet.as<SurNet>());
  SCK(cudaMalloc(&derr.p, sizeof(int)));
  SCK(cudaMemset(derr.p, 0, sizeof(int)));
  SCK(sur_grad_launch(dnet.as<SurNet>(), dx.as<float>(), dy.as<float>(), n, dg.as<float>(), dl.as<float>(),
                      derr.as<int>(), nullptr));
  int e = 0;
  SCK(cudaMemcpy(&e, derr.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) return MHD_ERR_CUDA;
  SCK(cudaMemcpy(grad, dg.p, SUR_NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
  if (loss) {
    SCK(cudaMemcpy(loss, dl.p, sizeof(float), cudaMemcpyDeviceToHost));
    *loss /= (float)n;
  }
  return MHD_OK;
}

// Trains from params (in/out) on n_data samples drawn in the training box
// and labelled by the plain integrator; Adam with the given learning rate,
// batch size and number of steps.  history (optional, steps entries)
// receives the mean squared error of each batch.
int mhd_surrogate_train(float *params, long long n_data, int batch, int steps, float lr,
                        unsigned long long seed, float *history, int device) {
  if (!params || n_data < batch || batch < 64 || steps < 0) return MHD_ERR_ARG;
  int r = sur_device(device);
  if (r) return r;
  DevBuf dm, m1, m2, dg, dnet, dx, dy, dl, derr;
  SCK(cudaMalloc(&derr.p, sizeof(int)));
  SCK(cudaMemset(derr.p, 0, sizeof(int)));
  SCK(cudaMalloc(&dm.p, SUR_NPARAM * sizeof(float)));
  SCK(cudaMalloc(&m1.p, SUR_NPARAM * sizeof(float)));
  SCK(cudaMalloc(&m2.p, SUR_NPARAM * sizeof(float)));
  SCK(cudaMalloc(&dg.p, SUR_NPARAM * sizeof(float)));
  SCK(cudaMalloc(&dnet.p, sizeof(SurNet)));
  SCK(cudaMalloc(&dx.p, n_data * 3 * sizeof(float)));
  SCK(cudaMalloc(&dy.p, n_data * sizeof(float)));
  SCK(cudaMalloc(&dl.p, (steps > 0 ? steps : 1) * sizeof(float)));
  SCK(cudaMemcpy(dm.p, params, SUR_NPARAM * sizeof(float), cudaMemcpyHostToDevice));
  SCK(cudaMemset(m1.p, 0, SUR_NPARAM * sizeof(float)));
  SCK(cudaMemset(m2.p, 0, SUR_NPARAM * sizeof(float)));
  SCK(cudaMemset(dg.p, 0, SUR_NPARAM * sizeof(float)));
  SCK(cudaMemset(dl.p, 0, (steps > 0 ? steps : 1) * sizeof(float)));
  sur_sample_kernel<<<nb(n_data, 128), 128>>>(dx.as<float>(), dy.as<float>(), n_data, seed, 8.63359);
  SCK(cudaGetLastError());
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  long long nbatch = n_data / batch;
  double c1 = 1.0, c2 = 1.0;
  for (int s = 0; s < steps; s++) {
    long long off = (long long)(s % nbatch) * batch;
    sur_pack_kernel<<<16, 256>>>(dm.as<float>(), dnet.as<SurNet>());
    SCK(sur_grad_launch(dnet.as<SurNet>(), dx.as<float>() + 3 * off, dy.as<float>() + off, batch, dg.as<float>(),
                        dl.as<float>() + s, derr.as<int>(), nullptr));
    c1 *= b1;
    c2 *= b2;
    sur_adam_kernel<<<nb(SUR_NPARAM, 256), 256>>>(dm.as<float>(), m1.as<float>(), m2.as<float>(), dg.as<float>(), lr,
                                                  b1, b2, eps, (float)(1.0 - c1), (float)(1.0 - c2));
  }
  SCK(cudaGetLastError());
  SCK(cudaDeviceSynchronize());
  int e = 0;
  SCK(cudaMemcpy(&e, derr.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) return MHD_ERR_CUDA;
  SCK(cudaMemcpy(params, dm.p, SUR_NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
  if (history && steps > 0) {
    std::vector<float> h(steps);
    SCK(cudaMemcpy(h.data(), dl.p, steps * sizeof(float), cudaMemcpyDeviceToHost));
    for (int s = 0; s < steps; s++) history[s] = h[s] / (float)batch;
  }
  return MHD_OK;
}

}  // extern "C"
