// mhd_surrogate.cu — training data, training and evaluation of the KI
// cooling surrogate on the GPU with the project's own kernels:
//   sur_label_kernel  labels from the plain integrator (FP64 IMC bisection,
//                     the same device code as the FP64 SOURCE)
//   sur_pack_kernel   FP32 master parameters -> BF16 packed SurNet
//   sur_grad_kernel   forward + backward on BF16 tensor-core tiles
//                     (mma.sync m16n8k16, FP32 accumulate), gradients of
//                     the mean squared error summed into an FP32 vector
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
    int o = t / 64, k = t % 64;
    __nv_bfloat16 w = __float2bfloat16_rn(m[SUR_OW2 + t]);
    net->W2[t] = w;
    net->W2T[k * 64 + o] = w;
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

// Forward + backward of one batch.  A CTA of 4 warps works on tiles of 64
// samples (16 per warp).  Per warp: FP32 first layer, BF16 tensor-core
// second and output layers, output gradients, dh2 = dy W3 (CUDA cores),
// dz2 = dh2 SiLU'(z2), dh1 = dz2 W2 (tensor cores), dz1 = dh1 SiLU'(z1).
// Per CTA: dW2 = dz2^T h1 over the 64 samples on tensor cores (each warp
// owns 16 rows of dW2); the small gradients (W1, b1, b2, W3, b3) are
// reduced with shuffles and shared-memory atomics.  Gradients are summed
// over the batch (divided by the batch size) into g (FP32).
__global__ void __launch_bounds__(128) sur_grad_kernel(const SurNet *net, const float *x, const float *y,
                                                       long long n, float inv_batch, float *gout, float *loss) {
  __shared__ __nv_bfloat16 s_h1[64][64 + 8];   // [sample][feature]
  __shared__ __nv_bfloat16 s_dz2[64][64 + 8];
  __shared__ float s_g[SUR_NPARAM];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  for (int q = threadIdx.x; q < SUR_NPARAM; q += blockDim.x) s_g[q] = 0.0f;
  float accW2[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; nt++) accW2[nt][0] = accW2[nt][1] = accW2[nt][2] = accW2[nt][3] = 0.0f;
  float lsum = 0.0f;
  __syncthreads();
  long long ntile = (n + 63) / 64;
  for (long long tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    long long s0 = tile * 64 + warp * 16;
    // lanes 0..15 bring one sample each (normalised inputs)
    long long sr = s0 + (lane & 15);
    bool ok = lane < 16 && sr < n;
    float n0 = ok ? (x[3 * sr] - SUR_C0) / SUR_S0 : 0.0f;
    float n1 = ok ? (x[3 * sr + 1] - SUR_C1) / SUR_S1 : 0.0f;
    float n2 = ok ? (x[3 * sr + 2] - SUR_C2) / SUR_S2 : 0.0f;
    // forward
    float z1[8][4];
    layer1_fp32(net, n0, n1, n2, 0, z1);
    uint32_t a1[4][4];
    act_frags(z1, a1);
    float z2[8][4];
    layer64<4>(net->W2, net->b2, a1, z2);
    uint32_t a2[4][4];
    act_frags(z2, a2);
    float yo[4];
    layer_out(net, a2, yo);
    // output gradients for rows g and g+8 (held by the t == 0 lanes)
    float d0g = 0, d1g = 0, d0h = 0, d1h = 0;
    if (t == 0) {
      long long ra = s0 + g, rb = s0 + g + 8;
      if (ra < n) {
        float e = yo[0] - y[ra];
        float tc = log10f(fabsf(e) + 1e-4f);
        d0g = 2.0f * e * inv_batch;
        d1g = kConfWeight * 2.0f * (yo[1] - tc) * inv_batch;
        lsum += e * e;
      }
      if (rb < n) {
        float e = yo[2] - y[rb];
        float tc = log10f(fabsf(e) + 1e-4f);
        d0h = 2.0f * e * inv_batch;
        d1h = kConfWeight * 2.0f * (yo[3] - tc) * inv_batch;
        lsum += e * e;
      }
    }
    d0g = __shfl_sync(0xffffffffu, d0g, g * 4);
    d1g = __shfl_sync(0xffffffffu, d1g, g * 4);
    d0h = __shfl_sync(0xffffffffu, d0h, g * 4);
    d1h = __shfl_sync(0xffffffffu, d1h, g * 4);
    // b3, W3 gradients; dh2 and dz2
    float dz2[8][4];
    float gb3a = (t == 0) ? d0g + d0h : 0.0f, gb3b = (t == 0) ? d1g + d1h : 0.0f;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
#pragma unroll
      for (int q = 0; q < 2; q++) {
        int k = nt * 8 + 2 * t + q;
        float hg = silu(z2[nt][q]), hh = silu(z2[nt][2 + q]);
        // the BF16-rounded activations the forward used
        hg = bf16_round(hg);
        hh = bf16_round(hh);
        float w30 = __bfloat162float(net->W3[k]), w31 = __bfloat162float(net->W3[64 + k]);
        float gw0 = d0g * hg + d0h * hh, gw1 = d1g * hg + d1h * hh;
        for (int o = 4; o < 32; o <<= 1) {
          gw0 += __shfl_xor_sync(0xffffffffu, gw0, o);
          gw1 += __shfl_xor_sync(0xffffffffu, gw1, o);
        }
        if (g == 0) {
          atomicAdd(&s_g[SUR_OW3 + k], gw0);
          atomicAdd(&s_g[SUR_OW3 + 64 + k], gw1);
        }
        dz2[nt][q] = (d0g * w30 + d1g * w31) * dsilu(z2[nt][q]);
        dz2[nt][2 + q] = (d0h * w30 + d1h * w31) * dsilu(z2[nt][2 + q]);
      }
    }
    for (int o = 4; o < 32; o <<= 1) {
      gb3a += __shfl_xor_sync(0xffffffffu, gb3a, o);
      gb3b += __shfl_xor_sync(0xffffffffu, gb3b, o);
    }
    if (lane == 0) {
      atomicAdd(&s_g[SUR_OB3], gb3a);
      atomicAdd(&s_g[SUR_OB3 + 1], gb3b);
    }
    // b2 gradient; stage dz2 and h1 (BF16) for the dW2 product
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
#pragma unroll
      for (int q = 0; q < 2; q++) {
        int k = nt * 8 + 2 * t + q;
        float gb = dz2[nt][q] + dz2[nt][2 + q];
        for (int o = 4; o < 32; o <<= 1) gb += __shfl_xor_sync(0xffffffffu, gb, o);
        if (g == 0) atomicAdd(&s_g[SUR_OB2 + k], gb);
        s_dz2[warp * 16 + g][k] = __float2bfloat16_rn(dz2[nt][q]);
        s_dz2[warp * 16 + g + 8][k] = __float2bfloat16_rn(dz2[nt][2 + q]);
        s_h1[warp * 16 + g][k] = __float2bfloat16_rn(silu(z1[nt][q]));
        s_h1[warp * 16 + g + 8][k] = __float2bfloat16_rn(silu(z1[nt][2 + q]));
      }
    }
    // dh1 = dz2 W2 on tensor cores (B operand from W2T rows)
    uint32_t adz[4][4];
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
      adz[kt][0] = pack_bf16(dz2[2 * kt][0], dz2[2 * kt][1]);
      adz[kt][1] = pack_bf16(dz2[2 * kt][2], dz2[2 * kt][3]);
      adz[kt][2] = pack_bf16(dz2[2 * kt + 1][0], dz2[2 * kt + 1][1]);
      adz[kt][3] = pack_bf16(dz2[2 * kt + 1][2], dz2[2 * kt + 1][3]);
    }
    float dh1[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      dh1[nt][0] = dh1[nt][1] = dh1[nt][2] = dh1[nt][3] = 0.0f;
      const __nv_bfloat16 *row = net->W2T + (nt * 8 + g) * 64;
#pragma unroll
      for (int kt = 0; kt < 4; kt++) mma_bf16(dh1[nt], adz[kt], ld32(row + kt * 16 + 2 * t), ld32(row + kt * 16 + 8 + 2 * t));
    }
    // dz1, b1 and W1 gradients (W1 against the FP32 inputs)
    float xa0 = __shfl_sync(0xffffffffu, n0, g), xa1 = __shfl_sync(0xffffffffu, n1, g),
          xa2 = __shfl_sync(0xffffffffu, n2, g);
    float xb0 = __shfl_sync(0xffffffffu, n0, g + 8), xb1 = __shfl_sync(0xffffffffu, n1, g + 8),
          xb2 = __shfl_sync(0xffffffffu, n2, g + 8);
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
#pragma unroll
      for (int q = 0; q < 2; q++) {
        int k = nt * 8 + 2 * t + q;
        float ga = dh1[nt][q] * dsilu(z1[nt][q]), gb = dh1[nt][2 + q] * dsilu(z1[nt][2 + q]);
        float gbias = ga + gb, gw0 = ga * xa0 + gb * xb0, gw1 = ga * xa1 + gb * xb1, gw2 = ga * xa2 + gb * xb2;
        for (int o = 4; o < 32; o <<= 1) {
          gbias += __shfl_xor_sync(0xffffffffu, gbias, o);
          gw0 += __shfl_xor_sync(0xffffffffu, gw0, o);
          gw1 += __shfl_xor_sync(0xffffffffu, gw1, o);
          gw2 += __shfl_xor_sync(0xffffffffu, gw2, o);
        }
        if (g == 0) {
          atomicAdd(&s_g[SUR_OB1 + k], gbias);
          atomicAdd(&s_g[SUR_OW1 + 3 * k], gw0);
          atomicAdd(&s_g[SUR_OW1 + 3 * k + 1], gw1);
          atomicAdd(&s_g[SUR_OW1 + 3 * k + 2], gw2);
        }
      }
    }
    __syncthreads();
    // dW2[n][k] += sum_s dz2[s][n] h1[s][k]; warp w owns rows n = 16w..16w+15
#pragma unroll
    for (int ks = 0; ks < 4; ks++) {
      int sa = ks * 16 + 2 * t;
      uint32_t a[4];
      int nr = warp * 16 + g;
      a[0] = (uint32_t)__bfloat16_as_ushort(s_dz2[sa][nr]) | ((uint32_t)__bfloat16_as_ushort(s_dz2[sa + 1][nr]) << 16);
      a[1] = (uint32_t)__bfloat16_as_ushort(s_dz2[sa][nr + 8]) | ((uint32_t)__bfloat16_as_ushort(s_dz2[sa + 1][nr + 8]) << 16);
      a[2] = (uint32_t)__bfloat16_as_ushort(s_dz2[sa + 8][nr]) | ((uint32_t)__bfloat16_as_ushort(s_dz2[sa + 9][nr]) << 16);
      a[3] = (uint32_t)__bfloat16_as_ushort(s_dz2[sa + 8][nr + 8]) | ((uint32_t)__bfloat16_as_ushort(s_dz2[sa + 9][nr + 8]) << 16);
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        int kc = nt * 8 + g;
        uint32_t b0 = (uint32_t)__bfloat16_as_ushort(s_h1[sa][kc]) | ((uint32_t)__bfloat16_as_ushort(s_h1[sa + 1][kc]) << 16);
        uint32_t b1 = (uint32_t)__bfloat16_as_ushort(s_h1[sa + 8][kc]) | ((uint32_t)__bfloat16_as_ushort(s_h1[sa + 9][kc]) << 16);
        mma_bf16(accW2[nt], a, b0, b1);
      }
    }
    __syncthreads();
  }
  // flush: dW2 fragment -> shared, then everything -> global
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    int r0 = warp * 16 + g, c0 = nt * 8 + 2 * t;
    s_g[SUR_OW2 + r0 * 64 + c0] += accW2[nt][0];
    s_g[SUR_OW2 + r0 * 64 + c0 + 1] += accW2[nt][1];
    s_g[SUR_OW2 + (r0 + 8) * 64 + c0] += accW2[nt][2];
    s_g[SUR_OW2 + (r0 + 8) * 64 + c0 + 1] += accW2[nt][3];
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0) atomicAdd(loss, lsum);
  __syncthreads();
  for (int q = threadIdx.x; q < SUR_NPARAM; q += blockDim.x) atomicAdd(&gout[q], s_g[q]);
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
  DevBuf dm, dnet, dx, dy, dg, dl;
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
  sur_grad_kernel<<<nb(n, 64) < 608 ? nb(n, 64) : 608, 128>>>(dnet.as<SurNet>(), dx.as<float>(), dy.as<float>(), n,
                                                              1.0f / (float)n, dg.as<float>(), dl.as<float>());
  SCK(cudaGetLastError());
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
  DevBuf dm, m1, m2, dg, dnet, dx, dy, dl;
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
  unsigned grid = nb(batch, 64) < 1216 ? nb(batch, 64) : 1216;
  double c1 = 1.0, c2 = 1.0;
  for (int s = 0; s < steps; s++) {
    long long off = (long long)(s % nbatch) * batch;
    sur_pack_kernel<<<16, 256>>>(dm.as<float>(), dnet.as<SurNet>());
    sur_grad_kernel<<<grid, 128>>>(dnet.as<SurNet>(), dx.as<float>() + 3 * off, dy.as<float>() + off, batch,
                                   1.0f / (float)batch, dg.as<float>(), dl.as<float>() + s);
    c1 *= b1;
    c2 *= b2;
    sur_adam_kernel<<<nb(SUR_NPARAM, 256), 256>>>(dm.as<float>(), m1.as<float>(), m2.as<float>(), dg.as<float>(), lr,
                                                  b1, b2, eps, (float)(1.0 - c1), (float)(1.0 - c2));
  }
  SCK(cudaGetLastError());
  SCK(cudaDeviceSynchronize());
  SCK(cudaMemcpy(params, dm.p, SUR_NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
  if (history && steps > 0) {
    std::vector<float> h(steps);
    SCK(cudaMemcpy(h.data(), dl.p, steps * sizeof(float), cudaMemcpyDeviceToHost));
    for (int s = 0; s < steps; s++) history[s] = h[s] / (float)batch;
  }
  return MHD_OK;
}

}  // extern "C"
