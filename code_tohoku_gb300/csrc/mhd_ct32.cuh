// mhd_ct32.cuh — chosen-form constrained transport: CC(1)-CC(3) of
// MCF3DSGincfca3.f90:2115-2445 with the face velocities, the characteristic
// EMF solve (CCT) and every limiter in FP32, and the face-field update in
// FP64.
//
//   face_velocity32   CC(1) face velocities, FP32 arithmetic, FP64 store
//                     (the ghost exchanges of the FP64 path follow it)
//   ct_prep32         one pass over the padded grid after those exchanges:
//                     FP32 copies of the face velocities, face B, rho and
//                     VLIMIT's T switch, so the EMF kernels load only FP32
//   emf32x2<E>        CC(2) + CCT for the edges along E, thread per edge,
//                     FP32 loads, FP32 arithmetic in packed pairs, FP32 EMF
//   face_b32          CC(3): B_face += dt/dy (E(j+1)-E(j)) - ..., the EMF
//                     differences taken in FP64 from the FP32 values, so the
//                     discrete div B of the update cancels to FP64 round-off
//                     exactly as in the FP64 path
//
// Conversions use the integer routines of mhd_conv.cuh (GB300 runs the
// hardware ones on its narrow FP64 pipe).
#pragma once

#include "mhd_conv.cuh"
#include "mhd_kernels.cuh"

namespace mhd {

struct CT32Args {
  Grid g;
  const float *vf[3];   // face velocities
  const float *bf[3];   // face B
  const float *rn;      // rho
  const float *sw;      // VLIMIT T switch (+-0.5) per cell
  float *emf[3];        // [0] Ez, [1] Ex, [2] Ey
  float dt, facm;       // facm = facdep / 2
};

#ifdef MHD_FP32_KERNELS
// Two faces per thread, blockDim apart (coalesced), the six loads of both
// issued before either is used.
__global__ void __launch_bounds__(256) face_velocity32_kernel(Grid g, Fields f, double *vf0, double *vf1,
                                                              double *vf2) {
  const int nx1 = g.n[0] + 1, ny1 = g.n[1] + 1, nz1 = g.n[2] + 1;
  const long long n = (long long)nx1 * ny1 * nz1;
  const long long t0 = (long long)blockIdx.x * (2 * blockDim.x) + threadIdx.x;
  const int sy = (int)g.st[1], sz = (int)g.st[2];
  double v[2][6];
  int aa[2], ijk[2][3];
#pragma unroll
  for (int u = 0; u < 2; u++) {
    const long long t = t0 + u * blockDim.x;
    aa[u] = -1;
    if (t < n) {
      int i, j, k;
      split3(t, nx1, ny1, i, j, k);
      i += 1; j += 1; k += 1;
      const int a = (int)gidx(g, i, j, k);
      aa[u] = a;
      ijk[u][0] = i; ijk[u][1] = j; ijk[u][2] = k;
      v[u][0] = f.U[1][a]; v[u][1] = f.U[1][a - 1];
      v[u][2] = f.U[2][a]; v[u][3] = f.U[2][a - sy];
      v[u][4] = f.U[3][a]; v[u][5] = f.U[3][a - sz];
    }
  }
  const float *dx = g.dxf[0], *dy = g.dxf[1], *dz = g.dxf[2];
#pragma unroll
  for (int u = 0; u < 2; u++) {
    const int a = aa[u];
    if (a < 0) continue;
    const int i = ijk[u][0], j = ijk[u][1], k = ijk[u][2];
    if (j <= g.n[1] && k <= g.n[2])
      vf0[a] = f2d(__fdividef(dx[i] * d2f(v[u][0]) + dx[i + 1] * d2f(v[u][1]), dx[i] + dx[i + 1]));
    if (i <= g.n[0] && k <= g.n[2])
      vf1[a] = f2d(__fdividef(dy[j] * d2f(v[u][2]) + dy[j + 1] * d2f(v[u][3]), dy[j] + dy[j + 1]));
    if (i <= g.n[0] && j <= g.n[1])
      vf2[a] = f2d(__fdividef(dz[k] * d2f(v[u][4]) + dz[k + 1] * d2f(v[u][5]), dz[k] + dz[k + 1]));
  }
}

// Two cells per thread (block-strided, so every warp access stays
// coalesced), all 16 loads issued before the first store: a copy-like
// kernel needs many loads in flight per SM to approach HBM bandwidth.
__global__ void __launch_bounds__(256) ct_prep32_kernel(long long ncell, Fields f, const double *vf0,
                                                        const double *vf1, const double *vf2, float kb,
                                                        CT32Args A) {
  const long long t0 = (long long)blockIdx.x * (2 * blockDim.x) + threadIdx.x;
  double v[2][8];
#pragma unroll
  for (int u = 0; u < 2; u++) {
    const long long t = t0 + u * blockDim.x;
    if (t < ncell) {
      v[u][0] = __ldg(vf0 + t); v[u][1] = __ldg(vf1 + t); v[u][2] = __ldg(vf2 + t);
      v[u][3] = __ldg(f.U[5] + t); v[u][4] = __ldg(f.U[6] + t); v[u][5] = __ldg(f.U[7] + t);
      v[u][6] = __ldg(f.U[0] + t); v[u][7] = __ldg(f.U[4] + t);
    }
  }
#pragma unroll
  for (int u = 0; u < 2; u++) {
    const long long t = t0 + u * blockDim.x;
    if (t >= ncell) continue;
    const_cast<float *>(A.vf[0])[t] = d2f(v[u][0]);
    const_cast<float *>(A.vf[1])[t] = d2f(v[u][1]);
    const_cast<float *>(A.vf[2])[t] = d2f(v[u][2]);
    for (int c = 0; c < 3; c++) const_cast<float *>(A.bf[c])[t] = d2f(v[u][3 + c]);
    float r = d2f(v[u][6]);
    const_cast<float *>(A.rn)[t] = r;
    // T = 1.27 p/(kb rho); sign(0.5, T-3)
    const_cast<float *>(A.sw)[t] = (1.27f * d2f(v[u][7]) >= 3.0f * kb * r) ? 0.5f : -0.5f;
  }
}

// Packed FP32 pairs: Blackwell's paired FP32 add, multiply and fused
// multiply-add (one instruction for both lanes).
__device__ __forceinline__ float2 p2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 pabs(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }

// vlim_w of two quantities (lanes) that share the widths and the switch
__device__ __forceinline__ float2 vlim_w2(float2 qm, float2 q0, float2 qp, const LimW &w) {
  if (w.s > 0.0f) {
    const float2 dp = pmul(psub(qp, q0), p2(w.rp, w.rp)), dm = pmul(psub(q0, qm), p2(w.rm, w.rm));
    const float2 pr = pmul(dp, dm);
    return p2(pr.x > 0.0f ? copysignf(fminf(fabsf(dp.x), fabsf(dm.x)), dp.x) : 0.0f,
              pr.y > 0.0f ? copysignf(fminf(fabsf(dp.y), fabsf(dm.y)), dp.y) : 0.0f);
  }
  const float2 delp = psub(qp, q0), delm = psub(q0, qm);
  const float2 eps = p2(1e-10f, 1e-10f);
  const float2 num = pfma(pmul(p2(2.0f, 2.0f), delp), delm, eps);
  const float2 den = pfma(delp, delp, pfma(delm, delm, eps));
  const float2 fl = p2(fmaxf(0.0f, __fdividef(num.x, den.x)), fmaxf(0.0f, __fdividef(num.y, den.y)));
  return pmul(pmul(fl, psub(qp, qm)), p2(w.ra, w.ra));
}

// CC(2) + CCT for the edge direction E (0: Ez on x/y, 1: Ex on y/z, 2: Ey on
// z/x): the arithmetic of emf_kernel (:2140-2157, :2186-2445) in FP32 on
// FP32 inputs, with the two characteristic combinations of every candidate
// in the two lanes of packed FP32 pairs: lane x the (+, -) pair (C1p, C2m),
// lane y the (-, +) pair (C1m, C2p), which do the same arithmetic on their
// own inputs; the slopes of V and B along a direction share their widths
// and switch, so they form a pair too.  32-bit cell offsets (the padded grid
// has fewer than 2^31 cells).
template <int E>
__global__ void __launch_bounds__(128) emf32x2_kernel(CT32Args A) {
  const Grid &g = A.g;
  constexpr int da = E, db = (E + 1) % 3, dc = (E + 2) % 3;
  int ext[3];
  ext[da] = g.n[da] + 1; ext[db] = g.n[db] + 1; ext[dc] = g.n[dc];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ext[0] * ext[1] * ext[2]) return;
  int c3[3];
  split3(t, ext[0], ext[1], c3[0], c3[1], c3[2]);
  c3[0] += 1; c3[1] += 1; c3[2] += 1;
  const int aa = c3[da], bb = c3[db];
  const int p0 = (int)gidx(g, c3[0], c3[1], c3[2]);
  const int sa = (int)g.st[da], sb = (int)g.st[db];
  const float *rn = A.rn, *sw = A.sw;
  const float dncv = 0.25f * (rn[p0] + rn[p0 - sa] + rn[p0 - sb] + rn[p0 - sa - sb]);
  const float dsqinv = rsqrtf(dncv);
  const float facm = A.facm, dt = A.dt;
  const float *Vx = A.vf[da], *Vy = A.vf[db], *Bxf = A.bf[da], *Byf = A.bf[db];
  const float *dxe = g.dxf[da], *dye = g.dxf[db];
  const float dxm = dxe[aa], dx0 = dxe[aa + 1], dym = dye[bb], dy0 = dye[bb + 1];
  const float2 sq = p2(dsqinv, -dsqinv), fm = p2(facm, facm);
  // (v + b s, v - b s) and ((q_v + q_b s) facm, (q_v - q_b s) facm), s = 1/sqrt(rho)
  auto chars = [&](const float *V, const float *B, int p, int sd, const float *dxx, int pos, float2 &a, float2 &d) {
    const LimW w = lim_w(dxx[pos], dxx[pos + 1], dxx[pos + 2], sw[p]);
    const float2 q = vlim_w2(p2(V[p - sd], B[p - sd]), p2(V[p], B[p]), p2(V[p + sd], B[p + sd]), w);
    const float v = V[p], b = B[p];
    a = pfma(p2(b, b), sq, p2(v, v));
    d = pmul(pfma(p2(q.y, q.y), sq, p2(q.x, q.x)), fm);
  };
  float2 a1L, d1L, a1R, d1R, a2L, d2L, a2R, d2R;
  chars(Vx, Bxf, p0 - sb, sb, dye, bb - 1, a1L, d1L);   // (a, b-1): (a1p, a1m), (da1p, da1m)
  chars(Vx, Bxf, p0, sb, dye, bb, a1R, d1R);            // (a, b)
  chars(Vy, Byf, p0 - sa, sa, dxe, aa - 1, a2L, d2L);   // (a-1, b): (a2p, a2m), (da2p, da2m)
  chars(Vy, Byf, p0, sa, dxe, aa, a2R, d2R);            // (a, b)
  auto swp = [](float2 v) { return make_float2(v.y, v.x); };
  const float2 mdt = p2(-dt, -dt), mdt2 = p2(-dt * dt, -dt * dt), one = p2(1.0f, 1.0f);
  auto cand = [&](float2 a1, float2 d1, float2 a2, float2 d2, float dyv, float dxv, float2 &C1, float2 &C2) {
    const float2 A1 = pfma(d1, p2(dyv, dyv), a1), A2 = pfma(d2, p2(dxv, dxv), a2);
    const float2 den = pfma(pmul(d1, d2), mdt2, one);
    const float2 r = p2(__fdividef(1.0f, den.x), __fdividef(1.0f, den.y));
    C1 = pmul(pfma(pmul(d1, A2), mdt, A1), r);
    C2 = pmul(pfma(pmul(d2, A1), mdt, A2), r);
  };
  // the second-side quantities enter as (a2m, a2p): the lanes swapped
  float2 C1LL, C2LL, C1RL, C2RL, C1LR, C2LR, C1RR, C2RR;
  cand(a1L, d1L, swp(a2L), swp(d2L), dym, dxm, C1LL, C2LL);     // S1 = +1, S2 = +1
  cand(a1R, d1R, swp(a2L), swp(d2L), -dy0, dxm, C1RL, C2RL);    // S1 = -1, S2 = +1
  cand(a1L, d1L, swp(a2R), swp(d2R), dym, -dx0, C1LR, C2LR);    // S1 = +1, S2 = -1
  cand(a1R, d1R, swp(a2R), swp(d2R), -dy0, -dx0, C1RR, C2RR);   // S1 = -1, S2 = -1
  const bool w11 = C1LL.x > 0.0f && C2LL.x > 0.0f, w12 = C1LL.y > 0.0f && C2LL.y > 0.0f;
  const bool w21 = C1RL.x > 0.0f && C2RL.x < 0.0f, w22 = C1RL.y > 0.0f && C2RL.y < 0.0f;
  const bool w31 = C1LR.x < 0.0f && C2LR.x > 0.0f, w32 = C1LR.y < 0.0f && C2LR.y > 0.0f;
  const bool w41 = C1RR.x < 0.0f && C2RR.x < 0.0f, w42 = C1RR.y < 0.0f && C2RR.y < 0.0f;
  // weight w + (1e13-1) * int(0.51 w1 + 0.51 w2): the boost is w1 AND w2
  const float big = 1.e13f - 1.0f;
  auto Wp = [&](bool x, bool y) {
    const float b = (x && y) ? big : 0.0f;
    return p2((x ? 1.0f : 0.0f) + b, (y ? 1.0f : 0.0f) + b);
  };
  float2 n1 = p2(0.0f, 0.0f), e1 = n1, n2 = n1, e2 = n1;
  auto acc = [&](float2 W, float2 C1, float2 C2) {
    const float2 u = pmul(W, pabs(C2)), v = pmul(W, pabs(C1));
    e1 = padd(e1, u);
    n1 = pfma(u, C1, n1);
    e2 = padd(e2, v);
    n2 = pfma(v, C2, n2);
  };
  acc(Wp(w11, w12), C1LL, C2LL);
  acc(Wp(w21, w22), C1RL, C2RL);
  acc(Wp(w31, w32), C1LR, C2LR);
  acc(Wp(w41, w42), C1RR, C2RR);
  const bool anyx = w11 || w21 || w31 || w41, anyy = w12 || w22 || w32 || w42;
  const float C1p = anyx ? __fdividef(n1.x, e1.x) : 0.0f, C2m = anyx ? __fdividef(n2.x, e2.x) : 0.0f;
  const float C1m = anyy ? __fdividef(n1.y, e1.y) : 0.0f, C2p = anyy ? __fdividef(n2.y, e2.y) : 0.0f;
  const float v1a = C1p + C1m, v2a = C2p + C2m, B1a = C1p - C1m, B2a = C2p - C2m;
  A.emf[E][p0] = 0.25f * (v1a * B2a - v2a * B1a) * (dncv * dsqinv);
}

// dt/dx(i) of every coordinate of the three axes (concatenated), once per
// CT: face_b32 reads them instead of forming three FP64 products per cell
// on the narrow FP64 pipe (the same products, so the update is unchanged)
__global__ void ct_coef32_kernel(Grid g, double dt, double *coef) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int s0 = g.s[0], s1 = g.s[1], s2 = g.s[2];
  if (t < s0) coef[t] = dt * g.rdxc[0][t];
  else if (t < s0 + s1) coef[t] = dt * g.rdxc[1][t - s0];
  else if (t < s0 + s1 + s2) coef[t] = dt * g.rdxc[2][t - s0 - s1];
}

// CC(3): face B from the EMF curl (:2159-2169); emf[0]=Ez, [1]=Ex, [2]=Ey
__global__ void __launch_bounds__(256) face_b32_kernel(Grid g, Fields f, const float *Ez, const float *Ex,
                                                       const float *Ey, const double *coef) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int nx1 = g.n[0] + 1, ny1 = g.n[1] + 1, nz1 = g.n[2] + 1;
  if (t >= (long long)nx1 * ny1 * nz1) return;
  int i, j, k;
  split3(t, nx1, ny1, i, j, k);
  i += 1; j += 1; k += 1;
  long long a = gidx(g, i, j, k);
  long long sx = 1, sy = g.st[1], sz = g.st[2];
  const double cx = coef[i + 1], cy = coef[g.s[0] + j + 1], cz = coef[g.s[0] + g.s[1] + k + 1];
  if (j <= g.n[1] && k <= g.n[2])
    f.U[5][a] = f.U[5][a] + cy * (f2d(Ez[a + sy]) - f2d(Ez[a])) - cz * (f2d(Ey[a + sz]) - f2d(Ey[a]));
  if (i <= g.n[0] && k <= g.n[2])
    f.U[6][a] = f.U[6][a] + cz * (f2d(Ex[a + sz]) - f2d(Ex[a])) - cx * (f2d(Ez[a + sx]) - f2d(Ez[a]));
  if (i <= g.n[0] && j <= g.n[1])
    f.U[7][a] = f.U[7][a] + cx * (f2d(Ey[a + sx]) - f2d(Ey[a])) - cy * (f2d(Ex[a + sy]) - f2d(Ex[a]));
}
#endif  // MHD_FP32_KERNELS

}  // namespace mhd
