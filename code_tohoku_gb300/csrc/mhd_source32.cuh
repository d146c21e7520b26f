// mhd_source32.cuh — chosen-form thermal SOURCE: the predictor/corrector of
// MCF3DSGincfca3.f90:2477-2572 with temperatures, conduction fluxes, the KI
// cooling function and the implicit solve in FP32, and the pressure
// accumulated in FP64 (p_new = p + dp).  The implicit solve is the same
// log-space bisection as IMC (:2898-2921); its midpoint
// 10^((log10 Pu + log10 Pd)/2) is evaluated as sqrt(Pu*Pd), which is the
// same number.  When a surrogate is attached (mhd_surrogate.cu) stiff cells
// first take the network's answer and fall back to the bisection when they
// are outside the training box or their implicit residual exceeds the
// tolerance.
#pragma once

#include "mhd_kernels.cuh"
#include "mhd_surrogate_net.cuh"

namespace mhd {

// KI cooling and its temperature derivative (FP32), for the Newton polish
__device__ __forceinline__ void fcool_ki_d(float T, float NN, float &L, float &dL) {
  float Tk = T * 1.0e3f;
  float el = __expf(-1.184e5f / (Tk + 1.0e3f));
  float Laml = 1.0e7f * el;
  float dLaml = 0.0f;
  if (Laml > 5.e3f) Laml = 5.e3f;
  else dLaml = Laml * 1.184e5f * 1.0e3f / ((Tk + 1.0e3f) * (Tk + 1.0e3f));
  float Lamc = 1.4e-2f * sqrtf(Tk) * __expf(-9.2e1f / Tk);
  float dLamc = Lamc * (0.5f / T + 9.2e1f / (T * Tk));
  L = (NN * NN * (Laml + Lamc) - NN) * 3.94656e1f;
  dL = NN * NN * (dLaml + dLamc) * 3.94656e1f;
}

__device__ __forceinline__ float imc32(float Pold, float nkbi, float c /* dt*g1 */, float NN) {
  float Pu = 1.e10f, Pd = 1.e-10f, Pm = 1.e1f, Pmold = -1.0f;
  for (int k = 0; k < 30; k++) {
    float CooL = fcool_ki(Pm * nkbi, NN);
    float fev = Pm + CooL * c - Pold;
    float iud = fev >= 0.0f ? 1.0f : -1.0f;
    Pd = fmx(-iud * Pm, Pd);
    Pu = fmn(2.0f * Pm / (iud + 1.0f + 1.e-10f), Pu);
    Pm = sqrtf(Pu * Pd);
    if (fabsf(Pm - Pmold) < 1.e-5f) break;
    Pmold = Pm;
  }
  return Pm;
}

struct Source32Args {
  Grid g;
  Phys ph;
  Fields f;
  const double *pin;
  const double *pold;
  double *pout;
  double dt;
  int pass;
  int *err;
  unsigned long long *imc_count;
  unsigned long long *sur_count;   // surrogate accepted
  unsigned long long *fb_count;    // surrogate rejected -> bisection
  const SurNet *W;                 // surrogate network (null: exact only)
  float tol;                       // residual tolerance for accepting it
};

}  // namespace mhd

namespace mhd {

#ifdef MHD_FP32_KERNELS
// One pass of the chosen-form SOURCE for one cell (thread per cell).
__global__ void __launch_bounds__(128) source32_kernel(Source32Args A) {
  const Grid &g = A.g;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  bool valid = t < (long long)nx * ny * nz;
  long long tt = valid ? t : 0;
  int i = 1 + (int)(tt % nx);
  int j = 1 + (int)((tt / nx) % ny);
  int k = 1 + (int)(tt / ((long long)nx * ny));
  long long a = gidx(g, i, j, k);
  const float kb = (float)A.ph.kb, Kc = (float)A.ph.kcond;
  const float dt = (float)A.dt;
  const double *pin = A.pin;
  const Fields &f = A.f;
  auto ntot = [&](long long c) { return (float)(f.sp[1][c] + f.sp[0][c] + f.sp[2][c] + f.sp[3][c] + f.sp[4][c]); };
  auto Tn = [&](long long c) { return (float)pin[c] / (kb * ntot(c)); };
  const double *dx = g.dx[0], *dy = g.dx[1], *dz = g.dx[2];
  long long sy = g.st[1], sz = g.st[2];
  float T0 = Tn(a);
  auto flux = [&](float Tl, float Tu, float dl, float du) {
    float rt = sqrtf((dl * Tu + du * Tl) / (dl + du));
    return Kc * fminf(rt, 3.873f) * (Tu - Tl) * 2.0f / (dl + du);
  };
  float dxm = (float)dx[i], dx0 = (float)dx[i + 1], dxp = (float)dx[i + 2];
  float dym = (float)dy[j], dy0 = (float)dy[j + 1], dyp = (float)dy[j + 2];
  float dzm = (float)dz[k], dz0 = (float)dz[k + 1], dzp = (float)dz[k + 2];
  float div = (flux(T0, Tn(a + 1), dx0, dxp) - flux(Tn(a - 1), T0, dxm, dx0)) / dx0 +
              (flux(T0, Tn(a + sy), dy0, dyp) - flux(Tn(a - sy), T0, dym, dy0)) / dy0 +
              (flux(T0, Tn(a + sz), dz0, dzp) - flux(Tn(a - sz), T0, dzm, dz0)) / dz0;
  float H = (float)f.sp[0][a], pr = (float)f.sp[1][a], H2 = (float)f.sp[2][a], He = (float)f.sp[3][a],
        Hep = (float)f.sp[4][a];
  float g1 = (2.0f * (H + pr + He + Hep) + 2.0f * H2) / (3.0f * (H + pr + He + Hep) + 5.0f * H2);
  float NN = (float)f.U[0][a] / 1.27f;
  float CooL = fcool_ki(T0, NN);
  double Pn = A.pold[a];
  float h = (A.pass == 0) ? 0.5f : 1.0f;          // predictor: half of dt
  float dts = dt * h;
  double base = (A.pass == 0) ? pin[a] : Pn;       // p the cooling acts on
  bool stiff = valid && !((float)dt <= 0.2f * (float)Pn / (g1 * fabsf(CooL)));
  double dp_cool = 0.0;
  bool need_imc = stiff;
  float nimc = H + pr + He + Hep + H2;
  float nkbi = 1.0f / (kb * nimc);
  float Tb = (float)base * nkbi;                  // temperature the implicit solve starts from
  if (A.W) {
    // surrogate: inputs log10 N, log10 T, log10(dts / t_cool) with
    // t_cool = P/((gamma-1)|Lambda|) at the starting state
    float Lb = fcool_ki(Tb, NN);
    float r = dts * g1 * fabsf(Lb) / (float)base;
    float x0 = log10f(NN), x1 = log10f(Tb), x2 = log10f(fmaxf(r, 1e-30f));
    bool inbox = stiff && x0 >= -2.0f && x0 <= 5.0f && x1 >= -2.0f && x1 <= 1.30103f && x2 >= -3.0f && x2 <= 3.0f;
    float conf;
    float y = surrogate_warp(A.W, x0, x1, x2, inbox, &conf);
    if (inbox) {
      // the network's answer, polished by two Newton steps on
      // f(P) = P + c Lambda(P) - P_start (c = dt (gamma-1)), then checked
      float c = dts * g1;
      float P = (Tb * exp10f(y)) / nkbi;
      for (int it = 0; it < 2; it++) {
        float L, dL;
        fcool_ki_d(P * nkbi, NN, L, dL);
        float fv = P + c * L - (float)base;
        float fp = 1.0f + c * dL * nkbi;
        if (fp > 0.0f) P = fmaxf(P - fv / fp, 0.1f * P);
      }
      // implicit residual |P + Lambda(P) dt (gamma-1) - P_old| / P_old
      float res = fabsf(P + fcool_ki(P * nkbi, NN) * c - (float)base) / (float)base;
      if (res <= A.tol) {
        dp_cool = (double)P - base;
        need_imc = false;
        atomicAdd(A.sur_count, 1ull);
      } else {
        atomicAdd(A.fb_count, 1ull);
      }
    }
  }
  if (!valid) return;
  if (!stiff) {
    dp_cool = -(double)(g1 * CooL * dts);
  } else if (need_imc) {
    float Pm = imc32((float)base, nkbi, dts * g1, NN);
    dp_cool = (double)Pm - base;
    atomicAdd(A.imc_count, 1ull);
  }
  float tcd = g1 * Kc * sqrtf(T0);
  tcd = 0.49f * nimc * kb / tcd * (dx0 * dx0);
  float w = (tcd - dt >= 0.0f) ? 1.0f : 0.0f;      // (sign(0.5, tcd-dt) + 0.5)
  double pnew = base + dp_cool + (double)(w * g1 * dts * div);
  pnew = fmx(pnew, A.ph.pmin);
  pnew = fmn(pnew, A.ph.pmax);
  A.pout[a] = pnew;
  if (!(pnew == pnew)) flag(A.err, ERRB_NONFINITE);
}

#endif  // MHD_FP32_KERNELS

}  // namespace mhd
