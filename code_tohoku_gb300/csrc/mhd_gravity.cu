// mhd_gravity.cu — self-gravity (ifgrv = 2): the potential of
// grad^2 Phi = 4 pi G rho, periodic in y and z and isolated in x, and the
// half kicks of the velocities by its gradient.
//
// The reference (3DMHD-CfCA/selfG_MPIfull8.f90, GRAVTY) takes the potential
// on the two x faces from the density's y-z Fourier modes through the
// Green's function of d^2/dx^2 - kap^2, kap^2 = 4 sin^2(pi l/Ny)/dy^2 +
// 4 sin^2(pi m/Nz)/dz^2 the eigenvalue of the discrete y-z Laplacian (PB
// :1133-1200), and relaxes the interior by multigrid with those faces as
// Dirichlet values.  Here the same discrete problem is solved directly:
//   1. complex FFTs of rho along y and along z (radix 2, shared memory);
//   2. per mode (l, m): the face values by the Green's function sums and
//      the tridiagonal system of the second-order x Laplacian minus kap^2
//      (the Thomas algorithm, one thread per mode), the faces entering
//      through the ghost reflection Phi_0 = 2 Phi_face - Phi_1;
//   3. the inverse FFTs, the real part, and the ghosts: x copies of the
//      edge cells (grad = 0, GRAVTY :70-75), y and z periodic.
// The half kick (GRAVTY mode 3, :90-97) is the fourth-order central
// difference with dx(0) in every direction.  FP64 throughout; the unit is
// built with --fmad=false like the plain form.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "mhd_launch.h"

namespace mhd {

namespace {

constexpr double kG4pi = 12.56637 * 1.11142e-4;   // MCF3DSGincfca3.f90:35

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__global__ void grav_load_kernel(Grid g, const double *rho, double2 *w) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nx = g.n[0], ny = g.n[1];
  if (t >= (long long)nx * ny * g.n[2]) return;
  w[t] = make_double2(rho[gidx_lin(g, t, nx, ny)], 0.0);
}

// Radix-2 FFT of lines of n = 2^logn complex values: line (a, b) starts at
// a + b * step_b and advances by `stride`; a CTA takes `lpc` lines of
// consecutive a (so the loads of one position are contiguous), n/2 threads
// per line.  Loaded in bit-reversed order, transformed in place
// (decimation in time); tw[k] = exp(sign 2 pi i k / n), k < n/2.
__global__ void fft_lines_kernel(double2 *w, int logn, long long stride, int na, long long step_b, int lpc,
                                 const double2 *tw) {
  extern __shared__ double2 fsm[];
  const int n = 1 << logn, half = n >> 1;
  const int l = threadIdx.x % lpc, q = threadIdx.x / lpc;   // line within the CTA, butterfly index
  const int a = blockIdx.x * lpc + l;
  const bool on = a < na;
  const long long base = (long long)a + (long long)blockIdx.y * step_b;
  double2 *x = fsm + (size_t)l * n;
  if (on) {
    for (int j = q; j < n; j += half) {
      const int r = (int)(__brev((unsigned)j) >> (32 - logn));
      x[r] = w[base + (long long)j * stride];
    }
  }
  __syncthreads();
  for (int len = 2; len <= n; len <<= 1) {
    const int h = len >> 1;
    if (on) {
      const int grp = q / h, pos = q - grp * h;
      const int i0 = grp * len + pos, i1 = i0 + h;
      const double2 u = x[i0], v = cmul(x[i1], tw[pos * (n / len)]);
      x[i0] = make_double2(u.x + v.x, u.y + v.y);
      x[i1] = make_double2(u.x - v.x, u.y - v.y);
    }
    __syncthreads();
  }
  if (on)
    for (int j = q; j < n; j += half) w[base + (long long)j * stride] = x[j];
}

// One thread per y-z mode: the face values and the x solve (row i of the
// system: (Phi_{i-1} - 2 Phi_i + Phi_{i+1}) / dx^2 - kap^2 Phi_i = G4pi rho_i).
// cp: nx doubles per mode of scratch for the Thomas coefficients.
__global__ void grav_modes_kernel(Grid g, double2 *w, double *cp, double dx, double dy, double dz, double x0,
                                  double lbox) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  if (t >= (long long)ny * nz) return;
  const int l = (int)(t % ny), m = (int)(t / ny);
  const double sy = sin(M_PI * l / ny), sz = sin(M_PI * m / nz);
  const double kap2 = 4.0 * sy * sy / (dy * dy) + 4.0 * sz * sz / (dz * dz);
  const double kap = sqrt(kap2);
  double2 *wl = w + (long long)t * nx;   // the mode's x line (x is the fastest index)
  double *c = cp + (long long)t * nx;
  const double *xe = g.x[0];
  double2 bl = make_double2(0.0, 0.0), br = make_double2(0.0, 0.0);
  for (int i = 0; i < nx; i++) {
    const double xcen = 0.5 * (xe[i + 1] + xe[i + 2]);   // centre of cell i+1: x(i), x(i+1) are its faces
    const double d1 = xcen - x0, d2 = lbox - d1;
    double f1, f2;
    if (l == 0 && m == 0) {
      f1 = 0.5 * kG4pi * dx * d1;
      f2 = 0.5 * kG4pi * dx * d2;
    } else {
      f1 = -0.5 * kG4pi * dx * exp(-kap * d1) / kap;
      f2 = -0.5 * kG4pi * dx * exp(-kap * d2) / kap;
    }
    const double2 r = wl[i];
    bl = make_double2(bl.x + r.x * f1, bl.y + r.y * f1);
    br = make_double2(br.x + r.x * f2, br.y + r.y * f2);
  }
  const double a = 1.0 / (dx * dx), b0 = -2.0 / (dx * dx) - kap2, be = -3.0 / (dx * dx) - kap2;
  // forward elimination (the right-hand side overwrites the line)
  const double d0 = (nx == 1) ? (-4.0 / (dx * dx) - kap2) : be;
  double2 rhs = make_double2(wl[0].x * kG4pi - 2.0 * a * bl.x, wl[0].y * kG4pi - 2.0 * a * bl.y);
  if (nx == 1) rhs = make_double2(rhs.x - 2.0 * a * br.x, rhs.y - 2.0 * a * br.y);
  double cprev = a / d0;
  double2 dprev = make_double2(rhs.x / d0, rhs.y / d0);
  c[0] = cprev;
  wl[0] = dprev;
  for (int i = 1; i < nx; i++) {
    const double bi = (i == nx - 1) ? be : b0;
    const double den = bi - a * cprev;
    double2 ri = make_double2(wl[i].x * kG4pi, wl[i].y * kG4pi);
    if (i == nx - 1) ri = make_double2(ri.x - 2.0 * a * br.x, ri.y - 2.0 * a * br.y);
    cprev = a / den;
    dprev = make_double2((ri.x - a * dprev.x) / den, (ri.y - a * dprev.y) / den);
    c[i] = cprev;
    wl[i] = dprev;
  }
  for (int i = nx - 2; i >= 0; i--) {
    const double2 nxt = wl[i + 1], cur = wl[i];
    wl[i] = make_double2(cur.x - c[i] * nxt.x, cur.y - c[i] * nxt.y);
  }
}

__global__ void grav_store_kernel(Grid g, const double2 *w, double *phi, double scale) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nx = g.n[0], ny = g.n[1];
  if (t >= (long long)nx * ny * g.n[2]) return;
  phi[gidx_lin(g, t, nx, ny)] = w[t].x * scale;
}

// ghosts: x (interior j, k) copies of the edge cells; then y over every i,
// interior k; then z over every i, j (the order of the oracle's passes)
__global__ void grav_ghost_x_kernel(Grid g, double *phi) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int ny = g.n[1], nz = g.n[2], nx = g.n[0];
  if (t >= (long long)ny * nz) return;
  const int j = 1 + (int)(t % ny), k = 1 + (int)(t / ny);
  const double lft = phi[gidx(g, 1, j, k)], rgt = phi[gidx(g, nx, j, k)];
  phi[gidx(g, 0, j, k)] = lft;
  phi[gidx(g, -1, j, k)] = lft;
  phi[gidx(g, nx + 1, j, k)] = rgt;
  phi[gidx(g, nx + 2, j, k)] = rgt;
}
__global__ void grav_ghost_y_kernel(Grid g, double *phi) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int sx = g.s[0], nz = g.n[2], ny = g.n[1];
  if (t >= (long long)sx * nz * 4) return;
  const int i = (int)(t % sx) - 1, k = 1 + (int)((t / sx) % nz), q = (int)(t / ((long long)sx * nz));
  const int j = q < 2 ? q - 1 : ny + q - 1;          // -1, 0, ny+1, ny+2
  const int js = j < 1 ? j + ny : j - ny;
  phi[gidx(g, i, j, k)] = phi[gidx(g, i, js, k)];
}
__global__ void grav_ghost_z_kernel(Grid g, double *phi) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int sx = g.s[0], sy = g.s[1], nz = g.n[2];
  if (t >= (long long)sx * sy * 4) return;
  const int i = (int)(t % sx) - 1, j = (int)((t / sx) % sy) - 1, q = (int)(t / ((long long)sx * sy));
  const int k = q < 2 ? q - 1 : nz + q - 1;
  const int ks = k < 1 ? k + nz : k - nz;
  phi[gidx(g, i, j, k)] = phi[gidx(g, i, j, ks)];
}

// GRAVTY mode 3 (:90-97)
__global__ void grav_kick_kernel(Grid g, Fields f, const double *phi, double dt, double dxi) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nx = g.n[0], ny = g.n[1];
  if (t >= (long long)nx * ny * g.n[2]) return;
  const long long a = gidx_lin(g, t, nx, ny), sy = g.st[1], sz = g.st[2];
  const double *F = phi;
  f.U[1][a] = f.U[1][a] - dt * (-F[a + 2] + 8.0 * F[a + 1] - 8.0 * F[a - 1] + F[a - 2]) * dxi * 0.5;
  f.U[2][a] = f.U[2][a] - dt * (-F[a + 2 * sy] + 8.0 * F[a + sy] - 8.0 * F[a - sy] + F[a - 2 * sy]) * dxi * 0.5;
  f.U[3][a] = f.U[3][a] - dt * (-F[a + 2 * sz] + 8.0 * F[a + sz] - 8.0 * F[a - sz] + F[a - 2 * sz]) * dxi * 0.5;
}

unsigned nblk(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

int ilog2(int n) {
  int l = 0;
  while ((1 << l) < n) l++;
  return l;
}

cudaError_t fft_lines(double2 *w, int n, long long stride, int na, int nb, long long step_b, const double2 *tw,
                      cudaStream_t s) {
  if (n == 1) return cudaSuccess;   // the transform of one value is itself
  const int half = n / 2 > 0 ? n / 2 : 1;
  int lpc = 1024 / half;
  const int cap = 3072 / n;   // at most 48 KB of lines in shared memory
  if (lpc > cap) lpc = cap;
  if (lpc > na) lpc = na;
  if (lpc < 1) lpc = 1;
  dim3 grid((unsigned)((na + lpc - 1) / lpc), (unsigned)nb);
  fft_lines_kernel<<<grid, lpc * half, (size_t)lpc * n * sizeof(double2), s>>>(w, ilog2(n), stride, na, step_b, lpc,
                                                                              tw);
  return cudaGetLastError();
}

}  // namespace

bool gravity_size_ok(int n) { return n >= 1 && n <= 1024 && (n & (n - 1)) == 0; }

// exp(sign 2 pi i k / n), k < n/2, for sign -1 then +1: 2 * (n/2) values
std::vector<double2> gravity_twiddles(int n) {
  std::vector<double2> t((size_t)(n / 2 > 0 ? n / 2 : 1) * 2);
  const int h = n / 2 > 0 ? n / 2 : 1;
  for (int k = 0; k < h; k++) {
    const double ang = 2.0 * M_PI * (double)k / (double)n;
    t[k] = make_double2(std::cos(ang), -std::sin(ang));
    t[h + k] = make_double2(std::cos(ang), std::sin(ang));
  }
  return t;
}

cudaError_t gravity_solve(const GravityArgs &a, cudaStream_t s) {
  const Grid &g = a.g;
  const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const long long ncells = (long long)nx * ny * nz, nmodes = (long long)ny * nz;
  const int hy = ny / 2 > 0 ? ny / 2 : 1, hz = nz / 2 > 0 ? nz / 2 : 1;
  cudaError_t e;
  grav_load_kernel<<<nblk(ncells, 256), 256, 0, s>>>(g, a.rho, a.w);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // y lines: stride nx, one per (i, k); z lines: stride nx ny, one per (i, j)
  if ((e = fft_lines(a.w, ny, nx, nx, nz, (long long)nx * ny, a.tw_y, s)) != cudaSuccess) return e;
  if ((e = fft_lines(a.w, nz, (long long)nx * ny, nx, ny, nx, a.tw_z, s)) != cudaSuccess) return e;
  grav_modes_kernel<<<nblk(nmodes, 128), 128, 0, s>>>(g, a.w, a.cp, a.dx, a.dy, a.dz, a.x0, a.lbox);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = fft_lines(a.w, nz, (long long)nx * ny, nx, ny, nx, a.tw_z + hz, s)) != cudaSuccess) return e;
  if ((e = fft_lines(a.w, ny, nx, nx, nz, (long long)nx * ny, a.tw_y + hy, s)) != cudaSuccess) return e;
  grav_store_kernel<<<nblk(ncells, 256), 256, 0, s>>>(g, a.w, a.phi, 1.0 / ((double)ny * (double)nz));
  grav_ghost_x_kernel<<<nblk(nmodes, 256), 256, 0, s>>>(g, a.phi);
  grav_ghost_y_kernel<<<nblk((long long)g.s[0] * nz * 4, 256), 256, 0, s>>>(g, a.phi);
  grav_ghost_z_kernel<<<nblk((long long)g.s[0] * g.s[1] * 4, 256), 256, 0, s>>>(g, a.phi);
  return cudaGetLastError();
}

cudaError_t gravity_kick(const Grid &g, const Fields &f, const double *phi, double dt, double dx0, cudaStream_t s) {
  const long long n = (long long)g.n[0] * g.n[1] * g.n[2];
  grav_kick_kernel<<<nblk(n, 256), 256, 0, s>>>(g, f, phi, dt, 1.0 / (12.0 * dx0));
  return cudaGetLastError();
}

}  // namespace mhd
