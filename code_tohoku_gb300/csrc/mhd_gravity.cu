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
//   1. y transforms of the real density, two z rows per complex FFT
//      (radix 4 in shared memory), unpacked into the half spectrum
//      l = 0..Ny/2 (the rest is its complex conjugate);
//   2. z transforms of the half spectrum (complex, radix 4);
//   3. per mode (l, m): the face values by the Green's function sums and the
//      tridiagonal system of the second-order x Laplacian minus kap^2 (the
//      Thomas algorithm, one thread per mode), the faces entering through
//      the ghost reflection Phi_0 = 2 Phi_face - Phi_1.  The Green's weights
//      and the elimination coefficients depend on the grid only, so they
//      are tabulated once per grid;
//   4. inverse z transforms, then inverse y transforms that pack two z rows
//      into one complex FFT again and write the two real rows;
//   5. the ghosts: x copies of the edge cells (grad = 0, GRAVTY :70-75),
//      y and z periodic.
// The spectrum is laid out [x][z][l] (x slowest), so the mode solve's
// threads read consecutive words at every x.  The half kick (GRAVTY mode 3,
// :90-97) is the fourth-order central difference with dx(0) in every
// direction.  FP64 throughout.
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

__device__ __forceinline__ int bitrev(int j, int logn) {
  return logn > 0 ? (int)(__brev((unsigned)j) >> (32 - logn)) : 0;
}

// exp(sign 2 pi i m / n) for m < n from the table of its first n/2 values
__device__ __forceinline__ double2 twid(const double2 *tw, int m, int n) {
  const int hn = n >> 1;
  if (m < hn) return tw[m];
  const double2 w = tw[m - hn];
  return make_double2(-w.x, -w.y);
}

// In-place decimation in time of a line of n = 2^logn values held in
// bit-reversed order: a radix-2 stage first when logn is odd, then radix-4
// stages, each combining four transforms of length h (at offsets 0, h, 2h,
// 3h: input residues 0, 2, 1, 3 mod 4 of the bit-reversed order) into one
// of length 4h with three twiddle products (none in the first stage).
// tw[k] = exp(sign 2 pi i k / n), k < n/2; inv: sign = +1.  Thread q < nt of
// the line takes butterflies q, q + nt, ...; every thread of the CTA calls
// it (barriers inside); `on` masks the lines beyond the grid.
__device__ __forceinline__ void fft_stages(double2 *x, int n, int logn, int q, int nt, bool on, const double2 *tw,
                                           bool inv) {
  int h = 1;
  if (logn & 1) {
    if (on)
      for (int b = q; b < (n >> 1); b += nt) {
        const double2 u = x[2 * b], v = x[2 * b + 1];
        x[2 * b] = make_double2(u.x + v.x, u.y + v.y);
        x[2 * b + 1] = make_double2(u.x - v.x, u.y - v.y);
      }
    __syncthreads();
    h = 2;
  }
  for (; h < n; h <<= 2) {
    if (on)
      for (int b = q; b < (n >> 2); b += nt) {
        const int grp = b / h, p = b - grp * h;
        const int i0 = grp * 4 * h + p;
        const double2 e0 = x[i0], e1 = x[i0 + h], e2 = x[i0 + 2 * h], e3 = x[i0 + 3 * h];
        double2 t1 = e2, t2 = e1, t3 = e3;
        if (h > 1) {
          const int st = n / (4 * h);
          t1 = cmul(e2, twid(tw, p * st, n));
          t2 = cmul(e1, twid(tw, 2 * p * st, n));
          t3 = cmul(e3, twid(tw, 3 * p * st, n));
        }
        const double2 ap = make_double2(e0.x + t2.x, e0.y + t2.y), am = make_double2(e0.x - t2.x, e0.y - t2.y);
        const double2 cp = make_double2(t1.x + t3.x, t1.y + t3.y), dm = make_double2(t1.x - t3.x, t1.y - t3.y);
        x[i0] = make_double2(ap.x + cp.x, ap.y + cp.y);
        x[i0 + 2 * h] = make_double2(ap.x - cp.x, ap.y - cp.y);
        // X1 = am + s dm, X3 = am - s dm, s = sign i
        if (inv) {
          x[i0 + h] = make_double2(am.x - dm.y, am.y + dm.x);
          x[i0 + 3 * h] = make_double2(am.x + dm.y, am.y - dm.x);
        } else {
          x[i0 + h] = make_double2(am.x + dm.y, am.y - dm.x);
          x[i0 + 3 * h] = make_double2(am.x - dm.y, am.y + dm.x);
        }
      }
    __syncthreads();
  }
}

// threads per line of n values
__host__ __device__ __forceinline__ int fft_threads(int n) { return n >= 4 ? n >> 2 : 1; }

// Forward y transforms: the CTA takes lpc lines of consecutive x (so the
// loads of one y position are contiguous) for the z rows k0 = 2 blockIdx.y
// and k0 + 1, packed as the real and imaginary parts of one complex line
// (k0 + 1 = nz: zero).  With Z the transform, the two real rows have
// A_l = (Z_l + conj Z_{n-l}) / 2 and B_l = (Z_l - conj Z_{n-l}) / 2i,
// stored for l = 0..ny/2 at S[(i nz + k) nyh + l].
__global__ void grav_fwd_y_kernel(Grid g, const double *rho, double2 *S, int logny, int lpc, const double2 *tw) {
  extern __shared__ double2 fsm[];
  const int nx = g.n[0], ny = g.n[1], nz = g.n[2], nyh = ny / 2 + 1;
  const int nt = fft_threads(ny);
  const int l = threadIdx.x % lpc, q = threadIdx.x / lpc;
  const int i = blockIdx.x * lpc + l;
  const int k0 = 2 * blockIdx.y, k1 = k0 + 1;
  const bool on = i < nx;
  double2 *x = fsm + (size_t)l * ny;
  if (on) {
    for (int j = q; j < ny; j += nt) {
      const double a = rho[gidx(g, i + 1, j + 1, k0 + 1)];
      const double b = k1 < nz ? rho[gidx(g, i + 1, j + 1, k1 + 1)] : 0.0;
      x[bitrev(j, logny)] = make_double2(a, b);
    }
  }
  __syncthreads();
  fft_stages(x, ny, logny, q, nt, on, tw, false);
  // consecutive threads store consecutive l of one line
  for (int e = threadIdx.x; e < lpc * nyh; e += blockDim.x) {
    const int ll = e / nyh, m = e - ll * nyh, ii = blockIdx.x * lpc + ll;
    if (ii >= nx) continue;
    const double2 *xl = fsm + (size_t)ll * ny;
    const double2 zl = xl[m], zn = xl[(ny - m) & (ny - 1)];
    S[((size_t)ii * nz + k0) * nyh + m] = make_double2(0.5 * (zl.x + zn.x), 0.5 * (zl.y - zn.y));
    if (k1 < nz) S[((size_t)ii * nz + k1) * nyh + m] = make_double2(0.5 * (zl.y + zn.y), -0.5 * (zl.x - zn.x));
  }
}

// Inverse y transforms of the rows k0, k0 + 1 of x lines i: Z_l = A_l + i B_l
// for every l (A_{n-l} = conj A_l, likewise B), transformed back and written
// as phi(i, j, k0) = Re, phi(i, j, k0 + 1) = Im, times `scale`.
__global__ void grav_inv_y_kernel(Grid g, const double2 *S, double *phi, int logny, int lpc, const double2 *tw,
                                  double scale) {
  extern __shared__ double2 fsm[];
  const int nx = g.n[0], ny = g.n[1], nz = g.n[2], nyh = ny / 2 + 1;
  const int nt = fft_threads(ny);
  const int k0 = 2 * blockIdx.y, k1 = k0 + 1;
  for (int e = threadIdx.x; e < lpc * nyh; e += blockDim.x) {
    const int ll = e / nyh, m = e - ll * nyh, ii = blockIdx.x * lpc + ll;
    if (ii >= nx) continue;
    double2 *xl = fsm + (size_t)ll * ny;
    const double2 A = S[((size_t)ii * nz + k0) * nyh + m];
    const double2 B = k1 < nz ? S[((size_t)ii * nz + k1) * nyh + m] : make_double2(0.0, 0.0);
    xl[bitrev(m & (ny - 1), logny)] = make_double2(A.x - B.y, A.y + B.x);
    if (m > 0 && m < ny - m) xl[bitrev(ny - m, logny)] = make_double2(A.x + B.y, B.x - A.y);
  }
  __syncthreads();
  const int l = threadIdx.x % lpc, q = threadIdx.x / lpc;
  const int i = blockIdx.x * lpc + l;
  const bool on = i < nx;
  double2 *x = fsm + (size_t)l * ny;
  fft_stages(x, ny, logny, q, nt, on, tw, true);
  if (on) {
    for (int j = q; j < ny; j += nt) {
      const double2 v = x[j];
      phi[gidx(g, i + 1, j + 1, k0 + 1)] = v.x * scale;
      if (k1 < nz) phi[gidx(g, i + 1, j + 1, k1 + 1)] = v.y * scale;
    }
  }
}

// FFT of lines of n = 2^logn complex values: line (a, b) starts at
// a + b * step_b and advances by `stride`; a CTA takes `lpc` lines of
// consecutive a (so the loads of one position are contiguous),
// fft_threads(n) threads per line.
__global__ void fft_lines_kernel(double2 *w, int logn, long long stride, int na, long long step_b, int lpc,
                                 const double2 *tw, bool inv) {
  extern __shared__ double2 fsm[];
  const int n = 1 << logn, nt = fft_threads(n);
  const int l = threadIdx.x % lpc, q = threadIdx.x / lpc;   // line within the CTA, thread of the line
  const int a = blockIdx.x * lpc + l;
  const bool on = a < na;
  const long long base = (long long)a + (long long)blockIdx.y * step_b;
  double2 *x = fsm + (size_t)l * n;
  if (on)
    for (int j = q; j < n; j += nt) x[bitrev(j, logn)] = w[base + (long long)j * stride];
  __syncthreads();
  fft_stages(x, n, logn, q, nt, on, tw, inv);
  if (on)
    for (int j = q; j < n; j += nt) w[base + (long long)j * stride] = x[j];
}

// The grid's tables, one thread per mode (l, m) of the half spectrum, for
// every x cell i (row of the system (Phi_{i-1} - 2 Phi_i + Phi_{i+1}) / dx^2
// - kap^2 Phi_i = G4pi rho_i): the Green's weights of the two faces and the
// elimination coefficients c_i = a / den_i and 1 / den_i.  Layout: table q
// at tab[(q nx + i) nmh + mode].
__global__ void grav_table_kernel(Grid g, double *tab, double dx, double dy, double dz, double x0, double lbox) {
  const int nx = g.n[0], ny = g.n[1], nz = g.n[2], nyh = ny / 2 + 1;
  const long long nmh = (long long)nyh * nz;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nmh) return;
  const int l = (int)(t % nyh), m = (int)(t / nyh);
  const double sy = sin(M_PI * l / ny), sz = sin(M_PI * m / nz);
  const double kap2 = 4.0 * sy * sy / (dy * dy) + 4.0 * sz * sz / (dz * dz);
  const double kap = sqrt(kap2);
  const double *xe = g.x[0];
  const double a = 1.0 / (dx * dx), b0 = -2.0 / (dx * dx) - kap2, be = -3.0 / (dx * dx) - kap2;
  const size_t N = (size_t)nx * nmh;
  double cprev = 0.0;
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
    double den;
    if (i == 0) den = (nx == 1) ? (-4.0 / (dx * dx) - kap2) : be;
    else den = ((i == nx - 1) ? be : b0) - a * cprev;
    const double inv = 1.0 / den;
    cprev = a * inv;
    const size_t o = (size_t)i * nmh + t;
    tab[o] = f1;
    tab[N + o] = f2;
    tab[2 * N + o] = cprev;
    tab[3 * N + o] = inv;
  }
}

// One thread per mode: the face values, the forward elimination (the
// right-hand side overwrites the line) and the back substitution; the
// mode's value at x cell i is S[i nmh + mode].  There are only ny/2+1 times
// nz modes (about seven warps per SM at 256^3), so each pass loads a batch
// of kGB x cells before it uses any: one memory wait per batch instead of
// one per cell.
constexpr int kGB = 8;
__global__ void grav_modes_kernel(Grid g, double2 *S, const double *tab, double dx) {
  const int nx = g.n[0], nyh = g.n[1] / 2 + 1;
  const long long nmh = (long long)nyh * g.n[2];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nmh) return;
  const size_t N = (size_t)nx * nmh;
  const double *f1 = tab, *f2 = tab + N, *cc = tab + 2 * N, *iv = tab + 3 * N;
  double2 *Sm = S + t;   // Sm[i nmh]: the mode at x cell i
  double2 bl = make_double2(0.0, 0.0), br = make_double2(0.0, 0.0);
  for (int i0 = 0; i0 < nx; i0 += kGB) {
    double2 r[kGB];
    double w1[kGB], w2[kGB];
#pragma unroll
    for (int u = 0; u < kGB; u++) {
      if (i0 + u < nx) {
        const size_t o = (size_t)(i0 + u) * nmh + t;
        r[u] = Sm[(size_t)(i0 + u) * nmh];
        w1[u] = f1[o];
        w2[u] = f2[o];
      }
    }
#pragma unroll
    for (int u = 0; u < kGB; u++) {
      if (i0 + u < nx) {
        bl = make_double2(bl.x + r[u].x * w1[u], bl.y + r[u].y * w1[u]);
        br = make_double2(br.x + r[u].x * w2[u], br.y + r[u].y * w2[u]);
      }
    }
  }
  const double a = 1.0 / (dx * dx);
  double2 d = make_double2(0.0, 0.0);
  for (int i0 = 0; i0 < nx; i0 += kGB) {
    double2 r[kGB];
    double inv[kGB];
#pragma unroll
    for (int u = 0; u < kGB; u++) {
      if (i0 + u < nx) {
        r[u] = Sm[(size_t)(i0 + u) * nmh];
        inv[u] = iv[(size_t)(i0 + u) * nmh + t];
      }
    }
#pragma unroll
    for (int u = 0; u < kGB; u++) {
      const int i = i0 + u;
      if (i < nx) {
        double2 ri = make_double2(r[u].x * kG4pi, r[u].y * kG4pi);
        if (i == 0) ri = make_double2(ri.x - 2.0 * a * bl.x, ri.y - 2.0 * a * bl.y);
        if (i == nx - 1) ri = make_double2(ri.x - 2.0 * a * br.x, ri.y - 2.0 * a * br.y);
        d = make_double2((ri.x - a * d.x) * inv[u], (ri.y - a * d.y) * inv[u]);
        Sm[(size_t)i * nmh] = d;
      }
    }
  }
  // back substitution, x cells nx-2 down to 0, in batches from the top
  for (int i1 = nx - 2; i1 >= 0; i1 -= kGB) {
    double2 r[kGB];
    double c[kGB];
#pragma unroll
    for (int u = 0; u < kGB; u++) {
      if (i1 - u >= 0) {
        r[u] = Sm[(size_t)(i1 - u) * nmh];
        c[u] = cc[(size_t)(i1 - u) * nmh + t];
      }
    }
#pragma unroll
    for (int u = 0; u < kGB; u++) {
      const int i = i1 - u;
      if (i >= 0) {
        d = make_double2(r[u].x - c[u] * d.x, r[u].y - c[u] * d.y);
        Sm[(size_t)i * nmh] = d;
      }
    }
  }
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

// GRAVTY mode 3 (:90-97): v -= dt (-F(+2) + 8 F(+1) - 8 F(-1) + F(-2)) / (24 dx0)
// in each direction, written as coef ((F(-2) - F(+2)) + 8 (F(+1) - F(-1))),
// coef = dt / (24 dx0): four FP64 operations per component on GB300's
// narrow FP64 pipe instead of seven (round-off apart, the same sum)
__global__ void grav_kick_kernel(Grid g, Fields f, const double *phi, double coef) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nx = g.n[0], ny = g.n[1];
  if (t >= (long long)nx * ny * g.n[2]) return;
  const long long a = gidx_lin(g, t, nx, ny), sy = g.st[1], sz = g.st[2];
  const double *F = phi;
  const double gx = (F[a - 2] - F[a + 2]) + 8.0 * (F[a + 1] - F[a - 1]);
  const double gy = (F[a - 2 * sy] - F[a + 2 * sy]) + 8.0 * (F[a + sy] - F[a - sy]);
  const double gz = (F[a - 2 * sz] - F[a + 2 * sz]) + 8.0 * (F[a + sz] - F[a - sz]);
  f.U[1][a] = f.U[1][a] - coef * gx;
  f.U[2][a] = f.U[2][a] - coef * gy;
  f.U[3][a] = f.U[3][a] - coef * gz;
}

unsigned nblk(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

int ilog2(int n) {
  int l = 0;
  while ((1 << l) < n) l++;
  return l;
}

// lines per CTA: up to 1024 threads (fft_threads(n) per line) and 32 KB of lines
int lines_per_cta(int n, int nlines) {
  int lpc = 1024 / fft_threads(n);
  const int cap = 2048 / n;
  if (lpc > cap) lpc = cap;
  if (lpc > nlines) lpc = nlines;
  return lpc < 1 ? 1 : lpc;
}

cudaError_t fft_lines(double2 *w, int n, long long stride, int na, int nb, long long step_b, const double2 *tw,
                      bool inv, cudaStream_t s) {
  if (n == 1) return cudaSuccess;   // the transform of one value is itself
  const int lpc = lines_per_cta(n, na);
  dim3 grid((unsigned)((na + lpc - 1) / lpc), (unsigned)nb);
  fft_lines_kernel<<<grid, lpc * fft_threads(n), (size_t)lpc * n * sizeof(double2), s>>>(w, ilog2(n), stride, na,
                                                                                         step_b, lpc, tw, inv);
  return cudaGetLastError();
}

}  // namespace

bool gravity_size_ok(int n) { return n >= 1 && n <= 1024 && (n & (n - 1)) == 0; }

size_t gravity_spectrum_size(const Grid &g) { return (size_t)g.n[0] * g.n[2] * (g.n[1] / 2 + 1); }

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

cudaError_t gravity_tables(const GravityArgs &a, cudaStream_t s) {
  const long long nmh = (long long)(a.g.n[1] / 2 + 1) * a.g.n[2];
  grav_table_kernel<<<nblk(nmh, 128), 128, 0, s>>>(a.g, a.tab, a.dx, a.dy, a.dz, a.x0, a.lbox);
  return cudaGetLastError();
}

cudaError_t gravity_solve(const GravityArgs &a, cudaStream_t s) {
  const Grid &g = a.g;
  const int nx = g.n[0], ny = g.n[1], nz = g.n[2], nyh = ny / 2 + 1;
  const long long nmh = (long long)nyh * nz;
  const int hy = ny / 2 > 0 ? ny / 2 : 1, hz = nz / 2 > 0 ? nz / 2 : 1, ty = fft_threads(ny);
  const int logny = ilog2(ny), lpcy = lines_per_cta(ny, nx);
  const dim3 ygrid((unsigned)((nx + lpcy - 1) / lpcy), (unsigned)((nz + 1) / 2));
  const size_t ysmem = (size_t)lpcy * ny * sizeof(double2);
  cudaError_t e;
  grav_fwd_y_kernel<<<ygrid, lpcy * ty, ysmem, s>>>(g, a.rho, a.S, logny, lpcy, a.tw_y);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // z lines of the half spectrum: mode l at S[(i nz + k) nyh + l], stride nyh
  if ((e = fft_lines(a.S, nz, nyh, nyh, nx, nmh, a.tw_z, false, s)) != cudaSuccess) return e;
  grav_modes_kernel<<<nblk(nmh, 128), 128, 0, s>>>(g, a.S, a.tab, a.dx);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = fft_lines(a.S, nz, nyh, nyh, nx, nmh, a.tw_z + hz, true, s)) != cudaSuccess) return e;
  grav_inv_y_kernel<<<ygrid, lpcy * ty, ysmem, s>>>(g, a.S, a.phi, logny, lpcy, a.tw_y + hy,
                                                    1.0 / ((double)ny * (double)nz));
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  grav_ghost_x_kernel<<<nblk((long long)ny * nz, 256), 256, 0, s>>>(g, a.phi);
  grav_ghost_y_kernel<<<nblk((long long)g.s[0] * nz * 4, 256), 256, 0, s>>>(g, a.phi);
  grav_ghost_z_kernel<<<nblk((long long)g.s[0] * g.s[1] * 4, 256), 256, 0, s>>>(g, a.phi);
  return cudaGetLastError();
}

cudaError_t gravity_kick(const Grid &g, const Fields &f, const double *phi, double dt, double dx0, cudaStream_t s) {
  const long long n = (long long)g.n[0] * g.n[1] * g.n[2];
  grav_kick_kernel<<<nblk(n, 256), 256, 0, s>>>(g, f, phi, dt / (24.0 * dx0));
  return cudaGetLastError();
}

}  // namespace mhd
