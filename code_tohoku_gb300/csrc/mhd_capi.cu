// mhd_capi.cu — the extern "C" boundary (include/mhd_gb300.h) and the host
// orchestration of one EVOLVE iteration (MCF3DSGincfca3.f90:562-657) on one
// GPU.  The handle owns the resident state (U, species, Bcc) and the step's
// scratch (face velocities, EMFs, the predictor pressure, DISSIP's divv);
// every ghost exchange the reference performs between its subroutines is
// issued here as a ghost exchange (ghost_fill_all) on the same fields and directions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/mhd_gb300.h"
#include "mhd_conv.cuh"
#include "mhd_launch.h"

// full-grid FP64 arrays of a handle, one allocation: 8 U + 8 species + 3 Bcc
// + 3 face velocities + 3 EMF + pnew + the chemistry's nde and ndtot
static constexpr int kStateArrays = 8 + 8 + 3 + 3 + 3 + 1 + 2;

using namespace mhd;

struct mhd_handle {
  mhd_params p{};
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  Grid g{};
  Phys ph{};
  Fields f{};
  double *block = nullptr;        // one allocation for all full-grid arrays
  double *coords = nullptr;
  double *vf[3] = {nullptr, nullptr, nullptr};
  double *emf[3] = {nullptr, nullptr, nullptr};
  double *pnew = nullptr;
  // chosen form only: FP32 scratch (cell temperatures for SOURCE; face
  // velocities, face B, rho, T switch and EMFs for CT) and FP32 widths
  float *fblock = nullptr;
  double *colblock = nullptr;     // SHIELD's ten column arrays (ifrad = 2)
  double *ctcoef = nullptr;       // chosen form's CC(3): dt/dx of every coordinate
  double dxh = 0.0;               // SHIELD's half width 0.5 dx(1)
  float *temp32 = nullptr;
  float *sh2_32 = nullptr;               // SOURCE's FP32 S = H+p+He+He+ and H2 (2 ncell floats)
  int *stiff_list = nullptr;             // SOURCE's stiff cells (guess-and-polish cooling modes)
  // sh2_32 holds S and H2 of the current species: set by SOURCE's first
  // pass, cleared by every writer of the species (upload, mhd_step_host,
  // the sweeps, the chemistry network)
  bool sh2_valid = false;
  float *vf32[3] = {nullptr, nullptr, nullptr};
  float *bf32[3] = {nullptr, nullptr, nullptr};
  float *rn32 = nullptr, *sw32 = nullptr;
  float *emf32[3] = {nullptr, nullptr, nullptr};
  float *coordsf = nullptr;
  // chosen form's time step: per-warp lower ends of the FP32 screen and
  // its four words (smallest upper ends, floor flag)
  float *dtlo = nullptr;
  unsigned *dtwords = nullptr;
  float *dtf = nullptr;                  // BC=4 reservoir (device)
  // self-gravity (ifgrv = 2): the potential, the complex work array, the
  // Thomas scratch, the twiddles for ny and nz, and the grid scalars the
  // solve and the kick read (from the last mhd_upload)
  double *phi = nullptr;
  void *gwork = nullptr;                  // the half spectrum
  double *gtab = nullptr;                 // the grid's tables (built at the first solve after an upload)
  bool gtab_ready = false;
  void *gtw = nullptr;
  double g_dx = 0.0, g_dy = 0.0, g_dz = 0.0, g_dx0 = 0.0, g_x0 = 0.0, g_lbox = 0.0;
  bool inflow_set = false;
  double *divv = nullptr;
  double *diag_part = nullptr;
  unsigned long long *dtred = nullptr;   // [0] tCFL, [1] tLMT bits, [2] IMC, [3] surrogate, [4] fallback,
                                         // [5] stiff-cell count
  float *sur_master = nullptr;           // FP32 surrogate parameters (device)
  SurNet *sur_net = nullptr;             // packed BF16 network (device)
  float sur_tol = 1e-3f;
  int *err = nullptr;
  unsigned long long *h_small = nullptr; // pinned readback
  double time = 0.0;
  int ifevo = 1;
  long long steps = 0;
  long long launches = 0;
  long long imc_cells = 0;
  bool uploaded = false;
  // mhd_step_host: copy-back stream and the events it waits on (created on
  // first use)
  cudaStream_t io_stream = nullptr;
  cudaEvent_t ev_io[3] = {nullptr, nullptr, nullptr};
  // mhd_step_host, chosen form: one event per slab of the last sweep, and
  // per slab of the late species copies the first sweep waits for
  cudaEvent_t ev_slab[9] = {};
  cudaEvent_t ev_late[8] = {};
  // ... and per z slab of the state's copy in, which CC(4) and the time
  // step's screen take slab by slab
  cudaEvent_t ev_in[9] = {};
  std::vector<double> rdx_host, rdxc_host;   // staging for the async coordinate copies
  std::vector<float> dxf_host;
  std::string msg;
};

namespace {

int fail(mhd_handle *h, int code, const char *fmt, ...) {
  if (h) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    h->msg = buf;
  }
  return code;
}

#define CK(call)                                                                             \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) return fail(h, MHD_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    h->launches++;                                                                           \
  } while (0)

#define CKR(call)                                                                            \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) return fail(h, MHD_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

#define TRY(call)              \
  do {                         \
    int r_ = (call);           \
    if (r_ != MHD_OK) return r_; \
  } while (0)

const double kNdMinH = 0.91, kNdMinHe = 0.09;

// BC_MPI-style exchange of up to 8 arrays along the directions in dirs (bit
// d), nol ghost layers; rules: the BC=4 rule of each array on an inflow side
// of x (IN_KEEP past nrules); spmask bit q: array q is a species array, whose
// free-boundary copy covers interior transverse lines only
int fill_mask(mhd_handle *h, const double *const *arrays, int n, int dirs, int nol, unsigned spmask,
              const int *rules, int nrules) {
  FillArgs a{};
  a.nf = n;
  for (int q = 0; q < n; q++) a.f[q] = const_cast<double *>(arrays[q]);
  for (int q = 0; q < nrules; q++) a.rule[q] = rules[q];
  a.spmask = spmask;
  a.in = h->ph.in;
  CK(ghost_fill_all(h->g, a, dirs, nol, h->stream));
  return MHD_OK;
}

int fill(mhd_handle *h, std::initializer_list<double *> arrays, int dirs, int nol, int species = 0,
         std::initializer_list<int> rules = {}) {
  const double *arr[8];
  int n = 0, nr = 0, r[8] = {IN_KEEP, IN_KEEP, IN_KEEP, IN_KEEP, IN_KEEP, IN_KEEP, IN_KEEP, IN_KEEP};
  for (double *p : arrays) arr[n++] = p;
  for (int x : rules) r[nr++] = x;
  return fill_mask(h, arr, n, dirs, nol, species ? (1u << n) - 1u : 0u, r, nr);
}

int check_err(mhd_handle *h) {
  int e = 0;
  CKR(cudaMemcpyAsync(&e, h->err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CKR(cudaStreamSynchronize(h->stream));
  if (e & ERRB_NONFINITE) return fail(h, MHD_ERR_NONFINITE, "non-finite value in the state (time %.17g)", h->time);
  if (e & ERRB_DT) return fail(h, MHD_ERR_DT, "non-positive time-step limit (err at Couran/Stblty)");
  if (e & ERRB_TC) return fail(h, MHD_ERR_CUDA, "tensor-core completion wait timed out in SOURCE");
  if (e & ERRB_TMA) return fail(h, MHD_ERR_CUDA, "a sweep's wait for its staged inputs timed out");
  return MHD_OK;
}

bool valid_bc(int b) { return b == 1 || b == 3; }

// a handle with BC=4 needs its inflow data before any exchange
int need_inflow(mhd_handle *h) {
  if ((h->p.bc[0] == 4 || h->p.bc[1] == 4) && !h->inflow_set)
    return fail(h, MHD_ERR_STATE, "BC code 4 needs mhd_set_inflow before the state is used");
  h->ph.in.time = h->time;   // the reference's module time during this step
  return MHD_OK;
}

// self-gravity (ifgrv = 2): GRAVTY mode 2 (the potential of the current
// density) and mode 3 (a half kick of the velocities by its gradient)
int gravity_potential(mhd_handle *h) {
  GravityArgs a{};
  a.g = h->g;
  a.rho = h->f.U[0];
  a.phi = h->phi;
  a.S = static_cast<double2 *>(h->gwork);
  a.tab = h->gtab;
  a.tw_y = static_cast<const double2 *>(h->gtw);
  a.tw_z = a.tw_y + (h->g.n[1] / 2 > 0 ? h->g.n[1] / 2 : 1) * 2;
  a.dx = h->g_dx; a.dy = h->g_dy; a.dz = h->g_dz; a.x0 = h->g_x0; a.lbox = h->g_lbox;
  if (!h->gtab_ready) {
    CK(gravity_tables(a, h->stream));
    h->launches += 1;
    h->gtab_ready = true;
  }
  CK(gravity_solve(a, h->stream));
  // the y transform, z transform, mode solve, inverse z, inverse y, three ghost passes
  h->launches += (h->g.n[2] > 1) ? 8 : 6;
  return MHD_OK;
}
int gravity_half_kick(mhd_handle *h, double dt) {
  CK(gravity_kick(h->g, h->f, h->phi, dt, h->g_dx0, h->stream));
  return MHD_OK;
}
int gravity(mhd_handle *h, double dt, bool kick) {
  TRY(gravity_potential(h));
  if (kick) TRY(gravity_half_kick(h, dt));
  return MHD_OK;
}

}  // namespace

extern "C" {

int mhd_create(const mhd_params *p, mhd_handle **out) {
  if (!p || !out) return MHD_ERR_ARG;
  *out = nullptr;
  if (p->nx < 4 || p->ny < 4 || p->nz < 4) return MHD_ERR_ARG;
  // linear cell indices are split in 32-bit arithmetic (split3)
  if ((long long)(p->nx + 4) * (p->ny + 4) * (p->nz + 4) >= (1LL << 31)) return MHD_ERR_ARG;
  for (int q = 0; q < 6; q++)   // codes 1 (free), 3 (periodic), 4 (inflow, x sides only)
    if (!(valid_bc(p->bc[q]) || (q < 2 && p->bc[q] == 4))) return MHD_ERR_ARG;
  if (p->precision != MHD_PREC_FP64 && p->precision != MHD_PREC_FP32) return MHD_ERR_ARG;
  if (p->cooling != MHD_COOL_EXACT && p->cooling != MHD_COOL_SURROGATE && p->cooling != MHD_COOL_NEWTON)
    return MHD_ERR_ARG;
  if (p->cooling != MHD_COOL_EXACT && p->precision != MHD_PREC_FP32) return MHD_ERR_ARG;
  if (p->ifchem != 0 && p->ifchem != 2) return MHD_ERR_ARG;
  if (p->ifrad != 0 && p->ifrad != 2) return MHD_ERR_ARG;
  if (p->ifgrv != 0 && p->ifgrv != 2) return MHD_ERR_ARG;
  if (p->ifgrv == 2 && !(gravity_size_ok(p->ny) && gravity_size_ok(p->nz))) return MHD_ERR_ARG;
  // the surrogate is trained on the KI cooling function only
  if (p->cooling != MHD_COOL_EXACT && p->ifchem == 2) return MHD_ERR_ARG;
  if (p->dissip && p->nx < 11) return MHD_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= p->device) return MHD_ERR_NO_DEVICE;
  mhd_handle *h = new (std::nothrow) mhd_handle();
  if (!h) return MHD_ERR_ARG;
  h->p = *p;
  if (cudaSetDevice(p->device) != cudaSuccess) { delete h; return MHD_ERR_NO_DEVICE; }
  Grid &g = h->g;
  g.n[0] = p->nx; g.n[1] = p->ny; g.n[2] = p->nz;
  for (int d = 0; d < 3; d++) g.s[d] = g.n[d] + 4;
  g.st[0] = 1; g.st[1] = g.s[0]; g.st[2] = (long long)g.s[0] * g.s[1];
  g.ncell = (long long)g.s[0] * g.s[1] * g.s[2];
  for (int d = 0; d < 3; d++) { g.bcl[d] = p->bc[2 * d]; g.bcr[d] = p->bc[2 * d + 1]; }
  Phys &ph = h->ph;
  ph.facdep = p->facdep; ph.pmin = p->pmin; ph.pmax = p->pmax; ph.rmin = p->rmin;
  ph.kb = p->kb; ph.kcond = p->kcond; ph.cfl = p->cfl; ph.tfinal = p->tfinal; ph.ifthrm = p->ifthrm;
  ph.ifchem = p->ifchem;
  ph.ifrad = p->ifrad;
  // species floors, MCF3DSGincfca3.f90:178-179 (slots H,p,H2,He,Hep,C,Cp,CO)
  double mins[8] = {p->rmin * kNdMinH, 1e-20, 1e-20, p->rmin * kNdMinHe, 1e-20, 1e-20, 1e-20, 1e-20};
  for (int s = 0; s < 8; s++) {
    ph.ndmin[s] = mins[s];
    ph.ndminf[s] = d2f(mins[s]);
  }
  ph.in.on[0] = p->bc[0] == 4;
  ph.in.on[1] = p->bc[1] == 4;

  // the full-grid arrays (kStateArrays), one allocation
  size_t bytes = (size_t)kStateArrays * (size_t)g.ncell * sizeof(double);
  if (cudaMalloc(&h->block, bytes) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return MHD_ERR_CUDA;
  }
  double *q = h->block;
  for (int f = 0; f < 8; f++) { h->f.U[f] = q; q += g.ncell; }
  for (int s = 0; s < 8; s++) { h->f.sp[s] = q; q += g.ncell; }
  for (int c = 0; c < 3; c++) { h->f.bcc[c] = q; q += g.ncell; }
  for (int c = 0; c < 3; c++) { h->vf[c] = q; q += g.ncell; }
  for (int c = 0; c < 3; c++) { h->emf[c] = q; q += g.ncell; }
  h->pnew = q; q += g.ncell;
  h->f.nde = q; q += g.ncell;
  h->f.ndtot = q;
  size_t ncoord = 4 * (size_t)(g.s[0] + g.s[1] + g.s[2]);
  size_t ndivv = 2 * 12 * (size_t)(g.n[1] + 2) * (g.n[2] + 2);
  size_t ndiag = 6 * (size_t)((g.n[0] * (long long)g.n[1] * g.n[2] + 255) / 256);
  bool ok = cudaMalloc(&h->coords, ncoord * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&h->coordsf, (size_t)(g.s[0] + g.s[1] + g.s[2]) * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&h->divv, ndivv * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&h->diag_part, ndiag * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&h->dtred, 8 * sizeof(unsigned long long)) == cudaSuccess &&
            cudaMalloc(&h->err, sizeof(int)) == cudaSuccess &&
            cudaMallocHost(&h->h_small, 8 * sizeof(unsigned long long)) == cudaSuccess &&
            cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    mhd_destroy(h);
    return MHD_ERR_CUDA;
  }
  h->own_stream = true;
  if (p->ifrad == 2) {
    // SHIELD's columns: Ntot, NH2, NnC, NCO, tCII from both x sides
    if (cudaMalloc(&h->colblock, 10 * (size_t)g.ncell * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      mhd_destroy(h);
      return MHD_ERR_CUDA;
    }
    for (int q = 0; q < 10; q++) h->f.col[q] = h->colblock + (size_t)q * g.ncell;
  }
  if (p->ifgrv == 2) {
    const size_t nspec = gravity_spectrum_size(g);
    std::vector<double2> ty = gravity_twiddles(g.n[1]), tz = gravity_twiddles(g.n[2]);
    bool okg = cudaMalloc(&h->phi, (size_t)g.ncell * sizeof(double)) == cudaSuccess &&
               cudaMalloc(&h->gwork, nspec * sizeof(double2)) == cudaSuccess &&
               cudaMalloc(&h->gtab, 4 * nspec * sizeof(double)) == cudaSuccess &&
               cudaMalloc(&h->gtw, (ty.size() + tz.size()) * sizeof(double2)) == cudaSuccess &&
               cudaMemcpy(h->gtw, ty.data(), ty.size() * sizeof(double2), cudaMemcpyHostToDevice) == cudaSuccess &&
               cudaMemcpy(static_cast<double2 *>(h->gtw) + ty.size(), tz.data(), tz.size() * sizeof(double2),
                          cudaMemcpyHostToDevice) == cudaSuccess &&
               cudaMemset(h->phi, 0, (size_t)g.ncell * sizeof(double)) == cudaSuccess;
    if (!okg) {
      cudaGetLastError();
      mhd_destroy(h);
      return MHD_ERR_CUDA;
    }
  }
  if (p->precision == MHD_PREC_FP32) {
    const size_t nf = 15;   // 14 FP32 arrays + the stiff-cell list of SOURCE
    size_t fbytes = nf * (size_t)g.ncell * sizeof(float);
    if (cudaMalloc(&h->fblock, fbytes) != cudaSuccess) {
      cudaGetLastError();
      mhd_destroy(h);
      return MHD_ERR_CUDA;
    }
    if (cudaMalloc(&h->ctcoef, (size_t)(g.s[0] + g.s[1] + g.s[2]) * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      mhd_destroy(h);
      return MHD_ERR_CUDA;
    }
    const size_t nw = (size_t)dt_screen_warps(g);
    if (cudaMalloc(&h->dtlo, (3 * nw + 4) * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      mhd_destroy(h);
      return MHD_ERR_CUDA;
    }
    h->dtwords = reinterpret_cast<unsigned *>(h->dtlo + 3 * nw);
    float *fq = h->fblock;
    h->temp32 = fq; fq += g.ncell;
    h->sh2_32 = fq; fq += 2 * g.ncell;
    for (int c = 0; c < 3; c++) { h->vf32[c] = fq; fq += g.ncell; }
    for (int c = 0; c < 3; c++) { h->bf32[c] = fq; fq += g.ncell; }
    h->rn32 = fq; fq += g.ncell;
    h->sw32 = fq; fq += g.ncell;
    for (int c = 0; c < 3; c++) { h->emf32[c] = fq; fq += g.ncell; }
    h->stiff_list = reinterpret_cast<int *>(fq); fq += g.ncell;
    cudaMemsetAsync(h->fblock, 0, fbytes, h->stream);
  }
  cudaMemsetAsync(h->block, 0, bytes, h->stream);
  cudaMemsetAsync(h->err, 0, sizeof(int), h->stream);
  cudaMemsetAsync(h->dtred, 0, 8 * sizeof(unsigned long long), h->stream);
  double *c = h->coords;
  float *cf = h->coordsf;
  for (int d = 0; d < 3; d++) {
    g.x[d] = c; c += g.s[d];
    g.dx[d] = c; c += g.s[d];
    g.rdx[d] = c; c += g.s[d];
    g.rdxc[d] = c; c += g.s[d];
    g.dxf[d] = cf; cf += g.s[d];
  }
  *out = h;
  return MHD_OK;
}

int mhd_destroy(mhd_handle *h) {
  if (!h) return MHD_OK;
  cudaSetDevice(h->p.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaFree(h->block);
  cudaFree(h->coords);
  cudaFree(h->coordsf);
  cudaFree(h->dtf);
  cudaFree(h->fblock);
  cudaFree(h->colblock);
  cudaFree(h->ctcoef);
  cudaFree(h->divv);
  cudaFree(h->diag_part);
  cudaFree(h->dtred);
  cudaFree(h->dtlo);
  cudaFree(h->phi);
  cudaFree(h->gwork);
  cudaFree(h->gtab);
  cudaFree(h->gtw);
  cudaFree(h->err);
  cudaFree(h->sur_master);
  cudaFree(h->sur_net);
  if (h->h_small) cudaFreeHost(h->h_small);
  if (h->io_stream) {
    cudaStreamSynchronize(h->io_stream);
    cudaStreamDestroy(h->io_stream);
  }
  for (int e = 0; e < 3; e++)
    if (h->ev_io[e]) cudaEventDestroy(h->ev_io[e]);
  for (cudaEvent_t e : h->ev_slab)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : h->ev_late)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : h->ev_in)
    if (e) cudaEventDestroy(e);
  if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return MHD_OK;
}

int mhd_set_stream(mhd_handle *h, void *stream) {
  if (!h) return MHD_ERR_ARG;
  CKR(cudaStreamSynchronize(h->stream));
  if (h->own_stream) cudaStreamDestroy(h->stream);
  if (stream) {
    h->stream = (cudaStream_t)stream;
    h->own_stream = false;
  } else {
    CKR(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->own_stream = true;
  }
  return MHD_OK;
}

namespace {
// SHIELD (:2924-3036): columns from both x sides of every cell; the
// predictor-pressure scratch holds the optical-depth source term
int shield(mhd_handle *h) {
  if (h->p.precision == MHD_PREC_FP32) CK(shield_fp32(h->g, h->ph, h->f, h->pnew, h->dxh, h->stream));
  else CK(shield(h->g, h->ph, h->f, h->pnew, h->dxh, h->stream));
  h->launches++;   // two kernels
  return MHD_OK;
}
}  // namespace

int mhd_upload(mhd_handle *h, const double *U, const double *species, const double *x, const double *dx,
               const double *y, const double *dy, const double *z, const double *dz) {
  if (!h || !U || !species || !x || !dx || !y || !dy || !z || !dz) return MHD_ERR_ARG;
  TRY(need_inflow(h));
  CKR(cudaSetDevice(h->p.device));
  const Grid &g = h->g;
  size_t nb = (size_t)g.ncell * sizeof(double);
  h->sh2_valid = false;
  for (int f = 0; f < 8; f++) CKR(cudaMemcpyAsync(h->f.U[f], U + (size_t)f * g.ncell, nb, cudaMemcpyHostToDevice, h->stream));
  for (int s = 0; s < 8; s++)
    CKR(cudaMemcpyAsync(h->f.sp[s], species + (size_t)s * g.ncell, nb, cudaMemcpyHostToDevice, h->stream));
  const double *src[6] = {x, dx, y, dy, z, dz};
  h->rdx_host.resize((size_t)(g.s[0] + g.s[1] + g.s[2]));
  h->rdxc_host.resize(h->rdx_host.size());
  h->dxf_host.resize(h->rdx_host.size());
  size_t off = 0;
  for (int d = 0; d < 3; d++) {
    CKR(cudaMemcpyAsync((void *)g.x[d], src[2 * d], g.s[d] * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CKR(cudaMemcpyAsync((void *)g.dx[d], src[2 * d + 1], g.s[d] * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    // reciprocal Euler widths for the chosen form's remap: 1/(x(i)-x(i-1))
    double *r = h->rdx_host.data() + off;
    const double *xx = src[2 * d];
    r[0] = 1.0 / src[2 * d + 1][0];
    for (int i = 1; i < g.s[d]; i++) r[i] = 1.0 / (xx[i] - xx[i - 1]);
    CKR(cudaMemcpyAsync((void *)g.rdx[d], r, g.s[d] * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    // chosen form: 1/dx(i) and dx(i) in FP32
    double *rc = h->rdxc_host.data() + off;
    float *wf = h->dxf_host.data() + off;
    for (int i = 0; i < g.s[d]; i++) {
      rc[i] = 1.0 / src[2 * d + 1][i];
      wf[i] = (float)src[2 * d + 1][i];
    }
    CKR(cudaMemcpyAsync((void *)g.rdxc[d], rc, g.s[d] * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CKR(cudaMemcpyAsync((void *)g.dxf[d], wf, g.s[d] * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    off += g.s[d];
  }
  // nde, ndtot (INITIA :471-474) and CC(4) as INITIA:470
  CK(chem_totals(h->g, h->f, 1, h->stream));
  // the columns start at 0 and INITIA iterates SHIELD 20 times (:475-479)
  if (h->p.ifrad == 2) {
    h->dxh = 0.5 * dx[2];   // dx(1), the first interior width along x (:2937)
    CKR(cudaMemsetAsync(h->colblock, 0, 10 * (size_t)g.ncell * sizeof(double), h->stream));
    for (int l = 0; l < 20; l++) TRY(shield(h));
  }
  CK(cell_b(h->g, h->f, h->stream));
  TRY(fill(h, {h->f.bcc[0], h->f.bcc[1], h->f.bcc[2]}, 7, 2, 0, {IN_BCC1, IN_B2, IN_B3}));
  if (h->p.ifgrv == 2) {
    // GRAVTY(0,2) of INITIA (:481-484); index 2 of the coordinate arrays is
    // cell 1, index 1 is x(0)
    h->g_dx = dx[2]; h->g_dy = dy[2]; h->g_dz = dz[2]; h->g_dx0 = dx[1];
    h->g_x0 = x[1]; h->g_lbox = x[g.n[0] + 1] - x[1];
    h->gtab_ready = false;   // new coordinates: new tables
    TRY(gravity(h, 0.0, false));
  }
  CKR(cudaStreamSynchronize(h->stream));
  h->uploaded = true;
  return MHD_OK;
}

int mhd_download_columns(mhd_handle *h, double *columns) {
  if (!h || !columns) return MHD_ERR_ARG;
  if (!h->uploaded) return fail(h, MHD_ERR_STATE, "no state uploaded");
  if (h->p.ifrad != 2) return fail(h, MHD_ERR_STATE, "the handle has no columns (ifrad != 2)");
  CKR(cudaSetDevice(h->p.device));
  CKR(cudaMemcpyAsync(columns, h->colblock, 10 * (size_t)h->g.ncell * sizeof(double), cudaMemcpyDeviceToHost,
                      h->stream));
  CKR(cudaStreamSynchronize(h->stream));
  return check_err(h);
}

int mhd_download_potential(mhd_handle *h, double *phi) {
  if (!h || !phi) return MHD_ERR_ARG;
  if (!h->uploaded) return fail(h, MHD_ERR_STATE, "no state uploaded");
  if (h->p.ifgrv != 2) return fail(h, MHD_ERR_STATE, "the handle has no potential (ifgrv != 2)");
  CKR(cudaSetDevice(h->p.device));
  CKR(cudaMemcpyAsync(phi, h->phi, (size_t)h->g.ncell * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CKR(cudaStreamSynchronize(h->stream));
  return check_err(h);
}

int mhd_download(mhd_handle *h, double *U, double *species, double *bcc) {
  if (!h || !U) return MHD_ERR_ARG;
  if (!h->uploaded) return fail(h, MHD_ERR_STATE, "no state uploaded");
  CKR(cudaSetDevice(h->p.device));
  const Grid &g = h->g;
  size_t nb = (size_t)g.ncell * sizeof(double);
  for (int f = 0; f < 8; f++) CKR(cudaMemcpyAsync(U + (size_t)f * g.ncell, h->f.U[f], nb, cudaMemcpyDeviceToHost, h->stream));
  if (species)
    for (int s = 0; s < 8; s++)
      CKR(cudaMemcpyAsync(species + (size_t)s * g.ncell, h->f.sp[s], nb, cudaMemcpyDeviceToHost, h->stream));
  if (bcc)
    for (int c = 0; c < 3; c++)
      CKR(cudaMemcpyAsync(bcc + (size_t)c * g.ncell, h->f.bcc[c], nb, cudaMemcpyDeviceToHost, h->stream));
  CKR(cudaStreamSynchronize(h->stream));
  return check_err(h);
}

}  // extern "C"

namespace {
// the reduction words of the time step at their starting values
int timestep_reset(mhd_handle *h) {
  CKR(cudaMemsetAsync(h->dtred, 0xff, 2 * sizeof(unsigned long long), h->stream));
  if (h->p.precision == MHD_PREC_FP32) {
    CKR(cudaMemsetAsync(h->dtwords, 0xff, 3 * sizeof(unsigned), h->stream));
    CKR(cudaMemsetAsync(h->dtwords + 3, 0, sizeof(unsigned), h->stream));
  }
  return MHD_OK;
}

// mhd_timestep; screened: the chosen form's words were reset and every cell
// screened by the caller (mhd_step_host, slab by slab as the state comes in)
int timestep_impl(mhd_handle *h, double *dt, int *st, bool screened) {
  if (!h || !dt || !st) return MHD_ERR_ARG;
  if (!h->uploaded) return fail(h, MHD_ERR_STATE, "no state uploaded");
  CKR(cudaSetDevice(h->p.device));
  const bool fp32 = h->p.precision == MHD_PREC_FP32;
  if (!screened) TRY(timestep_reset(h));
  if (fp32) {
    // an FP32 screen of every cell, then the FP64 limits of the cells that
    // can hold the minimum: the same dt as the plain form, bit for bit.  The
    // screen reads S and H2 of the interior cells from SOURCE's arrays while
    // the species are unchanged since (the same floats).
    if (!screened)
      CK(dt_screen_fp32(h->g, h->ph, h->f, h->sh2_valid ? h->sh2_32 : nullptr, h->dtlo, h->dtwords, h->err,
                        h->stream));
    CK(dt_refine(h->g, h->ph, h->f, h->dtlo, h->dtwords, h->dtred, h->stream));
    CKR(cudaMemcpyAsync(h->h_small + 6, h->dtwords + 3, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
  } else {
    CK(dt_reduce(h->g, h->ph, h->f, h->dtred, h->err, h->stream));
  }
  CKR(cudaMemcpyAsync(h->h_small, h->dtred, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
  TRY(check_err(h));
  double tcfl, tlmt;
  memcpy(&tcfl, &h->h_small[0], sizeof(double));
  memcpy(&tlmt, &h->h_small[1], sizeof(double));
  if (fp32) {
    // a limit no screened cell reached keeps its starting value, tfinal; a
    // cooling time at its floor is 2.5e-4 exactly (Stblty :2806)
    if (h->h_small[0] == ~0ull) tcfl = h->p.tfinal;
    if (h->h_small[1] == ~0ull) tlmt = h->p.tfinal;
    unsigned floored;
    memcpy(&floored, &h->h_small[6], sizeof floored);
    if (floored && h->p.ifthrm == 2 && 2.5e-4 < tlmt) tlmt = 2.5e-4;
  }
  // EVOLVE:569-596 with one rank
  double d = h->p.tfinal;
  double c = h->p.cfl * tcfl;
  d = (c < d) ? c : d;
  int s = 1;
  if (h->p.ifthrm == 2) {
    double stt = d;
    d = (tlmt < d) ? tlmt : d;
    if (d < stt) s = 2;
  }
  d = (d < h->p.tfinal) ? d : h->p.tfinal;
  if (!(d > 0.0)) return fail(h, MHD_ERR_DT, "err at Couran/Stblty: dt = %g", d);
  *dt = d;
  *st = s;
  return MHD_OK;
}
}  // namespace

extern "C" {

int mhd_timestep(mhd_handle *h, double *dt, int *st) { return timestep_impl(h, dt, st, false); }

namespace {
// the thermal branch of SOURCE (ifthrm = 2, :2477-2572); rho_sp_filled:
// the caller has already filled the ghosts of rho and the species with the
// same values (mhd_step_host, which copies those arrays back meanwhile).
// The predictor writes pnew, not U5; the reference updates U5 in place, so
// its exchange between the passes (:2526-2528) leaves the predictor's values
// in U5's one-layer ghost shell after SOURCE.  So pnew takes U5's outer
// shell before that exchange (which copies from it), and U5 takes pnew's
// one-layer shell after the corrector: every padded cell as the reference.
// fill_cco: the exchange also takes species 5-7 (C, C+, CO), which the
// thermal update does not read (the reference exchanges all eight), and U5
// takes the predictor's shell.  The first SOURCE of a step skips both: CT's
// exchanges and the second SOURCE rewrite those ghost cells before anything
// reads them.
int source_thermal(mhd_handle *h, double dt, bool rho_sp_filled = false, bool fill_cco = true) {
  // SOURCE :2481-2486 — rho, p and the species, one ghost layer, x y z
  if (rho_sp_filled) {
    TRY(fill(h, {h->f.U[4]}, 7, 1, 0, {IN_P}));
  } else {
    // rho and p, and the species (interior transverse lines), in one exchange
    const double *arr[7] = {h->f.U[0], h->f.U[4], h->f.sp[0], h->f.sp[1], h->f.sp[2], h->f.sp[3], h->f.sp[4]};
    const int rules[7] = {IN_RHO, IN_P, IN_SPEC + 0, IN_SPEC + 1, IN_SPEC + 2, IN_SPEC + 3, IN_SPEC + 4};
    TRY(fill_mask(h, arr, 7, 7, 1, 0x7cu, rules, 7));
    if (fill_cco) TRY(fill(h, {h->f.sp[5], h->f.sp[6], h->f.sp[7]}, 7, 1, 1, {IN_SPEC + 5, IN_SPEC + 6, IN_SPEC + 7}));
  }
  if (h->p.precision == MHD_PREC_FP32) {
    if (h->p.cooling == MHD_COOL_SURROGATE && !h->sur_net)
      return fail(h, MHD_ERR_STATE, "surrogate cooling selected but no network loaded (mhd_surrogate_load)");
    Source32Args a{};
    a.g = h->g; a.ph = h->ph; a.f = h->f;
    a.dt = dt; a.err = h->err;
    a.imc_count = h->dtred + 2; a.sur_count = h->dtred + 3; a.fb_count = h->dtred + 4;
    a.W = (h->p.cooling == MHD_COOL_SURROGATE) ? h->sur_net : nullptr;
    a.tol = h->sur_tol;
    a.T = h->temp32;
    a.sh2 = h->sh2_32;
    a.stiff_list = h->stiff_list; a.stiff_count = h->dtred + 5;
    a.pin = h->f.U[4]; a.pold = h->f.U[4]; a.pout = h->pnew; a.pass = 0;
    // how stiff cells start their implicit solve: the network, the
    // frozen-rate Newton start, or the bisection alone
    const int stiff_mode = h->p.cooling == MHD_COOL_SURROGATE ? STIFF_NETWORK
                           : h->p.cooling == MHD_COOL_NEWTON  ? STIFF_NEWTON
                                                              : 0;
    // S and H2 from the species, unless SOURCE formed them from the same
    // species before (the previous step's second SOURCE); an inflow side
    // refills the ghost species from the advected reservoir every time
    const bool inflow = h->ph.in.on[0] || h->ph.in.on[1];
    CK(temp_fp32(h->g, h->f, a.pin, h->ph.kb, h->temp32, h->sh2_32, !(h->sh2_valid && !inflow), h->stream));
    h->sh2_valid = true;
    CK(source_fp32(a, stiff_mode, h->stream));
    h->launches += stiff_mode ? 1 : 0;   // the stiff-cell kernel
    if (fill_cco) CK(shell_copy(h->g, h->f.U[4], h->pnew, 2, h->stream));
    TRY(fill(h, {h->pnew}, 7, 1, 0, {IN_P}));
    a.pin = h->pnew; a.pold = h->f.U[4]; a.pout = h->f.U[4]; a.pass = 1;
    CK(temp_fp32(h->g, h->f, a.pin, h->ph.kb, h->temp32, h->sh2_32, false, h->stream));
    CK(source_fp32(a, stiff_mode, h->stream));
    h->launches += stiff_mode ? 1 : 0;
    if (fill_cco) CK(shell_copy(h->g, h->pnew, h->f.U[4], 1, h->stream));
    return MHD_OK;
  }
  SourceArgs a{};
  a.g = h->g; a.ph = h->ph; a.f = h->f;
  a.dt = dt; a.err = h->err; a.imc_count = h->dtred + 2; a.skip = nullptr;
  a.pin = h->f.U[4]; a.pold = h->f.U[4]; a.pout = h->pnew; a.pass = 0;
  CK(source_pass(a, h->stream));
  if (fill_cco) CK(shell_copy(h->g, h->f.U[4], h->pnew, 2, h->stream));
  TRY(fill(h, {h->pnew}, 7, 1, 0, {IN_P}));   // :2526-2528
  a.pin = h->pnew; a.pold = h->f.U[4]; a.pout = h->f.U[4]; a.pass = 1;
  CK(source_pass(a, h->stream));
  if (fill_cco) CK(shell_copy(h->g, h->pnew, h->f.U[4], 1, h->stream));
  return MHD_OK;
}
}  // namespace

namespace {
int source_impl(mhd_handle *h, double dt, bool rho_sp_filled, bool fill_cco = true) {
  if (!h) return MHD_ERR_ARG;
  if (!h->uploaded) return fail(h, MHD_ERR_STATE, "no state uploaded");
  CKR(cudaSetDevice(h->p.device));
  TRY(need_inflow(h));
  // nde, ndtot from the species of cells 1..n (:2460-2463); read only by
  // the species cooling and the network
  if (h->p.ifchem == 2 || h->p.ifrad == 2) CK(chem_totals(h->g, h->f, 0, h->stream));
  if (h->p.ifrad == 2) TRY(shield(h));   // :2466-2468
  if (h->p.ifthrm == 2) TRY(source_thermal(h, dt, rho_sp_filled, fill_cco));
  // the chemistry network after the thermal update (ifchem = 2, :2576-2776)
  if (h->p.ifchem == 2) {
    if (h->p.precision == MHD_PREC_FP32) CK(chem_step_fp32(h->g, h->ph, h->f, dt, h->err, h->stream));
    else CK(chem_step(h->g, h->ph, h->f, dt, h->err, h->stream));
    h->sh2_valid = false;
  }
  return MHD_OK;
}
}  // namespace

int mhd_source(mhd_handle *h, double dt) { return source_impl(h, dt, false); }

int mhd_sweep(mhd_handle *h, int dir, double dt) {
  if (!h || dir < 0 || dir > 2) return MHD_ERR_ARG;
  if (!h->uploaded) return fail(h, MHD_ERR_STATE, "no state uploaded");
  TRY(need_inflow(h));
  CKR(cudaSetDevice(h->p.device));
  h->sh2_valid = false;   // the sweeps move the species
  SweepArgs a{};
  a.g = h->g; a.ph = h->ph; a.f = h->f; a.dt = dt; a.err = h->err;
  if (h->p.precision == MHD_PREC_FP32) CK(sweep_fp32(dir, a, h->block, kStateArrays, h->stream));
  else CK(sweep_fp64(dir, a, h->stream));
  return MHD_OK;
}

namespace {
int ct_impl(mhd_handle *h, double dt, bool rho_filled);
}
int mhd_ct(mhd_handle *h, double dt) { return ct_impl(h, dt, false); }

namespace {
// rho_filled: the caller has already filled rho's two ghost layers with the
// values CC(2) needs (mhd_step_host)
int ct_impl(mhd_handle *h, double dt, bool rho_filled) {
  if (!h) return MHD_ERR_ARG;
  if (!h->uploaded) return fail(h, MHD_ERR_STATE, "no state uploaded");
  CKR(cudaSetDevice(h->p.device));
  Fields &f = h->f;
  // CC(1) :2122-2137
  TRY(need_inflow(h));
  // with them, the x, y and z exchanges of p and rho that CC(2) needs
  // (:2142; nothing in between changes either)
  {
    const int n = rho_filled ? 4 : 5;
    const double *ax[5] = {f.U[1], f.U[6], f.U[7], f.U[4], f.U[0]};
    const double *ay[5] = {f.U[2], f.U[5], f.U[7], f.U[4], f.U[0]};
    const double *az[5] = {f.U[3], f.U[5], f.U[6], f.U[4], f.U[0]};
    const int rx[5] = {IN_V1, IN_B2, IN_B3, IN_P, IN_RHO};
    TRY(fill_mask(h, ax, n, 1, 2, 0u, rx, n));
    TRY(fill_mask(h, ay, n, 2, 2, 0u, nullptr, 0));
    TRY(fill_mask(h, az, n, 4, 2, 0u, nullptr, 0));
  }
  const bool fp32 = h->p.precision == MHD_PREC_FP32;
  if (fp32) CK(face_velocity_fp32(h->g, f, h->vf[0], h->vf[1], h->vf[2], h->stream));
  else CK(face_velocity(h->g, f, h->vf[0], h->vf[1], h->vf[2], h->stream));
  TRY(fill(h, {h->vf[1], h->vf[2]}, 1, 2, 0, {IN_VFC, IN_VFC}));
  TRY(fill(h, {h->vf[0], h->vf[2]}, 2, 2));
  TRY(fill(h, {h->vf[0], h->vf[1]}, 4, 2));
  // CC(2) for Ez :2142 (p and rho exchanged above)
  if (fp32) {
    CT32Args a{};
    a.g = h->g;
    for (int c = 0; c < 3; c++) { a.vf[c] = h->vf32[c]; a.bf[c] = h->bf32[c]; a.emf[c] = h->emf32[c]; }
    a.rn = h->rn32; a.sw = h->sw32;
    a.dt = (float)dt; a.facm = (float)(h->ph.facdep * 0.5);
    CK(ct_prep_fp32(h->g, f, h->vf, h->ph.kb, a, h->stream));
    for (int e = 0; e < 3; e++) CK(emf32(e, a, h->stream));
    CK(face_b_fp32(h->g, f, h->emf32, dt, h->ctcoef, h->stream));
    h->launches++;   // the coefficient kernel
  } else {
    CTArgs a{};
    a.g = h->g; a.ph = h->ph; a.f = f; a.dt = dt;
    for (int c = 0; c < 3; c++) { a.vf[c] = h->vf[c]; a.emf[c] = h->emf[c]; }
    for (int e = 0; e < 3; e++) CK(emf_fp64(e, a, h->stream));
    CK(face_b(h->g, f, h->emf[0], h->emf[1], h->emf[2], dt, h->stream));   // CC(3)
  }
  CK(cell_b(h->g, f, h->stream));   // CC(4)
  TRY(fill(h, {f.bcc[0], f.bcc[1], f.bcc[2]}, 7, 2, 0, {IN_BCC1, IN_B2, IN_B3}));
  return MHD_OK;
}
}  // namespace

int mhd_dissip(mhd_handle *h) {
  if (!h) return MHD_ERR_ARG;
  if (!h->uploaded) return fail(h, MHD_ERR_STATE, "no state uploaded");
  CKR(cudaSetDevice(h->p.device));
  TRY(need_inflow(h));
  TRY(fill(h, {h->f.U[1], h->f.U[2], h->f.U[3]}, 7, 2, 0, {IN_V1, IN_V2, IN_V3}));
  CK(divv(h->g, h->f, h->divv, h->stream));
  CK(dissip(h->g, h->f, h->divv, 0, h->stream));
  CK(dissip(h->g, h->f, h->divv, 1, h->stream));
  return MHD_OK;
}

int mhd_gravity(mhd_handle *h, double dt, int mode) {
  if (!h || (mode != 2 && mode != 3)) return MHD_ERR_ARG;
  if (!h->uploaded) return fail(h, MHD_ERR_STATE, "no state uploaded");
  if (h->p.ifgrv != 2) return fail(h, MHD_ERR_STATE, "the handle has no self-gravity (ifgrv != 2)");
  CKR(cudaSetDevice(h->p.device));
  return mode == 2 ? gravity_potential(h) : gravity_half_kick(h, dt);
}

int mhd_advance(mhd_handle *h, double dt) {
  if (!h) return MHD_ERR_ARG;
  if (!h->uploaded) return fail(h, MHD_ERR_STATE, "no state uploaded");
  static const int orders[6][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}, {0, 2, 1}, {1, 0, 2}, {2, 1, 0}};
  if (h->p.ifgrv == 2) TRY(gravity_half_kick(h, dt));   // EVOLVE :607
  // (the ghost values of species 5-7 the first SOURCE would exchange are
  // the second's to leave; no step reads them)
  TRY(source_impl(h, 0.5 * dt, false, false));
  for (int s = 0; s < 3; s++) TRY(mhd_sweep(h, orders[h->ifevo - 1][s], dt));
  h->ifevo = h->ifevo % 6 + 1;
  TRY(mhd_ct(h, dt));
  TRY(source_impl(h, 0.5 * dt, false, true));
  if (h->p.ifgrv == 2) TRY(gravity(h, dt, true));        // :653
  if (h->p.dissip) TRY(mhd_dissip(h));
  h->time = h->time + dt;
  h->steps++;
  return MHD_OK;
}

int mhd_step(mhd_handle *h, double tsave, double *dt, int *st) {
  if (!h || !dt || !st) return MHD_ERR_ARG;
  double d;
  int s;
  TRY(mhd_timestep(h, &d, &s));
  if (h->time + d > h->p.tfinal) d = h->p.tfinal - h->time;   // :603
  if (h->time + d > tsave) d = tsave - h->time;               // :604
  if (!(d > 0.0)) return fail(h, MHD_ERR_DT, "dt <= 0 after clipping (time %.17g)", h->time);
  TRY(mhd_advance(h, d));
  *dt = d;
  *st = s;
  return MHD_OK;
}

namespace {
// Slabs of the last sweep in mhd_step_host's chosen form.  Without
// chemistry rho and the species are final once the last sweep has passed
// over them, so that sweep runs as kCopySlabs launches, each over a slab of
// its pencil groups (z slabs for the x and y sweeps, y slabs for the z
// sweep); after each, the ghost cells of rho and the species that lie in
// the slab are filled (the passes of the exchange that stay inside it) and
// the copy stream takes the slab's planes or rows back while the next slab
// runs.  The ghost layers along the slab direction follow at the end, with
// every pass.  The link back to the host is the bound of the call, so it
// starts about a sweep earlier than after the whole sweep.
constexpr int kCopySlabs = 8;
// slabs of rows (after or before a z sweep) are copied with 2-D copies of
// one row range per plane, whose per-row cost makes fewer, wider slabs pay:
// calls whose last sweep is z took 26.7 ms with four row slabs against 27.3
// with eight (256^3)
#ifndef MHD_COPY_SLABS_ROWS
#define MHD_COPY_SLABS_ROWS 4
#endif
constexpr int kCopySlabsRows = MHD_COPY_SLABS_ROWS;
// slabs of the first sweep (and of the late species copies it waits for):
// 26.49 -> 26.39 ms per call at 256^3 with four instead of eight
#ifndef MHD_FIRST_SWEEP_SLABS
#define MHD_FIRST_SWEEP_SLABS 4
#endif
constexpr int kFirstSweepSlabs = MHD_FIRST_SWEEP_SLABS;
// the last sweep's first slab half as wide as the others: the copies back
// start sooner (26.47 -> 26.32 ms per call at 256^3)
#ifndef MHD_HALF_FIRST_SLAB
#define MHD_HALF_FIRST_SLAB 1
#endif
constexpr bool kHalfFirstSlab = MHD_HALF_FIRST_SLAB != 0;
// the handle's events: ev_slab[9] (a slab count plus one), ev_late[8], ev_in[9]
static_assert(kCopySlabs >= 1 && kCopySlabs <= 8 && kCopySlabsRows >= 1 && kCopySlabsRows <= 8 &&
                  kFirstSweepSlabs >= 1 && kFirstSweepSlabs <= 8,
              "slab counts are bounded by the handle's event arrays");
constexpr int kSweepOrders[6][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}, {0, 2, 1}, {1, 0, 2}, {2, 1, 0}};

// the slabs of a direction-dir sweep: K ranges of its transverse block index
// (z for the x and y sweeps, y for the z sweep), i.e. of the padded
// coordinate rdim from lo(s) + 2 to lo(s + 1) + 2
struct Slabs {
  int nby, rdim, K;
  int h;   // > 0: the first slab is h wide and the other K - 1 share the rest
  // kmax: at most that many slabs (0: kCopySlabs, kCopySlabsRows for rows);
  // half_first: the first slab half as wide as the others, so whatever
  // waits for it starts sooner
  Slabs(const Grid &g, int dir, int kmax = 0, bool half_first = false)
      : nby(dir == 2 ? g.n[1] : g.n[2]), rdim(dir == 2 ? 1 : 2),
        K(std::min(kmax > 0 ? kmax : (dir == 2 ? kCopySlabsRows : kCopySlabs), dir == 2 ? g.n[1] : g.n[2])),
        h(0) {
    if (half_first && K > 1 && nby >= 2 * K) h = nby / (2 * K - 1);
  }
  int lo(int s) const {
    if (h == 0 || s == 0) return (int)((long long)nby * s / K);
    return h + (int)((long long)(nby - h) * (s - 1) / (K - 1));
  }
};

// copy of one array over padded [lo, hi) along rdim: whole planes (rdim 2)
// or those rows of every plane (rdim 1)
cudaError_t copy_range(const Grid &g, int rdim, double *dst, const double *src, int lo, int hi, cudaMemcpyKind kind,
                       cudaStream_t st) {
  const size_t row = (size_t)g.s[0], plane = (size_t)g.s[0] * g.s[1];
  if (rdim == 2)
    return cudaMemcpyAsync(dst + lo * plane, src + lo * plane, (size_t)(hi - lo) * plane * sizeof(double), kind, st);
  return cudaMemcpy2DAsync(dst + lo * row, plane * sizeof(double), src + lo * row, plane * sizeof(double),
                           (size_t)(hi - lo) * row * sizeof(double), (size_t)g.s[2], kind, st);
}

int last_sweep_slabs(mhd_handle *h, int dir, double d, double *U_out, double *species_out) {
  const Grid &g = h->g;
  Fields &f = h->f;
  TRY(need_inflow(h));
  h->sh2_valid = false;   // the sweeps move the species
  const Slabs sb(g, dir, 0, kHalfFirstSlab);
  const int nby = sb.nby, rdim = sb.rdim, K = sb.K;
  const int fdirs = dir == 2 ? 5 : 3;   // exchange passes that stay inside a slab
  for (int e = 0; e <= K; e++)
    if (!h->ev_slab[e]) CKR(cudaEventCreateWithFlags(&h->ev_slab[e], cudaEventDisableTiming));
  const size_t nc = (size_t)g.ncell;
  FillArgs fr{};   // rho: two layers, every direction (:2481-2486, CC(2))
  fr.nf = 1;
  fr.f[0] = f.U[0];
  fr.rule[0] = IN_RHO;
  fr.in = h->ph.in;
  FillArgs fs{};   // the species (thermal SOURCE): one layer, interior transverse lines
  fs.nf = 8;
  for (int q = 0; q < 8; q++) {
    fs.f[q] = f.sp[q];
    fs.rule[q] = IN_SPEC + q;
  }
  fs.spmask = 255u;
  fs.in = h->ph.in;
  const bool sp_fill = h->p.ifthrm == 2;
  // the copies back of rho and the 8 species over padded [lo, hi) along rdim
  auto copy_back = [&](int lo, int hi) -> cudaError_t {
    for (int q = 0; q < 9; q++) {
      const double *src = q == 0 ? f.U[0] : f.sp[q - 1];
      double *dst = q == 0 ? U_out : species_out + (size_t)(q - 1) * nc;
      const cudaError_t e = copy_range(g, rdim, dst, src, lo, hi, cudaMemcpyDeviceToHost, h->io_stream);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  };
  SweepArgs a{};
  a.g = g; a.ph = h->ph; a.f = f; a.dt = d; a.err = h->err;
  for (int sl = 0; sl < K; sl++) {
    a.by0 = sb.lo(sl);
    a.by1 = sb.lo(sl + 1);
    CK(sweep_fp32(dir, a, h->block, kStateArrays, h->stream));
    CK(ghost_fill_slab(g, fr, fdirs, 2, rdim, a.by0 + 2, a.by1 + 2, false, h->stream));
    if (sp_fill) CK(ghost_fill_slab(g, fs, fdirs, 1, rdim, a.by0 + 2, a.by1 + 2, false, h->stream));
    CKR(cudaEventRecord(h->ev_slab[sl], h->stream));
    CKR(cudaStreamWaitEvent(h->io_stream, h->ev_slab[sl], 0));
    CKR(copy_back(a.by0 + 2, a.by1 + 2));
  }
  CK(ghost_fill_slab(g, fr, 7, 2, rdim, 2, nby + 2, true, h->stream));
  if (sp_fill) CK(ghost_fill_slab(g, fs, 7, 1, rdim, 2, nby + 2, true, h->stream));
  CKR(cudaEventRecord(h->ev_slab[K], h->stream));
  CKR(cudaStreamWaitEvent(h->io_stream, h->ev_slab[K], 0));
  CKR(copy_back(0, 2));
  CKR(copy_back(nby + 2, nby + 4));
  return MHD_OK;
}

// The first sweep of mhd_step_host's chosen form in the slabs of its
// direction, each waiting for that slab of species 5-7 (ev_late), which the
// copy stream brings in last: the sweep starts on the first slab while the
// others are still on the link.
int first_sweep_slabs(mhd_handle *h, int dir, double d) {
  TRY(need_inflow(h));
  h->sh2_valid = false;   // the sweeps move the species
  const Slabs sb(h->g, dir, std::min(kFirstSweepSlabs, dir == 2 ? kCopySlabsRows : kCopySlabs));
  SweepArgs a{};
  a.g = h->g; a.ph = h->ph; a.f = h->f; a.dt = d; a.err = h->err;
  for (int sl = 0; sl < sb.K; sl++) {
    a.by0 = sb.lo(sl);
    a.by1 = sb.lo(sl + 1);
    CKR(cudaStreamWaitEvent(h->stream, h->ev_late[sl], 0));
    CK(sweep_fp32(dir, a, h->block, kStateArrays, h->stream));
  }
  return MHD_OK;
}

// the EVOLVE iteration of mhd_advance for mhd_step_host, copying arrays
// back as soon as they are final: without chemistry rho and the species are
// final after the sweeps (once their ghosts are filled; in the chosen form
// slab by slab during the last sweep), the face field after CC
// late_species: species 5-7 are still coming in on the copy stream (event
// ev_io[2]; by slabs of the first sweep, events ev_late, when late_slabs);
// the first sweep, their first reader, waits for them
int step_host_body(mhd_handle *h, double d, double *U_out, double *species_out, bool late_species,
                   bool late_slabs) {
  const size_t nc = (size_t)h->g.ncell, nb = nc * sizeof(double);
  Fields &f = h->f;
  if (h->p.ifgrv == 2) TRY(gravity_half_kick(h, d));   // EVOLVE :607
  TRY(source_impl(h, 0.5 * d, false, false));   // species 5-7 may still be on the link
  if (late_species && !late_slabs) CKR(cudaStreamWaitEvent(h->stream, h->ev_io[2], 0));
  const int *order = kSweepOrders[h->ifevo - 1];
  h->ifevo = h->ifevo % 6 + 1;
  const bool early = h->p.ifchem != 2;
  const bool slabs = early && h->p.precision == MHD_PREC_FP32;
  if (late_species && late_slabs) TRY(first_sweep_slabs(h, order[0], d));
  for (int q = (late_species && late_slabs) ? 1 : 0; q < (slabs ? 2 : 3); q++) TRY(mhd_sweep(h, order[q], d));
  if (slabs) {
    TRY(last_sweep_slabs(h, order[2], d, U_out, species_out));
  } else if (early) {
    // the ghost fills CC(2) and SOURCE would make, made now
    TRY(fill(h, {f.U[0]}, 7, 2, 0, {IN_RHO}));
    if (h->p.ifthrm == 2)
      TRY(fill(h, {f.sp[0], f.sp[1], f.sp[2], f.sp[3], f.sp[4], f.sp[5], f.sp[6], f.sp[7]}, 7, 1, 1,
               {IN_SPEC + 0, IN_SPEC + 1, IN_SPEC + 2, IN_SPEC + 3, IN_SPEC + 4, IN_SPEC + 5, IN_SPEC + 6,
                IN_SPEC + 7}));
    CKR(cudaEventRecord(h->ev_io[0], h->stream));
    CKR(cudaStreamWaitEvent(h->io_stream, h->ev_io[0], 0));
    CKR(cudaMemcpyAsync(U_out, f.U[0], nb, cudaMemcpyDeviceToHost, h->io_stream));
    for (int q = 0; q < 8; q++)
      CKR(cudaMemcpyAsync(species_out + q * nc, f.sp[q], nb, cudaMemcpyDeviceToHost, h->io_stream));
  }
  TRY(ct_impl(h, d, early));
  CKR(cudaEventRecord(h->ev_io[1], h->stream));
  CKR(cudaStreamWaitEvent(h->io_stream, h->ev_io[1], 0));
  for (int q = 5; q < 8; q++)
    CKR(cudaMemcpyAsync(U_out + q * nc, f.U[q], nb, cudaMemcpyDeviceToHost, h->io_stream));
  TRY(source_impl(h, 0.5 * d, early));
  if (h->p.ifgrv == 2) TRY(gravity(h, d, true));        // :653
  if (h->p.dissip) TRY(mhd_dissip(h));
  h->time = h->time + d;
  h->steps++;
  for (int q = early ? 1 : 0; q < 5; q++)
    CKR(cudaMemcpyAsync(U_out + q * nc, f.U[q], nb, cudaMemcpyDeviceToHost, h->stream));
  if (!early)
    for (int q = 0; q < 8; q++)
      CKR(cudaMemcpyAsync(species_out + q * nc, f.sp[q], nb, cudaMemcpyDeviceToHost, h->stream));
  return MHD_OK;
}
}  // namespace

namespace {
// mhd_step_host after the copies in: CC(4), the time step (mhd_step's
// clipping), then the step with its copies back
// in_slabs: the state comes in by z slabs (events ev_in; the ghost planes
// with the first and the last), and CC(4) and the time step's screen take
// each slab once it and the next have arrived (CC(4) reads the z faces of
// the plane above)
int step_host_run(mhd_handle *h, double tsave, double *dt, int *st, double *U_out, double *species_out,
                  bool late_species, bool late_slabs, bool in_slabs) {
  Fields &f = h->f;
  double d;
  int s;
  if (in_slabs) {
    const Slabs zs(h->g, 0);
    const long long plane = (long long)h->g.n[0] * h->g.n[1];
    TRY(timestep_reset(h));
    for (int sl = 0; sl < zs.K; sl++) {
      const long long c0 = plane * zs.lo(sl), c1 = plane * zs.lo(sl + 1);
      CKR(cudaStreamWaitEvent(h->stream, h->ev_in[std::min(sl + 1, zs.K - 1)], 0));
      CK(cell_b_range(h->g, f, c0, c1, h->stream));   // CC(4) as after mhd_upload
      CK(dt_screen_fp32_range(h->g, h->ph, f, nullptr, h->dtlo, h->dtwords, h->err, c0, c1, h->stream));
    }
    TRY(fill(h, {f.bcc[0], f.bcc[1], f.bcc[2]}, 7, 2, 0, {IN_BCC1, IN_B2, IN_B3}));
    TRY(timestep_impl(h, &d, &s, true));
  } else {
    CK(cell_b(h->g, f, h->stream));   // CC(4) as after mhd_upload
    TRY(fill(h, {f.bcc[0], f.bcc[1], f.bcc[2]}, 7, 2, 0, {IN_BCC1, IN_B2, IN_B3}));
    TRY(mhd_timestep(h, &d, &s));
  }
  if (h->time + d > h->p.tfinal) d = h->p.tfinal - h->time;
  if (h->time + d > tsave) d = tsave - h->time;
  if (!(d > 0.0)) return fail(h, MHD_ERR_DT, "dt <= 0 after clipping (time %.17g)", h->time);
  *dt = d;
  *st = s;
  return step_host_body(h, d, U_out, species_out, late_species, late_slabs);
}
}  // namespace

int mhd_step_host(mhd_handle *h, const double *U_in, const double *species_in, double *U_out, double *species_out,
                  double tsave, double *dt, int *st) {
  if (!h || !U_in || !species_in || !U_out || !species_out || !dt || !st) return MHD_ERR_ARG;
  if (!h->uploaded) return fail(h, MHD_ERR_STATE, "mhd_step_host needs a first mhd_upload (coordinates)");
  CKR(cudaSetDevice(h->p.device));
  TRY(need_inflow(h));
  if (!h->io_stream) CKR(cudaStreamCreateWithFlags(&h->io_stream, cudaStreamNonBlocking));
  for (int e = 0; e < 3; e++)
    if (!h->ev_io[e]) CKR(cudaEventCreateWithFlags(&h->ev_io[e], cudaEventDisableTiming));
  const Grid &g = h->g;
  const size_t nc = (size_t)g.ncell, nb = nc * sizeof(double);
  Fields &f = h->f;
  // The state in.  Without chemistry or SHIELD neither the time step nor
  // the first SOURCE reads species 5-7 (C, C+, CO), so those three arrays
  // come in on the copy stream, after the other copies, while those kernels
  // run; the first sweep waits for them.
  const bool late = h->p.ifchem != 2 && h->p.ifrad != 2;
  // In the chosen form (with species 5-7 late) the other 13 arrays come in
  // on the copy stream by z slabs, an event after each, so that CC(4) and
  // the time step's screen run on each slab while the next ones are on the
  // link; the screen's blocks must not straddle a slab.
  const bool in_slabs = late && h->p.precision == MHD_PREC_FP32 &&
                        ((long long)g.n[0] * g.n[1]) % kDtScreenCells == 0;
  h->sh2_valid = false;
  if (in_slabs) {
    const Slabs zs(g, 0);
    const int nz = g.n[2];
    cudaError_t e = cudaEventRecord(h->ev_io[2], h->stream);   // after everything queued before (readers included)
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->io_stream, h->ev_io[2], 0);
    auto copy13 = [&](int lo, int hi) -> cudaError_t {
      cudaError_t r = cudaSuccess;
      for (int q = 0; q < 13 && r == cudaSuccess; q++) {
        double *dst = q < 8 ? f.U[q] : f.sp[q - 8];
        const double *src = q < 8 ? U_in + q * nc : species_in + (q - 8) * nc;
        r = copy_range(g, 2, dst, src, lo, hi, cudaMemcpyHostToDevice, h->io_stream);
      }
      return r;
    };
    // the ghost planes go with the first and the last slab (one copy per
    // array and slab: the copy engine pays per copy)
    for (int sl = 0; sl < zs.K && e == cudaSuccess; sl++) {
      e = copy13(sl == 0 ? 0 : zs.lo(sl) + 2, sl == zs.K - 1 ? nz + 4 : zs.lo(sl + 1) + 2);
      if (e == cudaSuccess && !h->ev_in[sl]) e = cudaEventCreateWithFlags(&h->ev_in[sl], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventRecord(h->ev_in[sl], h->io_stream);
    }
    if (e != cudaSuccess) {
      cudaStreamSynchronize(h->io_stream);   // no copy from the caller's buffers outlives the call
      return fail(h, MHD_ERR_CUDA, "state copy: %s", cudaGetErrorString(e));
    }
  } else {
    // a failed enqueue waits for the copies already queued from U_in and
    // species_in, so no copy from the caller's buffers outlives the call
    cudaError_t e = cudaSuccess;
    for (int q = 0; q < 8 && e == cudaSuccess; q++)
      e = cudaMemcpyAsync(f.U[q], U_in + q * nc, nb, cudaMemcpyHostToDevice, h->stream);
    for (int q = 0; q < (late ? 5 : 8) && e == cudaSuccess; q++)
      e = cudaMemcpyAsync(f.sp[q], species_in + q * nc, nb, cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) {
      cudaStreamSynchronize(h->stream);
      return fail(h, MHD_ERR_CUDA, "state copy: %s", cudaGetErrorString(e));
    }
  }
  // In the chosen form those three arrays come in by slabs of the first
  // sweep (the ghost layers with the first and the last slab), an event
  // after each slab, and the sweep's slabs wait for their own.
  const bool late_slabs = late && h->p.precision == MHD_PREC_FP32;
  if (late) {
    // (with in_slabs the copy stream already follows the main stream)
    cudaError_t e = cudaSuccess;
    if (!in_slabs) {
      e = cudaEventRecord(h->ev_io[2], h->stream);   // after everything queued before (readers included)
      if (e == cudaSuccess) e = cudaStreamWaitEvent(h->io_stream, h->ev_io[2], 0);
    }
    if (late_slabs) {
      const int first = kSweepOrders[h->ifevo - 1][0];
      const Slabs sb(g, first, std::min(kFirstSweepSlabs, first == 2 ? kCopySlabsRows : kCopySlabs));
      for (int sl = 0; sl < sb.K && e == cudaSuccess; sl++) {
        if (!h->ev_late[sl]) e = cudaEventCreateWithFlags(&h->ev_late[sl], cudaEventDisableTiming);
        const int lo = sl == 0 ? 0 : sb.lo(sl) + 2, hi = sl == sb.K - 1 ? sb.nby + 4 : sb.lo(sl + 1) + 2;
        for (int q = 5; q < 8 && e == cudaSuccess; q++)
          e = copy_range(g, sb.rdim, f.sp[q], species_in + q * nc, lo, hi, cudaMemcpyHostToDevice, h->io_stream);
        if (e == cudaSuccess) e = cudaEventRecord(h->ev_late[sl], h->io_stream);
      }
    } else {
      for (int q = 5; q < 8 && e == cudaSuccess; q++)
        e = cudaMemcpyAsync(f.sp[q], species_in + q * nc, nb, cudaMemcpyHostToDevice, h->io_stream);
    }
    if (e == cudaSuccess) e = cudaEventRecord(h->ev_io[2], h->io_stream);
    if (e != cudaSuccess) {
      cudaStreamSynchronize(h->io_stream);   // no copy from the caller's buffers outlives the call
      return fail(h, MHD_ERR_CUDA, "species copy stream: %s", cudaGetErrorString(e));
    }
  }
  // the copy stream may hold copies from the caller's input buffers and into
  // its output buffers: every exit below waits for it, so the buffers are
  // never touched after return
  double d = 0.0;
  int s = 0;
  const int r = step_host_run(h, tsave, &d, &s, U_out, species_out, late, late_slabs, in_slabs);
  const cudaError_t es = cudaStreamSynchronize(h->io_stream);
  if (r != MHD_OK) {
    cudaStreamSynchronize(h->stream);   // its copies into U_out too
    return r;
  }
  if (es != cudaSuccess) return fail(h, MHD_ERR_CUDA, "copy-back: %s", cudaGetErrorString(es));
  CKR(cudaStreamSynchronize(h->stream));
  *dt = d;
  *st = s;
  return check_err(h);
}

int mhd_evolve(mhd_handle *h, int nsteps, double tsave, int *steps_done) {
  if (!h || nsteps < 0) return MHD_ERR_ARG;
  int n = 0;
  for (; n < nsteps; n++) {
    if (h->time >= h->p.tfinal || h->time >= tsave) break;
    double dt;
    int st;
    int r = mhd_step(h, tsave, &dt, &st);
    if (r != MHD_OK) {
      if (steps_done) *steps_done = n;
      return r;
    }
  }
  if (steps_done) *steps_done = n;
  return MHD_OK;
}

int mhd_set_inflow(mhd_handle *h, const mhd_inflow *in, const float *reservoir, double uniform_density) {
  if (!h || !in) return MHD_ERR_ARG;
  if (h->p.bc[0] != 4 && h->p.bc[1] != 4) return fail(h, MHD_ERR_ARG, "no x side has BC code 4");
  if (!reservoir && !(uniform_density > 0.0)) return fail(h, MHD_ERR_ARG, "reservoir density must be positive");
  CKR(cudaSetDevice(h->p.device));
  const Grid &g = h->g;
  if (!h->dtf) CKR(cudaMalloc(&h->dtf, (size_t)g.ncell * sizeof(float)));
  if (reservoir) {
    CKR(cudaMemcpyAsync(h->dtf, reservoir, (size_t)g.ncell * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  } else {
    std::vector<float> u((size_t)g.ncell, (float)uniform_density);
    CKR(cudaMemcpyAsync(h->dtf, u.data(), u.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    CKR(cudaStreamSynchronize(h->stream));
  }
  CKR(cudaStreamSynchronize(h->stream));
  InflowDev &d = h->ph.in;
  d.rho_ref = in->rho_ref;
  for (int sd = 0; sd < 2; sd++) {
    d.p[sd] = in->p[sd];
    for (int c = 0; c < 3; c++) { d.v[sd][c] = in->v[sd][c]; d.b[sd][c] = in->b[sd][c]; }
  }
  for (int q = 0; q < 8; q++) d.cm[q] = in->species[q];
  d.dtf = h->dtf;
  h->inflow_set = true;
  return MHD_OK;
}

int mhd_get_time(mhd_handle *h, double *time, int *ifevo) {
  if (!h) return MHD_ERR_ARG;
  if (time) *time = h->time;
  if (ifevo) *ifevo = h->ifevo;
  return MHD_OK;
}

int mhd_set_time(mhd_handle *h, double time, int ifevo) {
  if (!h || ifevo < 1 || ifevo > 6) return MHD_ERR_ARG;
  h->time = time;
  h->ifevo = ifevo;
  return MHD_OK;
}

int mhd_diagnostics(mhd_handle *h, mhd_diag *out) {
  if (!h || !out) return MHD_ERR_ARG;
  if (!h->uploaded) return fail(h, MHD_ERR_STATE, "no state uploaded");
  CKR(cudaSetDevice(h->p.device));
  int nb = 0;
  CK(diag(h->g, h->ph, h->f, h->diag_part, &nb, h->stream));
  std::vector<double> part((size_t)nb * 6);
  CKR(cudaMemcpyAsync(part.data(), h->diag_part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CKR(cudaMemcpyAsync(h->h_small + 2, h->dtred + 2, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
  CKR(cudaStreamSynchronize(h->stream));
  memset(out, 0, sizeof *out);
  // fixed-order sum of the block partials (compensated)
  for (int q = 0; q < 5; q++) {
    double s = 0.0, c = 0.0;
    for (int b = 0; b < nb; b++) {
      double y = part[(size_t)b * 6 + q] - c;
      double t = s + y;
      c = (t - s) - y;
      s = t;
    }
    if (q == 0) out->mass = s;
    else if (q <= 3) out->momentum[q - 1] = s;
    else out->energy = s;
  }
  double m = 0.0;
  for (int b = 0; b < nb; b++) m = part[(size_t)b * 6 + 5] > m ? part[(size_t)b * 6 + 5] : m;
  out->divb_max = m;
  out->time = h->time;
  out->steps = h->steps;
  out->imc_cells = (long long)h->h_small[2];
  out->surrogate_cells = (long long)h->h_small[3];
  out->fallback_cells = (long long)h->h_small[4];
  return check_err(h);
}

int mhd_synchronize(mhd_handle *h) {
  if (!h) return MHD_ERR_ARG;
  CKR(cudaSetDevice(h->p.device));
  CKR(cudaStreamSynchronize(h->stream));
  return check_err(h);
}

int mhd_last_error(mhd_handle *h, char *buf, int len) {
  if (!h || !buf || len <= 0) return MHD_ERR_ARG;
  snprintf(buf, (size_t)len, "%s", h->msg.c_str());
  return MHD_OK;
}

long long mhd_kernel_launches(mhd_handle *h) { return h ? h->launches : 0; }

int mhd_surrogate_load(mhd_handle *h, const float *params, float tol) {
  if (!h || !params || !(tol > 0.0f)) return MHD_ERR_ARG;
  if (h->p.cooling != MHD_COOL_SURROGATE) return fail(h, MHD_ERR_ARG, "handle was created without surrogate cooling");
  CKR(cudaSetDevice(h->p.device));
  if (!h->sur_master) {
    CKR(cudaMalloc(&h->sur_master, SUR_NPARAM * sizeof(float)));
    CKR(cudaMalloc(&h->sur_net, sizeof(SurNet)));
  }
  CKR(cudaMemcpyAsync(h->sur_master, params, SUR_NPARAM * sizeof(float), cudaMemcpyHostToDevice, h->stream));
  CK(surrogate_pack(h->sur_master, h->sur_net, h->stream));
  CKR(cudaStreamSynchronize(h->stream));
  h->sur_tol = tol;
  return MHD_OK;
}

int mhd_reset_counters(mhd_handle *h) {
  if (!h) return MHD_ERR_ARG;
  CKR(cudaMemsetAsync(h->dtred + 2, 0, 3 * sizeof(unsigned long long), h->stream));
  return MHD_OK;
}

}  // extern "C"
