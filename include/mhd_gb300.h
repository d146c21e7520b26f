/* mhd_gb300.h — C ABI of the GB300 MHD + Koyama–Inutsuka cooling step.
 *
 * The reference program (3DMHD-CfCA/MCF3DSGincfca3.f90) advances its state
 * inside EVOLVE (:562-657) by calling Fortran subroutines on module arrays.
 * Each entry point below replaces one of those calls, so the Fortran driver,
 * its decks (INPUT3D.DAT) and its output writers stay as they are and a
 * bind(C) interface module routes the calls here:
 *
 *   mhd_timestep      Couran :1912-1930 + Stblty :2784-2822 + the dt
 *                     gather/min/bcast of EVOLVE :569-599
 *   mhd_source        SOURCE(dt) thermal branch :2477-2572 with the KI
 *                     Fcool of KIcool/1DMHDwCC3.f90:1148-1173 and IMC
 *   mhd_sweep         MHD(xelr,dxelr,dt) :1264-1324 (RHS, RIEMAN, MOC,
 *                     CHAREQ, REMAP, VLIMIT) for one direction
 *   mhd_ct            CC(1), CC(2)+CCT ×3, CC(3), CC(4) :639-649, :2115-2445
 *   mhd_dissip        DISSIP :3143-3173
 *   mhd_advance       one in20 iteration after dt is known :606-656
 *   mhd_step          the whole in20 iteration including dt :569-656
 *   mhd_upload/download  the module arrays U(-1:ndx,-1:ndy,-1:ndz,8), the
 *                     species ndH..ndCO and the coordinates (INITIA, SAVEU)
 *
 * All arrays are plain host pointers in the reference's Fortran layout:
 * U is U(-1:nx+2,-1:ny+2,-1:nz+2,8) column-major (x fastest, then y, z,
 * then field), i.e. 8 consecutive blocks of (nx+4)(ny+4)(nz+4) doubles.
 * U(:,:,:,1)=rho, 2..4 = velocity, 5 = pressure, 6..8 = face-centred B
 * (U(i,j,k,6) is Bx on the x-face i-1/2).  Species use the same block
 * layout in the order ndH, ndp, ndH2, ndHe, ndHep, ndC, ndCp, ndCO.
 * Coordinates are x(-1:nx+2) and dx(-1:nx+2), likewise y and z.
 *
 * The state lives on the GPU between calls; host copies happen only in
 * upload/download.  A handle is bound to one device and one CUDA stream and
 * is not safe for concurrent use from several threads.  Every function
 * returns MHD_OK (0) or one of the error codes below; mhd_last_error()
 * gives the message.  Device kernels never spin or trap: numerical failures
 * (NaN/Inf in the state, a non-positive dt) are recorded in a device error
 * word that the host reads after each call.
 */
#ifndef MHD_GB300_H
#define MHD_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define MHD_OK 0
#define MHD_ERR_ARG 1          /* invalid argument or unsupported option   */
#define MHD_ERR_CUDA 2         /* CUDA runtime error (allocation, launch)   */
#define MHD_ERR_NONFINITE 3    /* NaN or Inf appeared in the state          */
#define MHD_ERR_DT 4           /* dt <= 0 or not finite ('err at Couran')   */
#define MHD_ERR_STATE 5        /* call out of order (e.g. no upload yet)    */
#define MHD_ERR_NO_DEVICE 6    /* no CUDA device / kernels not loadable     */
#define MHD_ERR_TOO_LARGE 7    /* grid beyond MHD_NOALLOC_MAX_CELLS          */

#define MHD_PREC_FP64 0        /* plain form: every operation in FP64       */
#define MHD_PREC_FP32 1        /* FP32 reconstruction/flux, FP64 accumulate */

#define MHD_COOL_EXACT 0       /* explicit step or IMC bisection (reference) */
#define MHD_COOL_SURROGATE 1   /* MLP surrogate with exact fallback          */
#define MHD_COOL_NEWTON 2      /* the surrogate's Newton polish from the
                                  frozen-rate implicit start, no network,
                                  exact fallback (the comparison case)      */

typedef struct mhd_params {
  int nx, ny, nz;              /* interior cells (Ncellx, Ncelly, Ncellz);
                                  (nx+4)(ny+4)(nz+4) must be below 2^31  */
  double cfl, facdep, tfinal;  /* INPUT3D.DAT rows 13-14                    */
  int bc[6];                   /* BCx1,BCx2,BCy1,BCy2,BCz1,BCz2: 1 = free
                                  (zero-gradient), 3 = periodic, 4 = inflow
                                  (x sides only; see mhd_set_inflow)         */
  double pmin, pmax, rmin;     /* floors, MCF3DSGincfca3.f90:173-176        */
  double kb, kcond;            /* 8.63359, 1.6384e-2                        */
  int ifthrm;                  /* 2: KI source and thermal dt limit; 0: off */
  int dissip;                  /* 1: DISSIP edge damping after each step    */
  int precision;               /* MHD_PREC_FP64 or MHD_PREC_FP32            */
  int cooling;                 /* MHD_COOL_EXACT or MHD_COOL_SURROGATE      */
  int device;                  /* CUDA device ordinal                       */
  int ifchem;                  /* 2: the reference's chemistry network and
                                  species cooling (:2576-2776, :2825-2880);
                                  0: the KI cooling function                */
  int ifrad;                   /* 2: SHIELD column densities from both x
                                  sides (:2924-3036) for the species cooling
                                  and the rates; 0: columns 0 (the deck's) */
  int ifgrv;                   /* 2: self-gravity (GRAVTY, selfG_MPIfull8.f90):
                                  grad^2 Phi = 4 pi G rho, periodic y and z,
                                  isolated x, half kicks before the first and
                                  after the second SOURCE; needs ny and nz
                                  powers of two up to 1024 and uniform cells.
                                  0: off (the shipped deck's)               */
} mhd_params;

/* Inflow boundary data (BC code 4 on an x side): the values a ghost cell on
 * that side receives at each exchange, as INITIA sets them up
 * (MCF3DSGincfca3.f90:182-200) and BC_MPI / BC_MPI_OT apply them
 * (:814-890, :948-1080).  Side 0 is x = 0, side 1 the far end. */
typedef struct mhd_inflow {
  double rho_ref;        /* BBRV(1,*,*): the reference density dBC        */
  double v[2][3];        /* inflow velocity per side, BBRV(2..4,1,side)   */
  double p[2];           /* inflow pressure, BBRV(5,1,side)               */
  double b[2][3];        /* inflow field, BBRV(6..8,1,side)               */
  double species[8];     /* BBRV_cm: number density per unit mass density,
                            order H, p, H2, He, He+, C, C+, CO            */
} mhd_inflow;

typedef struct mhd_diag {
  double mass, momentum[3], energy;   /* sums over interior cells × volume  */
  double divb_max;                    /* max |div B| over interior cells    */
  double time;
  long long steps;
  long long imc_cells;                /* cells that took the implicit path  */
  long long surrogate_cells;          /* cells solved by the surrogate      */
  long long fallback_cells;           /* surrogate cells sent back to IMC   */
} mhd_diag;

typedef struct mhd_handle mhd_handle;

/* Allocates the resident state for p on p->device.  No data yet. */
int mhd_create(const mhd_params *p, mhd_handle **out);
/* Frees the handle and its device memory; a NULL handle is a no-op (MHD_OK). */
int mhd_destroy(mhd_handle *h);

/* INITIA/restart read: copies the full arrays (ghosts included) and runs
 * CC(4) (MCF3DSGincfca3.f90:470) to form the cell-centred field. */
int mhd_upload(mhd_handle *h, const double *U, const double *species,
               const double *x, const double *dx, const double *y,
               const double *dy, const double *z, const double *dz);
/* SAVEU: copies U and species back (bcc may be NULL; else 3 blocks). */
int mhd_download(mhd_handle *h, double *U, double *species, double *bcc);
/* SHIELD's column densities (ifrad = 2): ten blocks in the layout of U,
 * Ntot(:,:,:,1), Ntot(:,:,:,2), NH2(1), NH2(2), NnC(1), NnC(2), NCO(1),
 * NCO(2), tCII(1), tCII(2) (the module arrays of :30, side 1 = column from
 * x = 0, side 2 = from the far end). */
int mhd_download_columns(mhd_handle *h, double *columns);
/* The gravitational potential Phi (ifgrv = 2) in the layout of one block of
 * U, ghosts included (the module array Phi of :37, written by SAVEU). */
int mhd_download_potential(mhd_handle *h, double *phi);

/* Couran + Stblty + min (EVOLVE:569-599 for the whole grid).  *dt is
 * min(tfinal, CFL*tCFL, tLMT); *st is 1 (FastSpd) or 2 (Conduct).  Both
 * precisions return the FP64 minimum: the chosen form screens the cells in
 * FP32 and recomputes in FP64 those that can hold it. */
int mhd_timestep(mhd_handle *h, double *dt, int *st);
int mhd_source(mhd_handle *h, double dt);             /* SOURCE(dt)        */
int mhd_sweep(mhd_handle *h, int dir, double dt);     /* dir 0=x,1=y,2=z   */
int mhd_ct(mhd_handle *h, double dt);
int mhd_dissip(mhd_handle *h);
/* GRAVTY(dt, mode) of selfG_MPIfull8.f90:1-100 for a handle with ifgrv = 2:
 * mode 2 solves the potential of the current density, mode 3 gives the
 * half kick of the velocities by its fourth-order gradient (:90-97).
 * mhd_advance / mhd_step call both where EVOLVE does (:607, :653); a driver
 * that calls the step's parts one by one calls this itself. */
int mhd_gravity(mhd_handle *h, double dt, int mode);
/* SOURCE(dt/2), three sweeps in the order ifEVO (1..6, :611-634), CT,
 * SOURCE(dt/2), DISSIP, time += dt.  Advances ifEVO like the reference. */
int mhd_advance(mhd_handle *h, double dt);
/* Full iteration: dt from mhd_timestep clipped at tfinal and tsave
 * (:603-604), then mhd_advance.  Returns the dt used and the limiter. */
int mhd_step(mhd_handle *h, double tsave, double *dt, int *st);
/* One mhd_step from a host state to a host state, for a driver that keeps
 * its module arrays on the host and calls the library once per EVOLVE
 * iteration (the reference's loop body :569-656 with the arrays of
 * INITIA / SAVEU on either side).  U_in / species_in are copied in (the
 * layout of mhd_upload; the coordinates of the last mhd_upload are kept), the
 * step runs, and U_out / species_out receive the new state (the layout of
 * mhd_download).  The arrays are copied back while the step still runs as
 * soon as they are final: without chemistry rho and the species after the
 * sweeps, the face field after CT.  The results equal mhd_upload's state
 * copy + mhd_step + mhd_download bit for bit.  In and out may be the same
 * buffers; pinned host memory gives full copy speed.  Needs one
 * mhd_upload on the handle first. */
int mhd_step_host(mhd_handle *h, const double *U_in, const double *species_in, double *U_out,
                  double *species_out, double tsave, double *dt, int *st);
/* nsteps iterations of mhd_step; stops early at tfinal or tsave. */
int mhd_evolve(mhd_handle *h, int nsteps, double tsave, int *steps_done);

/* Inflow data for a handle with BC code 4 on an x side; required before
 * mhd_upload on such a handle.  reservoir: the DTF density field (REAL*4,
 * the padded layout of U, DTF(-1..nx+2,-1..ny+2,-1..nz+2), read by the
 * reference from D###.dat at :402-417), advected across the inflow ghosts
 * at the inflow speed; NULL gives a uniform reservoir of density
 * uniform_density (the shipped code's DTF = dinit1).  Replaces the BBRV /
 * BBRV_cm / DTF set-up of INITIA :182-200, :402-432. */
int mhd_set_inflow(mhd_handle *h, const mhd_inflow *in, const float *reservoir, double uniform_density);

int mhd_get_time(mhd_handle *h, double *time, int *ifevo);
int mhd_set_time(mhd_handle *h, double time, int ifevo);
int mhd_diagnostics(mhd_handle *h, mhd_diag *out);
/* Blocks until all work queued on the handle's stream has finished. */
int mhd_synchronize(mhd_handle *h);
/* Use an existing CUDA stream (cudaStream_t passed as void*); NULL = own. */
int mhd_set_stream(mhd_handle *h, void *stream);
/* Copies the last error message (NUL-terminated) into buf. */
int mhd_last_error(mhd_handle *h, char *buf, int len);
/* Number of kernels launched by this handle since creation. */
long long mhd_kernel_launches(mhd_handle *h);
/* Zeroes the IMC / surrogate / fallback cell counters of mhd_diagnostics. */
int mhd_reset_counters(mhd_handle *h);

/* ---- KI-cooling surrogate (chosen form; no counterpart in the reference,
 * whose stiff cells always take IMC, MCF3DSGincfca3.f90:2898-2921) ----
 * A 3->64->64->2 SiLU network maps (log10 N, log10 T, log10 dt/t_cool) to
 * log10(T_new/T) and a confidence; its FP32 master parameters are a vector
 * of mhd_surrogate_nparams() floats (W1[64][3], b1, W2[64][64], b2,
 * W3[2][64], b3).  Stiff cells inside the training box take the network's
 * answer polished by two Newton steps; a cell whose implicit residual
 * |P + Lambda(P) dt (gamma-1) - P_old| / P_old exceeds tol falls back to
 * the bisection. */
int mhd_surrogate_nparams(void);
/* Attaches a network to a handle created with cooling = MHD_COOL_SURROGATE. */
int mhd_surrogate_load(mhd_handle *h, const float *params, float tol);
/* Trains params in place on n_data states drawn log-uniformly in the box
 * N in [1e-2,1e5] cm^-3, T in [10 K, 2e4 K], dt/t_cool in [1e-3,1e3] and
 * labelled by the plain integrator (FP64 IMC); Adam, batch, steps, lr.
 * history[steps] (may be NULL) gets each batch's mean squared error. */
int mhd_surrogate_train(float *params, long long n_data, int batch, int steps, float lr,
                        unsigned long long seed, float *history, int device);
/* Plain-integrator labels log10(T_new/T) for inputs x[n][3]. */
int mhd_surrogate_label(const float *x, float *y, long long n, double kb, int device);
/* Network outputs out[n][2] for inputs x[n][3] (the fused kernel's code). */
int mhd_surrogate_eval(const float *params, const float *x, float *out, long long n, int device);
/* Gradient of the mean loss over (x, y) at params, computed by the
 * training kernels; loss gets the mean squared error. */
int mhd_surrogate_grad(const float *params, const float *x, const float *y, long long n, float *grad,
                       float *loss, int device);

/* ---- Device measurement (no counterpart in the reference) ----
 * Measured FP64 throughput of one device: fused multiply-adds (GFLOP/s, two
 * per FMA), divisions and square roots (billions per second), each from
 * eight independent dependent chains per thread, timed with CUDA events.
 * The plain FP64 form is bound by this pipe, not by HBM; bench.py quotes its
 * roofline against these numbers. */
int mhd_fp64_peak(int device, double *fma_gflops, double *div_gps, double *sqrt_gps);

/* ---- Time-step limits without device allocation ----
 * No counterpart in the reference (which has no device memory at all).
 * mhd_timestep needs a handle, and a handle allocates its state with
 * cudaMalloc.  Callers that cannot allocate device memory -- a code that
 * owns every device array through its own pool or arena, or one running
 * where new allocations are not allowed -- call this instead with device
 * pointers to arrays they already have, in the layout of mhd_upload: U
 * (8 blocks), species (8 blocks), Bcc (3 blocks, the cell-centred field of
 * CC(4)) and dx, dy, dz (n+4 each).  With p->ifchem == 2 the species
 * cooling also reads the chemistry's electron and particle densities nde
 * and ndtot (one block each, the module arrays of the same names), and
 * with ifchem == 2 and ifrad == 2 SHIELD's ten column blocks (the layout of
 * mhd_download_columns); a missing one gives MHD_ERR_ARG, and they are not
 * read otherwise.  The result equals mhd_timestep's on a handle of either
 * precision holding the same arrays (the chosen form keeps the CFL minimum
 * in FP64).
 *
 * The kernels' scratch is a fixed file-scope device array (about 1 MB) that
 * every GPU loading the library keeps until exit, so grids are limited to
 * MHD_NOALLOC_MAX_CELLS interior cells (256^3); larger grids return
 * MHD_ERR_TOO_LARGE before any GPU work.  The first call on a device looks
 * up the array's device address (cudaGetSymbolAddress); make that first
 * call before any stream capture.  All calls share the one array, so calls
 * whose kernels overlap on the GPU (different streams, or different host
 * threads, at the same time) race; the call synchronises its stream before
 * returning.  stream may be NULL (the legacy default stream). */
#define MHD_NOALLOC_MAX_CELLS 16777216LL
typedef struct mhd_device_state {
  const double *U, *species, *bcc;
  const double *dx, *dy, *dz;
  const double *nde, *ndtot;     /* ifchem == 2 only, else may be NULL     */
  const double *columns;         /* ifchem == 2 and ifrad == 2, else NULL  */
} mhd_device_state;
int mhd_timestep_noalloc(const mhd_params *p, const mhd_device_state *s, double *dt, int *st, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* MHD_GB300_H */
