// mhd_launch.h — host-side launchers shared by the two precision
// translation units (mhd_fp64.cu, mhd_fp32.cu) and the C-ABI layer.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "mhd_kernels.cuh"
#include "mhd_ct32.cuh"
#include "mhd_source32.cuh"

namespace mhd {

// largest pencil batch P in {4,2,1} that divides the batching direction
// and fits the shared-memory budget
int sweep_batch(const Grid &g, int dir);
size_t sweep_smem_bytes(const Grid &g, int dir, int P);

// plain form (every operation FP64, no contraction)
cudaError_t sweep_fp64(int dir, const SweepArgs &a, cudaStream_t s);
cudaError_t emf_fp64(int e, const CTArgs &a, cudaStream_t s);
// chosen form (FP32 reconstruction / Riemann / characteristics / EMF)
// block / narr: the allocation of narr equal-sized FP64 arrays that holds
// the state (the y and z sweeps stage their inputs from it with TMA)
cudaError_t sweep_fp32(int dir, const SweepArgs &a, const double *block, int narr, cudaStream_t s);
// stiff_mode 0: the bisection for stiff cells; STIFF_NETWORK / STIFF_NEWTON:
// the guess-and-polish path of source32_fused_kernel
cudaError_t source_fp32(const Source32Args &a, int stiff_mode, cudaStream_t s);
// FP32 temperatures of every padded cell; from_species: from the species
// (and store S = H+p+He+He+ and H2 in sh2, 2 ncell floats), else from them
cudaError_t temp_fp32(const Grid &g, const Fields &f, const double *pin, double kb, float *T, float *sh2,
                      bool from_species, cudaStream_t s);
// The chosen form's time step, first kernel (FP32 screen, see
// dt32_screen_kernel): lo gets 3 * nwarps lower ends, words[0..2] the
// smallest upper ends (start them at 0xffffffff) and words[3] the floor
// flag (start at 0).  sh2: S and H2 of every cell (SOURCE's arrays) when
// they are current, or null to form them from the species.
int dt_screen_warps(const Grid &g);
cudaError_t dt_screen_fp32(const Grid &g, const Phys &ph, const Fields &f, const float *sh2, float *lo,
                           unsigned *words, int *err, cudaStream_t s);
// the screen of the interior cells of linear index [c0, c1); c0 and c1 - c0
// multiples of kDtScreenCells (or c1 the last cell), so the slabs' blocks
// are the whole screen's
cudaError_t dt_screen_fp32_range(const Grid &g, const Phys &ph, const Fields &f, const float *sh2, float *lo,
                                 unsigned *words, int *err, long long c0, long long c1, cudaStream_t s);
cudaError_t face_velocity_fp32(const Grid &g, const Fields &f, double *v0, double *v1, double *v2, cudaStream_t s);
cudaError_t ct_prep_fp32(const Grid &g, const Fields &f, double *const vf[3], double kb, const CT32Args &a,
                         cudaStream_t s);
cudaError_t emf32(int e, const CT32Args &a, cudaStream_t s);
// CC(3) of the chosen form; coef: scratch of s[0]+s[1]+s[2] doubles for dt/dx
cudaError_t face_b_fp32(const Grid &g, const Fields &f, float *const emf[3], double dt, double *coef,
                        cudaStream_t s);
// pack FP32 master surrogate parameters into the BF16 device network
cudaError_t surrogate_pack(const float *master, SurNet *net, cudaStream_t s);

// precision-independent FP64 kernels (built in the FP64 unit)
// one ghost exchange over every direction in dirs, one launch
cudaError_t ghost_fill_all(const Grid &g, const FillArgs &f, int dirs, int nol, cudaStream_t s);
// the same exchange restricted to the ghost cells whose padded index along
// rdim lies in [rlo, rhi), or outside it (rdim = -1: all)
cudaError_t ghost_fill_slab(const Grid &g, const FillArgs &f, int dirs, int nol, int rdim, int rlo, int rhi,
                            bool outside, cudaStream_t s);
cudaError_t face_velocity(const Grid &g, const Fields &f, double *v0, double *v1, double *v2, cudaStream_t s);
cudaError_t face_b(const Grid &g, const Fields &f, const double *ez, const double *ex, const double *ey, double dt,
                   cudaStream_t s);
cudaError_t cell_b(const Grid &g, const Fields &f, cudaStream_t s);
// dst = src on the ghost shell of layer lay: 1 the cells with an index 0 or
// n+1 in some direction, 2 those with an index -1 or n+2
cudaError_t shell_copy(const Grid &g, const double *src, double *dst, int lay, cudaStream_t s);
// CC(4) for the interior cells of linear index [c0, c1) (i fastest, then j, k)
cudaError_t cell_b_range(const Grid &g, const Fields &f, long long c0, long long c1, cudaStream_t s);
cudaError_t source_pass(const SourceArgs &a, cudaStream_t s);
cudaError_t chem_step(const Grid &g, const Phys &ph, const Fields &f, double dt, int *err, cudaStream_t s);
cudaError_t chem_totals(const Grid &g, const Fields &f, int plus, cudaStream_t s);
// SHIELD: the optical-depth source term (FP64 / chosen form) into tau, then
// the columns from both x sides (FP64 sums)
cudaError_t shield(const Grid &g, const Phys &ph, const Fields &f, double *tau, double dxh, cudaStream_t s);
cudaError_t shield_fp32(const Grid &g, const Phys &ph, const Fields &f, double *tau, double dxh, cudaStream_t s);
cudaError_t shield_scan(const Grid &g, const Fields &f, const double *tau, double dxh, cudaStream_t s);
cudaError_t chem_step_fp32(const Grid &g, const Phys &ph, const Fields &f, double dt, int *err, cudaStream_t s);
cudaError_t dt_reduce(const Grid &g, const Phys &ph, const Fields &f, unsigned long long *out, int *err,
                      cudaStream_t s);
// second kernel of the chosen form's time step: the FP64 limits of the
// screened candidates, reduced into out like dt_reduce (start at ~0)
cudaError_t dt_refine(const Grid &g, const Phys &ph, const Fields &f, const float *lo, const unsigned *words,
                      unsigned long long *out, cudaStream_t s);
cudaError_t divv(const Grid &g, const Fields &f, double *d, cudaStream_t s);
cudaError_t dissip(const Grid &g, const Fields &f, const double *d, int e, cudaStream_t s);
cudaError_t diag(const Grid &g, const Phys &ph, const Fields &f, double *part, int *nblocks, cudaStream_t s);

// self-gravity (mhd_gravity.cu): the potential of rho on the grid, and the
// half kick of the velocities by its gradient
struct GravityArgs {
  Grid g;
  const double *rho;
  double *phi;                       // padded layout of U
  double2 *S;                        // the half spectrum, gravity_spectrum_size complex values
  double *tab;                       // the grid's tables: 4 gravity_spectrum_size doubles
  const double2 *tw_y, *tw_z;        // twiddles (gravity_twiddles) for ny and nz
  double dx, dy, dz, x0, lbox;       // dx(1), dy(1), dz(1), x(0), x(nx) - x(0)
};
bool gravity_size_ok(int n);          // a power of two up to 1024
size_t gravity_spectrum_size(const Grid &g);   // nx nz (ny/2 + 1)
std::vector<double2> gravity_twiddles(int n);
cudaError_t gravity_tables(const GravityArgs &a, cudaStream_t s);   // once per grid
cudaError_t gravity_solve(const GravityArgs &a, cudaStream_t s);
cudaError_t gravity_kick(const Grid &g, const Fields &f, const double *phi, double dt, double dx0, cudaStream_t s);

}  // namespace mhd
