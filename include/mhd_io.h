/* mhd_io.h — output and restart files of the reference driver.
 *
 * The reference writes, from SAVEU / SAVEU2D (3DMHD-CfCA/MCF3DSGincfca3.f90
 * :684-794) and reads back in INITIA (:454-465), Fortran unformatted
 * sequential files, one per MPI rank of its NSPLTx x NSPLTy x NSPLTz block
 * decomposition.  These functions write and read the same files from one
 * single-domain state (the padded arrays of mhd_upload / mhd_download), so a
 * run on one GPU produces the per-rank file set the reference's analysis and
 * restart code expect, for any decomposition that divides the grid, and a
 * per-rank restart set is merged back into one state.
 *
 *   NNNRRR.dat    snapshot, FP32: per (j,k) of the rank's block, k = 1..nz+1,
 *                 j = 1..ny+1, one record of i = 1..nx+1 cells x 17 values
 *                 U1..U8, H, p, H2, He, He+, C, CO, C+, Phi   (:704-710)
 *   000RRR.dat    restart, the same records in FP64             (:749-757)
 *   2DNNNRRR.dat  plane k = 1 of each rank's block, j = 1..ny, i = 1..nx,
 *                 FP32, with the cell-centred B in place of U6..U8 (:776-782)
 *
 * NNN is the output counter, RRR the rank (I3.3), nx/ny/nz the per-rank block
 * sizes; the cell i = nx+1 (j, k likewise) of a rank is the first cell of its
 * neighbour, or the ghost cell beyond the domain for the last rank.  Every
 * record is framed by 4-byte little-endian length markers (gfortran's
 * default).  Rank r sits at IS = r mod NSPLTx, JS = (r / NSPLTx) mod NSPLTy,
 * KS = r / (NSPLTx NSPLTy) (the reference's own numbering, :409 / INITIA).
 *
 * Species arrays here are in the order of mhd_upload (H, p, H2, He, He+, C,
 * C+, CO); the files hold C, CO, C+ as the reference writes them.  Phi (the
 * self-gravity potential, not part of this path) may be NULL and is then
 * written as zeros.
 *
 * Text files: time.DAT and tsave.DAT with the edit descriptors of the 3D
 * code (1P,D25.17 and I8) or of the 1D code (D25.17), and the info line of
 * SAVEU.  All functions return 0 on success, -1 on a bad argument, -2 on an
 * I/O error.  This interface has no device code; it needs no GPU. */
#ifndef MHD_IO_H
#define MHD_IO_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int nx, ny, nz;      /* interior cells of the whole domain */
  int nsplit[3];       /* ranks per direction; each must divide its extent */
} mhd_io_grid;

/* SAVEU's snapshot NNNRRR.dat (FP32) for every rank. replaces :697-711 */
int mhd_io_write_snapshot(const char *dir, int nunit, const mhd_io_grid *g, const double *U, const double *species,
                          const double *phi);
/* SAVEU's restart 000RRR.dat (FP64) for every rank. replaces :746-758 */
int mhd_io_write_restart(const char *dir, const mhd_io_grid *g, const double *U, const double *species,
                         const double *phi);
/* INITIA's restart read: 000RRR.dat of every rank into one padded state
 * (interior cells and the +1 overlap layer; other ghosts untouched).
 * replaces :454-465 */
int mhd_io_read_restart(const char *dir, const mhd_io_grid *g, double *U, double *species, double *phi);
/* SAVEU2D's plane 2DNNNRRR.dat (k = 1 of every rank's block). replaces :773-783 */
int mhd_io_write_plane(const char *dir, int nunit2d, const mhd_io_grid *g, const double *U, const double *bcc,
                       const double *species, const double *phi);

/* The DTF density reservoir of the inflow boundary as the density
 * generator writes it (GenDen/IGEN1.f90:156-161) and INITIA reads it
 * (MCF3DSGincfca3.f90:404-432): D%03d.dat per rank, for k = 1..nz, j = 1..ny
 * of the rank's block one record of its nx REAL*4 values.  write: every
 * rank's file from the padded single-domain array (the layout mhd_set_inflow
 * takes); read: all files into that array, then the two periodic ghost
 * layers in y and z (the reference's exchanges of DTF) and ghost_density in
 * the x ghosts (DTF's initial value there, dinit1). */
int mhd_io_write_reservoir(const char *dir, const mhd_io_grid *g, const float *dtf);
int mhd_io_read_reservoir(const char *dir, const mhd_io_grid *g, float *dtf, double ghost_density);

/* one value in the D25.17 edit descriptor: with_1p = 1 gives 1P,D25.17 (the
 * 3D code's time.DAT / tsave.DAT), 0 gives D25.17 (the 1D code's).  out must
 * hold 26 bytes. */
int mhd_io_format_d25_17(double v, int with_1p, char *out);
/* time.DAT: t[0..n-1], one value per line */
int mhd_io_write_time_dat(const char *path, const double *t, int n, int with_1p);
/* tsave.DAT: time then the unit counter (I8) */
int mhd_io_write_tsave(const char *path, double time, int nunit, int with_1p);
/* SAVEU's info line (:720): time, "  Step =", step (I8), "  dt =", dt
 * (1P,E11.3), the limiter name; out must hold 96 bytes */
int mhd_io_format_info_line(double time, int step, double dt, const char *limiter, char *out);

#ifdef __cplusplus
}
#endif
#endif
