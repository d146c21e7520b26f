// mhd_io.cpp — the reference's output and restart files from one
// single-domain state (include/mhd_io.h): SAVEU / SAVEU2D's per-rank
// Fortran unformatted files (3DMHD-CfCA/MCF3DSGincfca3.f90:684-794), the
// restart read of INITIA (:454-465), the DTF reservoir files of the inflow
// boundary (GenDen/IGEN1.f90:156-161, MCF3DSGincfca3.f90:404-432) and the
// text files time.DAT, tsave.DAT and the info line.  Host code only.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mhd_io.h"

namespace {

constexpr int kFields = 17;   // U1..U8, 8 species, Phi
// file slot -> species array of the mhd_upload order (H,p,H2,He,He+,C,C+,CO);
// the files hold ndH, ndp, ndH2, ndHe, ndHep, ndC, ndCO, ndCp
constexpr int kSpeciesOfSlot[8] = {0, 1, 2, 3, 4, 5, 7, 6};

bool valid(const mhd_io_grid *g) {
  if (!g || g->nx < 1 || g->ny < 1 || g->nz < 1) return false;
  const int n[3] = {g->nx, g->ny, g->nz};
  for (int d = 0; d < 3; d++)
    if (g->nsplit[d] < 1 || n[d] % g->nsplit[d] != 0) return false;
  return g->nsplit[0] * g->nsplit[1] * g->nsplit[2] <= 1000;   // RRR has three digits
}

struct Layout {
  long long sx, sy, ncell;   // padded strides
  int bx, by, bz;            // per-rank block sizes
  explicit Layout(const mhd_io_grid *g)
      : sx(g->nx + 4), sy(g->ny + 4), ncell((long long)(g->nx + 4) * (g->ny + 4) * (g->nz + 4)),
        bx(g->nx / g->nsplit[0]), by(g->ny / g->nsplit[1]), bz(g->nz / g->nsplit[2]) {}
  // offset of global cell (i, j, k), 1-based interior indices, ghosts -1..n+2
  long long at(int i, int j, int k) const { return (i + 1) + sx * ((j + 1) + sy * (long long)(k + 1)); }
};

void rank_origin(const mhd_io_grid *g, int r, int &is, int &js, int &ks) {
  is = r % g->nsplit[0];
  ks = r / (g->nsplit[0] * g->nsplit[1]);
  js = r / g->nsplit[0] - g->nsplit[1] * ks;
}

std::string join(const char *dir, const char *name) {
  std::string s = dir ? dir : ".";
  if (!s.empty() && s.back() != '/') s += '/';
  return s + name;
}

// one Fortran unformatted sequential record: marker, payload, marker
// (little-endian 4-byte markers; the payload is written in host order,
// which is little-endian on every platform this library builds for)
bool put_record(FILE *f, const void *data, size_t bytes) {
  if (bytes > 0x7fffffffu) return false;
  const uint32_t m = (uint32_t)bytes;
  unsigned char mk[4] = {(unsigned char)(m & 0xff), (unsigned char)((m >> 8) & 0xff),
                         (unsigned char)((m >> 16) & 0xff), (unsigned char)((m >> 24) & 0xff)};
  return fwrite(mk, 1, 4, f) == 4 && fwrite(data, 1, bytes, f) == bytes && fwrite(mk, 1, 4, f) == 4;
}

bool get_record(FILE *f, void *data, size_t bytes) {
  unsigned char mk[4], mk2[4];
  if (fread(mk, 1, 4, f) != 4) return false;
  const uint32_t m = mk[0] | (mk[1] << 8) | (mk[2] << 16) | ((uint32_t)mk[3] << 24);
  if (m != bytes) return false;
  if (fread(data, 1, bytes, f) != bytes || fread(mk2, 1, 4, f) != 4) return false;
  return memcmp(mk, mk2, 4) == 0;
}

// the 17 values of one cell in file order; b3 is U6..U8 or the cell-centred B
template <class T>
void gather_cell(const double *U, const double *sp, const double *phi, const double *b3, long long a,
                 long long ncell, T *out) {
  for (int q = 0; q < 5; q++) out[q] = (T)U[q * ncell + a];
  for (int q = 0; q < 3; q++) out[5 + q] = b3 ? (T)b3[q * ncell + a] : (T)U[(5 + q) * ncell + a];
  for (int s = 0; s < 8; s++) out[8 + s] = (T)sp[kSpeciesOfSlot[s] * ncell + a];
  out[16] = phi ? (T)phi[a] : (T)0;
}

// every rank's file: per (j,k) of its block incl. the +1 layer, one record
template <class T>
int write_blocks(const char *dir, const char *prefix, int nunit, const mhd_io_grid *g, const double *U,
                 const double *sp, const double *phi) {
  if (!valid(g) || !U || !sp) return -1;
  const Layout L(g);
  const int nranks = g->nsplit[0] * g->nsplit[1] * g->nsplit[2];
  std::vector<T> rec((size_t)(L.bx + 1) * kFields);
  for (int r = 0; r < nranks; r++) {
    int is, js, ks;
    rank_origin(g, r, is, js, ks);
    char name[64];
    if (nunit < 0) snprintf(name, sizeof name, "%s%03d.dat", prefix, r);
    else snprintf(name, sizeof name, "%s%03d%03d.dat", prefix, nunit, r);
    FILE *f = fopen(join(dir, name).c_str(), "wb");
    if (!f) return -2;
    bool ok = true;
    for (int k = 1; k <= L.bz + 1 && ok; k++)
      for (int j = 1; j <= L.by + 1 && ok; j++) {
        for (int i = 1; i <= L.bx + 1; i++)
          gather_cell<T>(U, sp, phi, nullptr, L.at(is * L.bx + i, js * L.by + j, ks * L.bz + k), L.ncell,
                         &rec[(size_t)(i - 1) * kFields]);
        ok = put_record(f, rec.data(), rec.size() * sizeof(T));
      }
    ok = (fclose(f) == 0) && ok;
    if (!ok) return -2;
  }
  return 0;
}

// Fortran D editing of one value, width 25, 17 digits: k = 1 (1P) gives
// one digit before the point and 17 after, k = 0 gives 0.<17 digits>.  The
// exponent is D+dd, or +ddd without the letter when it needs three digits.
void format_d(double v, int with_1p, char *out) {
  char buf[64];
  int e = 0;
  std::string mant;
  if (!std::isfinite(v)) {
    snprintf(out, 26, "%25s", std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity"));
    return;
  }
  const bool neg = std::signbit(v) && v != 0.0;
  if (with_1p) {
    snprintf(buf, sizeof buf, "%.17E", std::fabs(v));   // d.ddd...(17)E+xx, correctly rounded
    char *E = strchr(buf, 'E');
    e = v == 0.0 ? 0 : atoi(E + 1);
    mant.assign(buf, E - buf);
  } else {
    snprintf(buf, sizeof buf, "%.16E", std::fabs(v));   // 17 significant digits
    char *E = strchr(buf, 'E');
    e = v == 0.0 ? 0 : atoi(E + 1) + 1;
    std::string digits;
    for (char *c = buf; c < E; c++)
      if (*c != '.') digits += *c;
    mant = "0." + digits;
  }
  char ex[8];
  if (e >= -99 && e <= 99) snprintf(ex, sizeof ex, "D%c%02d", e < 0 ? '-' : '+', e < 0 ? -e : e);
  else snprintf(ex, sizeof ex, "%c%03d", e < 0 ? '-' : '+', e < 0 ? -e : e);
  std::string s = (neg ? "-" : "") + mant + ex;
  snprintf(out, 26, "%25s", s.c_str());
}

// Fortran 1P,E11.3
void format_e11_3(double v, char *out) {
  char buf[64];
  if (!std::isfinite(v)) {
    snprintf(out, 12, "%11s", std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity"));
    return;
  }
  snprintf(buf, sizeof buf, "%.3E", std::fabs(v));
  char *E = strchr(buf, 'E');
  int e = v == 0.0 ? 0 : atoi(E + 1);
  std::string mant(buf, E - buf);
  char ex[8];
  if (e >= -99 && e <= 99) snprintf(ex, sizeof ex, "E%c%02d", e < 0 ? '-' : '+', e < 0 ? -e : e);
  else snprintf(ex, sizeof ex, "%c%03d", e < 0 ? '-' : '+', e < 0 ? -e : e);
  std::string s = ((std::signbit(v) && v != 0.0) ? "-" : "") + mant + ex;
  snprintf(out, 12, "%11s", s.c_str());
}

}  // namespace

extern "C" {

int mhd_io_write_snapshot(const char *dir, int nunit, const mhd_io_grid *g, const double *U, const double *species,
                          const double *phi) {
  if (nunit < 0 || nunit > 999) return -1;
  return write_blocks<float>(dir, "", nunit, g, U, species, phi);
}

int mhd_io_write_restart(const char *dir, const mhd_io_grid *g, const double *U, const double *species,
                         const double *phi) {
  return write_blocks<double>(dir, "000", -1, g, U, species, phi);
}

int mhd_io_read_restart(const char *dir, const mhd_io_grid *g, double *U, double *species, double *phi) {
  if (!valid(g) || !U || !species) return -1;
  const Layout L(g);
  const int nranks = g->nsplit[0] * g->nsplit[1] * g->nsplit[2];
  std::vector<double> rec((size_t)(L.bx + 1) * kFields);
  for (int r = 0; r < nranks; r++) {
    int is, js, ks;
    rank_origin(g, r, is, js, ks);
    char name[32];
    snprintf(name, sizeof name, "000%03d.dat", r);
    FILE *f = fopen(join(dir, name).c_str(), "rb");
    if (!f) return -2;
    bool ok = true;
    for (int k = 1; k <= L.bz + 1 && ok; k++)
      for (int j = 1; j <= L.by + 1 && ok; j++) {
        ok = get_record(f, rec.data(), rec.size() * sizeof(double));
        for (int i = 1; ok && i <= L.bx + 1; i++) {
          const long long a = L.at(is * L.bx + i, js * L.by + j, ks * L.bz + k);
          const double *c = &rec[(size_t)(i - 1) * kFields];
          for (int q = 0; q < 8; q++) U[q * L.ncell + a] = c[q];
          for (int s = 0; s < 8; s++) species[kSpeciesOfSlot[s] * L.ncell + a] = c[8 + s];
          if (phi) phi[a] = c[16];
        }
      }
    fclose(f);
    if (!ok) return -2;
  }
  return 0;
}

int mhd_io_write_plane(const char *dir, int nunit2d, const mhd_io_grid *g, const double *U, const double *bcc,
                       const double *species, const double *phi) {
  if (!valid(g) || !U || !bcc || !species || nunit2d < 0 || nunit2d > 999) return -1;
  const Layout L(g);
  const int nranks = g->nsplit[0] * g->nsplit[1] * g->nsplit[2];
  std::vector<float> rec((size_t)L.bx * kFields);
  for (int r = 0; r < nranks; r++) {
    int is, js, ks;
    rank_origin(g, r, is, js, ks);
    char name[32];
    snprintf(name, sizeof name, "2D%03d%03d.dat", nunit2d, r);
    FILE *f = fopen(join(dir, name).c_str(), "wb");
    if (!f) return -2;
    bool ok = true;
    const int k = 1;
    for (int j = 1; j <= L.by && ok; j++) {
      for (int i = 1; i <= L.bx; i++)
        gather_cell<float>(U, species, phi, bcc, L.at(is * L.bx + i, js * L.by + j, ks * L.bz + k), L.ncell,
                           &rec[(size_t)(i - 1) * kFields]);
      ok = put_record(f, rec.data(), rec.size() * sizeof(float));
    }
    ok = (fclose(f) == 0) && ok;
    if (!ok) return -2;
  }
  return 0;
}

int mhd_io_write_reservoir(const char *dir, const mhd_io_grid *g, const float *dtf) {
  if (!valid(g) || !dtf) return -1;
  const Layout L(g);
  const int nranks = g->nsplit[0] * g->nsplit[1] * g->nsplit[2];
  std::vector<float> rec((size_t)L.bx);
  for (int r = 0; r < nranks; r++) {
    int is, js, ks;
    rank_origin(g, r, is, js, ks);
    char name[32];
    snprintf(name, sizeof name, "D%03d.dat", r);
    FILE *f = fopen(join(dir, name).c_str(), "wb");
    if (!f) return -2;
    bool ok = true;
    for (int k = 1; k <= L.bz && ok; k++)
      for (int j = 1; j <= L.by && ok; j++) {
        for (int i = 1; i <= L.bx; i++) rec[(size_t)(i - 1)] = dtf[L.at(is * L.bx + i, js * L.by + j, ks * L.bz + k)];
        ok = put_record(f, rec.data(), rec.size() * sizeof(float));
      }
    ok = (fclose(f) == 0) && ok;
    if (!ok) return -2;
  }
  return 0;
}

int mhd_io_read_reservoir(const char *dir, const mhd_io_grid *g, float *dtf, double ghost_density) {
  if (!valid(g) || !dtf) return -1;
  const Layout L(g);
  for (long long q = 0; q < L.ncell; q++) dtf[q] = (float)ghost_density;   // DTF(:,:,:) = dinit1
  const int nranks = g->nsplit[0] * g->nsplit[1] * g->nsplit[2];
  std::vector<float> rec((size_t)L.bx);
  for (int r = 0; r < nranks; r++) {
    int is, js, ks;
    rank_origin(g, r, is, js, ks);
    char name[32];
    snprintf(name, sizeof name, "D%03d.dat", r);
    FILE *f = fopen(join(dir, name).c_str(), "rb");
    if (!f) return -2;
    bool ok = true;
    for (int k = 1; k <= L.bz && ok; k++)
      for (int j = 1; j <= L.by && ok; j++) {
        ok = get_record(f, rec.data(), rec.size() * sizeof(float));
        for (int i = 1; ok && i <= L.bx; i++) dtf[L.at(is * L.bx + i, js * L.by + j, ks * L.bz + k)] = rec[(size_t)(i - 1)];
      }
    fclose(f);
    if (!ok) return -2;
  }
  // periodic ghost layers in y, then z (:418-432), every x index
  for (int k = 1; k <= g->nz; k++)
    for (int i = -1; i <= g->nx + 2; i++) {
      dtf[L.at(i, -1, k)] = dtf[L.at(i, g->ny - 1, k)];
      dtf[L.at(i, 0, k)] = dtf[L.at(i, g->ny, k)];
      dtf[L.at(i, g->ny + 1, k)] = dtf[L.at(i, 1, k)];
      dtf[L.at(i, g->ny + 2, k)] = dtf[L.at(i, 2, k)];
    }
  for (int j = -1; j <= g->ny + 2; j++)
    for (int i = -1; i <= g->nx + 2; i++) {
      dtf[L.at(i, j, -1)] = dtf[L.at(i, j, g->nz - 1)];
      dtf[L.at(i, j, 0)] = dtf[L.at(i, j, g->nz)];
      dtf[L.at(i, j, g->nz + 1)] = dtf[L.at(i, j, 1)];
      dtf[L.at(i, j, g->nz + 2)] = dtf[L.at(i, j, 2)];
    }
  return 0;
}

int mhd_io_format_d25_17(double v, int with_1p, char *out) {
  if (!out) return -1;
  format_d(v, with_1p, out);
  return 0;
}

int mhd_io_write_time_dat(const char *path, const double *t, int n, int with_1p) {
  if (!path || (n > 0 && !t) || n < 0) return -1;
  FILE *f = fopen(path, "w");
  if (!f) return -2;
  char line[32];
  bool ok = true;
  for (int i = 0; i < n && ok; i++) {
    format_d(t[i], with_1p, line);
    ok = fprintf(f, "%s\n", line) > 0;
  }
  ok = (fclose(f) == 0) && ok;
  return ok ? 0 : -2;
}

int mhd_io_write_tsave(const char *path, double time, int nunit, int with_1p) {
  if (!path) return -1;
  FILE *f = fopen(path, "w");
  if (!f) return -2;
  char line[32];
  format_d(time, with_1p, line);
  bool ok = fprintf(f, "%s\n%8d\n", line, nunit) > 0;
  ok = (fclose(f) == 0) && ok;
  return ok ? 0 : -2;
}

int mhd_io_format_info_line(double time, int step, double dt, const char *limiter, char *out) {
  if (!out || !limiter) return -1;
  char t25[32], d11[16];
  format_d(time, 1, t25);
  format_e11_3(dt, d11);
  snprintf(out, 96, "%s  Step =%8d  dt =%s%.7s", t25, step, d11, limiter);
  return 0;
}

}  // extern "C"
