// field_io.cu -- the reference's field files (host code).
//
// Field form, written by DEALII_SCFT/src/scft.cc:317-333 and read by
// DEALII_SCFT/src/scft_util.cc:14-41 (read_yita_middle_1D):
//
//   N= <nodes>, ERROR= <%e>
//   mean_field_free_energy, <%2.15f>
//   <i>,<x_i %2.15f>,<w_i %2.15f>          one line per node
//
// The MATLAB inputs (Matlab_files/inputFiles/solution_yita_1D_N=*.txt) carry
// only "N= <nodes>" on the first line and no energy line; read_yita_middle_1D
// skips the second line whatever it holds, which there drops node 0.  This
// reader keeps every data line instead and reports which optional values were
// present.
//
// Result tables (.res) of the external implicit-Euler code, read by
// 1D_FEM.c:321-342: nine header lines ("m = <m>   n = <steps>", a line of
// N= l= cp= mphi= t=, a line of Z= f= |f|max=, column titles and rules, blank
// lines), then one row of five numbers per node: x/l, phi, eta, phie, phij.
// 1D_FEM.c skips ten lines (the header and the wall row) and takes the eta
// column of the interior rows; this reader returns every row, walls included,
// and the header values.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "scft.h"

int scft_internal_set_error(int code, const char *msg);  // runtime.cu: records the message for scft_last_error

namespace {

int fail(int code, const std::string &msg) { return scft_internal_set_error(code, msg.c_str()); }

// Value after `key` on the line (strtod), or NAN when the key is absent.
double keyed(const char *line, const char *key) {
  const char *p = std::strstr(line, key);
  if (!p) return NAN;
  p += std::strlen(key);
  char *end = nullptr;
  const double v = std::strtod(p, &end);
  return end == p ? NAN : v;
}

struct File {
  FILE *f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

}  // namespace

extern "C" {

int scft_field_read(const char *path, int max_nodes, int *n_nodes, double *x, double *w, double *err,
                    double *free_energy) {
  if (!path || !n_nodes || max_nodes < 0) return fail(SCFT_EINVAL, "scft_field_read: null argument");
  File F;
  F.f = std::fopen(path, "r");
  if (!F.f) return fail(SCFT_EIO, std::string("scft_field_read: cannot open ") + path + ": " + std::strerror(errno));
  char line[512];
  if (!std::fgets(line, sizeof line, F.f)) return fail(SCFT_EIO, "scft_field_read: empty file");
  int N = 0;
  if (std::sscanf(line, " N= %d", &N) != 1 || N < 1)
    return fail(SCFT_EINVAL, std::string("scft_field_read: first line is not \"N= <nodes>\": ") + line);
  if (err) *err = keyed(line, "ERROR=");
  if (free_energy) *free_energy = NAN;
  *n_nodes = N;
  if (N > max_nodes) return fail(SCFT_EINVAL, "scft_field_read: " + std::to_string(N) + " nodes exceed max_nodes");
  std::vector<char> seen(N, 0);
  int count = 0;
  while (std::fgets(line, sizeof line, F.f)) {
    if (std::strncmp(line, "mean_field_free_energy", 22) == 0) {
      const char *c = std::strchr(line, ',');
      if (free_energy && c) *free_energy = std::strtod(c + 1, nullptr);
      continue;
    }
    int i;
    double xi, wi;
    if (std::sscanf(line, "%d ,%lf ,%lf", &i, &xi, &wi) != 3) {
      bool blank = true;
      for (const char *p = line; *p; p++) blank &= (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n');
      if (blank) continue;
      return fail(SCFT_EINVAL, std::string("scft_field_read: unreadable line: ") + line);
    }
    if (i < 0 || i >= N) return fail(SCFT_EINVAL, "scft_field_read: node index " + std::to_string(i) + " out of range");
    if (!seen[i]) count++;
    seen[i] = 1;
    if (x) x[i] = xi;
    if (w) w[i] = wi;
  }
  if (count != N)
    return fail(SCFT_EINVAL, "scft_field_read: " + std::to_string(count) + " of " + std::to_string(N) + " nodes present");
  return SCFT_OK;
}

int scft_field_write(const char *path, int n_nodes, const double *x, const double *w, double err, double free_energy) {
  if (!path || !x || !w || n_nodes < 1) return fail(SCFT_EINVAL, "scft_field_write: bad argument");
  File F;
  F.f = std::fopen(path, "w");
  if (!F.f) return fail(SCFT_EIO, std::string("scft_field_write: cannot create ") + path + ": " + std::strerror(errno));
  bool ok = std::fprintf(F.f, "N= %d, ERROR= %e \n", n_nodes, err) > 0;
  ok = ok && std::fprintf(F.f, "mean_field_free_energy, %2.15f \n", free_energy) > 0;
  for (int i = 0; ok && i < n_nodes; i++) ok = std::fprintf(F.f, "%d,%2.15f,%2.15f\n", i, x[i], w[i]) > 0;
  ok = ok && std::fflush(F.f) == 0;
  if (!ok) return fail(SCFT_EIO, std::string("scft_field_write: write failed on ") + path);
  return SCFT_OK;
}

int scft_res_read(const char *path, int max_rows, int *rows, double *table, int *m, int *nsteps, double *header) {
  if (!path || !rows || max_rows < 0 || (max_rows > 0 && !table))
    return fail(SCFT_EINVAL, "scft_res_read: null argument");
  File F;
  F.f = std::fopen(path, "r");
  if (!F.f) return fail(SCFT_EIO, std::string("scft_res_read: cannot open ") + path + ": " + std::strerror(errno));
  char line[512];
  double hv[6] = {NAN, NAN, NAN, NAN, NAN, NAN};  // l, mphi, t, Z, f, |f|max
  int mm = -1, nn = -1, r = 0;
  while (std::fgets(line, sizeof line, F.f)) {
    double v[5];
    if (std::sscanf(line, "%lf %lf %lf %lf %lf", v, v + 1, v + 2, v + 3, v + 4) == 5) {
      if (r < max_rows)
        for (int c = 0; c < 5; c++) table[5 * r + c] = v[c];
      r++;
      continue;
    }
    int a, b;
    if (std::sscanf(line, " m = %d n = %d", &a, &b) == 2) { mm = a; nn = b; }
    const double l = keyed(line, " l="), mphi = keyed(line, "mphi="), t = keyed(line, " t=");
    if (!std::isnan(l)) hv[0] = l;
    if (!std::isnan(mphi)) hv[1] = mphi;
    if (!std::isnan(t)) hv[2] = t;
    if (std::strncmp(line, "Z=", 2) == 0) {
      hv[3] = keyed(line, "Z=");
      hv[4] = keyed(line, " f=");
      hv[5] = keyed(line, "|f|max=");
    }
  }
  if (m) *m = mm;
  if (nsteps) *nsteps = nn;
  if (header)
    for (int k = 0; k < 6; k++) header[k] = hv[k];
  *rows = r;
  if (r > max_rows) return fail(SCFT_EINVAL, "scft_res_read: " + std::to_string(r) + " rows exceed max_rows");
  return SCFT_OK;
}

}  // extern "C"
