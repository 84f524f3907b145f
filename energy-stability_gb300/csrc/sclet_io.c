/*
 * Host-side input handling of the ScLETD step: the reference's positional
 * file formats, the eigen-data files, restart text and the seeded initial
 * values.  Plain C; no CUDA.
 */
#include "sclet_gb300.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void sclet_params_default(sclet_params *p) {
  int i;
  memset(p, 0, sizeof *p);
  p->nx = p->ny = p->nz = 68;
  p->px = p->py = p->pz = 1;
  p->nghost = 2;
  strcpy(p->work_dir, "./output/");
  strcpy(p->data_dir, "./data/");
  p->dt = 0.01;
  p->t_total = 9.995;
  p->epn2 = 0.5;
  p->periodic = 1;
  p->nac = 4;
  p->nch = 0;
  strcpy(p->restart_dir, "./restart/");
  p->xmax = p->ymax = p->zmax = 32.0;
  p->elastic = 1;
  p->kkx = p->kky = p->kkz = 1.0;
  p->elastic_scale = 50.0;
  for (i = 0; i < 3; i++) {
    int j;
    for (j = 0; j < 3; j++) p->voigt[i * 6 + j] = (i == j) ? 1.0 : 0.6;
    p->voigt[(3 + i) * 6 + 3 + i] = 0.4;
  }
  {
    static const int dirs[4][3] = {{1, 1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, 1}};
    int v, a, b;
    for (v = 0; v < 4; v++)
      for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) p->eigenstrain[v][a * 3 + b] = a == b ? 0.01 : 0.005 * dirs[v][a] * dirs[v][b];
  }
  {
    static const double lan[11] = {-1.0, -1.0, 2.0, 1.5, 0.8, 0.5, 1.0, 1.0, 6.0, 1.0, 2.0};
    memcpy(p->landau, lan, sizeof lan);
  }
}

/* Positional parse with the same fscanf formats as main() (ScLETD.c:18-34). */
int sclet_read_ini(const char *path, sclet_params *p) {
  FILE *f = fopen(path, "r");
  int ok = 1;
  if (!f) return SCLET_ERR_IO;
  ok &= fscanf(f, "%d,%d,%d", &p->nx, &p->ny, &p->nz) == 3;
  ok &= fscanf(f, "%d,%d,%d", &p->px, &p->py, &p->pz) == 3;
  ok &= fscanf(f, "%d", &p->nghost) == 1;
  ok &= fscanf(f, "%1023s", p->work_dir) == 1;
  ok &= fscanf(f, "%1023s", p->data_dir) == 1;
  ok &= fscanf(f, "%lf,%lf", &p->dt, &p->t_total) == 2;
  ok &= fscanf(f, "%lf", &p->epn2) == 1;
  ok &= fscanf(f, "%d", &p->periodic) == 1;
  ok &= fscanf(f, "%d, %d", &p->nac, &p->nch) == 2;
  ok &= fscanf(f, "%d, %d, %1023s", &p->restart, &p->restart_iter, p->restart_dir) == 3;
  ok &= fscanf(f, "%lf,%lf,%lf", &p->xmin, &p->ymin, &p->zmin) == 3;
  ok &= fscanf(f, "%lf,%lf,%lf", &p->xmax, &p->ymax, &p->zmax) == 3;
  ok &= fscanf(f, "%d", &p->etd2) == 1;
  ok &= fscanf(f, "%d", &p->elastic) == 1;
  ok &= fscanf(f, "%d", &p->anisotropic) == 1;
  ok &= fscanf(f, "%lf,%lf,%lf", &p->kkx, &p->kky, &p->kkz) == 3;
  ok &= fscanf(f, "%d", &p->variable_mobility) == 1;
  fclose(f);
  return ok ? SCLET_OK : SCLET_ERR_IO;
}

/* elastic_input(), elastic.c:349-439: ElasticScale, 36 stiffness values,
 * then four 3x3 eigenstrains. */
int sclet_read_elastic_input(const char *path, sclet_params *p) {
  FILE *f = fopen(path, "r");
  int i, ok = 1;
  if (!f) return SCLET_ERR_IO;
  ok &= fscanf(f, "%lf", &p->elastic_scale) == 1;
  for (i = 0; i < 36 && ok; i++) ok &= fscanf(f, "%lf", &p->voigt[i]) == 1;
  for (i = 0; i < 36 && ok; i++) ok &= fscanf(f, "%lf", &p->eigenstrain[i / 9][i % 9]) == 1;
  fclose(f);
  return ok ? SCLET_OK : SCLET_ERR_IO;
}

/* anisotropic_input(), anisotropic.c:630-674: nac 3x3 tensors. */
int sclet_read_anisotropic_input(const char *path, sclet_params *p) {
  FILE *f = fopen(path, "r");
  int i, ok = 1;
  if (!f) return SCLET_ERR_IO;
  if (p->nac > 4) {
    fclose(f);
    return SCLET_ERR_ARG;
  }
  for (i = 0; i < 9 * p->nac && ok; i++) ok &= fscanf(f, "%lf", &p->lambda_file[i / 9][i % 9]) == 1;
  fclose(f);
  return ok ? SCLET_OK : SCLET_ERR_IO;
}

int sclet_read_landau_input(const char *path, sclet_params *p) {
  FILE *f = fopen(path, "r");
  int i, ok = 1;
  if (!f) return SCLET_ERR_IO;
  for (i = 0; i < 11 && ok; i++) ok &= fscanf(f, "%lf", &p->landau[i]) == 1;
  fclose(f);
  return ok ? SCLET_OK : SCLET_ERR_IO;
}

int sclet_read_case(const char *dir, const char *suffix, sclet_params *p) {
  char path[2300];
  int rc;
  sclet_params_default(p);
  snprintf(path, sizeof path, "%s/input%s.ini", dir, suffix);
  if ((rc = sclet_read_ini(path, p)) != SCLET_OK) return rc;
  if (p->elastic != 0) {
    snprintf(path, sizeof path, "%s/elastic_input.txt", dir);
    if ((rc = sclet_read_elastic_input(path, p)) != SCLET_OK) return rc;
  }
  if (p->anisotropic == 1) {
    snprintf(path, sizeof path, "%s/anisotropic_input.txt", dir);
    if ((rc = sclet_read_anisotropic_input(path, p)) != SCLET_OK) return rc;
  }
  snprintf(path, sizeof path, "%s/landau_input.txt", dir);
  {
    FILE *f = fopen(path, "r");
    if (f) {
      fclose(f);
      if ((rc = sclet_read_landau_input(path, p)) != SCLET_OK) return rc;
    }
  }
  snprintf(path, sizeof path, "%s/physics_input.txt", dir);
  {
    FILE *f = fopen(path, "r");
    if (f) {
      char name[64] = {0};
      int ok = fscanf(f, "%63s", name) == 1;
      fclose(f);
      if (!ok) return SCLET_ERR_IO;
      if (strcmp(name, "landau246") == 0) p->physics = SCLET_PHYSICS_LANDAU246;
      else if (strcmp(name, "formula234") == 0) p->physics = SCLET_PHYSICS_FORMULA234;
      else return SCLET_ERR_ARG;
    }
  }
  return SCLET_OK;
}

/* read_matrices(), vars.c:375-476: eigenvalues one per token; V and V^-1 row
 * by row. */
int sclet_read_eigen(const char *dir, int n, int variant, double *d, double *v, double *vi) {
  char path[2300];
  FILE *f;
  int i, ok = 1;
  snprintf(path, sizeof path, "%s/d%d%d.dat", dir, variant, n);
  if (!(f = fopen(path, "r"))) return SCLET_ERR_IO;
  for (i = 0; i < n && ok; i++) ok &= fscanf(f, "%lf", &d[i]) == 1;
  fclose(f);
  snprintf(path, sizeof path, "%s/v%d%d.dat", dir, variant, n);
  if (!(f = fopen(path, "r"))) return SCLET_ERR_IO;
  for (i = 0; i < n * n && ok; i++) ok &= fscanf(f, "%lf", &v[i]) == 1;
  fclose(f);
  snprintf(path, sizeof path, "%s/vi%d%d.dat", dir, variant, n);
  if (!(f = fopen(path, "r"))) return SCLET_ERR_IO;
  for (i = 0; i < n * n && ok; i++) ok &= fscanf(f, "%lf", &vi[i]) == 1;
  fclose(f);
  return ok ? SCLET_OK : SCLET_ERR_IO;
}

/* DST-I: T = V diag(d) V^T for the Dirichlet second difference, eigenvalues
 * -4 sin^2(k pi / (2(n+1))) in ascending order (k = n .. 1). */
void sclet_eigen_dirichlet(int n, double *d, double *v, double *vi) {
  const double pi = 3.14159265358979323846;
  double s = sqrt(2.0 / (n + 1));
  int i, j;
  for (j = 0; j < n; j++) {
    double k = (double)(n - j);
    double t = sin(k * pi / (2.0 * (n + 1)));
    d[j] = -4.0 * t * t;
  }
  for (i = 0; i < n; i++)
    for (j = 0; j < n; j++) {
      double k = (double)(n - j);
      double val = s * sin(pi * (double)(i + 1) * k / (n + 1));
      v[i * n + j] = val;
      vi[j * n + i] = val;
    }
}

static unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}

double sclet_seeded_value(unsigned long long seed, int field, long long cell, double lo, double hi) {
  unsigned long long key = seed * 0xD1B54A32D192ED03ULL + (unsigned long long)(field + 1) * 0xA0761D6478BD642FULL;
  unsigned long long z = splitmix64(splitmix64((unsigned long long)cell ^ key));
  double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
  return lo + (hi - lo) * u;
}

int sclet_write_restart(const char *path, int n, const double *block) {
  FILE *f = fopen(path, "w");
  int x, y, z;
  if (!f) return SCLET_ERR_IO;
  for (z = 2; z < n - 2; z++)
    for (y = 2; y < n - 2; y++)
      for (x = 2; x < n - 2; x++) fprintf(f, "%.17g\n", block[((size_t)z * n + y) * n + x]);
  fclose(f);
  return SCLET_OK;
}

int sclet_read_restart(const char *path, int n, double *block) {
  FILE *f = fopen(path, "r");
  int x, y, z, ok = 1;
  if (!f) return SCLET_ERR_IO;
  for (z = 2; z < n - 2 && ok; z++)
    for (y = 2; y < n - 2 && ok; y++)
      for (x = 2; x < n - 2 && ok; x++) ok &= fscanf(f, "%lf", &block[((size_t)z * n + y) * n + x]) == 1;
  fclose(f);
  return ok ? SCLET_OK : SCLET_ERR_IO;
}

/* ---- checkpoint and 16-bit field files (the alpha driver's output) ------ */

/* File names of one block: the rank's z coordinate names a sub-directory and
 * the three coordinates end the name (vars.c:975 and :1079 of
 * source_beta_to_alpha/src); a single block is rank (0, 0, 0). */
int sclet_chk_path(char *out, size_t len, const char *dir, int m, int chk) {
  int w = snprintf(out, len, "%s%02d/eta%d_chk%d_%02d%02d%02d.dat", dir, 0, m, chk, 0, 0, 0);
  return (w < 0 || (size_t)w >= len) ? SCLET_ERR_ARG : SCLET_OK;
}

int sclet_field2b_path(char *out, size_t len, const char *dir, int kind, int m, int irun) {
  int w = snprintf(out, len, "%s%02d/%s%d_%06d_%02d%02d%02d.dat", dir, 0, kind == SCLET_CH ? "c" : "eta", m, irun, 0,
                   0, 0);
  return (w < 0 || (size_t)w >= len) ? SCLET_ERR_ARG : SCLET_OK;
}

/* write_chk (vars.c:966-989): the step counter as one int, then every cell of
 * the n^3 block (ghost layers included) as a double, native byte order. */
int sclet_write_chk_file(const char *path, int irun, int n, const double *block) {
  FILE *f = fopen(path, "wb");
  size_t cells = (size_t)n * n * n;
  int ok;
  if (!f) return SCLET_ERR_IO;
  ok = fwrite(&irun, sizeof(int), 1, f) == 1 && fwrite(block, sizeof(double), cells, f) == cells;
  ok &= fclose(f) == 0;
  return ok ? SCLET_OK : SCLET_ERR_IO;
}

/* read_chk (vars.c:1012-1035).  A file shorter than the block is an error
 * (the reference reads past its end unchecked). */
int sclet_read_chk_file(const char *path, int n, int *irun, double *block) {
  FILE *f = fopen(path, "rb");
  size_t cells = (size_t)n * n * n;
  int ok;
  if (!f) return SCLET_ERR_IO;
  ok = fread(irun, sizeof(int), 1, f) == 1 && fread(block, sizeof(double), cells, f) == cells;
  fclose(f);
  return ok ? SCLET_OK : SCLET_ERR_IO;
}

/* ---- plain-text VTK of the order parameters (post-processing) ---------- */
/* The layout of visualisation/write_vtk.py:57-101: a legacy ASCII structured grid
 * of the whole n^3 block, points listed with x fastest and written as
 * (z, y, x), then one float scalar block "eta<m>" per field, every value in
 * %14.6e. */
int sclet_write_vtk_file(const char *path, int istep, int n, int nfields, const double *blocks) {
  FILE *f = fopen(path, "w");
  const size_t cells = (size_t)n * n * n;
  int x, y, z, m, ok = 1;
  size_t l;
  if (!f) return SCLET_ERR_IO;
  ok &= fprintf(f, "# vtk DataFile Version 2.0\ntime_%d.vtk\nASCII\nDATASET STRUCTURED_GRID\n", istep) > 0;
  ok &= fprintf(f, "DIMENSIONS %5d  %5d  %5d\n", n, n, n) > 0;
  ok &= fprintf(f, "POINTS %7zu float\n", cells) > 0;
  for (z = 0; z < n && ok; z++)
    for (y = 0; y < n; y++)
      for (x = 0; x < n; x++) ok &= fprintf(f, "%14.6e   %14.6e   %14.6e\n", (double)z, (double)y, (double)x) > 0;
  ok &= fprintf(f, "POINT_DATA %5zu\n", cells) > 0;
  for (m = 0; m < nfields && ok; m++) {
    ok &= fprintf(f, "SCALARS eta%d  float  1\nLOOKUP_TABLE default\n", m) > 0;
    for (l = 0; l < cells && ok; l++) ok &= fprintf(f, "%14.6e\n", blocks[(size_t)m * cells + l]) > 0;
  }
  ok &= fclose(f) == 0;
  return ok ? SCLET_OK : SCLET_ERR_IO;
}

/* ---- diagnostics logs of check_soln_new (field.c:419-455, 524, 591, 647) --- */
/* One row per field "iter,max,min,vol,eng" appended to phi_ac_<m>.csv /
 * phi_ch_<m>.csv under work_dir, and "iter,eng" to phi_couple.csv when couple
 * is given; iter 0 starts each file with its header line. */
static int soln_row(const char *path, int iter, const char *header, const double *v, int nv) {
  FILE *f;
  int ok = 1, k;
  if (iter == 0) {
    f = fopen(path, "w");
    if (!f) return SCLET_ERR_IO;
    ok &= fprintf(f, "%s\n", header) > 0;
    ok &= fclose(f) == 0;
    if (!ok) return SCLET_ERR_IO;
  }
  f = fopen(path, "a");
  if (!f) return SCLET_ERR_IO;
  ok &= fprintf(f, "%d", iter) > 0;
  for (k = 0; k < nv; k++) ok &= fprintf(f, ",%+1.15f", v[k]) > 0;
  ok &= fprintf(f, "\n") > 0;
  ok &= fclose(f) == 0;
  return ok ? SCLET_OK : SCLET_ERR_IO;
}

int sclet_append_soln_log(const char *work_dir, int iter, int nac, int nch, const sclet_diag *d, const double *couple) {
  char path[4096];
  int m, rc;
  if (couple && nac > 0 && nch > 0) {
    snprintf(path, sizeof path, "%sphi_couple.csv", work_dir);
    if ((rc = soln_row(path, iter, "iter,eng", couple, 1)) != SCLET_OK) return rc;
  }
  for (m = 0; m < nac + nch; m++) {
    const double v[4] = {d[m].max, d[m].min, d[m].vol, d[m].energy};
    snprintf(path, sizeof path, m < nac ? "%sphi_ac_%d.csv" : "%sphi_ch_%d.csv", work_dir, m < nac ? m : m - nac);
    rc = soln_row(path, iter, m < nac ? "iter,maxphiE,minphiE,volE,engE" : "iter,maxphiCI,minphiCI,volCI,engCI", v, 4);
    if (rc != SCLET_OK) return rc;
  }
  return SCLET_OK;
}
