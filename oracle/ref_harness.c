/*
 * Step-by-step driver for the reference's own omega code, compiled into
 * oracle/_ref/libsclet_ref*.so (test infrastructure only).
 *
 * ref_init() performs the set-up sequence of main()
 * (source_beta_to_omega/src/ScLETD.c:15-83: positional ini parse, then
 * elastic_input, alloc_vars, init_vars, anisotropic_input, define_mpi_type,
 * sw_cart_creat, init_para, read_matrices, init_field, elastic_init).
 * ref_step() performs one pass of the time loop body (ScLETD.c:86-190), calling
 * the reference's functions in the same order.  Accessors return the
 * reference's own arrays so a test can read or overwrite them.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "mpi.h"
#include "ScLETD.h"

void elastic_input(void);
void alloc_vars(void);
void init_vars(void);
void anisotropic_input(void);
void define_mpi_type(void);
void sw_cart_creat(void);
void init_para(void);
void read_matrices(void);
void init_field(void);
void elastic_init(void);
void elastic_calculate(void);
void check_soln_new(double);
void transfer(void);
void calc_mu(void);
void ac_calc_FU(int, double *);
void ch_calc_FU(int, double *);
void PUX(double *, double *, double *, double *);
void PUY(double *, double *, double *, double *);
void PUZ(double *, double *, double *, double *, double *);
void ac_updateU_new(int, double *, double *);
void ch_updateU_new(int, double *, double *);
void prepare_U1_new(double *, double *);
void prepare_U2_new(double *, double *, double *);
void correct_U_new(double *, double *);
void zxy_xyz(double *, double *);
void start_mpi(int, char **);

static double g_tt;
static int g_check = 1;

void ref_set_check(int on) { g_check = on; }
double ref_time(void) { return g_tt; }

/* update_M_C (mobility.c:860-922) writes the mobility of three
 * concentrations (ch[0..2].M and .C) whatever nch is.  With fewer than three
 * conserved fields the harness gives ch[] three entries (the reference's own
 * ones first, then two with only an M array), so that the reference's
 * routine runs within bounds; only ch[0..nch-1] enter the step. */
static void pad_ch_for_mobility(void) {
  struct Cahn_Hilliard *p;
  int m;
  if (!VariableMobility || nch >= 3) return;
  p = (struct Cahn_Hilliard *)calloc(3, sizeof *p);
  memcpy(p, ch, (size_t)nch * sizeof *p);
  for (m = nch; m < 3; m++) p[m].M = (double *)calloc((size_t)nx * ny * nz, sizeof(double));
  ch = p;
}

/* Parses input<suffix>.ini in the working directory (format of ScLETD.c:16-34)
 * and runs the reference's set-up.  Returns 0 on success. */
int ref_init(const char *suffix) {
  char filename[1024];
  FILE *file;
  start_mpi(0, NULL);
  snprintf(filename, sizeof filename, "input%s.ini", suffix);
  file = fopen(filename, "r");
  if (!file) return 1;
  if (fscanf(file, "%d,%d,%d", &nx, &ny, &nz) != 3) return 2;
  if (fscanf(file, "%d,%d,%d", &procs[0], &procs[1], &procs[2]) != 3) return 2;
  if (fscanf(file, "%d", &nghost) != 1) return 2;
  if (fscanf(file, "%s", work_dir) != 1) return 2;
  if (fscanf(file, "%s", data_dir) != 1) return 2;
  if (fscanf(file, "%lf,%lf", &dt, &t_total) != 2) return 2;
  if (fscanf(file, "%lf", &epn2) != 1) return 2;
  if (fscanf(file, "%d", &periodic) != 1) return 2;
  if (fscanf(file, "%d, %d", &nac, &nch) != 2) return 2;
  if (fscanf(file, "%d, %d, %s", &restart, &restart_iter, restart_dir) != 3) return 2;
  if (fscanf(file, "%lf,%lf,%lf", &xmin, &ymin, &zmin) != 3) return 2;
  if (fscanf(file, "%lf,%lf,%lf", &xmax, &ymax, &zmax) != 3) return 2;
  if (fscanf(file, "%d", &ETD2) != 1) return 2;
  if (fscanf(file, "%d", &ELASTIC) != 1) return 2;
  if (fscanf(file, "%d", &ANISOTROPIC) != 1) return 2;
  if (fscanf(file, "%lf,%lf,%lf", &kkx, &kky, &kkz) != 3) return 2;
  if (fscanf(file, "%d", &VariableMobility) != 1) return 2;
  fclose(file);
  if (ELASTIC != NEITHER_FUNCTION) elastic_input();
  alloc_vars();
  pad_ch_for_mobility();
  init_vars();
  if (ANISOTROPIC == 1) anisotropic_input();
  define_mpi_type();
  sw_cart_creat();
  init_para();
  read_matrices();
  init_field();
  if (ELASTIC != NEITHER_FUNCTION) elastic_init();
  iter = 0;
  if (restart == 1) iter = restart_iter;
  g_tt = iter * dt;
  ioutput = iter / 100;
  return 0;
}

/* The first half of a loop pass: halo, elastic force, boundary values and the
 * nonlinear right-hand sides into fieldE1 / fieldCI1 (ScLETD.c:86-103). */
void ref_rhs(void) {
  int n;
  transfer();
  if (ELASTIC != NEITHER_FUNCTION) elastic_calculate();
  calc_mu();
  for (n = 0; n < nac; n++) ac_calc_FU(n, ac[n].fieldE1);
  for (n = 0; n < nch; n++) ch_calc_FU(n, ch[n].fieldCI1);
}

/* One pass of the time loop (ScLETD.c:86-190). */
void ref_step(void) {
  int n;
  if (g_check) check_soln_new(g_tt);
  iter++;
  g_tt += dt;
  ref_rhs();
  for (n = 0; n < nac; n++) {
    stage = 0;
    PUX(MPXI, ac[n].fieldE, ac[n].fieldEt, ac[n].fieldEp);
    PUY(MPYI, ac[n].fieldEt, ac[n].fieldE, ac[n].fieldEp);
    PUZ(MPZI, ac[n].fieldE, ac[n].fieldEt, ac[n].fieldEp, ac[n].fieldEt);
    stage = 1;
    PUX(MPXI, ac[n].fieldE1, ac[n].fieldE, ac[n].fieldEp);
    PUY(MPYI, ac[n].fieldE, ac[n].fieldE1p, ac[n].fieldEp);
    PUZ(MPZI, ac[n].fieldE1p, ac[n].fieldE, ac[n].fieldEp, ac[n].fieldEt);
    ac_updateU_new(n, ac[n].fieldEt, ac[n].fieldEp);
    zxy_xyz(ac[n].fieldEt, ac[n].fieldE);
    stage = 2;
    PUX(MPX, ac[n].fieldE, ac[n].fieldE1p, ac[n].fieldEp);
    PUY(MPY, ac[n].fieldE1p, ac[n].fieldEt, ac[n].fieldEp);
    PUZ(MPZ, ac[n].fieldEt, ac[n].fieldE, ac[n].fieldEp, ac[n].fieldEt);
  }
  for (n = 0; n < nch; n++) {
    stage = 0;
    PUX(MPXI, ch[n].fieldCI, ch[n].fieldCIt, ch[n].fieldCIp);
    PUY(MPYI, ch[n].fieldCIt, ch[n].fieldCI, ch[n].fieldCIp);
    PUZ(MPZI, ch[n].fieldCI, ch[n].fieldCIt, ch[n].fieldCIp, ch[n].fieldCIt);
    stage = 1;
    PUX(MPXI, ch[n].fieldCI1, ch[n].fieldCI, ch[n].fieldCIp);
    PUY(MPYI, ch[n].fieldCI, ch[n].fieldCI1p, ch[n].fieldCIp);
    PUZ(MPZI, ch[n].fieldCI1p, ch[n].fieldCI, ch[n].fieldCIp, ch[n].fieldCIt);
    ch_updateU_new(n, ch[n].fieldCIt, ch[n].fieldCIp);
    zxy_xyz(ch[n].fieldCIt, ch[n].fieldCI);
    stage = 2;
    PUX(MPX, ch[n].fieldCI, ch[n].fieldCI1p, ch[n].fieldCIp);
    PUY(MPY, ch[n].fieldCI1p, ch[n].fieldCIt, ch[n].fieldCIp);
    PUZ(MPZ, ch[n].fieldCIt, ch[n].fieldCI, ch[n].fieldCIp, ch[n].fieldCIt);
  }
  if (ETD2 == 1) {
    transfer();
    if (ELASTIC != NEITHER_FUNCTION) elastic_calculate();
    calc_mu();
    for (n = 0; n < nac; n++) ac_calc_FU(n, ac[n].fieldE2);
    for (n = 0; n < nch; n++) ch_calc_FU(n, ch[n].fieldCI2);
    for (n = 0; n < nac; n++) {
      prepare_U1_new(ac[n].fieldE1, ac[n].fieldE2);
      stage = 0;
      PUX(MPXI, ac[n].fieldE2, ac[n].fieldEt, ac[n].fieldEp);
      PUY(MPYI, ac[n].fieldEt, ac[n].fieldE1p, ac[n].fieldEp);
      PUZ(MPZI, ac[n].fieldE1p, ac[n].fieldE2, ac[n].fieldEp, ac[n].fieldEt);
      prepare_U2_new(ac[n].phiE2, ac[n].fieldE1, ac[n].fieldE2);
      zxy_xyz(ac[n].fieldE2, ac[n].fieldE1);
      stage = 2;
      PUX(MPX, ac[n].fieldE1, ac[n].fieldE1p, ac[n].fieldEp);
      PUY(MPY, ac[n].fieldE1p, ac[n].fieldEt, ac[n].fieldEp);
      PUZ(MPZ, ac[n].fieldEt, ac[n].fieldE1, ac[n].fieldEp, ac[n].fieldEt);
      correct_U_new(ac[n].fieldE, ac[n].fieldE1);
    }
    for (n = 0; n < nch; n++) {
      prepare_U1_new(ch[n].fieldCI1, ch[n].fieldCI2);
      stage = 0;
      PUX(MPXI, ch[n].fieldCI2, ch[n].fieldCIt, ch[n].fieldCIp);
      PUY(MPYI, ch[n].fieldCIt, ch[n].fieldCI1p, ch[n].fieldCIp);
      PUZ(MPZI, ch[n].fieldCI1p, ch[n].fieldCI2, ch[n].fieldCIp, ch[n].fieldCIt);
      prepare_U2_new(ch[n].phiCI2, ch[n].fieldCI1, ch[n].fieldCI2);
      zxy_xyz(ch[n].fieldCI2, ch[n].fieldCI1);
      stage = 2;
      PUX(MPX, ch[n].fieldCI1, ch[n].fieldCI1p, ch[n].fieldCIp);
      PUY(MPY, ch[n].fieldCI1p, ch[n].fieldCIt, ch[n].fieldCIp);
      PUZ(MPZ, ch[n].fieldCIt, ch[n].fieldCI1, ch[n].fieldCIp, ch[n].fieldCIt);
      correct_U_new(ch[n].fieldCI, ch[n].fieldCI1);
    }
  }
}

/* Accessors.  which: 0 field, 1 field1 (RHS), 2 felas, 3..8 boundary values
 * u_left,right,top,bottom,front,back, 9..14 boundary mu (same order),
 * 15 phi, 16 phi2, 17..22 enlarged halo slabs (left,right,top,bottom,front,
 * back; (n+4)x(n+4)x4 each), 23 field2.  kind: 0 = Allen-Cahn, 1 = Cahn-Hilliard. */
double *ref_ptr(int kind, int n, int which) {
  if (kind == 0) {
    struct Allen_Cahn *a = &ac[n];
    double *t[] = {a->fieldE, a->fieldE1, a->felas, a->fieldEu_left, a->fieldEu_right, a->fieldEu_top,
                   a->fieldEu_bottom, a->fieldEu_front, a->fieldEu_back, a->fieldEmu_left, a->fieldEmu_right,
                   a->fieldEmu_top, a->fieldEmu_bottom, a->fieldEmu_front, a->fieldEmu_back, a->phiE, a->phiE2,
                   a->fieldEe_left, a->fieldEe_right, a->fieldEe_top, a->fieldEe_bottom, a->fieldEe_front,
                   a->fieldEe_back, a->fieldE2};
    return t[which];
  } else {
    struct Cahn_Hilliard *c = &ch[n];
    double *t[] = {c->fieldCI, c->fieldCI1, c->felas, c->fieldCIu_left, c->fieldCIu_right, c->fieldCIu_top,
                   c->fieldCIu_bottom, c->fieldCIu_front, c->fieldCIu_back, c->fieldCImu_left, c->fieldCImu_right,
                   c->fieldCImu_top, c->fieldCImu_bottom, c->fieldCImu_front, c->fieldCImu_back, c->phiCI, c->phiCI2,
                   c->fieldCIe_left, c->fieldCIe_right, c->fieldCIe_top, c->fieldCIe_bottom, c->fieldCIe_front,
                   c->fieldCIe_back, c->fieldCI2};
    return t[which];
  }
}

/* Per-axis matrices after read_matrices: 0 MPX 1 MPY 2 MPZ 3 MPXI 4 MPYI 5 MPZI
 * 6 DDX 7 DDY 8 DDZ. */
double *ref_mat(int which) {
  double *t[] = {MPX, MPY, MPZ, MPXI, MPYI, MPZI, DDX, DDY, DDZ};
  return t[which];
}

double ref_h(int axis) { return axis == 0 ? hx : axis == 1 ? hy : hz; }
int ref_iter(void) { return iter; }
