/*
 * CPU restatement of the reference's ScLETD ETD step (single periodic rank),
 * TEST INFRASTRUCTURE ONLY: tests, __graft_entry__.smoke() and the bench's
 * CPU baseline use it as the oracle; the product never links it.
 *
 * Every routine cites the reference function it restates
 * (paths relative to the reference project, source_beta_to_omega/src/...).
 * Layout: each field is an n^3 block (n = N + 4: N owned cells plus two ghost
 * layers per side), index z*n*n + y*n + x.  Owned cells are 2..n-3 per axis.
 */
#ifndef SCLET_ORACLE_H
#define SCLET_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int n;            /* block edge incl. ghosts (reference nx = ny = nz) */
  int nac, nch;     /* Allen-Cahn and Cahn-Hilliard field counts */
  int etd2;         /* 1: second-order ETD corrector */
  int elastic;      /* 0 none, 1 elastic force on AC fields */
  int anisotropic;  /* 1: explicit div(lambda grad eta) correction */
  double dt, epn2;
  double h[3];      /* grid spacing per axis */
  double kk[3];     /* per-axis weights of the implicit AC operator */
  double lam[4][3][3]; /* F2 tensors = diag(kk) - file tensor, per AC field */
  double elastic_scale;
  /* physics plugin (numbered as SCLET_PHYSICS_* of include/sclet_gb300.h)
   * and its constants K (for the Landau plugin: a2 a4 a6 g th c0 A LE KE LCI
   * KCI); LE, KE, LCI, KCI from the plugin's init_KL (orc_physics_setup) */
  int physics;
  double K[16];
  double LE, KE, LCI, KCI;
  /* per-axis eigen data: V and V^-1 stored column-major (element (r, c) at
   * c*n + r) as the reference keeps MPX / MPXI; eigenvalues already / h^2. */
  const double *mp[3], *mpi[3], *dd[3];
  /* Green-tensor kernel B_pq(k) on the N^3 FFT grid, [p][q][z][y][x]. */
  const double *bn;
  /* energy: per-AC-field gradient tensors and which Landau polynomial
   * (0: the reference's hard-coded 2-3-4 form, 1: the 2-4-6 plugin form). */
  double elam[4][3][3];
  int energy_form;
  /* 1: variable-mobility Cahn-Hilliard right-hand side (VariableMobility of
   * the ini, ch_calc_FU_VariableMobility, mobility.c:838-858) */
  int variable_mobility;
} orc_cfg;

/* Ghost fill of one n^3 block in place (transfer(), trans.c:1939-1996, on a
 * periodic self-neighbour). */
void orc_ghost_fill(int n, double *f);

/* Boundary values: the periodic image of the cell just outside each face
 * (calc_mu() -> ac_mu/ch_mu fieldu_*, trans.c:927-1937).  faces = 6*n*n:
 * left,right [z][y]; top,bottom [z][x]; front,back [y][x]. */
void orc_boundary_values(int n, const double *f, double *faces);

/* Green-tensor kernel (elastic_calculate_BN, elastic.c:460-605).  voigt: 6x6
 * row-major; eps: 4 x 3x3 row-major eigenstrains.  out: 4*4*N^3. */
void orc_compute_bn(int big_n, const double *voigt, const double *eps, double *out);

/* Elastic force of all AC fields (elastic_calculate, elastic.c:689-763):
 * felas (nac*n^3) keeps the reference's scratch semantics: each field's ghost
 * cells come from the fill of the shared scratch block, whose stale cells hold
 * the previous field's result.  fstate: the scratch block (n^3), persistent. */
void orc_elastic(const orc_cfg *c, const double *eta, double *felas, double *fstate);

/* Right-hand sides of all fields (ac_calc_FU, calc.c:8-68 -> anisotropic.c;
 * ch_calc_FU_ConstantMobility, calc.c:70-473).  u: filled fields
 * ((nac+nch)*n^3), felas as from orc_elastic, out: (nac+nch)*n^3. */
void orc_rhs(const orc_cfg *c, const double *u, const double *felas, double *out);

/* Constants of update_M_C (mobility.c:860-922) for the first concentration:
 * M(eta0) = m0 (1 (1 - eta0) + dg eta0). */
void orc_mobility_constants(double *m0, double *dg);

/* Mode-n product with cyclic rotation: out[b + n*c + n*n*a'] =
 * sum_a M(a', a) * in[a + n*b + n*n*c], M column-major (PUX/PUY/PUZ,
 * calc.c:631-684, one contraction plus its layout rotation). */
void orc_mode_product(int n, const double *m, const double *in, double *out);

/* One pass of the time loop (ScLETD.c:86-190) on state u ((nac+nch)*n^3,
 * updated in place).  felas / fstate: elastic scratch (see orc_elastic). */
void orc_step(const orc_cfg *c, double *u, double *felas, double *fstate);

/* Diagnostics of check_soln_new (field.c:407-678): per field max, min, vol,
 * and the free energy.  out: (nac+nch)*4 doubles. */
void orc_check_soln(const orc_cfg *c, const double *u, double *out);

/* init_KL of the plugin c->physics (formula.c:9-19): fills LE, KE, LCI, KCI
 * from K.  Returns 0, or -1 for an unknown plugin. */
int orc_physics_setup(orc_cfg *c);

/* Threads used by the oracle's parallel loops (OpenMP when built with it). */
int orc_threads(void);

#ifdef __cplusplus
}
#endif
#endif
