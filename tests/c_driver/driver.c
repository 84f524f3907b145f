/*
 * The reference's time loop (source_beta_to_omega/src/ScLETD.c:15-191) as a
 * plain C driver on the C ABI of libsclet_gb300.so, the binding a
 * maintainer would add on the reference side (the loop of INTEGRATION.md).
 * Test program: built by tests/test_c_driver.py.
 *
 *   driver RUN_DIR SUFFIX STEPS PRECISION OUT.bin
 *
 * Reads the run directory (ini, elastic/anisotropic/landau/physics inputs,
 * the eigen files d3<n>.dat / v3<n>.dat / vi3<n>.dat when present, the
 * restart fields input/field_iter0_{ac,ch}<m>_000.txt), runs STEPS passes
 * stage by stage, prints one "diag" line per pass and field (check_soln_new)
 * and writes the final field blocks (F n^3 doubles, AC fields first) to
 * OUT.bin.  Exit status 0 on success, 1 with the library's message on error.
 */
#include <stdio.h>
#include <stdlib.h>

#include "sclet_gb300.h"

static int fail(const char *what, int rc, const sclet_ctx *ctx) {
  fprintf(stderr, "%s failed (%d): %s\n", what, rc, sclet_last_error(ctx));
  return 1;
}

int main(int argc, char **argv) {
  sclet_params p;
  sclet_ctx *ctx = NULL;
  char path[2048];
  int rc, it, m, steps, precision, n, F;
  double *d, *v, *vi, *out;
  sclet_diag diag[5];
  FILE *fo;
  if (argc != 6) {
    fprintf(stderr, "usage: driver RUN_DIR SUFFIX STEPS PRECISION OUT.bin\n");
    return 2;
  }
  steps = atoi(argv[3]);
  precision = atoi(argv[4]);
  /* main(): ScLETD.c:15-72 */
  if ((rc = sclet_read_case(argv[1], argv[2], &p)) != SCLET_OK) return fail("sclet_read_case", rc, NULL);
  /* alloc_vars, init_para, read_matrices, *_init_phi, elastic_init (vars.c:58-591) */
  if ((rc = sclet_create(&p, precision, 0, &ctx)) != SCLET_OK) return fail("sclet_create", rc, NULL);
  n = sclet_block_edge(ctx);
  F = sclet_field_count(ctx);
  d = malloc(sizeof(double) * n);
  v = malloc(sizeof(double) * n * n);
  vi = malloc(sizeof(double) * n * n);
  if (sclet_read_eigen(argv[1], n, 3, d, v, vi) == SCLET_OK &&
      (rc = sclet_set_eigen(ctx, d, v, vi)) != SCLET_OK)
    return fail("sclet_set_eigen", rc, ctx);
  /* init_field() with restart = 1 (field.c:746-754) */
  for (m = 0; m < p.nac; m++) {
    snprintf(path, sizeof path, "%s/input/field_iter0_ac%d_000.txt", argv[1], m);
    if ((rc = sclet_load_restart(ctx, SCLET_AC, m, path)) != SCLET_OK) return fail("sclet_load_restart", rc, ctx);
  }
  for (m = 0; m < p.nch; m++) {
    snprintf(path, sizeof path, "%s/input/field_iter0_ch%d_000.txt", argv[1], m);
    if ((rc = sclet_load_restart(ctx, SCLET_CH, m, path)) != SCLET_OK) return fail("sclet_load_restart", rc, ctx);
  }
  for (it = 0; it < steps; it++) {
    /* one pass of ScLETD.c:86-190, stage by stage */
    if ((rc = sclet_transfer(ctx)) != SCLET_OK) return fail("sclet_transfer", rc, ctx);
    if ((rc = sclet_elastic_calculate(ctx)) != SCLET_OK) return fail("sclet_elastic_calculate", rc, ctx);
    if ((rc = sclet_calc_rhs(ctx, 1)) != SCLET_OK) return fail("sclet_calc_rhs", rc, ctx);
    if ((rc = sclet_etd_update(ctx)) != SCLET_OK) return fail("sclet_etd_update", rc, ctx);
    if (p.etd2) {
      if ((rc = sclet_transfer(ctx)) != SCLET_OK) return fail("sclet_transfer", rc, ctx);
      if ((rc = sclet_elastic_calculate(ctx)) != SCLET_OK) return fail("sclet_elastic_calculate", rc, ctx);
      if ((rc = sclet_calc_rhs(ctx, 2)) != SCLET_OK) return fail("sclet_calc_rhs", rc, ctx);
      if ((rc = sclet_etd2_correct(ctx)) != SCLET_OK) return fail("sclet_etd2_correct", rc, ctx);
    }
    /* check_soln_new (field.c:407-678) */
    if ((rc = sclet_check_soln(ctx, 1, diag)) != SCLET_OK) return fail("sclet_check_soln", rc, ctx);
    for (m = 0; m < F; m++)
      printf("diag %d %d %.17g %.17g %.17g %.17g\n", it, m, diag[m].max, diag[m].min, diag[m].vol, diag[m].energy);
  }
  out = malloc(sizeof(double) * (size_t)F * n * n * n);
  if ((rc = sclet_get_fields(ctx, out)) != SCLET_OK) return fail("sclet_get_fields", rc, ctx);
  fo = fopen(argv[5], "wb");
  if (!fo || fwrite(out, sizeof(double), (size_t)F * n * n * n, fo) != (size_t)F * n * n * n) {
    fprintf(stderr, "cannot write %s\n", argv[5]);
    return 1;
  }
  fclose(fo);
  sclet_destroy(ctx); /* dealloc_vars, vars.c:593-732 */
  free(d);
  free(v);
  free(vi);
  free(out);
  return 0;
}
