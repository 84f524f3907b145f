/*
 * Physics plugin "formula234" (SCLET_PHYSICS_FORMULA234): the reference's own
 * default physics, source_beta_to_omega/src/formula.c:9-38, restated in the
 * plugin form of sclet_plugin.h.
 *
 *   init_KL: LE = 1, KE = 42 for every order parameter (formula.c:9-19)
 *   AC_f(n) = f_A e_n - f_B e_n^2 + f_C (sum_m e_m^2) e_n       (:28-38)
 *     f_A = 2376/2372, f_B = (7128 + 12 * 2372)/2372,
 *     f_C = (4752 + 12 * 2372)/2372
 *   bulk energy: f_A/2 sum e^2 - f_B/3 sum e^3 + f_C/4 (sum e^2)^2, the
 *     polynomial AC_f derives from (and the one check_soln_new hard-codes,
 *     field.c:508)
 *
 * The reference's AC_f sums the squares of ac[0..3] whatever nac is; this
 * plugin sums the nac order parameters (the same for nac = 4, the only count
 * at which the reference reads no stale entries).  Its CH_f has no
 * concentration physics (formula.c:40-56: case 0 returns an unset value), so
 * the plugin takes no concentration.  The constants K are not used.
 */
#define SCLET_F234_A (2376.0 / 2372.0)
#define SCLET_F234_B ((7128.0 + 12.0 * 2372.0) / 2372.0)
#define SCLET_F234_C ((4752.0 + 12.0 * 2372.0) / 2372.0)

SCLET_MAX_NCH(0)
SCLET_C0_INDEX(-1)
SCLET_DEFAULTS = {0.0};

SCLET_INIT_KL {
  (void)Kp;
  kl->LE = 1.0;
  kl->KE = 42.0;
  kl->LCI = 0.0;
  kl->KCI = 0.0;
}

SCLET_AC_F {
  real sumh22 = 0, e = ac[n].u;
  int m;
  (void)ch;
  (void)nch;
  (void)Kp;
  for (m = 0; m < nac; m++) sumh22 += ac[m].u * ac[m].u;
  return (real)SCLET_F234_A * e - (real)SCLET_F234_B * e * e + (real)SCLET_F234_C * sumh22 * e;
}

SCLET_CH_F {
  (void)ac;
  (void)ch;
  (void)nac;
  (void)nch;
  (void)Kp;
  (void)n;
  return 0;
}

SCLET_F_BULK {
  real s2 = 0, s3 = 0;
  int m;
  (void)ch;
  (void)nch;
  (void)Kp;
  for (m = 0; m < nac; m++) {
    s2 += ac[m].u * ac[m].u;
    s3 += ac[m].u * ac[m].u * ac[m].u;
  }
  return (real)(SCLET_F234_A / 2.0) * s2 - (real)(SCLET_F234_B / 3.0) * s3 + (real)(SCLET_F234_C / 4.0) * s2 * s2;
}
