/*
 * Physics plugin "landau246" (SCLET_PHYSICS_LANDAU246): Landau 2-4-6 free
 * energy with a cross term and a c-eta coupling, written against the
 * reference's plugin interface (init_KL / AC_f / CH_f,
 * source_beta_to_omega/src/formula.c:9-56) through sclet_plugin.h.
 *
 *   f = sum_n [a2/2 e_n^2 + a4/4 e_n^4 + a6/6 e_n^6] + g sum_{m<n} e_m^2 e_n^2
 *       + A/2 (c - c0)^2 - th (c - c0) sum_n e_n^2      (c terms when nch = 1)
 *   AC_f(n) = df/de_n = a2 e + a4 e^3 + a6 e^5 + 2 g e_n sum_{m!=n} e_m^2
 *                       - 2 th (c - c0) e_n
 *   CH_f(0) = df/dc   = A (c - c0) - th sum_n e_n^2
 *
 * Constants (landau_input.txt, one line):
 *   K(0..10) = a2 a4 a6 g th c0 A LE KE LCI KCI
 */
SCLET_MAX_NCH(1)
SCLET_C0_INDEX(5)
SCLET_DEFAULTS = {-1.0, -1.0, 2.0, 1.5, 0.8, 0.5, 1.0, 1.0, 6.0, 1.0, 2.0};

SCLET_INIT_KL {
  kl->LE = K(7);
  kl->KE = K(8);
  kl->LCI = K(9);
  kl->KCI = K(10);
}

SCLET_AC_F {
  real e = ac[n].u, e2 = e * e, others = 0, f;
  int m;
  for (m = 0; m < nac; m++)
    if (m != n) others += ac[m].u * ac[m].u;
  f = K(0) * e + K(1) * e2 * e + K(2) * e2 * e2 * e + 2 * K(3) * e * others;
  if (nch > 0) f -= 2 * K(4) * (ch[0].c - K(5)) * e;
  return f;
}

SCLET_CH_F {
  real s = 0;
  int m;
  (void)n;
  (void)nch;
  for (m = 0; m < nac; m++) s += ac[m].u * ac[m].u;
  return K(6) * (ch[0].c - K(5)) - K(4) * s;
}

SCLET_F_BULK {
  real f = 0, s = 0;
  int m, q;
  for (m = 0; m < nac; m++) {
    real u2 = ac[m].u * ac[m].u;
    s += u2;
    f += K(0) / 2 * u2 + K(1) / 4 * u2 * u2 + K(2) / 6 * u2 * u2 * u2;
    for (q = m + 1; q < nac; q++) f += K(3) * u2 * ac[q].u * ac[q].u;
  }
  if (nch > 0) {
    real d = ch[0].c - K(5);
    f += K(6) / 2 * d * d - K(4) * d * s;
  }
  return f;
}
