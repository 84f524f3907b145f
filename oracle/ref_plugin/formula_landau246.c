/*
 * Physics plugin for the reference's extension point (the four functions of
 * source_beta_to_omega/src/formula.c:9-56, read through the globals that the
 * macros SWTICH_AC_FIELD1 / SWITCH_CH_FIELD1 / SWITCH_CH_FIELDMU set,
 * src/ScLETD.h:108-158).  Compiled in place of the reference's formula.c when
 * the reference is built into the test oracle (oracle/_ref).  Test
 * infrastructure.
 *
 * Free energy density (Landau 2-4-6 with a cross term and a c-eta coupling):
 *   f = sum_n [a2/2 e_n^2 + a4/4 e_n^4 + a6/6 e_n^6] + g sum_{m<n} e_m^2 e_n^2
 *       + A/2 (c - c0)^2 - th (c - c0) sum_n e_n^2          (CH part if nch > 0)
 *   AC_f(n) = df/de_n = a2 e + a4 e^3 + a6 e^5 + 2 g e_n sum_{m!=n} e_m^2
 *             - 2 th (c - c0) e_n
 *   CH_f(0) = df/dc   = A (c - c0) - th sum_n e_n^2
 * Linear-operator constants: LE, KE (AC), LCI, KCI (CH).
 *
 * Parameters come from "landau_input.txt" in the working directory when it
 * exists (one line: a2 a4 a6 g th c0 A LE KE LCI KCI), else the defaults below.
 */
#include <stdio.h>
#include <stdlib.h>
#include "mpi.h"
#include "ScLETD.h"

double sclet_a2 = -1.0, sclet_a4 = -1.0, sclet_a6 = 2.0, sclet_g = 1.5;
double sclet_th = 0.8, sclet_c0 = 0.5, sclet_A = 1.0;
double sclet_LE = 1.0, sclet_KE = 6.0, sclet_LCI = 1.0, sclet_KCI = 2.0;

void init_KL()
{
  int n;
  FILE *fp = fopen("landau_input.txt", "r");
  if (fp) {
    if (fscanf(fp, "%lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf", &sclet_a2, &sclet_a4, &sclet_a6, &sclet_g,
               &sclet_th, &sclet_c0, &sclet_A, &sclet_LE, &sclet_KE, &sclet_LCI, &sclet_KCI) != 11) {
      printf("landau_input.txt: expected 11 numbers\n");
      exit(1);
    }
    fclose(fp);
  }
  for (n = 0; n < nac; n++) {
    ac[n].LE = sclet_LE;
    ac[n].KE = sclet_KE;
  }
  for (n = 0; n < nch; n++) {
    ch[n].LCI = sclet_LCI;
    ch[n].KCI = sclet_KCI;
  }
}

double EF()
{
  return 0;
}

double AC_f(int n)
{
  int m;
  double e = ac[n].u, e2 = e * e, others = 0.0, f;
  for (m = 0; m < nac; m++)
    if (m != n) others += ac[m].u * ac[m].u;
  f = sclet_a2 * e + sclet_a4 * e2 * e + sclet_a6 * e2 * e2 * e + 2.0 * sclet_g * e * others;
  if (nch > 0) f -= 2.0 * sclet_th * (ch[0].c - sclet_c0) * e;
  return f;
}

double CH_f(int n)
{
  int m;
  double s = 0.0;
  if (n != 0) {
    printf("error:please choose correct CH_FIELD function.\n");
    exit(1);
  }
  for (m = 0; m < nac; m++) s += ac[m].u * ac[m].u;
  return sclet_A * (ch[0].c - sclet_c0) - sclet_th * s;
}
