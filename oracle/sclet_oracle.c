/*
 * CPU restatement of the reference's ScLETD ETD step on one periodic rank.
 * TEST INFRASTRUCTURE ONLY (the reference results for tests, smoke() and the
 * CPU baseline); see sclet_oracle.h.  Citations are relative to the reference's
 * source_beta_to_omega/src/.
 */
#include "sclet_oracle.h"
#include "ref_shims/oracle_fft.h"

/* the physics plugins: the same sources the device kernels compile */
#include "../energy-stability_gb300/plugins/sclet_plugin.h"
#define SCLET_PLUGIN_NS(x) landau246_##x
#include "../energy-stability_gb300/plugins/landau246.h"
#undef SCLET_PLUGIN_NS
#define SCLET_PLUGIN_NS(x) formula234_##x
#include "../energy-stability_gb300/plugins/formula234.h"
#undef SCLET_PLUGIN_NS
#undef K
#undef real

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(n, z, y, x) (((size_t)(z) * (n) + (size_t)(y)) * (n) + (size_t)(x))

int orc_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Periodic image inside the owned range 2..n-3 (period N = n - 4). */
static inline int img(int n, int v) {
  int N = n - 4;
  int r = (v - 2) % N;
  if (r < 0) r += N;
  return 2 + r;
}

/* One-axis wrap used by the ghost exchange: ghosts 0,1 take cells N, N+1 and
 * ghosts n-2, n-1 take cells 2, 3. */
static inline int wrap1(int n, int v) {
  int N = n - 4;
  if (v < 2) return v + N;
  if (v >= n - 2) return v - N;
  return v;
}

/* transfer(), trans.c:1939-1996, with every neighbour the rank itself: the
 * front/back planes travel first, then top/bottom slabs, then left/right, all
 * packed from the block as it was before the exchange; unpack() (trans.c:
 * 154-251) writes left, right, top, bottom, front, back in that order, so a
 * ghost cell takes the value of its one-axis periodic image along the
 * highest-priority ghost axis (z over y over x), copied from the pre-exchange
 * block (whose own ghost cells there are the block's evolved values). */
void orc_ghost_fill(int n, double *f) {
  size_t n3 = (size_t)n * n * n;
  double *old = (double *)malloc(sizeof(double) * n3);
  int z;
  memcpy(old, f, sizeof(double) * n3);
#pragma omp parallel for
  for (z = 0; z < n; z++) {
    int y, x;
    int gz = (z < 2 || z >= n - 2);
    for (y = 0; y < n; y++) {
      int gy = (y < 2 || y >= n - 2);
      for (x = 0; x < n; x++) {
        int gx = (x < 2 || x >= n - 2);
        if (gz)
          f[IDX(n, z, y, x)] = old[IDX(n, wrap1(n, z), y, x)];
        else if (gy)
          f[IDX(n, z, y, x)] = old[IDX(n, z, wrap1(n, y), x)];
        else if (gx)
          f[IDX(n, z, y, x)] = old[IDX(n, z, y, wrap1(n, x))];
      }
    }
  }
  free(old);
}

/* fieldEu_* of ac_mu / ch_mu (trans.c:927-1937) via enlarge() (trans.c:
 * 253-925): the value at the cell just outside each face, i.e. the periodic
 * image of x = -1 / x = n (resp. y, z), for every in-face position. */
void orc_boundary_values(int n, const double *f, double *faces) {
  size_t nn = (size_t)n * n;
  int a, b;
  for (a = 0; a < n; a++) {
    for (b = 0; b < n; b++) {
      int wa = img(n, a), wb = img(n, b);
      faces[0 * nn + a * n + b] = f[IDX(n, wa, wb, img(n, -1))];
      faces[1 * nn + a * n + b] = f[IDX(n, wa, wb, img(n, n))];
      faces[2 * nn + a * n + b] = f[IDX(n, wa, img(n, -1), wb)];
      faces[3 * nn + a * n + b] = f[IDX(n, wa, img(n, n), wb)];
      faces[4 * nn + a * n + b] = f[IDX(n, img(n, -1), wa, wb)];
      faces[5 * nn + a * n + b] = f[IDX(n, img(n, n), wa, wb)];
    }
  }
}

/* ---------------------------------------------------------------------- */
/* Physics plugin of the run: AC_f / CH_f at one cell (formula.c:28-56, as  */
/* SWTICH_AC_FIELD1 / SWITCH_CH_FIELD1 load ac[m].u and ch[m].c,            */
/* ScLETD.h:108-135).                                                       */
/* ---------------------------------------------------------------------- */
static void load_cell(const orc_cfg *c, const double *e, double cval, sclet_acv *ac, sclet_chv *ch) {
  int k;
  for (k = 0; k < 4; k++) ac[k].u = k < c->nac ? e[k] : 0.0;
  ch[0].c = cval;
}

static double ac_f(const orc_cfg *c, const double *e, double cval, int m) {
  sclet_acv ac[4];
  sclet_chv ch[1];
  load_cell(c, e, cval, ac, ch);
  if (c->physics == 1) return formula234_AC_f(ac, ch, c->nac, c->nch, c->K, m);
  return landau246_AC_f(ac, ch, c->nac, c->nch, c->K, m);
}

static double ch_f(const orc_cfg *c, const double *e, double cval) {
  sclet_acv ac[4];
  sclet_chv ch[1];
  load_cell(c, e, cval, ac, ch);
  if (c->physics == 1) return formula234_CH_f(ac, ch, c->nac, c->nch, c->K, 0);
  return landau246_CH_f(ac, ch, c->nac, c->nch, c->K, 0);
}

static double f_bulk(const orc_cfg *c, const double *e, double cval) {
  sclet_acv ac[4];
  sclet_chv ch[1];
  load_cell(c, e, cval, ac, ch);
  if (c->physics == 1) return formula234_F_bulk(ac, ch, c->nac, c->nch, c->K);
  return landau246_F_bulk(ac, ch, c->nac, c->nch, c->K);
}

int orc_physics_setup(orc_cfg *c) {
  sclet_kl kl;
  if (c->physics == 0) landau246_init_KL(c->K, &kl);
  else if (c->physics == 1) formula234_init_KL(c->K, &kl);
  else return -1;
  c->LE = kl.LE;
  c->KE = kl.KE;
  c->LCI = kl.LCI;
  c->KCI = kl.KCI;
  return 0;
}

/* ---------------------------------------------------------------------- */
/* Elastic force                                                           */
/* ---------------------------------------------------------------------- */
static void inverse3(const double *a, double *out) {
  /* inverse_3x3, elastic.c:442-458 (cofactors over the determinant). */
  double det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
               a[2] * (a[3] * a[7] - a[4] * a[6]);
  out[0] = (a[4] * a[8] - a[5] * a[7]) / det;
  out[1] = -(a[3] * a[8] - a[6] * a[5]) / det;
  out[2] = (a[3] * a[7] - a[6] * a[4]) / det;
  out[3] = -(a[1] * a[8] - a[7] * a[2]) / det;
  out[4] = (a[0] * a[8] - a[2] * a[6]) / det;
  out[5] = -(a[0] * a[7] - a[6] * a[1]) / det;
  out[6] = (a[1] * a[5] - a[4] * a[2]) / det;
  out[7] = -(a[0] * a[5] - a[3] * a[2]) / det;
  out[8] = (a[0] * a[4] - a[1] * a[3]) / det;
}

static int voigt_index(int i, int j) {
  /* elastic_index_3to6, elastic.c:321-347: 11,22,33,23,13,12. */
  if (i == j) return i;
  if ((i == 1 && j == 2) || (i == 2 && j == 1)) return 3;
  if ((i == 0 && j == 2) || (i == 2 && j == 0)) return 4;
  return 5;
}

/* elastic_input (elastic.c:349-439) and elastic_calculate_BN (460-605):
 * B_pq(n) = C_ijkl e0p_ij e0q_kl - n_i s0p_ij Om_jk s0q_kl n_l with
 * Om = (C_ijkl n_j n_l)^-1, s0p = C : e0p, n = k/|k|, n = (0,1,0) at k = 0.
 * Wave numbers follow the FFT order: 0..N/2-1, then -N/2..-1. */
void orc_compute_bn(int big_n, const double *voigt, const double *eps, double *out) {
  double C[81], sig[4][9];
  int i, j, k, l, p, z;
  size_t N3 = (size_t)big_n * big_n * big_n;
  for (i = 0; i < 3; i++)
    for (j = 0; j < 3; j++)
      for (k = 0; k < 3; k++)
        for (l = 0; l < 3; l++) C[((i * 3 + j) * 3 + k) * 3 + l] = voigt[voigt_index(i, j) * 6 + voigt_index(k, l)];
  for (p = 0; p < 4; p++)
    for (i = 0; i < 3; i++)
      for (j = 0; j < 3; j++) {
        double s = 0.0;
        for (k = 0; k < 3; k++)
          for (l = 0; l < 3; l++) s += C[((i * 3 + j) * 3 + k) * 3 + l] * eps[p * 9 + k * 3 + l];
        sig[p][i * 3 + j] = s;
      }
#pragma omp parallel for
  for (z = 0; z < big_n; z++) {
    int y, x, pp, qq, a, b, cc, d;
    for (y = 0; y < big_n; y++) {
      for (x = 0; x < big_n; x++) {
        double nv[3], om_inv[9], om[9];
        double kx = x < big_n / 2 ? x : -(double)(big_n - x);
        double ky = y < big_n / 2 ? y : -(double)(big_n - y);
        double kz = z < big_n / 2 ? z : -(double)(big_n - z);
        if (x == 0 && y == 0 && z == 0) {
          nv[0] = 0.0;
          nv[1] = 1.0;
          nv[2] = 0.0;
        } else {
          double r = sqrt(kx * kx + ky * ky + kz * kz);
          nv[0] = kx / r;
          nv[1] = ky / r;
          nv[2] = kz / r;
        }
        for (a = 0; a < 3; a++)
          for (cc = 0; cc < 3; cc++) {
            double s = 0.0;
            for (b = 0; b < 3; b++)
              for (d = 0; d < 3; d++) s += C[((a * 3 + b) * 3 + cc) * 3 + d] * nv[b] * nv[d];
            om_inv[a * 3 + cc] = s;
          }
        inverse3(om_inv, om);
        for (pp = 0; pp < 4; pp++)
          for (qq = 0; qq < 4; qq++) {
            double t0 = 0.0, t1 = 0.0;
            for (a = 0; a < 3; a++)
              for (b = 0; b < 3; b++)
                for (cc = 0; cc < 3; cc++)
                  for (d = 0; d < 3; d++) {
                    t0 += C[((a * 3 + b) * 3 + cc) * 3 + d] * eps[pp * 9 + a * 3 + b] * eps[qq * 9 + cc * 3 + d];
                    t1 += nv[a] * sig[pp][a * 3 + b] * om[b * 3 + cc] * sig[qq][cc * 3 + d] * nv[d];
                  }
            out[(size_t)(pp * 4 + qq) * N3 + ((size_t)z * big_n + y) * big_n + x] = t0 - t1;
          }
      }
    }
  }
}

/* elastic_calculate (elastic.c:689-763) with ELASTIC == AC_FUNCTION and
 * elastic_calculate_ElasDri (617-687): for each p, sum over q of
 * IFFT(B_pq * FFT(eta_q)) on the N^3 interior, written into the shared
 * scratch block whose ghost cells are then exchanged like a field. */
void orc_elastic(const orc_cfg *c, const double *eta, double *felas, double *fstate) {
  int n = c->n, N = n - 4, p, q;
  size_t n3 = (size_t)n * n * n, N3 = (size_t)N * N * N, m;
  double *spec = (double *)malloc(sizeof(double) * 2 * N3);
  double *acc = (double *)malloc(sizeof(double) * N3);
  for (p = 0; p < c->nac; p++) {
    int z;
    memset(acc, 0, sizeof(double) * N3);
    for (q = 0; q < 4; q++) {
      /* fields beyond nac are zero (the reference's zero-filled tmpy_re). */
      for (z = 0; z < N; z++) {
        int y, x;
        for (y = 0; y < N; y++)
          for (x = 0; x < N; x++) {
            size_t g = ((size_t)z * N + y) * N + x;
            spec[2 * g] = q < c->nac ? eta[(size_t)q * n3 + IDX(n, z + 2, y + 2, x + 2)] : 0.0;
            spec[2 * g + 1] = 0.0;
          }
      }
      oracle_fft3d(spec, N, N, N, -1);
      for (m = 0; m < N3; m++) {
        double b = c->bn[(size_t)(p * 4 + q) * N3 + m];
        spec[2 * m] *= b;
        spec[2 * m + 1] *= b;
      }
      oracle_fft3d(spec, N, N, N, +1);
      for (m = 0; m < N3; m++) acc[m] += spec[2 * m] * (1.0 / (double)N3);
    }
    for (z = 0; z < N; z++) {
      int y, x;
      for (y = 0; y < N; y++)
        for (x = 0; x < N; x++) fstate[IDX(n, z + 2, y + 2, x + 2)] = acc[((size_t)z * N + y) * N + x];
    }
    orc_ghost_fill(n, fstate);
    memcpy(felas + (size_t)p * n3, fstate, sizeof(double) * n3);
  }
  free(spec);
  free(acc);
}

/* ---------------------------------------------------------------------- */
/* Right-hand sides                                                        */
/* ---------------------------------------------------------------------- */
/* ac_calc_F2, anisotropic.c:164-628: grad = lambda . (central differences),
 * then its central divergence, with every value outside the block taken as
 * zero; y and z differences are (previous - next) as the reference writes. */
static void ac_f2(const orc_cfg *c, int m, const double *u, double *f2, double *g) {
  int n = c->n, z;
  size_t n3 = (size_t)n * n * n;
  double hx = c->h[0], hy = c->h[1], hz = c->h[2];
  const double(*L)[3] = c->lam[m];
#pragma omp parallel for
  for (z = 0; z < n; z++) {
    int y, x;
    for (y = 0; y < n; y++)
      for (x = 0; x < n; x++) {
        double al = x > 0 ? u[IDX(n, z, y, x - 1)] : 0.0, ar = x < n - 1 ? u[IDX(n, z, y, x + 1)] : 0.0;
        double at = y > 0 ? u[IDX(n, z, y - 1, x)] : 0.0, ab = y < n - 1 ? u[IDX(n, z, y + 1, x)] : 0.0;
        double af = z > 0 ? u[IDX(n, z - 1, y, x)] : 0.0, ak = z < n - 1 ? u[IDX(n, z + 1, y, x)] : 0.0;
        double gx = (ar - al) / (2.0 * hx), gy = (at - ab) / (2.0 * hy), gz = (af - ak) / (2.0 * hz);
        size_t l = IDX(n, z, y, x);
        g[l] = L[0][0] * gx + L[0][1] * gy + L[0][2] * gz;
        g[n3 + l] = L[1][0] * gx + L[1][1] * gy + L[1][2] * gz;
        g[2 * n3 + l] = L[2][0] * gx + L[2][1] * gy + L[2][2] * gz;
      }
  }
#pragma omp parallel for
  for (z = 0; z < n; z++) {
    int y, x;
    for (y = 0; y < n; y++)
      for (x = 0; x < n; x++) {
        double al = x > 0 ? g[IDX(n, z, y, x - 1)] : 0.0, ar = x < n - 1 ? g[IDX(n, z, y, x + 1)] : 0.0;
        double at = y > 0 ? g[n3 + IDX(n, z, y - 1, x)] : 0.0, ab = y < n - 1 ? g[n3 + IDX(n, z, y + 1, x)] : 0.0;
        double af = z > 0 ? g[2 * n3 + IDX(n, z - 1, y, x)] : 0.0;
        double ak = z < n - 1 ? g[2 * n3 + IDX(n, z + 1, y, x)] : 0.0;
        double t = 0.0;
        t += (ar - al) / 2.0 / hx;
        t += (at - ab) / 2.0 / hy;
        t += (af - ak) / 2.0 / hz;
        f2[IDX(n, z, y, x)] = t;
      }
  }
}

/* Adds v / h^2 * w to the cells of each block face, faces in the order
 * left, right, top, bottom, front, back (the loops of anisotropic.c:88-158
 * and calc.c:104-174, 402-472). */
static void add_faces(int n, double *f, const double *faces, double w, const double *h) {
  size_t nn = (size_t)n * n;
  int a, b;
  for (a = 0; a < n; a++)
    for (b = 0; b < n; b++) f[IDX(n, a, b, 0)] += w * faces[0 * nn + a * n + b] / h[0] / h[0];
  for (a = 0; a < n; a++)
    for (b = 0; b < n; b++) f[IDX(n, a, b, n - 1)] += w * faces[1 * nn + a * n + b] / h[0] / h[0];
  for (a = 0; a < n; a++)
    for (b = 0; b < n; b++) f[IDX(n, a, 0, b)] += w * faces[2 * nn + a * n + b] / h[1] / h[1];
  for (a = 0; a < n; a++)
    for (b = 0; b < n; b++) f[IDX(n, a, n - 1, b)] += w * faces[3 * nn + a * n + b] / h[1] / h[1];
  for (a = 0; a < n; a++)
    for (b = 0; b < n; b++) f[IDX(n, 0, a, b)] += w * faces[4 * nn + a * n + b] / h[2] / h[2];
  for (a = 0; a < n; a++)
    for (b = 0; b < n; b++) f[IDX(n, n - 1, a, b)] += w * faces[5 * nn + a * n + b] / h[2] / h[2];
}

/* ch_mu (trans.c:1433-1937) with every neighbour present: at the periodic
 * image P of the cell just outside each face,
 * mu = LCI * (epn2 * lap(c)(P) - CH_f(fields at P)), the 7-point Laplacian
 * summed x, y, z in that order over periodic images. */
static void ch_boundary_mu(const orc_cfg *c, const double *u, double *mu) {
  int n = c->n, a, b, face, m;
  size_t n3 = (size_t)n * n * n, nn = (size_t)n * n;
  const double *cc = u + (size_t)c->nac * n3;
  for (face = 0; face < 6; face++)
    for (a = 0; a < n; a++)
      for (b = 0; b < n; b++) {
        int z, y, x;
        double e[4], lap, cv;
        int outside = (face % 2 == 0) ? -1 : n;
        if (face < 2) {
          z = img(n, a); y = img(n, b); x = img(n, outside);
        } else if (face < 4) {
          z = img(n, a); y = img(n, outside); x = img(n, b);
        } else {
          z = img(n, outside); y = img(n, a); x = img(n, b);
        }
        cv = cc[IDX(n, z, y, x)];
        lap = (cc[IDX(n, z, y, img(n, x - 1))] + (-2.0) * cv + cc[IDX(n, z, y, img(n, x + 1))]) / c->h[0] / c->h[0];
        lap += (cc[IDX(n, z, img(n, y - 1), x)] + (-2.0) * cv + cc[IDX(n, z, img(n, y + 1), x)]) / c->h[1] / c->h[1];
        lap += (cc[IDX(n, img(n, z - 1), y, x)] + (-2.0) * cv + cc[IDX(n, img(n, z + 1), y, x)]) / c->h[2] / c->h[2];
        for (m = 0; m < c->nac; m++) e[m] = u[(size_t)m * n3 + IDX(n, z, y, x)];
        lap = c->LCI * c->epn2 * lap;
        lap -= c->LCI * ch_f(c, e, cv);
        mu[face * nn + a * n + b] = lap;
      }
}

/* update_M_C (mobility.c:860-922): the mobility of the first concentration
 * (Cu) from the first order parameter, M = cu0 (1 - cu0) (DA (1 - eta0) +
 * DG eta0), with DA = 1 and DG the ratio of the two phases' Arrhenius
 * diffusivities D0 exp(-Q / RT) at T = 823 K (R = 8.314472). */
void orc_mobility_constants(double *m0, double *dg) {
  const double rt = 8.314472 * 823.0, cu0 = 0.15;
  const double da = 4.7e-5 * exp(-2.44e5 / rt);
  *dg = (4.3e-5 * exp(-2.80e5 / rt)) / da;
  *m0 = cu0 * (1.0 - cu0);
}

/* laplace (mobility.c:12-239) on a periodic single rank: the 7-point
 * Laplacian with values outside the block taken as zero. */
static void lap_zero_outside(const orc_cfg *c, const double *a, double *la) {
  int n = c->n, z;
  size_t nn = (size_t)n * n;
#pragma omp parallel for
  for (z = 0; z < n; z++) {
    int y, x;
    for (y = 0; y < n; y++)
      for (x = 0; x < n; x++) {
        size_t l = IDX(n, z, y, x);
        double al = x > 0 ? a[l - 1] : 0.0, ar = x < n - 1 ? a[l + 1] : 0.0;
        double at = y > 0 ? a[l - n] : 0.0, ab = y < n - 1 ? a[l + n] : 0.0;
        double af = z > 0 ? a[l - nn] : 0.0, ak = z < n - 1 ? a[l + nn] : 0.0;
        double tmp = 0.0;
        tmp += (al + ar - 2.0 * a[l]) / c->h[0] / c->h[0];
        tmp += (at + ab - 2.0 * a[l]) / c->h[1] / c->h[1];
        tmp += (af + ak - 2.0 * a[l]) / c->h[2] / c->h[2];
        la[l] = tmp;
      }
  }
}

/* ch_calc_FU_VariableMobility (mobility.c:838-858) of the single conserved
 * field with update_M_C run first (calc.c:475-481):
 *   f0 = -LCI KCI c + LCI CH_f                       (ch_calc_F0, SWITCH_CH_FIELD1)
 *   f1 = -C lap0(-f0 + KCI c + epn2 c_out / h^2) - C mu_out / h^2   (ch_calc_F1)
 *   f2 = -div0((M - C) grad(epn2 lap0(c) - f0 + epn2 c_out / h^2))  (ch_calc_F2)
 *   N  = LCI (f1 + f2)
 * with C the largest M over the block (update_M_C), lap0 and div0 zero
 * outside the block (ch_divergence_M_gradient, mobility.c:435-722: the
 * face flux (m_q + m) (a_q - a) / (2 h^2), m_q = a_q = 0 outside), c_out
 * the periodic image outside each face and mu_out the boundary chemical
 * potential there (ch_mu). */
static void ch_rhs_variable_mobility(const orc_cfg *c, const double *u, double *f, double *faces, double *tmp) {
  int n = c->n, z;
  size_t n3 = (size_t)n * n * n, nn = (size_t)n * n, l;
  const double *cm = u + (size_t)c->nac * n3, *e0 = u;
  double *M = tmp, *f0 = tmp + n3, *t = tmp + 2 * n3, *g = tmp + 3 * n3;
  double m0, dg, C = -1.0e30;
  orc_mobility_constants(&m0, &dg);
  for (l = 0; l < n3; l++) {
    M[l] = m0 * (1.0 * (1.0 - e0[l]) + dg * e0[l]);
    C = C > M[l] ? C : M[l];
  }
#pragma omp parallel for
  for (z = 0; z < n; z++) {
    int y, x, k;
    for (y = 0; y < n; y++)
      for (x = 0; x < n; x++) {
        double e[4];
        size_t q = IDX(n, z, y, x);
        for (k = 0; k < c->nac; k++) e[k] = u[(size_t)k * n3 + q];
        f0[q] = -c->LCI * c->KCI * cm[q];
        f0[q] += c->LCI * ch_f(c, e, cm[q]);
      }
  }
  orc_boundary_values(n, cm, faces);
  /* f1 */
  for (l = 0; l < n3; l++) t[l] = -f0[l] + c->KCI * cm[l];
  add_faces(n, t, faces, c->epn2, c->h);
  lap_zero_outside(c, t, f);
  for (l = 0; l < n3; l++) f[l] = -C * f[l];
  ch_boundary_mu(c, u, g);
  add_faces(n, f, g, -C, c->h);
  /* f2 */
  lap_zero_outside(c, cm, t);
  for (l = 0; l < n3; l++) t[l] = c->epn2 * t[l] - f0[l];
  add_faces(n, t, faces, c->epn2, c->h);
  for (l = 0; l < n3; l++) M[l] = M[l] - C;
#pragma omp parallel for
  for (z = 0; z < n; z++) {
    int y, x;
    for (y = 0; y < n; y++)
      for (x = 0; x < n; x++) {
        size_t q = IDX(n, z, y, x);
        const double am = t[q], mm = M[q];
        const double al = x > 0 ? t[q - 1] : 0.0, ml = x > 0 ? M[q - 1] : 0.0;
        const double ar = x < n - 1 ? t[q + 1] : 0.0, mr = x < n - 1 ? M[q + 1] : 0.0;
        const double at = y > 0 ? t[q - n] : 0.0, mt = y > 0 ? M[q - n] : 0.0;
        const double ab = y < n - 1 ? t[q + n] : 0.0, mb = y < n - 1 ? M[q + n] : 0.0;
        const double af = z > 0 ? t[q - nn] : 0.0, mf = z > 0 ? M[q - nn] : 0.0;
        const double ak = z < n - 1 ? t[q + nn] : 0.0, mk = z < n - 1 ? M[q + nn] : 0.0;
        double d = 0.0;
        d += (ml + mm) * (al - am) / 2.0 / c->h[0] / c->h[0];
        d += (mr + mm) * (ar - am) / 2.0 / c->h[0] / c->h[0];
        d += (mt + mm) * (at - am) / 2.0 / c->h[1] / c->h[1];
        d += (mb + mm) * (ab - am) / 2.0 / c->h[1] / c->h[1];
        d += (mf + mm) * (af - am) / 2.0 / c->h[2] / c->h[2];
        d += (mk + mm) * (ak - am) / 2.0 / c->h[2] / c->h[2];
        g[q] = -d;
      }
  }
  for (l = 0; l < n3; l++) f[l] = c->LCI * (f[l] + g[l]);
}

void orc_rhs(const orc_cfg *c, const double *u, const double *felas, double *out) {
  int n = c->n, m, z;
  size_t n3 = (size_t)n * n * n, nn = (size_t)n * n;
  double *faces = (double *)malloc(sizeof(double) * 6 * nn);
  double *tmp = (double *)malloc(sizeof(double) * n3 * 4);
  /* ac_calc_FU (calc.c:8-68) -> ac_calc_F1 (anisotropic.c:9-161). */
  for (m = 0; m < c->nac; m++) {
    const double *um = u + (size_t)m * n3;
    double *f = out + (size_t)m * n3;
#pragma omp parallel for
    for (z = 0; z < n; z++) {
      int y, x, k;
      for (y = 0; y < n; y++)
        for (x = 0; x < n; x++) {
          double e[4], cv = 0.0, v;
          size_t l = IDX(n, z, y, x);
          for (k = 0; k < c->nac; k++) e[k] = u[(size_t)k * n3 + l];
          if (c->nch > 0) cv = u[(size_t)c->nac * n3 + l];
          v = c->LE * c->KE * um[l];
          v -= c->LE * ac_f(c, e, cv, m);
          f[l] = v;
        }
    }
    orc_boundary_values(n, um, faces);
    add_faces(n, f, faces, c->LE * c->epn2, c->h);
    if (c->anisotropic) {
      size_t l;
      ac_f2(c, m, um, tmp, tmp + n3);
      for (l = 0; l < n3; l++) f[l] -= c->epn2 * c->LE * tmp[l];
    }
    if (c->elastic == 1) {
      size_t l;
      for (l = 0; l < n3; l++) f[l] -= c->LE * c->elastic_scale * felas[(size_t)m * n3 + l];
    }
  }
  if (c->variable_mobility && c->nch > 0) ch_rhs_variable_mobility(c, u, out + (size_t)c->nac * n3, faces, tmp);
  /* ch_calc_FU_ConstantMobility (calc.c:70-473). */
  for (m = 0; m < (c->variable_mobility ? 0 : c->nch); m++) {
    const double *cm = u + (size_t)(c->nac + m) * n3;
    double *f = out + (size_t)(c->nac + m) * n3;
    double *t = tmp;
    double *mu = tmp + n3;
#pragma omp parallel for
    for (z = 0; z < n; z++) {
      int y, x, k;
      for (y = 0; y < n; y++)
        for (x = 0; x < n; x++) {
          double e[4], v;
          size_t l = IDX(n, z, y, x);
          for (k = 0; k < c->nac; k++) e[k] = u[(size_t)k * n3 + l];
          v = -c->LCI * c->KCI * cm[l];
          v += c->LCI * ch_f(c, e, cm[l]);
          t[l] = v;
        }
    }
    orc_boundary_values(n, cm, faces);
    add_faces(n, t, faces, -c->LCI * c->epn2, c->h);
#pragma omp parallel for
    for (z = 0; z < n; z++) {
      int y, x;
      for (y = 0; y < n; y++)
        for (x = 0; x < n; x++) {
          size_t l = IDX(n, z, y, x);
          double fl = x > 0 ? t[l - 1] : 0.0, fr = x < n - 1 ? t[l + 1] : 0.0;
          double ft = y > 0 ? t[l - n] : 0.0, fb = y < n - 1 ? t[l + n] : 0.0;
          double ff = z > 0 ? t[l - nn] : 0.0, fk = z < n - 1 ? t[l + nn] : 0.0;
          double v = (fl + fr - 2.0 * t[l]) / c->h[0] / c->h[0];
          v += (ft + fb - 2.0 * t[l]) / c->h[1] / c->h[1];
          v += (ff + fk - 2.0 * t[l]) / c->h[2] / c->h[2];
          f[l] = v;
        }
    }
    ch_boundary_mu(c, u, mu);
    add_faces(n, f, mu, -1.0, c->h);
  }
  free(faces);
  free(tmp);
}

/* ---------------------------------------------------------------------- */
/* Eigenbasis transforms and the ETD update                                */
/* ---------------------------------------------------------------------- */
void orc_mode_product(int n, const double *mat, const double *in, double *out) {
  int c;
  size_t nn = (size_t)n * n;
#pragma omp parallel for
  for (c = 0; c < n; c++) {
    int b, a, ap;
    double col[1024];
    for (b = 0; b < n; b++) {
      const double *src = in + (size_t)c * nn + (size_t)b * n;
      for (ap = 0; ap < n; ap++) col[ap] = 0.0;
      for (a = 0; a < n; a++) {
        double s = src[a];
        const double *mc = mat + (size_t)a * n;
        for (ap = 0; ap < n; ap++) col[ap] += mc[ap] * s;
      }
      for (ap = 0; ap < n; ap++) out[(size_t)ap * nn + (size_t)c * n + b] = col[ap];
    }
  }
}

/* V^-1 along x, y, z (PUX/PUY/PUZ with MP*I, calc.c:631-684): three rotating
 * products return to x-fastest order, indices now eigen-modes. */
static void to_eigen(const orc_cfg *c, double *a, double *tmp) {
  orc_mode_product(c->n, c->mpi[0], a, tmp);
  orc_mode_product(c->n, c->mpi[1], tmp, a);
  orc_mode_product(c->n, c->mpi[2], a, tmp);
  memcpy(a, tmp, sizeof(double) * (size_t)c->n * c->n * c->n);
}

static void from_eigen(const orc_cfg *c, double *a, double *tmp) {
  orc_mode_product(c->n, c->mp[0], a, tmp);
  orc_mode_product(c->n, c->mp[1], tmp, a);
  orc_mode_product(c->n, c->mp[2], a, tmp);
  memcpy(a, tmp, sizeof(double) * (size_t)c->n * c->n * c->n);
}

/* H of the linear operator at eigen-mode (i, j, k): ac_updateU_new /
 * ch_updateU_new (calc.c:489-535); phi1, phi2: ac_init_phi / ch_init_phi
 * (vars.c:302-359). */
static void etd_coeffs(const orc_cfg *c, int is_ch, int i, int j, int k, double *H, double *phi1, double *phi2) {
  double tmp, h;
  if (!is_ch) {
    tmp = c->kk[2] * c->dd[2][k] + c->kk[1] * c->dd[1][j] + c->kk[0] * c->dd[0][i];
    h = -c->LE * (tmp * c->epn2 - c->KE);
  } else {
    tmp = c->dd[2][k] + c->dd[1][j] + c->dd[0][i];
    h = c->LCI * (tmp * tmp * c->epn2 - c->KCI * tmp);
  }
  if (fabs(h) > 1.0e-8) {
    double e = exp(-c->dt * h);
    *phi1 = (1.0 - e) / h;
    *phi2 = (1.0 - *phi1 / c->dt) / h;
  } else {
    *phi1 = c->dt;
    *phi2 = c->dt / 2;
  }
  *H = fabs(h) < 1.0e-8 ? 0.0 : h;
}

/* One time-loop pass (ScLETD.c:86-190).  The reference's check_soln_new at
 * the top of the loop only reports; it is orc_check_soln here. */
void orc_step(const orc_cfg *c, double *u, double *felas, double *fstate) {
  int n = c->n, F = c->nac + c->nch, m;
  size_t n3 = (size_t)n * n * n;
  double *N1 = (double *)malloc(sizeof(double) * n3 * F);
  double *N2 = c->etd2 ? (double *)malloc(sizeof(double) * n3 * F) : NULL;
  double *tmp = (double *)malloc(sizeof(double) * n3);
  double *b = (double *)malloc(sizeof(double) * n3);
  int pass;
  for (pass = 0; pass < (c->etd2 ? 2 : 1); pass++) {
    double *R = pass == 0 ? N1 : N2;
    for (m = 0; m < F; m++) orc_ghost_fill(n, u + (size_t)m * n3);
    if (c->elastic == 1) orc_elastic(c, u, felas, fstate);
    orc_rhs(c, u, felas, R);
    for (m = 0; m < F; m++) {
      double *um = u + (size_t)m * n3;
      int is_ch = m >= c->nac, k;
      if (pass == 0) {
        /* u <- V [(1 - phi1 H) V^-1 u + phi1 V^-1 N1] */
        memcpy(b, N1 + (size_t)m * n3, sizeof(double) * n3);
        to_eigen(c, um, tmp);
        to_eigen(c, b, tmp);
#pragma omp parallel for
        for (k = 0; k < n; k++) {
          int j, i;
          for (j = 0; j < n; j++)
            for (i = 0; i < n; i++) {
              double H, p1, p2;
              size_t l = IDX(n, k, j, i);
              etd_coeffs(c, is_ch, i, j, k, &H, &p1, &p2);
              um[l] = (1.0 - p1 * H) * um[l] + p1 * b[l];
            }
        }
        from_eigen(c, um, tmp);
      } else {
        /* ETD2 corrector: u += V phi2 V^-1 (N2 - N1) (prepare_U1_new,
         * prepare_U2_new, correct_U_new: calc.c:537-583). */
        size_t l;
        for (l = 0; l < n3; l++) b[l] = N2[(size_t)m * n3 + l] - N1[(size_t)m * n3 + l];
        to_eigen(c, b, tmp);
#pragma omp parallel for
        for (k = 0; k < n; k++) {
          int j, i;
          for (j = 0; j < n; j++)
            for (i = 0; i < n; i++) {
              double H, p1, p2;
              size_t ll = IDX(n, k, j, i);
              etd_coeffs(c, is_ch, i, j, k, &H, &p1, &p2);
              b[ll] = p2 * b[ll];
            }
        }
        from_eigen(c, b, tmp);
        for (l = 0; l < n3; l++) um[l] += b[l];
      }
    }
  }
  free(N1);
  free(N2);
  free(tmp);
  free(b);
}

/* ---------------------------------------------------------------------- */
/* Diagnostics                                                             */
/* ---------------------------------------------------------------------- */
static double landau_energy(const orc_cfg *c, const double *e, double cv) {
  if (c->energy_form == 0) {
    /* the reference's hard-coded polynomial, field.c:508 (four fields) */
    double s2 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2] + e[3] * e[3];
    double s3 = e[0] * e[0] * e[0] + e[1] * e[1] * e[1] + e[2] * e[2] * e[2] + e[3] * e[3] * e[3];
    return (2376.0 / 2372.0 / 2.0) * s2 - ((7128.0 + 12.0 * 2372.0) / 2372.0 / 3.0) * s3 +
           ((4752.0 + 12.0 * 2372.0) / 2372.0 / 4.0) * s2 * s2;
  }
  return f_bulk(c, e, cv);
}

/* check_soln_new, field.c:407-678.  Per field: max, min, vol = sum(u + 1) h^3
 * over owned cells, and the energy over the owned cells' corner cubes:
 * 8-corner average and corner-difference gradients, gradient energy
 * epn2/2 grad.lambda.grad of every AC field (plus epn2/2 |grad c|^2 of the CH
 * field when energy_form == 1) and the Landau energy of the averages. */
void orc_check_soln(const orc_cfg *c, const double *u, double *out) {
  int n = c->n, F = c->nac + c->nch, m;
  size_t n3 = (size_t)n * n * n;
  double hx = c->h[0], hy = c->h[1], hz = c->h[2];
  double eng_ac = 0.0, eng_ch = 0.0;
  int k, j, i, q;
  for (m = 0; m < F; m++) {
    const double *f = u + (size_t)m * n3;
    double mx = -1.0e30, mn = 1.0e30, vol = 0.0;
    for (k = 2; k < n - 2; k++)
      for (j = 2; j < n - 2; j++)
        for (i = 2; i < n - 2; i++) {
          double t = f[IDX(n, k, j, i)];
          if (t > mx) mx = t;
          if (t < mn) mn = t;
          vol += t + 1.0;
        }
    out[m * 4 + 0] = mx;
    out[m * 4 + 1] = mn;
    out[m * 4 + 2] = vol * hx * hy * hz;
  }
  for (k = 2; k < n - 3; k++)
    for (j = 2; j < n - 3; j++)
      for (i = 2; i < n - 3; i++) {
        double avg[5] = {0, 0, 0, 0, 0}, cbar = 0.0;
        for (q = 0; q < F; q++) {
          const double *f = u + (size_t)q * n3;
          double v[8], ux, uy, uz;
          v[0] = f[IDX(n, k, j, i)];
          v[1] = f[IDX(n, k, j, i + 1)];
          v[2] = f[IDX(n, k, j + 1, i)];
          v[3] = f[IDX(n, k, j + 1, i + 1)];
          v[4] = f[IDX(n, k + 1, j, i)];
          v[5] = f[IDX(n, k + 1, j, i + 1)];
          v[6] = f[IDX(n, k + 1, j + 1, i)];
          v[7] = f[IDX(n, k + 1, j + 1, i + 1)];
          avg[q] = (v[0] + v[1] + v[2] + v[3] + v[4] + v[5] + v[6] + v[7]) / 8;
          ux = ((v[1] - v[0]) + (v[3] - v[2]) + (v[5] - v[4]) + (v[7] - v[6])) / 4 / hx;
          uy = ((v[2] - v[0]) + (v[3] - v[1]) + (v[6] - v[4]) + (v[7] - v[5])) / 4 / hy;
          uz = ((v[4] - v[0]) + (v[5] - v[1]) + (v[6] - v[2]) + (v[7] - v[3])) / 4 / hz;
          if (q < c->nac) {
            const double(*L)[3] = c->elam[q];
            double fx = ux * L[0][0] + uy * L[1][0] + uz * L[2][0];
            double fy = ux * L[0][1] + uy * L[1][1] + uz * L[2][1];
            double fz = ux * L[0][2] + uy * L[1][2] + uz * L[2][2];
            eng_ac += c->epn2 * (fx * ux + fy * uy + fz * uz) / 2;
          } else {
            double g = c->epn2 * (ux * ux + uy * uy + uz * uz) / 2;
            if (c->energy_form == 0) eng_ch += g; else eng_ac += g;
            cbar = avg[q];
          }
        }
        if (c->nac > 0 || c->energy_form == 1) eng_ac += landau_energy(c, avg, cbar);
        if (c->nch > 0 && c->energy_form == 0) eng_ch += (cbar * cbar - 1) * (cbar * cbar - 1) / 4;
      }
  for (m = 0; m < F; m++) {
    double e = (c->energy_form == 0 && m >= c->nac) ? eng_ch : eng_ac;
    out[m * 4 + 3] = e * hx * hy * hz;
  }
}
