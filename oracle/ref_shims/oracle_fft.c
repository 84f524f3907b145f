/* Mixed-radix complex DFT for the test oracle; see oracle_fft.h. */
#include "oracle_fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static int smallest_factor(int n) {
  int p;
  if (n % 2 == 0) return 2;
  for (p = 3; p * p <= n; p += 2)
    if (n % p == 0) return p;
  return n;
}

/* out[0..n) = DFT of in[0], in[s], in[2s], ...; w = table of exp(sign 2 pi i j / ntab),
 * wstep = ntab / n. */
static void fft_rec(const double *in, ptrdiff_t s, double *out, int n, const double *w, int wstep, int ntab) {
  int p, m, r, k, q;
  if (n == 1) {
    out[0] = in[0];
    out[1] = in[1];
    return;
  }
  p = smallest_factor(n);
  m = n / p;
  for (r = 0; r < p; r++) fft_rec(in + 2 * r * s, s * p, out + 2 * r * m, m, w, wstep * p, ntab);
  {
    double *tmp = (double *)malloc(sizeof(double) * 2 * n);
    for (k = 0; k < m; k++) {
      for (q = 0; q < p; q++) {
        double re = 0.0, im = 0.0;
        int kk = k + q * m;
        for (r = 0; r < p; r++) {
          long e = ((long)r * kk) % n;
          double wr = w[2 * (e * wstep % ntab)], wi = w[2 * (e * wstep % ntab) + 1];
          double xr = out[2 * (r * m + k)], xi = out[2 * (r * m + k) + 1];
          re += xr * wr - xi * wi;
          im += xr * wi + xi * wr;
        }
        tmp[2 * kk] = re;
        tmp[2 * kk + 1] = im;
      }
    }
    memcpy(out, tmp, sizeof(double) * 2 * n);
    free(tmp);
  }
}

void oracle_fft1d(double *data, int n, ptrdiff_t stride, int sign) {
  int j;
  double *w = (double *)malloc(sizeof(double) * 2 * n);
  double *in = (double *)malloc(sizeof(double) * 2 * n);
  double *out = (double *)malloc(sizeof(double) * 2 * n);
  const double two_pi = 6.283185307179586476925286766559;
  for (j = 0; j < n; j++) {
    w[2 * j] = cos(two_pi * j / n);
    w[2 * j + 1] = sign * sin(two_pi * j / n);
    in[2 * j] = data[2 * j * stride];
    in[2 * j + 1] = data[2 * j * stride + 1];
  }
  fft_rec(in, 1, out, n, w, 1, n);
  for (j = 0; j < n; j++) {
    data[2 * j * stride] = out[2 * j];
    data[2 * j * stride + 1] = out[2 * j + 1];
  }
  free(w);
  free(in);
  free(out);
}

void oracle_fft3d(double *data, int nx, int ny, int nz, int sign) {
  int i, j, k;
  for (k = 0; k < nz; k++)
    for (j = 0; j < ny; j++) oracle_fft1d(data + 2 * ((size_t)k * nx * ny + (size_t)j * nx), nx, 1, sign);
  for (k = 0; k < nz; k++)
    for (i = 0; i < nx; i++) oracle_fft1d(data + 2 * ((size_t)k * nx * ny + i), ny, nx, sign);
  for (j = 0; j < ny; j++)
    for (i = 0; i < nx; i++) oracle_fft1d(data + 2 * ((size_t)j * nx + i), nz, (ptrdiff_t)nx * ny, sign);
}
