/* Mixed-radix complex DFT for the test oracle; see oracle_fft.h.
 * Recursive decimation in time over the prime factors of n (Cooley-Tukey),
 * twiddles from one table exp(sign 2 pi i j / n); the 3D transform runs its
 * lines in parallel (OpenMP) with per-thread scratch. */
#include "oracle_fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static int smallest_factor(int n) {
  int p;
  if (n % 4 == 0) return 4;
  if (n % 2 == 0) return 2;
  for (p = 3; p * p <= n; p += 2)
    if (n % p == 0) return p;
  return n;
}

/* out[0..n) = DFT of in[0], in[s], ...; w: table of size ntab (w^j =
 * exp(sign 2 pi i j / ntab)), wstep = ntab / n; tmp: 2n doubles of scratch
 * for this level and below (levels use disjoint parts). */
static void fft_rec(const double *in, ptrdiff_t s, double *out, int n, const double *w, int wstep, int ntab,
                    double *tmp) {
  int p, m, r, k, q;
  if (n == 1) {
    out[0] = in[0];
    out[1] = in[1];
    return;
  }
  p = smallest_factor(n);
  m = n / p;
  for (r = 0; r < p; r++) fft_rec(in + 2 * r * s, s * p, out + 2 * r * m, m, w, wstep * p, ntab, tmp + 2 * n);
  for (k = 0; k < m; k++) {
    for (q = 0; q < p; q++) {
      double re = 0.0, im = 0.0;
      int kk = k + q * m;
      for (r = 0; r < p; r++) {
        long e = ((long)r * kk) % n;
        double wr = w[2 * (e * wstep)], wi = w[2 * (e * wstep) + 1];
        double xr = out[2 * (r * m + k)], xi = out[2 * (r * m + k) + 1];
        re += xr * wr - xi * wi;
        im += xr * wi + xi * wr;
      }
      tmp[2 * kk] = re;
      tmp[2 * kk + 1] = im;
    }
  }
  memcpy(out, tmp, sizeof(double) * 2 * n);
}

/* Levels shrink by at least 2, so 4n doubles of scratch cover all levels. */
static void fft_line(double *data, int n, ptrdiff_t stride, const double *w, double *work) {
  int j;
  double *in = work, *out = work + 2 * n, *tmp = work + 4 * n;
  for (j = 0; j < n; j++) {
    in[2 * j] = data[2 * j * stride];
    in[2 * j + 1] = data[2 * j * stride + 1];
  }
  fft_rec(in, 1, out, n, w, 1, n, tmp);
  for (j = 0; j < n; j++) {
    data[2 * j * stride] = out[2 * j];
    data[2 * j * stride + 1] = out[2 * j + 1];
  }
}

static double *twiddles(int n, int sign) {
  const double two_pi = 6.283185307179586476925286766559;
  double *w = (double *)malloc(sizeof(double) * 2 * n);
  int j;
  for (j = 0; j < n; j++) {
    w[2 * j] = cos(two_pi * j / n);
    w[2 * j + 1] = sign * sin(two_pi * j / n);
  }
  return w;
}

void oracle_fft1d(double *data, int n, ptrdiff_t stride, int sign) {
  double *w = twiddles(n, sign);
  double *work = (double *)malloc(sizeof(double) * 8 * n);
  fft_line(data, n, stride, w, work);
  free(w);
  free(work);
}

void oracle_fft3d(double *data, int nx, int ny, int nz, int sign) {
  double *wx = twiddles(nx, sign), *wy = twiddles(ny, sign), *wz = twiddles(nz, sign);
  int nmax = nx > ny ? (nx > nz ? nx : nz) : (ny > nz ? ny : nz);
  int line;
#pragma omp parallel
  {
    double *work = (double *)malloc(sizeof(double) * 8 * nmax);
#pragma omp for
    for (line = 0; line < ny * nz; line++) fft_line(data + 2 * (size_t)line * nx, nx, 1, wx, work);
#pragma omp for
    for (line = 0; line < nx * nz; line++) {
      int k = line / nx, i = line % nx;
      fft_line(data + 2 * ((size_t)k * nx * ny + i), ny, nx, wy, work);
    }
#pragma omp for
    for (line = 0; line < nx * ny; line++) fft_line(data + 2 * (size_t)line, nz, (ptrdiff_t)nx * ny, wz, work);
    free(work);
  }
  free(wx);
  free(wy);
  free(wz);
}
