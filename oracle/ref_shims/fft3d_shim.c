/* fftMPI stand-in for oracle/_ref (single rank); see fft3d_wrap.h. */
#include "fft3d_wrap.h"
#include "oracle_fft.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int nfast, nmid, nslow;
} shim_fft;

void fft3d_create(MPI_Comm comm, int precision, void **handle) {
  (void)comm;
  if (precision != 2) {
    fprintf(stderr, "fft3d shim: only double precision\n");
    exit(3);
  }
  *handle = calloc(1, sizeof(shim_fft));
}

void fft3d_destroy(void *handle) { free(handle); }

void fft3d_set(void *handle, const char *key, int value) { (void)handle; (void)key; (void)value; }

void fft3d_setup(void *handle, int nfast, int nmid, int nslow,
                 int in_ilo, int in_ihi, int in_jlo, int in_jhi, int in_klo, int in_khi,
                 int out_ilo, int out_ihi, int out_jlo, int out_jhi, int out_klo, int out_khi,
                 int permute, int *fftsize, int *sendsize, int *recvsize) {
  shim_fft *f = (shim_fft *)handle;
  (void)in_ilo; (void)in_ihi; (void)in_jlo; (void)in_jhi; (void)in_klo; (void)in_khi;
  (void)out_ilo; (void)out_ihi; (void)out_jlo; (void)out_jhi; (void)out_klo; (void)out_khi;
  if (permute != 0) {
    fprintf(stderr, "fft3d shim: permute must be 0\n");
    exit(3);
  }
  f->nfast = nfast;
  f->nmid = nmid;
  f->nslow = nslow;
  *fftsize = nfast * nmid * nslow;
  *sendsize = 0;
  *recvsize = 0;
}

void fft3d_compute(void *handle, FFT_SCALAR *in, FFT_SCALAR *out, int flag) {
  shim_fft *f = (shim_fft *)handle;
  size_t n = (size_t)f->nfast * f->nmid * f->nslow, m;
  if (out != in) memcpy(out, in, sizeof(double) * 2 * n);
  oracle_fft3d(out, f->nfast, f->nmid, f->nslow, flag == 1 ? -1 : +1);
  if (flag == -1) {
    double s = 1.0 / (double)n;
    for (m = 0; m < 2 * n; m++) out[m] *= s;
  }
}
