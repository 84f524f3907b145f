/*
 * Stand-in for the fftMPI C interface (libfft3dmpi, LAMMPS-derived; not
 * vendored in the reference, version unpinned: source_beta_to_omega/makefile:17,
 * src/fft3d.h:3-4), used ONLY to compile the reference into the test oracle
 * (oracle/_ref).  Test infrastructure.
 *
 * Restated published behaviour (single rank, brick in == brick out):
 *   - data: interleaved complex doubles (precision 2), x fastest;
 *   - fft3d_compute(..., +1): forward DFT, X[k] = sum_j x[j] exp(-2 pi i jk/N),
 *     unscaled;
 *   - fft3d_compute(..., -1): backward DFT with exp(+2 pi i jk/N), scaled by
 *     1/(nfast*nmid*nslow) (fftMPI's default "scaled" = 1), so that
 *     backward(forward(x)) == x as fft_test assumes (src/fft3d.c:27-32).
 */
#ifndef SCLET_ORACLE_FFT3D_WRAP_H
#define SCLET_ORACLE_FFT3D_WRAP_H

#include "mpi.h"

typedef double FFT_SCALAR;

void fft3d_create(MPI_Comm comm, int precision, void **handle);
void fft3d_destroy(void *handle);
void fft3d_set(void *handle, const char *key, int value);
void fft3d_setup(void *handle, int nfast, int nmid, int nslow,
                 int in_ilo, int in_ihi, int in_jlo, int in_jhi, int in_klo, int in_khi,
                 int out_ilo, int out_ihi, int out_jlo, int out_jhi, int out_klo, int out_khi,
                 int permute, int *fftsize, int *sendsize, int *recvsize);
void fft3d_compute(void *handle, FFT_SCALAR *in, FFT_SCALAR *out, int flag);

#endif
