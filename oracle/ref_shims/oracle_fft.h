/*
 * Mixed-radix complex DFT used by the test oracle (both the fftMPI stand-in
 * for oracle/_ref and the C restatement in oracle/sclet_oracle.c).  Test
 * infrastructure.  Recursive decimation in time over the prime factors of N
 * (Cooley-Tukey); twiddles exp(sign * 2 pi i j / N) taken from one table.
 */
#ifndef SCLET_ORACLE_FFT_H
#define SCLET_ORACLE_FFT_H
#include <stddef.h>

/* In-place 1D DFT of n complex values spaced `stride` complex elements apart.
 * sign = -1: forward (exp(-i..)); sign = +1: backward, unscaled. */
void oracle_fft1d(double *data, int n, ptrdiff_t stride, int sign);

/* In-place 3D DFT of an nx*ny*nz interleaved complex array, x fastest.
 * sign = -1 forward (unscaled), +1 backward (unscaled). */
void oracle_fft3d(double *data, int nx, int ny, int nz, int sign);

#endif
