// Declarations of the tensor-core (tcgen05) mode-n product, see k_modeprod_tc.cu.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace sclet {

constexpr int TC_PLANES = 4;    // fixed-point slices per data operand (tc_slice_bits each)
constexpr int TC_PLANES_M = 5;  // slices per matrix: four 6-bit slices and a fifth
                                // stored pre-scaled by 1/64 (see k_modeprod_tc.cu)

struct TcArgs {
  int n, kp, kblocks, count;
  int bits;                 // slice width (set by launch_modeprod_tc)
  int epi;                  // 0 none, 1 ETD1 update (aux = uhat), 2 phi2 scaling
  int outmode;              // 1 FP32 store, 2 FP32 accumulate
  const float *aux;         // [count][n^3] FP32 uhat, same layout as out
  float *out;               // [count][n^3] FP32, rotated layout
  const float *in_scale;    // [count][n*n] power-of-two scale of each input row's slices
  const float *row_scale;   // [n] power-of-two scale of each matrix row's slices
  // per field kind (0 AC, 1 CH), per eigen-mode [k][j][i]: ETD1
  // (e = 1 - phi1 H, phi1) and ETD2 (phi2) coefficients computed in FP64
  // (ac_init_phi / ch_init_phi, vars.c:302-359) as hi + lo FP32 pairs
  const float4 *coef[2];
  const float2 *coef2[2];
  int nac, F;
  int *err;                 // set to 1 when a bounded wait gives up
  int max_ctas;             // persistent CTAs (0: as many as can be resident)
  int idle;                 // 1: the producer issues no loads (the bounded-wait self-test)
};

// kp = n rounded up to whole k-blocks of 32: the slice planes are k-blocked,
// [p][kp / 32][rows][32], columns n .. kp - 1 zero
int tc_kp(int n);
int tc_slice_bits(int n);
// Row-major FP64 n x n matrix -> TC_PLANES_M k-blocked slice planes
// [p][kp / 32][n][32] (zero padded columns) and the power-of-two scale of each row.
cudaError_t tc_slice_matrix(const double *m, __nv_bfloat16 *planes, float *row_scale, int n, cudaStream_t s);
// FP32 blocks (x - sub; sub may be null), rows of n -> k-blocked slice planes
// [count][p][kp / 32][n*n][32] with the power-of-two scale of each row in
// scale[count][n*n]; the pad columns are never written (zero from allocation).
cudaError_t tc_slice_fields(const float *x, const float *sub, float *scale, __nv_bfloat16 *planes, int n, int count,
                            cudaStream_t s);
// ETD coefficient tables of one field kind (see TcArgs::coef)
cudaError_t tc_make_coefs(float4 *coef, float2 *coef2, int n, int kind, const double *dx, const double *dy,
                          const double *dz, const double *kk, double epn2, double dt, double L, double K,
                          cudaStream_t s);
// out[t] = mat x in[t] (contracting the row axis, rotating), count tensors
cudaError_t launch_modeprod_tc(const __nv_bfloat16 *mat, const __nv_bfloat16 *planes, int count, const TcArgs &args,
                               cudaStream_t s);

}  // namespace sclet
