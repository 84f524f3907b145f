// Declarations of the tensor-core (tcgen05) mode-n product, see k_modeprod_tc.cu.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace sclet {

struct TcArgs {
  int n, kp, kblocks, count;
  int epi;                    // 0 none, 1 ETD1 update with aux = uhat planes, 2 phi2 scaling
  int outmode;                // 0 split planes, 1 FP32 store, 2 FP32 accumulate
  const __nv_bfloat16 *aux;   // split planes of uhat (same layout as out_split)
  __nv_bfloat16 *out_split;   // [count][3][n*n][kp]
  float *out_f32;             // [count][n^3]
  const float *dd[3];         // eigenvalues / h^2 per axis
  float kk[3], epn2, dt, LE, KE, LCI, KCI;
  int nac, F;
  int *err;                   // set to 1 when a bounded wait gives up
};

int tc_kp(int n);
// [3][n][kp] split planes of a row-major FP64 matrix (zero padded columns)
cudaError_t tc_split_matrix(const double *m, __nv_bfloat16 *out, int n, cudaStream_t s);
// FP32 field blocks (minus `sub` when given) -> split planes [count][3][n*n][kp]
cudaError_t tc_split_fields(const float *u, const float *sub, __nv_bfloat16 *out, int n, int count, cudaStream_t s);
// out[t] = mat x in[t] (contracting the row axis, rotating), count tensors
cudaError_t launch_modeprod_tc(const __nv_bfloat16 *mat, const __nv_bfloat16 *in, int count, const TcArgs &args,
                               cudaStream_t s);

}  // namespace sclet
