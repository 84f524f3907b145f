// Declarations of the corrector network's kernels (k_conv.cu, k_conv_train.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace sclet {

constexpr int CH = 32;    // channels of every activation (inputs and outputs zero padded)
constexpr int TAPS = 27;  // 3 x 3 x 3 taps, t = (dz + 1) 9 + (dy + 1) 3 + (dx + 1)

// Activation layout, chunk-planar: a sample is Np = N + 2 haloed planes (zh),
// each plane 4 chunks of 8 channels (16 bytes per cell), each chunk the plane's
// Np^2 cells (slot = yh Np + xh) padded to a multiple of 8 slots (so every
// chunk starts on a 128-byte boundary).  Positions below are in 16-byte units.
__host__ __device__ inline long long conv_chunk_slots(int N) {
  const long long s = (long long)(N + 2) * (N + 2);
  return (s + 7) / 8 * 8;
}
// chunk k (channels 8k .. 8k+7) of cell (zh, slot) of sample b
__host__ __device__ inline long long conv_at(int N, int b, int zh, int k, long long slot) {
  return (((long long)b * (N + 2) + zh) * 4 + k) * conv_chunk_slots(N) + slot;
}
// 16-byte units of `batch` samples
__host__ __device__ inline long long conv_units(int N, int batch) {
  return (long long)batch * (N + 2) * 4 * conv_chunk_slots(N);
}

// Epilogue of conv_tc_kernel (acc = the convolution, b = bias, a = aux at the cell):
enum ConvMode {
  CONV_RELU = 0,      // out = max(acc + b, 0)                       (BF16)
  CONV_RESIDUAL = 1,  // out = a + acc + b                           (BF16)
  CONV_MASK = 2,      // out = acc where a > 0, else 0 (ReLU adjoint) (BF16)
  CONV_OUT_F32 = 3,   // outf = (acc + b) * scale, channels < cout, FP32 planar owned cells
  CONV_LINEAR = 4,    // out = acc + b                               (BF16)
};

struct ConvArgs {
  int N, batch;              // grid edge and samples
  int mode;
  int cout;                  // CONV_OUT_F32: channels written
  float scale;               // CONV_OUT_F32: output scale
  const float *bias;         // CH values or null
  const __nv_bfloat16 *aux;  // residual / mask source, same layout as the input
  __nv_bfloat16 *out;        // BF16 activation output (owned cells; halo untouched)
  float *outf;               // CONV_OUT_F32: [batch][cout][N^3]
  int *err;                  // set to 1 when a bounded wait gives up
};

// in: batch haloed samples in the chunk-planar layout; w: TAPS x CH (co) x CH
// (ci) BF16, ci fastest.
cudaError_t launch_conv(const __nv_bfloat16 *in, const __nv_bfloat16 *w, const ConvArgs &args, cudaStream_t s);
// Input runs per tile of launch_conv (sclet_net_set_conv_runs); returns the
// previous setting, -1 for an invalid one.
int conv_set_runs(int runs_per_plane);

// Periodic halo of batch haloed blocks, in place.
cudaError_t launch_conv_halo(__nv_bfloat16 *a, int N, int batch, cudaStream_t s);
// FP32 planar fields [batch][cin][N^3] (owned cells) -> haloed BF16 activations,
// channels >= cin zero, halo filled.
cudaError_t launch_conv_pack(const float *in, int cin, int N, int batch, __nv_bfloat16 *a, cudaStream_t s);
// FP32 planar [batch][cout][N^3] -> haloed BF16 (channels >= cout zero, halo filled),
// times `scale`.
cudaError_t launch_conv_pack_grad(const float *g, int cout, float scale, int N, int batch, __nv_bfloat16 *a,
                                  cudaStream_t s);
// dW[t][co][ci] += sum over owned cells of g[cell][co] x in[cell + off(t)][ci];
// db[co] += sum of g[cell][co] (FP32 accumulators).
cudaError_t launch_conv_wgrad(const __nv_bfloat16 *in, const __nv_bfloat16 *g, int N, int batch, float *dw, float *db,
                              cudaStream_t s);
// FP32 master weights [layers][TAPS][CH][CH] -> BF16 forward copies (same layout)
// and adjoint copies (taps flipped, co and ci swapped).
cudaError_t launch_conv_weights(const float *w, int layers, __nv_bfloat16 *wf, __nv_bfloat16 *wt, cudaStream_t s);
// g = 0 where act <= 0 (the ReLU adjoint), owned cells and halo alike.
cudaError_t launch_conv_relu_mask(__nv_bfloat16 *g, const __nv_bfloat16 *act, int N, int batch, cudaStream_t s);
// Adam on count parameters (FP32 master p, moments m, v; gradient g, zeroed after).
cudaError_t launch_adam(float *p, float *m, float *v, float *g, long long count, float lr, float b1, float b2,
                        float eps, float c1, float c2, cudaStream_t s);
// r = pred - target over count values into r; partial sums of r^2 into part
// (blocks of the launch) for the loss.
cudaError_t launch_residual(const float *pred, const float *target, float *r, long long count, double *part,
                            int nparts, cudaStream_t s);

}  // namespace sclet
