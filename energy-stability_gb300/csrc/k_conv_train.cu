// Element-wise and reduction kernels of the corrector network: periodic halo,
// packing FP32 fields into haloed BF16 activations, the weight gradient of a
// 3x3x3 convolution (FP32 accumulation), the BF16 weight copies, Adam and the
// training residual.  Activations in the chunk-planar layout of
// sclet_conv.cuh (conv_at).
#include <cuda_bf16.h>
#include <stdint.h>

#include "sclet_conv.cuh"
#include "sclet_internal.cuh"

namespace sclet {
namespace {

__device__ __forceinline__ int wrap_h(int h, int N) { return 1 + (h - 1 + N) % N; }

__host__ __device__ inline long long shell_cells(int N) {
  const long long Np = N + 2;
  return 2 * Np * Np + 2LL * N * Np + 2LL * N * N;
}

// one 16-byte chunk (8 channels) of a halo cell per thread
__global__ void halo_kernel(__nv_bfloat16 *a, int N, int batch) {
  const int Np = N + 2;
  const long long per = shell_cells(N), plane = (long long)Np * Np;
  const long long total = per * batch * 4;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i & 3);
    long long s = i >> 2;
    const int b = (int)(s / per);
    s -= (long long)b * per;
    int z, y, x;
    if (s < 2 * plane) {
      z = s < plane ? 0 : Np - 1;
      const long long r = s % plane;
      y = (int)(r / Np);
      x = (int)(r % Np);
    } else if ((s -= 2 * plane) < 2LL * N * Np) {
      z = 1 + (int)(s / (2 * Np));
      const long long r = s % (2 * Np);
      y = r < Np ? 0 : Np - 1;
      x = (int)(r % Np);
    } else {
      s -= 2LL * N * Np;
      z = 1 + (int)(s / (2 * N));
      const long long r = s % (2 * N);
      y = 1 + (int)(r % N);
      x = r < N ? 0 : Np - 1;
    }
    const long long dst = conv_at(N, b, z, k, (long long)y * Np + x);
    const long long src = conv_at(N, b, wrap_h(z, N), k, (long long)wrap_h(y, N) * Np + wrap_h(x, N));
    reinterpret_cast<uint4 *>(a)[dst] = reinterpret_cast<const uint4 *>(a)[src];
  }
}

// every haloed cell from its periodic image in the planar FP32 input
__global__ void pack_kernel(const float *__restrict__ in, int cin, float scale, int N, int batch,
                            __nv_bfloat16 *__restrict__ a) {
  const int Np = N + 2;
  const long long n3 = (long long)N * N * N, cells = (long long)Np * Np * Np;
  const long long total = cells * batch;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(i / cells);
    long long r = i - (long long)b * cells;
    const int z = (int)(r / ((long long)Np * Np));
    r -= (long long)z * Np * Np;
    const int y = (int)(r / Np), x = (int)(r - (long long)y * Np);
    const long long own = ((long long)(wrap_h(z, N) - 1) * N + (wrap_h(y, N) - 1)) * N + (wrap_h(x, N) - 1);
    const float *src = in + (long long)b * cin * n3 + own;
    uint32_t w[CH / 2];
#pragma unroll
    for (int c = 0; c < CH; c += 2) {
      const float v0 = c < cin ? src[c * n3] * scale : 0.0f;
      const float v1 = c + 1 < cin ? src[(c + 1) * n3] * scale : 0.0f;
      const __nv_bfloat162 p = __floats2bfloat162_rn(v0, v1);
      w[c / 2] = *reinterpret_cast<const uint32_t *>(&p);
    }
    uint4 *dst = reinterpret_cast<uint4 *>(a);
    const long long c0 = conv_at(N, b, z, 0, (long long)y * Np + x), cs = conv_chunk_slots(N);
#pragma unroll
    for (int k = 0; k < 4; k++) dst[c0 + k * cs] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
  }
}

// Weight gradient: one tap per blockIdx.y; a CTA of 64 threads walks its
// share of the owned cells 64 at a time, the gradient and the shifted input
// of those cells in shared memory as FP32; thread (co4, ci4) accumulates a
// 4 x 4 block of dW over them, then adds it to the FP32 accumulator.
constexpr int WG_CELLS = 64;
__global__ void __launch_bounds__(64) wgrad_kernel(const __nv_bfloat16 *__restrict__ in,
                                                   const __nv_bfloat16 *__restrict__ g, int N, int batch,
                                                   float *__restrict__ dw, float *__restrict__ db) {
  __shared__ __align__(16) float gs[WG_CELLS][CH];
  __shared__ __align__(16) float xs[WG_CELLS][CH];
  const int tap = blockIdx.y;
  const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
  const int Np = N + 2;
  const long long n3 = (long long)N * N * N;
  const long long total = n3 * batch;
  const int tid = threadIdx.x;
  const int co0 = (tid >> 3) * 4, ci0 = (tid & 7) * 4;
  float acc[4][4] = {};
  float bacc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  const long long nblk = (total + WG_CELLS - 1) / WG_CELLS;
  for (long long blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    // 64 cells x 4 chunks of 8 channels per array: 4 chunk loads per thread each
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int idx = tid + 64 * r;  // 0..255
      const int c = idx >> 2, k = idx & 3;
      const long long i = blk * WG_CELLS + c;
      uint4 gv = make_uint4(0, 0, 0, 0), xv = make_uint4(0, 0, 0, 0);
      if (i < total) {
        const int b = (int)(i / n3);
        long long rr = i - (long long)b * n3;
        const int z = (int)(rr / ((long long)N * N));
        rr -= (long long)z * N * N;
        const int y = (int)(rr / N), x = (int)(rr - (long long)y * N);
        gv = reinterpret_cast<const uint4 *>(g)[conv_at(N, b, z + 1, k, (long long)(y + 1) * Np + x + 1)];
        xv = reinterpret_cast<const uint4 *>(in)[conv_at(N, b, z + 1 + dz, k, (long long)(y + 1 + dy) * Np + x + 1 + dx)];
      }
      const uint32_t gw[4] = {gv.x, gv.y, gv.z, gv.w}, xw[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
      for (int h = 0; h < 4; h++) {
        gs[c][k * 8 + 2 * h] = __uint_as_float(gw[h] << 16);
        gs[c][k * 8 + 2 * h + 1] = __uint_as_float(gw[h] & 0xffff0000u);
        xs[c][k * 8 + 2 * h] = __uint_as_float(xw[h] << 16);
        xs[c][k * 8 + 2 * h + 1] = __uint_as_float(xw[h] & 0xffff0000u);
      }
    }
    __syncthreads();
#pragma unroll 8
    for (int c = 0; c < WG_CELLS; c++) {
      const float4 gv = *reinterpret_cast<const float4 *>(&gs[c][co0]);
      const float4 xv = *reinterpret_cast<const float4 *>(&xs[c][ci0]);
      const float gg[4] = {gv.x, gv.y, gv.z, gv.w}, xx[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = fmaf(gg[a], xx[b], acc[a][b]);
      if (tap == 13 && ci0 == 0) {
#pragma unroll
        for (int a = 0; a < 4; a++) bacc[a] += gg[a];
      }
    }
    __syncthreads();
  }
  float *d = dw + (long long)tap * CH * CH;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) atomicAdd(&d[(co0 + a) * CH + ci0 + b], acc[a][b]);
  if (tap == 13 && ci0 == 0 && db) {
#pragma unroll
    for (int a = 0; a < 4; a++) atomicAdd(&db[co0 + a], bacc[a]);
  }
}

__global__ void relu_mask_kernel(uint4 *__restrict__ g, const uint4 *__restrict__ act, long long chunks) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < chunks; i += (long long)gridDim.x * blockDim.x) {
    uint4 gv = g[i];
    const uint4 av = act[i];
    uint32_t *gw = reinterpret_cast<uint32_t *>(&gv);
    const uint32_t aw[4] = {av.x, av.y, av.z, av.w};
#pragma unroll
    for (int h = 0; h < 4; h++) {
      // a BF16 value is > 0 when its sign bit is clear and it is not zero
      const uint32_t lo = aw[h] & 0xffffu, hi = aw[h] >> 16;
      const uint32_t keep_lo = (lo != 0 && !(lo & 0x8000u)) ? 0xffffu : 0u;
      const uint32_t keep_hi = (hi != 0 && !(hi & 0x8000u)) ? 0xffff0000u : 0u;
      gw[h] &= keep_lo | keep_hi;
    }
    g[i] = gv;
  }
}

__global__ void weights_kernel(const float *__restrict__ w, int layers, __nv_bfloat16 *__restrict__ wf,
                               __nv_bfloat16 *__restrict__ wt) {
  const long long per = (long long)TAPS * CH * CH, total = per * layers;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const long long l = i / per;
    const int r = (int)(i - l * per);
    const int t = r / (CH * CH), co = (r / CH) % CH, ci = r % CH;
    const __nv_bfloat16 v = __float2bfloat16_rn(w[i]);
    wf[i] = v;
    if (wt) wt[l * per + ((long long)(TAPS - 1 - t) * CH + ci) * CH + co] = v;
  }
}

__global__ void adam_kernel(float *p, float *m, float *v, float *g, long long count, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    g[i] = 0.0f;
  }
}

__global__ void residual_kernel(const float *__restrict__ pred, const float *__restrict__ target, float *__restrict__ r,
                                long long count, double *__restrict__ part) {
  __shared__ double red[256];
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
    const float d = pred[i] - target[i];
    r[i] = d;
    s += (double)d * d;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

int grid_for(long long total, int block) {
  const long long b = (total + block - 1) / block;
  return (int)(b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

}  // namespace

cudaError_t launch_conv_halo(__nv_bfloat16 *a, int N, int batch, cudaStream_t s) {
  halo_kernel<<<grid_for(shell_cells(N) * batch * 4, 256), 256, 0, s>>>(a, N, batch);
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t launch_conv_pack(const float *in, int cin, int N, int batch, __nv_bfloat16 *a, cudaStream_t s) {
  if (cin < 1 || cin > CH) return cudaErrorInvalidValue;
  const long long cells = (long long)(N + 2) * (N + 2) * (N + 2) * batch;
  pack_kernel<<<grid_for(cells, 256), 256, 0, s>>>(in, cin, 1.0f, N, batch, a);
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t launch_conv_pack_grad(const float *g, int cout, float scale, int N, int batch, __nv_bfloat16 *a,
                                  cudaStream_t s) {
  if (cout < 1 || cout > CH) return cudaErrorInvalidValue;
  const long long cells = (long long)(N + 2) * (N + 2) * (N + 2) * batch;
  pack_kernel<<<grid_for(cells, 256), 256, 0, s>>>(g, cout, scale, N, batch, a);
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t launch_conv_relu_mask(__nv_bfloat16 *g, const __nv_bfloat16 *act, int N, int batch, cudaStream_t s) {
  const long long chunks = conv_units(N, batch);
  relu_mask_kernel<<<grid_for(chunks, 256), 256, 0, s>>>(reinterpret_cast<uint4 *>(g),
                                                          reinterpret_cast<const uint4 *>(act), chunks);
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t launch_conv_wgrad(const __nv_bfloat16 *in, const __nv_bfloat16 *g, int N, int batch, float *dw, float *db,
                              cudaStream_t s) {
  const long long blocks = ((long long)N * N * N * batch + WG_CELLS - 1) / WG_CELLS;
  const int gx = (int)(blocks < 256 ? blocks : 256);
  wgrad_kernel<<<dim3(gx, TAPS), 64, 0, s>>>(in, g, N, batch, dw, db);
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t launch_conv_weights(const float *w, int layers, __nv_bfloat16 *wf, __nv_bfloat16 *wt, cudaStream_t s) {
  weights_kernel<<<grid_for((long long)TAPS * CH * CH * layers, 256), 256, 0, s>>>(w, layers, wf, wt);
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t launch_adam(float *p, float *m, float *v, float *g, long long count, float lr, float b1, float b2,
                        float eps, float c1, float c2, cudaStream_t s) {
  adam_kernel<<<grid_for(count, 256), 256, 0, s>>>(p, m, v, g, count, lr, b1, b2, eps, c1, c2);
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t launch_residual(const float *pred, const float *target, float *r, long long count, double *part,
                            int nparts, cudaStream_t s) {
  residual_kernel<<<nparts, 256, 0, s>>>(pred, target, r, count, part);
  launch_counter()++;
  return cudaGetLastError();
}

}  // namespace sclet
