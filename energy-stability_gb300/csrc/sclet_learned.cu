// Coarse ETD steps corrected by the learned network and judged, step by
// step, by the checks of the plain scheme (sclet_learned_step in
// include/sclet_gb300.h): discrete energy non-increasing, conserved mass
// unchanged, and a periodic bound on the distance from the fine steps the
// coarse step replaces.  A step that fails is re-run as fine ETD steps.
//
// The reference has no learned step.  The closest of its pieces are the
// alpha driver's (disabled) adaptive-step rollback,
// source_beta_to_alpha/src/anisotropic_hip.c:4230-4262, which re-runs a step
// that failed a check, and check_cahn_hilliard_min,
// source_beta_to_alpha/src/field.c:193-266, a per-step sanity check.
#include <math.h>
#include <string.h>

#include <string>
#include <vector>

#include "sclet_conv.cuh"
#include "sclet_gb300.h"
#include "sclet_internal.cuh"

namespace sclet {
int ctx_export_owned(sclet_ctx *ctx, float *dst);
int ctx_import_owned(sclet_ctx *ctx, const float *src);
int ctx_device(const sclet_ctx *ctx);
double ctx_dt(const sclet_ctx *ctx);
int ctx_nac(const sclet_ctx *ctx);
int ctx_fail(sclet_ctx *ctx, int code, const char *msg);
int net_forward_on(sclet_net *net, int N, int batch, const float *in, float *out, cudaStream_t s);
const char *net_error(const sclet_net *net);
}  // namespace sclet

using namespace sclet;

namespace {

// per-field sums over the owned cells: sums[f] of d (f >= from, else
// untouched) for the mean of a conserved field's correction
__global__ void field_sum_kernel(const float *__restrict__ d, long long n3, int from, double *__restrict__ sums) {
  const int f = from + blockIdx.y;
  __shared__ double red[256];
  double s = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3; i += (long long)gridDim.x * blockDim.x)
    s += (double)d[f * n3 + i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(&sums[f], red[0]);
}

// dx = xc - x0 (all fields); sums of squares of dx into sq[0] and of x0 into sq[1]
__global__ void increment_kernel(const float *__restrict__ xc, const float *__restrict__ x0, float *__restrict__ dx,
                                 long long count, double *__restrict__ sq) {
  __shared__ double red[2][256];
  double s = 0.0, u = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
    const float a = x0[i], d = xc[i] - a;
    dx[i] = d;
    s += (double)d * d;
    u += (double)a * a;
  }
  red[0][threadIdx.x] = s;
  red[1][threadIdx.x] = u;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicAdd(&sq[0], red[0][0]);
    atomicAdd(&sq[1], red[1][0]);
  }
}

// the pair's scale: the RMS of the coarse increment plus SCLET_NET_FLOOR
// times the RMS of the start state (the floor keeps the scale away from zero
// where the state has stopped moving)
__device__ __forceinline__ double pair_scale(const double *sq, long long count) {
  return sqrt(sq[0] / (double)count) + SCLET_NET_FLOOR * sqrt(sq[1] / (double)count);
}

// dx /= s (dx stays 0 when s = 0)
__global__ void normalise_kernel(float *__restrict__ dx, long long count, const double *__restrict__ sq) {
  const double sc = pair_scale(sq, count);
  const float inv = sc > 0.0 ? (float)(1.0 / sc) : 0.0f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    dx[i] *= inv;
}

// x = xc + s d (s the pair's scale), minus the mean of s d for the conserved
// fields (f >= nac)
__global__ void correct_kernel(float *__restrict__ x, const float *__restrict__ xc, const float *__restrict__ d,
                               long long n3, int nac, const double *__restrict__ sums, const double *__restrict__ sq,
                               long long count) {
  const int f = blockIdx.y;
  const float sc = (float)pair_scale(sq, count);
  const float mean = f >= nac ? (float)(sums[f] / (double)n3) * sc : 0.0f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3; i += (long long)gridDim.x * blockDim.x)
    x[f * n3 + i] = xc[f * n3 + i] + (sc * d[f * n3 + i] - mean);
}

// per field: sums[2 f] += (a - b)^2, sums[2 f + 1] += b^2
__global__ void dist_kernel(const float *__restrict__ a, const float *__restrict__ b, long long n3,
                            double *__restrict__ sums) {
  const int f = blockIdx.y;
  __shared__ double r0[256], r1[256];
  double s0 = 0.0, s1 = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3; i += (long long)gridDim.x * blockDim.x) {
    const double u = a[f * n3 + i], v = b[f * n3 + i];
    s0 += (u - v) * (u - v);
    s1 += v * v;
  }
  r0[threadIdx.x] = s0;
  r1[threadIdx.x] = s1;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      r0[threadIdx.x] += r0[threadIdx.x + w];
      r1[threadIdx.x] += r1[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicAdd(&sums[2 * f], r0[0]);
    atomicAdd(&sums[2 * f + 1], r1[0]);
  }
}

int blocks_for(long long n) {
  const long long b = (n + 255) / 256;
  return (int)(b > 152 * 8 ? 152 * 8 : (b < 1 ? 1 : b));
}

struct Buffers {
  float *xin = nullptr;    // [2F][N^3]: the start state u0, then the normalised coarse increment
  float *xc = nullptr;     // [F][N^3]: the coarse step's result, then the corrected state
  float *delta = nullptr;  // [F][N^3]: the network's output
  float *xf = nullptr;     // [F][N^3]: fine steps from u0
  double *sums = nullptr;  // 2F + 2
  ~Buffers() {
    cudaFree(xin);
    cudaFree(xc);
    cudaFree(delta);
    cudaFree(xf);
    cudaFree(sums);
  }
};

}  // namespace

#define LK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      std::string m_ = std::string(#call) + ": " + cudaGetErrorString(e_);         \
      return ctx_fail(coarse, SCLET_ERR_CUDA, m_.c_str());                         \
    }                                                                              \
  } while (0)
#define LR(call)                \
  do {                          \
    int r_ = (call);            \
    if (r_ != SCLET_OK) return r_; \
  } while (0)

extern "C" int sclet_learned_step(sclet_ctx *coarse, sclet_ctx *fine, sclet_net *net, int ratio, int nsteps,
                                  int check_every, double deviation_bound, double energy_tol,
                                  sclet_learned_stats *st) {
  if (!coarse || !fine || !st || ratio < 1 || nsteps < 0) return SCLET_ERR_ARG;
  const int n = sclet_block_edge(coarse), F = sclet_field_count(coarse), nac = ctx_nac(coarse);
  if (sclet_block_edge(fine) != n || sclet_field_count(fine) != F || ctx_device(fine) != ctx_device(coarse))
    return ctx_fail(coarse, SCLET_ERR_ARG, "coarse and fine contexts differ in size, fields or device");
  if (fabs(ctx_dt(coarse) - ratio * ctx_dt(fine)) > 1e-12 * ctx_dt(coarse))
    return ctx_fail(coarse, SCLET_ERR_ARG, "the coarse step must be ratio times the fine step");
  if (net && F != SCLET_NET_OUT)
    return ctx_fail(coarse, SCLET_ERR_UNSUPPORTED, "the corrector takes runs of four fields");
  LK(cudaSetDevice(ctx_device(coarse)));
  const int N = n - 4;
  const long long n3 = (long long)N * N * N;
  cudaStream_t s = (cudaStream_t)sclet_stream(coarse), sf = (cudaStream_t)sclet_stream(fine);
  Buffers b;
  LK(cudaMalloc(&b.xin, sizeof(float) * 2 * F * n3));
  LK(cudaMalloc(&b.xc, sizeof(float) * F * n3));
  LK(cudaMalloc(&b.delta, sizeof(float) * F * n3));
  LK(cudaMalloc(&b.xf, sizeof(float) * F * n3));
  LK(cudaMalloc(&b.sums, sizeof(double) * (2 * F + 2)));
  float *x0 = b.xin, *dx = b.xin + F * n3;
  double *sq = b.sums + 2 * F;
  std::vector<sclet_diag> d0(F), d1(F);
  LR(sclet_check_soln(coarse, 1, d0.data()));
  const dim3 grid(blocks_for(n3), F);
  for (int k = 0; k < nsteps; k++) {
    LR(ctx_export_owned(coarse, x0));
    LR(sclet_step(coarse, 1));
    if (net) {
      // input: u0 and the coarse increment scaled to unit RMS; the output is
      // the correction in units of that RMS
      LR(ctx_export_owned(coarse, b.xc));
      LK(cudaMemsetAsync(b.sums, 0, sizeof(double) * (2 * F + 2), s));
      increment_kernel<<<blocks_for(F * n3), 256, 0, s>>>(b.xc, x0, dx, F * n3, sq);
      LK(cudaGetLastError());
      normalise_kernel<<<blocks_for(F * n3), 256, 0, s>>>(dx, F * n3, sq);
      LK(cudaGetLastError());
      int rc = net_forward_on(net, N, 1, b.xin, b.delta, s);
      if (rc != SCLET_OK) return ctx_fail(coarse, rc, net_error(net));
      if (F > nac) {
        field_sum_kernel<<<dim3(blocks_for(n3), F - nac), 256, 0, s>>>(b.delta, n3, nac, b.sums);
        LK(cudaGetLastError());
      }
      correct_kernel<<<grid, 256, 0, s>>>(b.xc, b.xc, b.delta, n3, nac, b.sums, sq, F * n3);
      LK(cudaGetLastError());
      LR(ctx_import_owned(coarse, b.xc));
    }
    LR(sclet_check_soln(coarse, 1, d1.data()));
    bool ok = true, have_fine = false;
    const double e0 = d0[0].energy, e1 = d1[0].energy;
    if (!(e1 <= e0 + energy_tol * fabs(e0))) {
      ok = false;
      st->energy_fail++;
    }
    for (int f = nac; f < F; f++)
      if (!(fabs(d1[f].vol - d0[f].vol) <= 1e-10 * fabs(d0[f].vol))) {
        ok = false;
        st->mass_fail++;
        break;
      }
    if (check_every > 0 && (k + 1) % check_every == 0) {
      LK(cudaStreamSynchronize(s));
      LR(ctx_import_owned(fine, x0));
      LR(sclet_step(fine, ratio));
      LR(ctx_export_owned(fine, b.xf));
      LR(ctx_export_owned(coarse, b.xc));
      LK(cudaStreamSynchronize(sf));
      LK(cudaMemsetAsync(b.sums, 0, sizeof(double) * 2 * F, s));
      dist_kernel<<<grid, 256, 0, s>>>(b.xc, b.xf, n3, b.sums);
      LK(cudaGetLastError());
      std::vector<double> h(2 * F);
      LK(cudaMemcpyAsync(h.data(), b.sums, sizeof(double) * 2 * F, cudaMemcpyDeviceToHost, s));
      LK(cudaStreamSynchronize(s));
      double dev = 0.0;
      for (int f = 0; f < F; f++) dev = fmax(dev, sqrt(h[2 * f] / fmax(h[2 * f + 1], 1e-300)));
      st->deviation_checks++;
      st->max_deviation = fmax(st->max_deviation, dev);
      have_fine = true;
      if (!(dev <= deviation_bound)) {
        ok = false;
        st->deviation_fail++;
      }
    }
    if (!ok) {
      if (!have_fine) {
        LK(cudaStreamSynchronize(s));
        LR(ctx_import_owned(fine, x0));
        LR(sclet_step(fine, ratio));
        LR(ctx_export_owned(fine, b.xf));
        LK(cudaStreamSynchronize(sf));
      }
      LR(ctx_import_owned(coarse, b.xf));
      LR(sclet_check_soln(coarse, 1, d1.data()));
      st->fallbacks++;
    }
    st->steps++;
    d0 = d1;
  }
  LK(cudaStreamSynchronize(s));
  return SCLET_OK;
}
