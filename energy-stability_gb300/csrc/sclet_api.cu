// C ABI of sclet_gb300: context, device state and the step sequence of the
// reference's time loop (source_beta_to_omega/src/ScLETD.c:84-191) on one GPU.
//
// Two arithmetic forms share the sequence:
//   SCLET_FP64  -- FP64 state, FP64 SIMT mode-n products (k_modeprod_f64.cu);
//   SCLET_MIXED -- FP32 state and stencils/FFT, eigenbasis products as
//                  split-BF16 tcgen05 products with FP32 accumulation
//                  (k_modeprod_tc.cu), FP64-compensated diagnostics.
#include <cuda_bf16.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>
#include <sys/stat.h>

#include "sclet_gb300.h"
#include "sclet_internal.cuh"
#include "sclet_physics.cuh"
#include "sclet_tc.cuh"

namespace sclet {
void set_phi_tables(const double *phi1_ac, const double *phi1_ch, const double *phi2_ac, const double *phi2_ch);
}

using namespace sclet;

struct StageEv {
  int cls;
  cudaEvent_t a, b;
};

struct sclet_ctx {
  sclet_params p;
  int precision = SCLET_FP64, device = 0;
  int step_diag = -1;  // energy form of the diagnostics sclet_step queues after each step; -1 none
  int n = 0, F = 0, nac = 0, nch = 0;
  // runs of the same size side by side (sclet_create_runs): FT = runs F
  // stored fields, run r's at r F n^3; krun = per-run plugin constant 0
  int runs = 1, FT = 0;
  double *krun = nullptr;
  long long n3 = 0;
  Phys ph;
  cudaStream_t stream = nullptr;
  std::string err;
  // shared
  double *dd[3] = {nullptr, nullptr, nullptr};  // eigenvalues / h^2 (FP64)
  double *elam = nullptr, *partials = nullptr;
  // the diagnostics record: page-locked host memory mapped into the device,
  // written by the reduction kernel, so reading it needs no copy (a copy would
  // queue behind large transfers on the copy engines)
  double *diag_host = nullptr, *diag = nullptr;
  int npart = 0;
  ElasticPlan *elastic = nullptr;
  int *dev_err = nullptr;  // bounded-wait failures of device kernels
  // FP64 form: state2 = [u (F) | rhs1 (F)]
  double *state2 = nullptr, *rhs2 = nullptr, *A = nullptr, *B = nullptr;
  double *felas = nullptr, *scratch = nullptr, *shell = nullptr;
  double *V[3] = {nullptr, nullptr, nullptr}, *Vi[3] = {nullptr, nullptr, nullptr};
  double *phi1[2] = {nullptr, nullptr}, *phi2[2] = {nullptr, nullptr};
  // MIXED form: fstate2 = [u (F) | rhs1 (F)] in FP32; FP32 work tensors W1, W2
  // (2F blocks each); slice planes P of up to 2F tensors with their row scales
  // scaleP; sliced matrices with row scales
  float *fstate2 = nullptr, *frhs2 = nullptr, *ffelas = nullptr, *fscratch = nullptr, *fshell = nullptr;
  float *W1 = nullptr, *W2 = nullptr, *scaleP = nullptr, *rsV = nullptr, *rsVi = nullptr;
  __nv_bfloat16 *P = nullptr, *matV = nullptr, *matVi = nullptr;
  float4 *coef[2] = {nullptr, nullptr};   // ETD1 coefficient pairs per field kind
  float2 *coef2[2] = {nullptr, nullptr};  // ETD2 phi2 pairs per field kind
  double *stage64 = nullptr;  // n^3 FP64 staging block for host transfers
  // variable-mobility CH: two scratch blocks per run in the state's type and
  // the block maxima of the mobility (Phys::mob_t, Phys::mob_part)
  void *mob_t = nullptr;
  double *mob_part = nullptr;
  // pipelined transfers of all fields (sclet_set_fields_async /
  // sclet_get_fields_async): an FP64 staging area per direction, filled and
  // drained by the copy engines on one stream per direction, while the
  // context's stream only converts between staging and state
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  double *in_stage = nullptr, *out_stage = nullptr;
  cudaEvent_t in_ready = nullptr, in_free = nullptr, out_ready = nullptr, out_free = nullptr;
  // conserved-field mass of the mixed form: FP64 weights wE, wP (, w2) of n^3
  // each, target / after partial sums, last (target, before, shift)
  double *massW = nullptr, *massPart = nullptr, *massRes = nullptr;
  // profiling
  bool profiling = false;
  std::vector<StageEv> evs;
  float stage_ms[8] = {0};
  int stage_launches[8] = {0};
  long long launches0 = 0;
  long long steps_done = 0;
  // one step captured as a CUDA graph (sclet_graph_step)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
};

static std::string g_create_error;

#define CK(call)                                                                  \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) {                                                      \
      ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);              \
      return e_ == cudaErrorMemoryAllocation ? SCLET_ERR_NOMEM : SCLET_ERR_CUDA;  \
    }                                                                             \
  } while (0)

namespace {

bool mixed(const sclet_ctx *ctx) { return ctx->precision == SCLET_MIXED; }
double *u_of(sclet_ctx *ctx) { return ctx->state2; }
double *rhs1_of(sclet_ctx *ctx) { return ctx->state2 + (long long)ctx->FT * ctx->n3; }
float *fu_of(sclet_ctx *ctx) { return ctx->fstate2; }
float *frhs1_of(sclet_ctx *ctx) { return ctx->fstate2 + (long long)ctx->FT * ctx->n3; }

// phi1, phi2 of each field kind at eigen-mode (i, j, k), layout [k][j][i]
// (ac_init_phi / ch_init_phi, vars.c:302-359).
__global__ void phi_kernel(double *phi1, double *phi2, int n, int kind, const double *dx, const double *dy,
                           const double *dz, double kkx, double kky, double kkz, double epn2, double dt, double L,
                           double K) {
  long long n3 = (long long)n * n * n;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < n3; o += (long long)gridDim.x * blockDim.x) {
    int i = (int)(o % n), j = (int)((o / n) % n), k = (int)(o / ((long long)n * n));
    double tmp, H;
    if (kind == 0) {
      tmp = kkz * dz[k] + kky * dy[j] + kkx * dx[i];
      H = -L * (tmp * epn2 - K);
    } else {
      tmp = dz[k] + dy[j] + dx[i];
      H = L * (tmp * tmp * epn2 - K * tmp);
    }
    double p1, p2;
    if (fabs(H) > 1.0e-8) {
      double e = exp(-dt * H);
      p1 = (1.0 - e) / H;
      p2 = (1.0 - p1 / dt) / H;
    } else {
      p1 = dt;
      p2 = dt / 2;
    }
    phi1[o] = p1;
    phi2[o] = p2;
  }
}

__global__ void f64_to_f32(const double *__restrict__ a, float *__restrict__ b, long long count, double shift) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)(a[i] - shift);
}
__global__ void f32_to_f64(const float *__restrict__ a, double *__restrict__ b, long long count, double shift) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    b[i] = (double)a[i] + shift;
}

// all F fields between the FP64 host layout and the state: FP32 states hold
// the conserved fields (f >= nac) relative to shift; grid y = field.  Four
// values per thread and pass (16-byte FP32 and two 16-byte FP64 accesses)
// where every field block starts on a 32-byte boundary (n^3 % 4 == 0).
__global__ void fields_to_state(const double *__restrict__ a, float *__restrict__ b, long long n3, int nac,
                                double shift, int F) {
  const double sh = (int)blockIdx.y % F >= nac ? shift : 0.0;
  const double *s = a + blockIdx.y * n3;
  float *d = b + blockIdx.y * n3;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x, st = (long long)gridDim.x * blockDim.x;
  long long done = 0;
  if (n3 % 4 == 0) {
    const double4_32a *s4 = reinterpret_cast<const double4_32a *>(s);
    float4 *d4 = reinterpret_cast<float4 *>(d);
    for (long long i = t0; i < n3 / 4; i += st) {
      const double4_32a v = s4[i];
      d4[i] = make_float4((float)(v.x - sh), (float)(v.y - sh), (float)(v.z - sh), (float)(v.w - sh));
    }
    done = n3;
  }
  for (long long i = done + t0; i < n3; i += st) d[i] = (float)(s[i] - sh);
}
__global__ void fields_from_state(const float *__restrict__ a, double *__restrict__ b, long long n3, int nac,
                                  double shift, int F) {
  const double sh = (int)blockIdx.y % F >= nac ? shift : 0.0;
  const float *s = a + blockIdx.y * n3;
  double *d = b + blockIdx.y * n3;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x, st = (long long)gridDim.x * blockDim.x;
  long long done = 0;
  if (n3 % 4 == 0) {
    const float4 *s4 = reinterpret_cast<const float4 *>(s);
    double4_32a *d4 = reinterpret_cast<double4_32a *>(d);
    for (long long i = t0; i < n3 / 4; i += st) {
      const float4 v = s4[i];
      d4[i] = make_double4_32a((double)v.x + sh, (double)v.y + sh, (double)v.z + sh, (double)v.w + sh);
    }
    done = n3;
  }
  for (long long i = done + t0; i < n3; i += st) d[i] = (double)s[i] + sh;
}

int grid_of(long long total) {
  long long b = (total + 255) / 256;
  return (int)(b > 152LL * 16 ? 152LL * 16 : (b < 1 ? 1 : b));
}

int fail(sclet_ctx *ctx, int code, const std::string &msg) {
  ctx->err = msg;
  return code;
}

int mass_weights_setup(sclet_ctx *ctx, const double *v, const double *vi);
int queue_diagnostics(sclet_ctx *ctx, int energy_form);
int read_diagnostics(sclet_ctx *ctx, sclet_diag *out);

int upload_eigen(sclet_ctx *ctx, const double *d, const double *v, const double *vi) {
  const int n = ctx->n;
  std::vector<double> ds(n);
  for (int ax = 0; ax < 3; ax++) {
    double h = ctx->ph.h[ax];
    // DDX[l] = DDX_b[l] / hx / hx (vars.c:510-513)
    for (int l = 0; l < n; l++) {
      ds[l] = d[l] / h / h;
    }
    CK(cudaMemcpyAsync(ctx->dd[ax], ds.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  if (mixed(ctx)) {
    // the stage block holds the FP64 matrices while they are split
    CK(cudaMemcpyAsync(ctx->stage64, vi, sizeof(double) * n * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(tc_slice_matrix(ctx->stage64, ctx->matVi, ctx->rsVi, n, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpyAsync(ctx->stage64, v, sizeof(double) * n * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(tc_slice_matrix(ctx->stage64, ctx->matV, ctx->rsV, n, ctx->stream));
    const sclet_params &p = ctx->p;
    const double kk[3] = {p.kkx, p.kky, p.kkz};
    for (int kind = 0; kind < 2; kind++)
      CK(tc_make_coefs(ctx->coef[kind], ctx->coef2[kind], n, kind, ctx->dd[0], ctx->dd[1], ctx->dd[2], kk, p.epn2,
                       p.dt, kind == 0 ? ctx->ph.LE : ctx->ph.LCI, kind == 0 ? ctx->ph.KE : ctx->ph.KCI,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->nch > 0) return mass_weights_setup(ctx, v, vi);
    return SCLET_OK;
  }
  for (int ax = 0; ax < 3; ax++) {
    CK(cudaMemcpyAsync(ctx->V[ax], v, sizeof(double) * n * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->Vi[ax], vi, sizeof(double) * n * n, cudaMemcpyHostToDevice, ctx->stream));
  }
  const sclet_params &p = ctx->p;
  const Phys &ph = ctx->ph;  // LE, KE, LCI, KCI from the plugin's init_KL
  phi_kernel<<<grid_of(ctx->n3), 256, 0, ctx->stream>>>(ctx->phi1[0], ctx->phi2[0], n, 0, ctx->dd[0], ctx->dd[1],
                                                        ctx->dd[2], p.kkx, p.kky, p.kkz, p.epn2, p.dt, ph.LE, ph.KE);
  phi_kernel<<<grid_of(ctx->n3), 256, 0, ctx->stream>>>(ctx->phi1[1], ctx->phi2[1], n, 1, ctx->dd[0], ctx->dd[1],
                                                        ctx->dd[2], p.kkx, p.kky, p.kkz, p.epn2, p.dt, ph.LCI, ph.KCI);
  launch_counter() += 2;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ctx->stream));
  return SCLET_OK;
}

EtdCoef etd_coef(sclet_ctx *ctx);

// FP64 mass weights of the conserved field (see k_mass.cu) from the FP64 basis:
// g = column sums of V over the owned rows, V^-T as a row-major matrix.
int mass_weights_setup(sclet_ctx *ctx, const double *v, const double *vi) {
  const int n = ctx->n;
  std::vector<double> g(n, 0.0), viT((size_t)n * n);
  for (int i = 2; i < n - 2; i++)
    for (int q = 0; q < n; q++) g[q] += v[(size_t)i * n + q];
  for (int i = 0; i < n; i++)
    for (int q = 0; q < n; q++) viT[(size_t)i * n + q] = vi[(size_t)q * n + i];
  double *dg = nullptr, *dm = nullptr;
  cudaError_t e = cudaMalloc(&dg, sizeof(double) * n);
  if (e == cudaSuccess) e = cudaMalloc(&dm, sizeof(double) * n * n);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dg, g.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dm, viT.data(), sizeof(double) * n * n, cudaMemcpyHostToDevice, ctx->stream);
  const EtdCoef ec = etd_coef(ctx);
  const int nw = ctx->p.etd2 ? 3 : 2;
  for (int w = 0; w < nw && e == cudaSuccess; w++)
    e = mass_weight(ctx->massW + w * ctx->n3, ctx->stage64, dg, dm, n, w, ec, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(dg);
  cudaFree(dm);
  CK(e);
  return SCLET_OK;
}

EtdCoef etd_coef(sclet_ctx *ctx) {
  EtdCoef ec;
  for (int a = 0; a < 3; a++) ec.dd[a] = ctx->dd[a];
  ec.kk[0] = ctx->p.kkx;
  ec.kk[1] = ctx->p.kky;
  ec.kk[2] = ctx->p.kkz;
  ec.epn2 = ctx->p.epn2;
  ec.dt = ctx->p.dt;
  ec.LE = ctx->ph.LE;
  ec.KE = ctx->ph.KE;
  ec.LCI = ctx->ph.LCI;
  ec.KCI = ctx->ph.KCI;
  ec.nac = ctx->nac;
  ec.F = ctx->F;
  return ec;
}

// Elements of one sliced tensor (TC_PLANES planes of n*n rows of kp)
long long plane_stride(const sclet_ctx *ctx) { return (long long)TC_PLANES * ctx->n * ctx->n * tc_kp(ctx->n); }

void stage_begin(sclet_ctx *ctx, int cls, StageEv &ev) {
  if (!ctx->profiling) return;
  ev.cls = cls;
  cudaEventCreate(&ev.a);
  cudaEventCreate(&ev.b);
  cudaEventRecord(ev.a, ctx->stream);
}
void stage_end(sclet_ctx *ctx, StageEv &ev, long long l0) {
  if (!ctx->profiling) return;
  cudaEventRecord(ev.b, ctx->stream);
  ctx->evs.push_back(ev);
  ctx->stage_launches[ev.cls] += (int)(launch_counter() - l0);
}

int field_index(sclet_ctx *ctx, int kind, int m) {
  if (kind == SCLET_AC && m >= 0 && m < ctx->nac) return m;
  if (kind == SCLET_CH && m >= 0 && m < ctx->nch) return ctx->nac + m;
  return -1;
}

// host FP64 block -> device block of the working precision (FP32 blocks store
// value - shift)
int put_block(sclet_ctx *ctx, const double *host, double *dst64, float *dst32, double shift = 0.0) {
  if (!mixed(ctx)) {
    CK(cudaMemcpyAsync(dst64, host, sizeof(double) * ctx->n3, cudaMemcpyHostToDevice, ctx->stream));
  } else {
    CK(cudaMemcpyAsync(ctx->stage64, host, sizeof(double) * ctx->n3, cudaMemcpyHostToDevice, ctx->stream));
    f64_to_f32<<<grid_of(ctx->n3), 256, 0, ctx->stream>>>(ctx->stage64, dst32, ctx->n3, shift);
    launch_counter()++;
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return SCLET_OK;
}

int get_block(sclet_ctx *ctx, const double *src64, const float *src32, double *host, double shift = 0.0) {
  if (!mixed(ctx)) {
    CK(cudaMemcpyAsync(host, src64, sizeof(double) * ctx->n3, cudaMemcpyDeviceToHost, ctx->stream));
  } else {
    f32_to_f64<<<grid_of(ctx->n3), 256, 0, ctx->stream>>>(src32, ctx->stage64, ctx->n3, shift);
    launch_counter()++;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(host, ctx->stage64, sizeof(double) * ctx->n3, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return SCLET_OK;
}

// staging areas, copy streams and events of the pipelined transfers, on first use
int ensure_io(sclet_ctx *ctx) {
  if (ctx->copy_in) return SCLET_OK;
  const size_t bytes = sizeof(double) * ctx->FT * ctx->n3;
  if (!ctx->in_stage) CK(cudaMalloc(&ctx->in_stage, bytes));
  if (!ctx->out_stage) CK(cudaMalloc(&ctx->out_stage, bytes));
  cudaEvent_t *evs[] = {&ctx->in_ready, &ctx->in_free, &ctx->out_ready, &ctx->out_free};
  for (cudaEvent_t *e : evs)
    if (!*e) CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  // the "free" events start out complete
  CK(cudaEventRecord(ctx->in_free, ctx->stream));
  CK(cudaEventRecord(ctx->out_free, ctx->stream));
  if (!ctx->copy_out) CK(cudaStreamCreateWithFlags(&ctx->copy_out, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&ctx->copy_in, cudaStreamNonBlocking));
  return SCLET_OK;
}

}  // namespace

extern "C" {

int sclet_set_fields_async(sclet_ctx *ctx, const double *host) {
  int rc = ensure_io(ctx);
  if (rc != SCLET_OK) return rc;
  const size_t bytes = sizeof(double) * ctx->FT * ctx->n3;
  CK(cudaStreamWaitEvent(ctx->copy_in, ctx->in_free, 0));
  CK(cudaMemcpyAsync(ctx->in_stage, host, bytes, cudaMemcpyHostToDevice, ctx->copy_in));
  CK(cudaEventRecord(ctx->in_ready, ctx->copy_in));
  CK(cudaStreamWaitEvent(ctx->stream, ctx->in_ready, 0));
  if (mixed(ctx)) {
    fields_to_state<<<dim3(grid_of(ctx->n3), ctx->FT), 256, 0, ctx->stream>>>(ctx->in_stage, fu_of(ctx), ctx->n3,
                                                                             ctx->nac, ctx->ph.cshift, ctx->F);
    launch_counter()++;
    CK(cudaGetLastError());
  } else {
    CK(cudaMemcpyAsync(u_of(ctx), ctx->in_stage, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  CK(cudaEventRecord(ctx->in_free, ctx->stream));
  return SCLET_OK;
}

int sclet_get_fields_async(sclet_ctx *ctx, double *host) {
  int rc = ensure_io(ctx);
  if (rc != SCLET_OK) return rc;
  const size_t bytes = sizeof(double) * ctx->FT * ctx->n3;
  CK(cudaStreamWaitEvent(ctx->stream, ctx->out_free, 0));
  if (mixed(ctx)) {
    fields_from_state<<<dim3(grid_of(ctx->n3), ctx->FT), 256, 0, ctx->stream>>>(fu_of(ctx), ctx->out_stage,
                                                                               ctx->n3, ctx->nac, ctx->ph.cshift,
                                                                               ctx->F);
    launch_counter()++;
    CK(cudaGetLastError());
  } else {
    CK(cudaMemcpyAsync(ctx->out_stage, u_of(ctx), bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  CK(cudaEventRecord(ctx->out_ready, ctx->stream));
  CK(cudaStreamWaitEvent(ctx->copy_out, ctx->out_ready, 0));
  CK(cudaMemcpyAsync(host, ctx->out_stage, bytes, cudaMemcpyDeviceToHost, ctx->copy_out));
  CK(cudaEventRecord(ctx->out_free, ctx->copy_out));
  return SCLET_OK;
}

int sclet_set_fields(sclet_ctx *ctx, const double *host) {
  int rc = sclet_set_fields_async(ctx, host);
  if (rc != SCLET_OK) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return SCLET_OK;
}

int sclet_get_fields(sclet_ctx *ctx, double *host) {
  int rc = sclet_get_fields_async(ctx, host);
  if (rc != SCLET_OK) return rc;
  CK(cudaStreamSynchronize(ctx->copy_out));
  return SCLET_OK;
}

const char *sclet_last_error(const sclet_ctx *ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

int sclet_block_edge(const sclet_ctx *ctx) { return ctx->n; }
int sclet_field_count(const sclet_ctx *ctx) { return ctx->FT; }
void *sclet_stream(const sclet_ctx *ctx) { return (void *)ctx->stream; }
long long sclet_launch_count(const sclet_ctx *ctx) { return launch_counter() - ctx->launches0; }

void sclet_destroy(sclet_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->copy_in) cudaStreamSynchronize(ctx->copy_in);
  if (ctx->copy_out) cudaStreamSynchronize(ctx->copy_out);
  void *bufs[] = {ctx->state2, ctx->rhs2, ctx->A, ctx->B, ctx->felas, ctx->scratch, ctx->shell, ctx->elam,
                  ctx->partials, ctx->phi1[0], ctx->phi1[1], ctx->phi2[0], ctx->phi2[1], ctx->dev_err,
                  ctx->fstate2, ctx->frhs2, ctx->ffelas, ctx->fscratch, ctx->fshell, ctx->W1, ctx->W2, ctx->P,
                  ctx->scaleP, ctx->rsV, ctx->rsVi, ctx->matV, ctx->matVi, ctx->stage64,
                  ctx->coef[0], ctx->coef[1], ctx->coef2[0], ctx->coef2[1], ctx->massW, ctx->massPart,
                  ctx->massRes, ctx->in_stage, ctx->out_stage, ctx->krun, ctx->mob_t, ctx->mob_part};
  for (void *b : bufs) cudaFree(b);
  if (ctx->diag_host) cudaFreeHost(ctx->diag_host);
  for (int a = 0; a < 3; a++) {
    cudaFree(ctx->V[a]);
    cudaFree(ctx->Vi[a]);
    cudaFree(ctx->dd[a]);
  }
  for (auto &e : ctx->evs) {
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  elastic_plan_destroy(ctx->elastic);
  cudaEvent_t ioev[] = {ctx->in_ready, ctx->in_free, ctx->out_ready, ctx->out_free};
  for (cudaEvent_t e : ioev)
    if (e) cudaEventDestroy(e);
  if (ctx->copy_in) cudaStreamDestroy(ctx->copy_in);
  if (ctx->copy_out) cudaStreamDestroy(ctx->copy_out);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int sclet_create(const sclet_params *p, int precision, int device, sclet_ctx **out) {
  return sclet_create_runs(p, 1, nullptr, precision, device, out);
}

int sclet_create_runs(const sclet_params *p, int runs, const double *krun, int precision, int device,
                      sclet_ctx **out) {
  *out = nullptr;
  g_create_error.clear();
  if (runs < 1) {
    g_create_error = "runs must be at least 1";
    return SCLET_ERR_ARG;
  }
  if (runs > 1 && (precision != SCLET_MIXED || p->nch != 0)) {
    g_create_error = "several runs in one context: the mixed form, order parameters only (nch = 0)";
    return SCLET_ERR_UNSUPPORTED;
  }
  auto bad = [&](const char *m) {
    g_create_error = m;
    return SCLET_ERR_ARG;
  };
  if (p->nx != p->ny || p->nx != p->nz) return bad("nx, ny, nz must be equal (one cubic block)");
  if (p->px != 1 || p->py != 1 || p->pz != 1) return bad("one block per GPU: px = py = pz = 1");
  if (p->nghost != 2) return bad("nghost must be 2");
  if (p->periodic != 1) return bad("periodic must be 1 (single block with self-neighbours)");
  if (p->nx < 8 || p->nx > 1028) return bad("block edge out of range [8, 1028]");
  if (p->nac < 0 || p->nac > 4 || p->nch < 0 || p->nch > 1 || p->nac + p->nch < 1)
    return bad("supported: 0..4 Allen-Cahn fields and 0..1 Cahn-Hilliard field");
  if (p->variable_mobility != 0 && p->variable_mobility != 1) return bad("VariableMobility must be 0 or 1");
  if (p->variable_mobility == 1 && (p->nch != 1 || p->nac < 1)) {
    // update_M_C takes the mobility from the first order parameter
    g_create_error = "VariableMobility = 1 needs one Cahn-Hilliard field and at least one Allen-Cahn field";
    return SCLET_ERR_UNSUPPORTED;
  }
  if (p->elastic != 0 && p->elastic != 1) {
    g_create_error = "ELASTIC must be 0 or 1 (elastic force on the Allen-Cahn fields)";
    return SCLET_ERR_UNSUPPORTED;
  }
  if (p->elastic == 1 && p->nac < 1) return bad("ELASTIC = 1 needs Allen-Cahn fields");
  if (precision != SCLET_FP64 && precision != SCLET_MIXED) return bad("precision must be SCLET_FP64 or SCLET_MIXED");
  sclet_ctx *ctx = new sclet_ctx();
  ctx->p = *p;
  ctx->precision = precision;
  ctx->device = device;
  ctx->n = p->nx;
  ctx->nac = p->nac;
  ctx->nch = p->nch;
  ctx->F = p->nac + p->nch;
  ctx->runs = runs;
  ctx->FT = runs * ctx->F;
  ctx->n3 = (long long)ctx->n * ctx->n * ctx->n;
  ctx->launches0 = launch_counter();
  const int n = ctx->n, F = ctx->F, N = n - 4, FT = ctx->FT;
  Phys &ph = ctx->ph;
  memset(&ph, 0, sizeof ph);
  ph.n = n;
  ph.nac = ctx->nac;
  ph.nch = ctx->nch;
  ph.F = F;
  ph.runs = runs;
  ph.anisotropic = p->anisotropic;
  ph.elastic = p->elastic;
  ph.dt = p->dt;
  ph.epn2 = p->epn2;
  // h = (max - min) / gN with gN = n - 2 nghost on one periodic block (vars.c:58-157)
  ph.h[0] = (p->xmax - p->xmin) / N;
  ph.h[1] = (p->ymax - p->ymin) / N;
  ph.h[2] = (p->zmax - p->zmin) / N;
  ph.kk[0] = p->kkx;
  ph.kk[1] = p->kky;
  ph.kk[2] = p->kkz;
  // lambda = diag(kk) - file tensor (anisotropic_input, anisotropic.c:653-672)
  for (int m = 0; m < 4; m++)
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) ph.lam[m][i * 3 + j] = (i == j ? ph.kk[i] : 0.0) - p->lambda_file[m][i * 3 + j];
  ph.elastic_scale = p->elastic_scale;
  // init_KL and the plugin's constants (formula.c:9-19)
  if (const char *why = physics_setup(p, precision, &ph)) {
    g_create_error = why;
    delete ctx;
    return SCLET_ERR_UNSUPPORTED;
  }

  int rc = SCLET_OK;
  cudaError_t e;
#define CC(call)                                                                   \
  if ((e = (call)) != cudaSuccess) {                                               \
    ctx->err = std::string(#call) + ": " + cudaGetErrorString(e);                  \
    rc = e == cudaErrorMemoryAllocation ? SCLET_ERR_NOMEM : SCLET_ERR_CUDA;         \
    g_create_error = ctx->err;                                                     \
    sclet_destroy(ctx);                                                            \
    return rc;                                                                     \
  }
  CC(cudaSetDevice(device));
  CC(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  cudaStream_t s = ctx->stream;
  for (int a = 0; a < 3; a++) CC(cudaMalloc(&ctx->dd[a], sizeof(double) * n));
  CC(cudaMalloc(&ctx->elam, sizeof(double) * 36));
  ctx->npart = check_soln_partials(n);
  CC(cudaMalloc(&ctx->partials, sizeof(double) * ctx->npart * (4 * F + 4) * runs));
  CC(cudaHostAlloc(&ctx->diag_host, sizeof(double) * 4 * FT, cudaHostAllocMapped | cudaHostAllocPortable));
  if (krun) {
    CC(cudaMalloc(&ctx->krun, sizeof(double) * runs));
    CC(cudaMemcpy(ctx->krun, krun, sizeof(double) * runs, cudaMemcpyHostToDevice));
    ph.krun = ctx->krun;
  }
  CC(cudaHostGetDevicePointer(&ctx->diag, ctx->diag_host, 0));
  CC(cudaMalloc(&ctx->dev_err, sizeof(int)));
  CC(cudaMemsetAsync(ctx->dev_err, 0, sizeof(int), s));
  const int nfel = ctx->nac > 0 ? ctx->nac : 1;
  if (!mixed(ctx)) {
    const size_t blk = sizeof(double) * ctx->n3;
    CC(cudaMalloc(&ctx->state2, 2 * F * blk));
    CC(cudaMemsetAsync(ctx->state2, 0, 2 * F * blk, s));
    if (p->etd2) CC(cudaMalloc(&ctx->rhs2, F * blk));
    CC(cudaMalloc(&ctx->A, 2 * F * blk));
    CC(cudaMalloc(&ctx->B, 2 * F * blk));
    CC(cudaMalloc(&ctx->felas, nfel * blk));
    CC(cudaMemsetAsync(ctx->felas, 0, nfel * blk, s));
    CC(cudaMalloc(&ctx->scratch, 2 * blk));
    CC(cudaMalloc(&ctx->shell, sizeof(double) * F * shell_count(n)));
    for (int a = 0; a < 3; a++) {
      CC(cudaMalloc(&ctx->V[a], sizeof(double) * n * n));
      CC(cudaMalloc(&ctx->Vi[a], sizeof(double) * n * n));
    }
    for (int k = 0; k < 2; k++) {
      CC(cudaMalloc(&ctx->phi1[k], blk));
      CC(cudaMalloc(&ctx->phi2[k], blk));
    }
  } else {
    const size_t blk = sizeof(float) * ctx->n3;
    CC(cudaMalloc(&ctx->fstate2, 2 * FT * blk));
    CC(cudaMemsetAsync(ctx->fstate2, 0, 2 * FT * blk, s));
    if (p->etd2) CC(cudaMalloc(&ctx->frhs2, FT * blk));
    CC(cudaMalloc(&ctx->ffelas, nfel * runs * blk));
    CC(cudaMemsetAsync(ctx->ffelas, 0, nfel * runs * blk, s));
    // elastic ghost shells of every run (and the zero block of the first
    // call) or the CH scratch of every run
    CC(cudaMalloc(&ctx->fscratch, (runs + 1) * blk));
    CC(cudaMalloc(&ctx->fshell, sizeof(float) * FT * shell_count(n)));
    CC(cudaMalloc(&ctx->W1, 2 * FT * blk));
    CC(cudaMalloc(&ctx->W2, 2 * FT * blk));
    {
      const size_t pbytes = sizeof(__nv_bfloat16) * plane_stride(ctx) * 2 * FT;
      // pad columns of the slice planes are never written and must stay zero
      CC(cudaMalloc(&ctx->P, pbytes));
      CC(cudaMemsetAsync(ctx->P, 0, pbytes, s));
      CC(cudaMalloc(&ctx->scaleP, sizeof(float) * 2 * FT * n * n));
    }
    CC(cudaMalloc(&ctx->matV, sizeof(__nv_bfloat16) * TC_PLANES_M * n * tc_kp(n)));
    CC(cudaMalloc(&ctx->matVi, sizeof(__nv_bfloat16) * TC_PLANES_M * n * tc_kp(n)));
    CC(cudaMalloc(&ctx->rsV, sizeof(float) * n));
    CC(cudaMalloc(&ctx->rsVi, sizeof(float) * n));
    CC(cudaMalloc(&ctx->stage64, sizeof(double) * ctx->n3));
    for (int k = 0; k < 2; k++) {
      CC(cudaMalloc(&ctx->coef[k], sizeof(float4) * ctx->n3));
      if (p->etd2) CC(cudaMalloc(&ctx->coef2[k], sizeof(float2) * ctx->n3));
    }
    if (ctx->nch > 0) {
      CC(cudaMalloc(&ctx->massW, sizeof(double) * ctx->n3 * (p->etd2 ? 3 : 2)));
      CC(cudaMalloc(&ctx->massPart, sizeof(double) * 4 * mass_partials()));
      CC(cudaMalloc(&ctx->massRes, sizeof(double) * 4));
    }
  }
  if (p->variable_mobility == 1) {
    CC(cudaMalloc(&ctx->mob_t, (mixed(ctx) ? sizeof(float) : sizeof(double)) * 2 * runs * ctx->n3));
    CC(cudaMalloc(&ctx->mob_part, sizeof(double) * (MOB_PARTS + 1) * runs));
    ph.mob_t = ctx->mob_t;
    ph.mob_part = ctx->mob_part;
  }
  {
    // energy tensors: the gradient operator of the dynamics
    double el[36] = {0};
    for (int m = 0; m < 4; m++)
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
          el[m * 9 + i * 3 + j] = p->anisotropic ? p->lambda_file[m][i * 3 + j] : (i == j ? ph.kk[i] : 0.0);
    CC(cudaMemcpyAsync(ctx->elam, el, sizeof el, cudaMemcpyHostToDevice, s));
    CC(cudaStreamSynchronize(s));
  }
  {
    std::vector<double> d(n), v((size_t)n * n), vi((size_t)n * n);
    sclet_eigen_dirichlet(n, d.data(), v.data(), vi.data());
    rc = upload_eigen(ctx, d.data(), v.data(), vi.data());
    if (rc != SCLET_OK) {
      g_create_error = ctx->err;
      sclet_destroy(ctx);
      return rc;
    }
  }
  if (p->elastic == 1) {
    CC(elastic_plan_create(&ctx->elastic, N, ctx->nac, p->voigt, &p->eigenstrain[0][0], mixed(ctx) ? 1 : 0, s, runs));
  }
  CC(cudaStreamSynchronize(s));
#undef CC
  *out = ctx;
  return SCLET_OK;
}

int sclet_set_eigen(sclet_ctx *ctx, const double *d, const double *v, const double *vi) {
  CK(cudaSetDevice(ctx->device));
  return upload_eigen(ctx, d, v, vi);
}

int sclet_set_energy_tensors(sclet_ctx *ctx, const double *lam) {
  double el[36] = {0};
  memcpy(el, lam, sizeof(double) * 9 * ctx->nac);
  CK(cudaMemcpyAsync(ctx->elam, el, sizeof el, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return SCLET_OK;
}

int sclet_set_field(sclet_ctx *ctx, int kind, int m, const double *block) {
  if (ctx->runs > 1) return fail(ctx, SCLET_ERR_UNSUPPORTED, "per-field access to a context of several runs");
  int f = field_index(ctx, kind, m);
  if (f < 0) return fail(ctx, SCLET_ERR_ARG, "no such field");
  return mixed(ctx) ? put_block(ctx, block, nullptr, fu_of(ctx) + f * ctx->n3, f >= ctx->nac ? ctx->ph.cshift : 0.0)
                    : put_block(ctx, block, u_of(ctx) + f * ctx->n3, nullptr);
}

int sclet_get_field(sclet_ctx *ctx, int kind, int m, double *block) {
  if (ctx->runs > 1) return fail(ctx, SCLET_ERR_UNSUPPORTED, "per-field access to a context of several runs");
  int f = field_index(ctx, kind, m);
  if (f < 0) return fail(ctx, SCLET_ERR_ARG, "no such field");
  return mixed(ctx) ? get_block(ctx, nullptr, fu_of(ctx) + f * ctx->n3, block, f >= ctx->nac ? ctx->ph.cshift : 0.0)
                    : get_block(ctx, u_of(ctx) + f * ctx->n3, nullptr, block);
}

// the rank's sub-directory "<dir>00/" of the alpha driver's files
static void make_rank_dir(const char *dir) { mkdir((std::string(dir) + "00").c_str(), 0755); }

int sclet_write_chk(sclet_ctx *ctx, const char *dir, int chk, int irun) {
  if (ctx->runs > 1) return fail(ctx, SCLET_ERR_UNSUPPORTED, "per-field access to a context of several runs");
  std::vector<double> blk(ctx->n3);
  char path[4096];
  make_rank_dir(dir);
  for (int m = 0; m < ctx->nac; m++) {
    int rc = sclet_get_field(ctx, SCLET_AC, m, blk.data());
    if (rc != SCLET_OK) return rc;
    if (sclet_chk_path(path, sizeof path, dir, m, chk) != SCLET_OK) return fail(ctx, SCLET_ERR_ARG, "path too long");
    if (sclet_write_chk_file(path, irun, ctx->n, blk.data()) != SCLET_OK)
      return fail(ctx, SCLET_ERR_IO, std::string("cannot write ") + path);
  }
  return SCLET_OK;
}

int sclet_read_chk(sclet_ctx *ctx, const char *dir, int chk, int *irun) {
  if (ctx->runs > 1) return fail(ctx, SCLET_ERR_UNSUPPORTED, "per-field access to a context of several runs");
  std::vector<double> blk(ctx->n3);
  char path[4096];
  for (int m = 0; m < ctx->nac; m++) {
    if (sclet_chk_path(path, sizeof path, dir, m, chk) != SCLET_OK) return fail(ctx, SCLET_ERR_ARG, "path too long");
    if (sclet_read_chk_file(path, ctx->n, irun, blk.data()) != SCLET_OK)
      return fail(ctx, SCLET_ERR_IO, std::string("cannot read checkpoint ") + path);
    int rc = sclet_set_field(ctx, SCLET_AC, m, blk.data());
    if (rc != SCLET_OK) return rc;
  }
  return SCLET_OK;
}

int sclet_field_u16(sclet_ctx *ctx, int kind, int m, unsigned short *out) {
  if (ctx->runs > 1) return fail(ctx, SCLET_ERR_UNSUPPORTED, "per-field access to a context of several runs");
  int f = field_index(ctx, kind, m);
  if (f < 0) return fail(ctx, SCLET_ERR_ARG, "no such field");
  const int k = kind == SCLET_CH ? 1 : 0;
  // the work block of the context holds the codes (no step is in flight between calls)
  unsigned short *dev = mixed(ctx) ? reinterpret_cast<unsigned short *>(ctx->fscratch)
                                   : reinterpret_cast<unsigned short *>(ctx->scratch);
  if (mixed(ctx))
    CK(launch_field_u16<float>(fu_of(ctx) + f * ctx->n3, k, f >= ctx->nac ? ctx->ph.cshift : 0.0, ctx->n3, dev,
                               ctx->stream));
  else
    CK(launch_field_u16<double>(u_of(ctx) + f * ctx->n3, k, 0.0, ctx->n3, dev, ctx->stream));
  CK(cudaMemcpyAsync(out, dev, sizeof(unsigned short) * ctx->n3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return SCLET_OK;
}

int sclet_write_field2b(sclet_ctx *ctx, const char *data_dir, int irun, int mode) {
  if (ctx->runs > 1) return fail(ctx, SCLET_ERR_UNSUPPORTED, "per-field access to a context of several runs");
  if (mode != 0 && mode != 1) return fail(ctx, SCLET_ERR_ARG, "mode must be 0 (order parameters) or 1 (concentrations)");
  const int kind = mode == 0 ? SCLET_AC : SCLET_CH, count = mode == 0 ? ctx->nac : ctx->nch;
  std::vector<unsigned short> codes(ctx->n3);
  char path[4096];
  make_rank_dir(data_dir);
  for (int m = 0; m < count; m++) {
    int rc = sclet_field_u16(ctx, kind, m, codes.data());
    if (rc != SCLET_OK) return rc;
    if (sclet_field2b_path(path, sizeof path, data_dir, kind, m, irun) != SCLET_OK)
      return fail(ctx, SCLET_ERR_ARG, "path too long");
    FILE *fp = fopen(path, "wb");
    if (!fp) return fail(ctx, SCLET_ERR_IO, std::string("cannot write ") + path);
    const bool ok = fwrite(codes.data(), sizeof(unsigned short), codes.size(), fp) == codes.size();
    if (fclose(fp) != 0 || !ok) return fail(ctx, SCLET_ERR_IO, std::string("cannot write ") + path);
  }
  return SCLET_OK;
}

int sclet_log_soln(sclet_ctx *ctx, const char *work_dir, int iter, int energy_form) {
  if (ctx->runs > 1) return fail(ctx, SCLET_ERR_UNSUPPORTED, "per-field access to a context of several runs");
  std::vector<sclet_diag> d(ctx->nac + ctx->nch);
  int rc = sclet_check_soln(ctx, energy_form, d.data());
  if (rc != SCLET_OK) return rc;
  double couple = d[0].energy;
  if (energy_form != 1 && ctx->nac > 0 && ctx->nch > 0) {
    std::vector<sclet_diag> t(d.size());
    if ((rc = sclet_check_soln(ctx, 1, t.data())) != SCLET_OK) return rc;
    couple = t[0].energy;
  }
  if (sclet_append_soln_log(work_dir, iter, ctx->nac, ctx->nch, d.data(), &couple) != SCLET_OK)
    return fail(ctx, SCLET_ERR_IO, std::string("cannot append the diagnostics logs under ") + work_dir);
  return SCLET_OK;
}

int sclet_write_vtk(sclet_ctx *ctx, const char *path, int istep) {
  if (ctx->runs > 1) return fail(ctx, SCLET_ERR_UNSUPPORTED, "per-field access to a context of several runs");
  std::vector<double> blk((size_t)ctx->nac * ctx->n3);
  for (int m = 0; m < ctx->nac; m++) {
    int rc = sclet_get_field(ctx, SCLET_AC, m, blk.data() + (size_t)m * ctx->n3);
    if (rc != SCLET_OK) return rc;
  }
  if (sclet_write_vtk_file(path, istep, ctx->n, ctx->nac, blk.data()) != SCLET_OK)
    return fail(ctx, SCLET_ERR_IO, std::string("cannot write ") + path);
  return SCLET_OK;
}

int sclet_load_restart(sclet_ctx *ctx, int kind, int m, const char *path) {
  if (ctx->runs > 1) return fail(ctx, SCLET_ERR_UNSUPPORTED, "per-field access to a context of several runs");
  std::vector<double> blk(ctx->n3, 0.0);
  int f = field_index(ctx, kind, m);
  if (f < 0) return fail(ctx, SCLET_ERR_ARG, "no such field");
  int rc = sclet_get_field(ctx, kind, m, blk.data());
  if (rc != SCLET_OK) return rc;
  rc = sclet_read_restart(path, ctx->n, blk.data());
  if (rc != SCLET_OK) return fail(ctx, rc, std::string("cannot read restart file ") + path);
  return sclet_set_field(ctx, kind, m, blk.data());
}

int sclet_get_rhs(sclet_ctx *ctx, int slot, int kind, int m, double *block) {
  if (ctx->runs > 1) return fail(ctx, SCLET_ERR_UNSUPPORTED, "per-field access to a context of several runs");
  int f = field_index(ctx, kind, m);
  bool have2 = mixed(ctx) ? ctx->frhs2 != nullptr : ctx->rhs2 != nullptr;
  if (f < 0 || (slot != 1 && slot != 2) || (slot == 2 && !have2)) return fail(ctx, SCLET_ERR_ARG, "bad rhs slot");
  if (mixed(ctx)) return get_block(ctx, nullptr, (slot == 1 ? frhs1_of(ctx) : ctx->frhs2) + f * ctx->n3, block);
  return get_block(ctx, (slot == 1 ? rhs1_of(ctx) : ctx->rhs2) + f * ctx->n3, nullptr, block);
}

int sclet_get_felas(sclet_ctx *ctx, int m, double *block) {
  if (ctx->runs > 1) return fail(ctx, SCLET_ERR_UNSUPPORTED, "per-field access to a context of several runs");
  if (m < 0 || m >= ctx->nac) return fail(ctx, SCLET_ERR_ARG, "no such field");
  if (mixed(ctx)) return get_block(ctx, nullptr, ctx->ffelas + m * ctx->n3, block);
  return get_block(ctx, ctx->felas + m * ctx->n3, nullptr, block);
}

int sclet_transfer(sclet_ctx *ctx) {
  StageEv ev;
  long long l0 = launch_counter();
  stage_begin(ctx, 3, ev);
  if (mixed(ctx)) CK(launch_ghost_fill<float>(fu_of(ctx), ctx->FT, ctx->n, ctx->fshell, ctx->stream));
  else CK(launch_ghost_fill<double>(u_of(ctx), ctx->F, ctx->n, ctx->shell, ctx->stream));
  stage_end(ctx, ev, l0);
  return SCLET_OK;
}

int sclet_elastic_calculate(sclet_ctx *ctx) {
  if (!ctx->elastic) return SCLET_OK;
  StageEv ev;
  long long l0 = launch_counter();
  stage_begin(ctx, 2, ev);
  if (mixed(ctx))
    CK(elastic_compute<float>(ctx->elastic, fu_of(ctx), ctx->ffelas, ctx->n, ctx->fscratch, ctx->stream,
                              (long long)ctx->F * ctx->n3));
  else
    CK(elastic_compute<double>(ctx->elastic, u_of(ctx), ctx->felas, ctx->n, ctx->scratch, ctx->stream));
  stage_end(ctx, ev, l0);
  return SCLET_OK;
}

int sclet_calc_rhs(sclet_ctx *ctx, int slot) {
  if (slot != 1 && slot != 2) return fail(ctx, SCLET_ERR_ARG, "slot must be 1 or 2");
  if (slot == 2 && !ctx->p.etd2) return fail(ctx, SCLET_ERR_ARG, "slot 2 needs ETD2 = 1");
  StageEv ev;
  long long l0 = launch_counter();
  stage_begin(ctx, 1, ev);
  if (mixed(ctx)) {
    float *dst = slot == 1 ? frhs1_of(ctx) : ctx->frhs2;
    CK(launch_rhs<float>(ctx->ph, fu_of(ctx), ctx->ffelas, dst, ctx->fscratch, ctx->stream));
  } else {
    double *dst = slot == 1 ? rhs1_of(ctx) : ctx->rhs2;
    CK(launch_rhs<double>(ctx->ph, u_of(ctx), ctx->felas, dst, ctx->scratch, ctx->stream));
  }
  stage_end(ctx, ev, l0);
  return SCLET_OK;
}

static TcArgs tc_args(sclet_ctx *ctx, bool inverse, int count, float *out, int epi, const float *aux, int outmode) {
  TcArgs g;
  memset(&g, 0, sizeof g);
  g.n = ctx->n;
  g.count = count;
  g.epi = epi;
  g.outmode = outmode;
  g.aux = aux;
  g.out = out;
  g.row_scale = inverse ? ctx->rsV : ctx->rsVi;
  for (int k = 0; k < 2; k++) {
    g.coef[k] = ctx->coef[k];
    g.coef2[k] = ctx->coef2[k];
  }
  g.nac = ctx->nac;
  g.F = ctx->F;
  g.err = ctx->dev_err;
  g.max_ctas = ctx->ph.tc_ctas;
  return g;
}

// One fixed-point tensor-core product of `count` sliced tensors (planes at
// `planes`, row scales at `scale`) into FP32 `out`.
static cudaError_t tc_prod(sclet_ctx *ctx, bool inverse, const __nv_bfloat16 *planes, const float *scale, int count,
                           float *out, int epi, const float *aux, int outmode) {
  StageEv ev;
  long long l0 = launch_counter();
  stage_begin(ctx, 5, ev);
  TcArgs g = tc_args(ctx, inverse, count, out, epi, aux, outmode);
  g.in_scale = scale;
  cudaError_t e = launch_modeprod_tc(inverse ? ctx->matV : ctx->matVi, planes, count, g, ctx->stream);
  stage_end(ctx, ev, l0);
  return e;
}

// x (count FP32 blocks, minus sub) -> slice planes P and row scales
static cudaError_t tc_slice(sclet_ctx *ctx, const float *x, const float *sub, int count) {
  StageEv ev;
  long long l0 = launch_counter();
  stage_begin(ctx, 6, ev);
  cudaError_t e = tc_slice_fields(x, sub, ctx->scaleP, ctx->P, ctx->n, count, ctx->stream);
  stage_end(ctx, ev, l0);
  return e;
}

// Mixed form of the transforms (ScLETD.c:105-142): V^-1 along x and y for u
// and N1 together, along z for u, then for N1 with the ETD update fused; V
// along x, y, z back to the FP32 state.
static int etd_update_mixed(sclet_ctx *ctx) {
  const int F = ctx->FT;  // every run's fields
  const long long ps = plane_stride(ctx), rows = (long long)ctx->n * ctx->n, n3 = ctx->n3;
  if (ctx->nch > 0)  // target mass of the conserved field from (u, N1)
    CK(mass_target(fu_of(ctx) + ctx->nac * n3, ctx->massW, frhs1_of(ctx) + ctx->nac * n3, nullptr, ctx->massW + n3,
                   ctx->n, ctx->massPart, ctx->stream));
  CK(tc_slice(ctx, ctx->fstate2, nullptr, 2 * F));
  CK(tc_prod(ctx, false, ctx->P, ctx->scaleP, 2 * F, ctx->W1, 0, nullptr, 1));
  CK(tc_slice(ctx, ctx->W1, nullptr, 2 * F));
  CK(tc_prod(ctx, false, ctx->P, ctx->scaleP, 2 * F, ctx->W2, 0, nullptr, 1));
  CK(tc_slice(ctx, ctx->W2, nullptr, 2 * F));
  // uhat into W2 (free once sliced), so that the fused update reads it from a
  // buffer it does not write
  CK(tc_prod(ctx, false, ctx->P, ctx->scaleP, F, ctx->W2, 0, nullptr, 1));
  CK(tc_prod(ctx, false, ctx->P + F * ps, ctx->scaleP + F * rows, F, ctx->W1, 1, ctx->W2, 1));
  CK(tc_slice(ctx, ctx->W1, nullptr, F));
  CK(tc_prod(ctx, true, ctx->P, ctx->scaleP, F, ctx->W2, 0, nullptr, 1));
  CK(tc_slice(ctx, ctx->W2, nullptr, F));
  CK(tc_prod(ctx, true, ctx->P, ctx->scaleP, F, ctx->W1, 0, nullptr, 1));
  CK(tc_slice(ctx, ctx->W1, nullptr, F));
  CK(tc_prod(ctx, true, ctx->P, ctx->scaleP, F, fu_of(ctx), 0, nullptr, 1));
  if (ctx->nch > 0)
    CK(mass_fix(fu_of(ctx) + ctx->nac * n3, ctx->n, ctx->massPart, ctx->massPart + 2 * mass_partials(), ctx->massRes,
                ctx->stream));
  return SCLET_OK;
}

// ETD2 corrector (ScLETD.c:159-188): u += V phi2 V^-1 (N2 - N1).
static int etd2_correct_mixed(sclet_ctx *ctx) {
  const int F = ctx->FT;  // every run's fields
  const long long n3 = ctx->n3, off = ctx->nac * n3;
  if (ctx->nch > 0)  // target: current mass plus <w2, N2 - N1>
    CK(mass_target(fu_of(ctx) + off, nullptr, ctx->frhs2 + off, frhs1_of(ctx) + off, ctx->massW + 2 * n3, ctx->n,
                   ctx->massPart, ctx->stream));
  CK(tc_slice(ctx, ctx->frhs2, frhs1_of(ctx), F));
  CK(tc_prod(ctx, false, ctx->P, ctx->scaleP, F, ctx->W1, 0, nullptr, 1));
  CK(tc_slice(ctx, ctx->W1, nullptr, F));
  CK(tc_prod(ctx, false, ctx->P, ctx->scaleP, F, ctx->W2, 0, nullptr, 1));
  CK(tc_slice(ctx, ctx->W2, nullptr, F));
  CK(tc_prod(ctx, false, ctx->P, ctx->scaleP, F, ctx->W1, 2, nullptr, 1));
  CK(tc_slice(ctx, ctx->W1, nullptr, F));
  CK(tc_prod(ctx, true, ctx->P, ctx->scaleP, F, ctx->W2, 0, nullptr, 1));
  CK(tc_slice(ctx, ctx->W2, nullptr, F));
  CK(tc_prod(ctx, true, ctx->P, ctx->scaleP, F, ctx->W1, 0, nullptr, 1));
  CK(tc_slice(ctx, ctx->W1, nullptr, F));
  CK(tc_prod(ctx, true, ctx->P, ctx->scaleP, F, fu_of(ctx), 0, nullptr, 2));
  if (ctx->nch > 0)
    CK(mass_fix(fu_of(ctx) + off, ctx->n, ctx->massPart, ctx->massPart + 2 * mass_partials(), ctx->massRes,
                ctx->stream));
  return SCLET_OK;
}

int sclet_etd_update(sclet_ctx *ctx) {
  StageEv ev;
  long long l0 = launch_counter();
  stage_begin(ctx, 0, ev);
  if (mixed(ctx)) {
    int rc = etd_update_mixed(ctx);
    if (rc != SCLET_OK) return rc;
    stage_end(ctx, ev, l0);
    return SCLET_OK;
  }
  const int F = ctx->F;
  const long long n3 = ctx->n3;
  EtdCoef ec = etd_coef(ctx);
  set_phi_tables(ctx->phi1[0], ctx->phi1[1], ctx->phi2[0], ctx->phi2[1]);
  cudaStream_t s = ctx->stream;
  // V^-1 along x, y for u and N1 together; along z for u, then for N1 with
  // the ETD1 update fused (uhat in A[0..F) is updated in place).
  CK(launch_modeprod_f64(ctx->Vi[0], ctx->state2, nullptr, ctx->A, nullptr, 2 * F, ctx->n, 0, ec, n3, n3, s));
  CK(launch_modeprod_f64(ctx->Vi[1], ctx->A, nullptr, ctx->B, nullptr, 2 * F, ctx->n, 0, ec, n3, n3, s));
  CK(launch_modeprod_f64(ctx->Vi[2], ctx->B, nullptr, ctx->A, nullptr, F, ctx->n, 0, ec, n3, n3, s));
  CK(launch_modeprod_f64(ctx->Vi[2], ctx->B + F * n3, nullptr, ctx->A, ctx->A, F, ctx->n, 1, ec, n3, n3, s));
  // V along x, y, z back to physical space
  CK(launch_modeprod_f64(ctx->V[0], ctx->A, nullptr, ctx->B, nullptr, F, ctx->n, 0, ec, n3, n3, s));
  CK(launch_modeprod_f64(ctx->V[1], ctx->B, nullptr, ctx->A, nullptr, F, ctx->n, 0, ec, n3, n3, s));
  CK(launch_modeprod_f64(ctx->V[2], ctx->A, nullptr, u_of(ctx), nullptr, F, ctx->n, 0, ec, n3, n3, s));
  stage_end(ctx, ev, l0);
  return SCLET_OK;
}

int sclet_etd2_correct(sclet_ctx *ctx) {
  if (!ctx->p.etd2) return fail(ctx, SCLET_ERR_ARG, "ETD2 = 0");
  StageEv ev;
  long long l0 = launch_counter();
  stage_begin(ctx, 0, ev);
  if (mixed(ctx)) {
    int rc = etd2_correct_mixed(ctx);
    if (rc != SCLET_OK) return rc;
    stage_end(ctx, ev, l0);
    return SCLET_OK;
  }
  const int F = ctx->F;
  const long long n3 = ctx->n3;
  EtdCoef ec = etd_coef(ctx);
  set_phi_tables(ctx->phi1[0], ctx->phi1[1], ctx->phi2[0], ctx->phi2[1]);
  cudaStream_t s = ctx->stream;
  CK(launch_modeprod_f64(ctx->Vi[0], ctx->rhs2, rhs1_of(ctx), ctx->A, nullptr, F, ctx->n, 0, ec, n3, n3, s));
  CK(launch_modeprod_f64(ctx->Vi[1], ctx->A, nullptr, ctx->B, nullptr, F, ctx->n, 0, ec, n3, n3, s));
  CK(launch_modeprod_f64(ctx->Vi[2], ctx->B, nullptr, ctx->A, nullptr, F, ctx->n, 2, ec, n3, n3, s));
  CK(launch_modeprod_f64(ctx->V[0], ctx->A, nullptr, ctx->B, nullptr, F, ctx->n, 0, ec, n3, n3, s));
  CK(launch_modeprod_f64(ctx->V[1], ctx->B, nullptr, ctx->A, nullptr, F, ctx->n, 0, ec, n3, n3, s));
  CK(launch_modeprod_f64(ctx->V[2], ctx->A, nullptr, u_of(ctx), nullptr, F, ctx->n, 3, ec, n3, n3, s));
  stage_end(ctx, ev, l0);
  return SCLET_OK;
}

int sclet_step(sclet_ctx *ctx, int nsteps) {
  int rc;
  CK(cudaSetDevice(ctx->device));
  for (int s = 0; s < nsteps; s++) {
    if ((rc = sclet_transfer(ctx)) != SCLET_OK) return rc;
    if ((rc = sclet_elastic_calculate(ctx)) != SCLET_OK) return rc;
    if ((rc = sclet_calc_rhs(ctx, 1)) != SCLET_OK) return rc;
    if ((rc = sclet_etd_update(ctx)) != SCLET_OK) return rc;
    if (ctx->p.etd2) {
      if ((rc = sclet_transfer(ctx)) != SCLET_OK) return rc;
      if ((rc = sclet_elastic_calculate(ctx)) != SCLET_OK) return rc;
      if ((rc = sclet_calc_rhs(ctx, 2)) != SCLET_OK) return rc;
      if ((rc = sclet_etd2_correct(ctx)) != SCLET_OK) return rc;
    }
    if (ctx->step_diag >= 0 && (rc = queue_diagnostics(ctx, ctx->step_diag)) != SCLET_OK) return rc;
    ctx->steps_done++;
  }
  return SCLET_OK;
}

int sclet_set_step_diagnostics(sclet_ctx *ctx, int energy_form) {
  if (energy_form < -1 || energy_form > 1) return fail(ctx, SCLET_ERR_ARG, "energy_form must be -1, 0 or 1");
  ctx->step_diag = energy_form;
  return SCLET_OK;
}

int sclet_last_diagnostics(sclet_ctx *ctx, sclet_diag *out) { return read_diagnostics(ctx, out); }

int sclet_check_soln(sclet_ctx *ctx, int energy_form, sclet_diag *out) {
  int rc = queue_diagnostics(ctx, energy_form);
  if (rc != SCLET_OK) return rc;
  return read_diagnostics(ctx, out);
}

}  // extern "C"

namespace {
// check_soln_new's reductions on the context's stream into the device record
int queue_diagnostics(sclet_ctx *ctx, int energy_form) {
  StageEv ev;
  long long l0 = launch_counter();
  stage_begin(ctx, 4, ev);
  if (mixed(ctx))
    CK(launch_check_soln<float>(ctx->ph, fu_of(ctx), ctx->elam, energy_form, ctx->partials, ctx->npart, ctx->diag,
                                ctx->stream));
  else
    CK(launch_check_soln<double>(ctx->ph, u_of(ctx), ctx->elam, energy_form, ctx->partials, ctx->npart, ctx->diag,
                                 ctx->stream));
  stage_end(ctx, ev, l0);
  return SCLET_OK;
}

// waits for the stream and copies the last diagnostics record out
int read_diagnostics(sclet_ctx *ctx, sclet_diag *out) {
  CK(cudaStreamSynchronize(ctx->stream));
  const double *h = ctx->diag_host;
  int nonfinite = 0;
  for (int f = 0; f < ctx->FT; f++) {
    out[f].max = h[4 * f];
    out[f].min = h[4 * f + 1];
    out[f].vol = h[4 * f + 2];
    out[f].energy = h[4 * f + 3];
    if (!isfinite(out[f].max) || !isfinite(out[f].min) || !isfinite(out[f].energy)) nonfinite = 1;
  }
  if (nonfinite) return fail(ctx, SCLET_ERR_NONFINITE, "non-finite value in the state");
  return SCLET_OK;
}
}  // namespace

extern "C" {

int sclet_mode_product(sclet_ctx *ctx, int inverse, const double *in, double *out) {
  if (ctx->runs > 1) return fail(ctx, SCLET_ERR_UNSUPPORTED, "per-field access to a context of several runs");
  const long long n3 = ctx->n3;
  if (mixed(ctx)) {
    // in -> FP32 scratch, slices, product, FP32 -> host FP64
    float *tmp = ctx->fscratch;
    CK(cudaMemcpyAsync(ctx->stage64, in, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
    f64_to_f32<<<grid_of(n3), 256, 0, ctx->stream>>>(ctx->stage64, tmp, n3, 0.0);
    launch_counter()++;
    CK(cudaGetLastError());
    CK(tc_slice(ctx, tmp, nullptr, 1));
    CK(tc_prod(ctx, inverse != 0, ctx->P, ctx->scaleP, 1, tmp + n3, 0, nullptr, 1));
    f32_to_f64<<<grid_of(n3), 256, 0, ctx->stream>>>(tmp + n3, ctx->stage64, n3, 0.0);
    launch_counter()++;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, ctx->stage64, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
    return sclet_sync(ctx);
  }
  EtdCoef ec = etd_coef(ctx);
  CK(cudaMemcpyAsync(ctx->A, in, sizeof(double) * n3, cudaMemcpyHostToDevice, ctx->stream));
  CK(launch_modeprod_f64(inverse ? ctx->V[0] : ctx->Vi[0], ctx->A, nullptr, ctx->B, nullptr, 1, ctx->n, 0, ec, n3, n3,
                         ctx->stream));
  CK(cudaMemcpyAsync(out, ctx->B, sizeof(double) * n3, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return SCLET_OK;
}

int sclet_sync(sclet_ctx *ctx) {
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->copy_in) CK(cudaStreamSynchronize(ctx->copy_in));
  if (ctx->copy_out) CK(cudaStreamSynchronize(ctx->copy_out));
  int e = 0;
  CK(cudaMemcpyAsync(&e, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (e) {
    // reported once: the flag starts clear again for the next work
    CK(cudaMemsetAsync(ctx->dev_err, 0, sizeof(int), ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return fail(ctx, SCLET_ERR_TIMEOUT, "a bounded device wait gave up (tensor-core pipeline)");
  }
  return SCLET_OK;
}

int sclet_selftest_wait_timeout(sclet_ctx *ctx) {
  CK(cudaSetDevice(ctx->device));
  if (!mixed(ctx)) return fail(ctx, SCLET_ERR_UNSUPPORTED, "the self-test runs the tensor-core product (mixed form)");
  int rc = sclet_sync(ctx);
  if (rc != SCLET_OK) return rc;
  // one product whose producer issues no loads: the MMA and epilogue warps
  // wait on barriers nothing arrives on, give up, record the error, free
  // their tensor memory and return
  TcArgs g = tc_args(ctx, false, 1, ctx->W1, 0, nullptr, 1);
  g.in_scale = ctx->scaleP;
  g.idle = 1;
  CK(launch_modeprod_tc(ctx->matVi, ctx->P, 1, g, ctx->stream));
  return sclet_sync(ctx);
}

int sclet_set_profiling(sclet_ctx *ctx, int on) {
  ctx->profiling = on != 0;
  return SCLET_OK;
}

int sclet_time_steps(sclet_ctx *ctx, int nsteps, float *ms) {
  cudaEvent_t a, b;
  CK(cudaSetDevice(ctx->device));
  for (auto &e : ctx->evs) {
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  ctx->evs.clear();
  memset(ctx->stage_ms, 0, sizeof ctx->stage_ms);
  memset(ctx->stage_launches, 0, sizeof ctx->stage_launches);
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  CK(cudaEventRecord(a, ctx->stream));
  int rc = sclet_step(ctx, nsteps);
  CK(cudaEventRecord(b, ctx->stream));
  CK(cudaEventSynchronize(b));
  CK(cudaEventElapsedTime(ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  for (auto &e : ctx->evs) {
    float t = 0;
    cudaEventElapsedTime(&t, e.a, e.b);
    ctx->stage_ms[e.cls] += t;
  }
  if (rc == SCLET_OK) rc = sclet_sync(ctx);
  return rc;
}

void *sclet_host_alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
  return p;
}

void sclet_host_free(void *ptr) {
  if (ptr) cudaFreeHost(ptr);
}

int sclet_stage_times(const sclet_ctx *ctx, float *ms, int *launches, int nclasses) {
  for (int k = 0; k < nclasses && k < 8; k++) {
    ms[k] = ctx->stage_ms[k];
    launches[k] = ctx->stage_launches[k];
  }
  return SCLET_OK;
}

}  // extern "C"

// ---- owned cells as FP32 planar device blocks (the learned step) ----------
namespace {
template <typename T>
__global__ void owned_export_kernel(const T *__restrict__ u, float *__restrict__ dst, int n, int nac, double shift,
                                    int F) {
  const int N = n - 4;
  const long long n3 = (long long)N * N * N, b3 = (long long)n * n * n;
  const int f = blockIdx.y;
  const double sh = f % F >= nac ? shift : 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3; i += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(i / ((long long)N * N)), y = (int)((i / N) % N), x = (int)(i % N);
    dst[f * n3 + i] = (float)((double)u[f * b3 + ((long long)(z + 2) * n + y + 2) * n + x + 2] + sh);
  }
}
template <typename T>
__global__ void owned_import_kernel(const float *__restrict__ src, T *__restrict__ u, int n, int nac, double shift,
                                    int F) {
  const int N = n - 4;
  const long long n3 = (long long)N * N * N, b3 = (long long)n * n * n;
  const int f = blockIdx.y;
  const double sh = f % F >= nac ? shift : 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3; i += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(i / ((long long)N * N)), y = (int)((i / N) % N), x = (int)(i % N);
    u[f * b3 + ((long long)(z + 2) * n + y + 2) * n + x + 2] = (T)((double)src[f * n3 + i] - sh);
  }
}
}  // namespace

namespace sclet {
int ctx_export_owned(sclet_ctx *ctx, float *dst) {
  const long long n3 = (long long)(ctx->n - 4) * (ctx->n - 4) * (ctx->n - 4);
  const dim3 grid(grid_of(n3), ctx->FT);
  if (mixed(ctx))
    owned_export_kernel<float><<<grid, 256, 0, ctx->stream>>>(fu_of(ctx), dst, ctx->n, ctx->nac, ctx->ph.cshift,
                                                              ctx->F);
  else
    owned_export_kernel<double><<<grid, 256, 0, ctx->stream>>>(u_of(ctx), dst, ctx->n, ctx->nac, 0.0, ctx->F);
  launch_counter()++;
  CK(cudaGetLastError());
  return SCLET_OK;
}
int ctx_import_owned(sclet_ctx *ctx, const float *src) {
  const long long n3 = (long long)(ctx->n - 4) * (ctx->n - 4) * (ctx->n - 4);
  const dim3 grid(grid_of(n3), ctx->FT);
  if (mixed(ctx))
    owned_import_kernel<float><<<grid, 256, 0, ctx->stream>>>(src, fu_of(ctx), ctx->n, ctx->nac, ctx->ph.cshift,
                                                              ctx->F);
  else
    owned_import_kernel<double><<<grid, 256, 0, ctx->stream>>>(src, u_of(ctx), ctx->n, ctx->nac, 0.0, ctx->F);
  launch_counter()++;
  CK(cudaGetLastError());
  return SCLET_OK;
}
int ctx_device(const sclet_ctx *ctx) { return ctx->device; }
double ctx_dt(const sclet_ctx *ctx) { return ctx->p.dt; }
int ctx_nac(const sclet_ctx *ctx) { return ctx->nac; }
int ctx_fail(sclet_ctx *ctx, int code, const char *msg) {
  ctx->err = msg;
  return code;
}
}  // namespace sclet

// ---- CUDA graphs and the autotuner ------------------------------------------
namespace {
void drop_graph(sclet_ctx *ctx) {
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  ctx->graph_exec = nullptr;
  ctx->graph = nullptr;
}
}  // namespace

namespace sclet {
// one step of ctx captured on its own stream into the capture that stream is
// part of (the caller began it)
int ctx_capture_step(sclet_ctx *ctx) { return sclet_step(ctx, 1); }
long long ctx_steps_done(const sclet_ctx *ctx) { return ctx->steps_done; }
}  // namespace sclet

extern "C" {

int sclet_graph_step(sclet_ctx *ctx, int nsteps) {
  CK(cudaSetDevice(ctx->device));
  if (nsteps <= 0) return SCLET_OK;
  if (ctx->profiling) return fail(ctx, SCLET_ERR_ARG, "graph steps are not profiled per stage");
  if (ctx->steps_done == 0) {
    // the first step has its own set-up (elastic scratch, launch attributes)
    int rc = sclet_step(ctx, 1);
    if (rc != SCLET_OK) return rc;
    nsteps--;
  }
  if (!ctx->graph_exec) {
    const long long before = ctx->steps_done;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
    int rc = sclet_step(ctx, 1);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    ctx->steps_done = before;  // captured, not run
    if (rc != SCLET_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    CK(e);
    ctx->graph = g;
    CK(cudaGraphInstantiate(&ctx->graph_exec, ctx->graph, 0));
  }
  for (int k = 0; k < nsteps; k++) {
    CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    ctx->steps_done++;
  }
  return SCLET_OK;
}

int sclet_tune(sclet_ctx *ctx, int trials, int *choice) {
  CK(cudaSetDevice(ctx->device));
  if (!mixed(ctx)) return fail(ctx, SCLET_ERR_UNSUPPORTED, "the autotuner tunes the mixed form");
  if (trials < 1) trials = 1;
  if (ctx->steps_done == 0) {
    int rc = sclet_step(ctx, 1);
    if (rc != SCLET_OK) return rc;
  }
  // the state and the elastic force (whose ghost cells carry over between
  // steps) are put back after every trial, so tuning changes no result
  const size_t ub = sizeof(float) * ctx->FT * ctx->n3;
  const size_t fb = sizeof(float) * (ctx->nac > 0 ? ctx->nac : 1) * ctx->runs * ctx->n3;
  float *su = nullptr, *sf = nullptr;
  CK(cudaMalloc(&su, ub));
  cudaError_t e = cudaMalloc(&sf, fb);
  if (e != cudaSuccess) {
    cudaFree(su);
    CK(e);
  }
  CK(cudaMemcpyAsync(su, fu_of(ctx), ub, cudaMemcpyDeviceToDevice, ctx->stream));
  CK(cudaMemcpyAsync(sf, ctx->ffelas, fb, cudaMemcpyDeviceToDevice, ctx->stream));
  const int step_diag = ctx->step_diag;
  auto trial = [&](int zc, int ctas, float *ms) -> int {
    ctx->ph.rhs_zc = zc;
    ctx->ph.tc_ctas = ctas;
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    int rc = sclet_step(ctx, 1);  // warm-up of this shape
    CK(cudaEventRecord(a, ctx->stream));
    if (rc == SCLET_OK) rc = sclet_step(ctx, trials);
    CK(cudaEventRecord(b, ctx->stream));
    CK(cudaEventSynchronize(b));
    CK(cudaEventElapsedTime(ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    ctx->steps_done -= trials + 1;
    CK(cudaMemcpyAsync(fu_of(ctx), su, ub, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->ffelas, sf, fb, cudaMemcpyDeviceToDevice, ctx->stream));
    return rc;
  };
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  // coordinate search: z-planes per CTA of the RHS, then the persistent CTAs
  // of the tensor-core products
  const int zcs[] = {8, 16, 32, 64};
  const int ctas[] = {sms, sms * 3 / 4, sms / 2};
  int best_zc = 32, best_ctas = 0, rc = SCLET_OK;
  float best = 1e30f, ms = 0.0f;
  for (int zc : zcs) {
    if ((rc = trial(zc, 0, &ms)) != SCLET_OK) break;
    if (ms < best) best = ms, best_zc = zc;
  }
  best = 1e30f;
  for (int c : ctas) {
    if (rc != SCLET_OK) break;
    if ((rc = trial(best_zc, c, &ms)) != SCLET_OK) break;
    if (ms < best) best = ms, best_ctas = c;
  }
  ctx->step_diag = step_diag;
  ctx->ph.rhs_zc = best_zc;
  ctx->ph.tc_ctas = best_ctas;
  cudaStreamSynchronize(ctx->stream);
  cudaFree(su);
  cudaFree(sf);
  drop_graph(ctx);  // captured launches keep their old shapes
  if (choice) {
    choice[0] = best_zc;
    choice[1] = best_ctas;
  }
  return rc;
}

}  // extern "C"

// ---- FP64 issue rate of the device (the bound of the plain form's stages) ----
namespace {
// eight independent FMA chains per thread; the result is stored so the
// chains are not removed
__global__ void fp64_fma_kernel(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = threadIdx.x * 1e-9 + k;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  if (s == 12345.678) out[0] = s;  // never true for these inputs; keeps the work
}
}  // namespace

extern "C" int sclet_measure_fp64_rate(int device, double *tflops) {
  if (!tflops) return SCLET_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return SCLET_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return SCLET_ERR_CUDA;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return SCLET_ERR_NOMEM;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  float best = 1e30f;
  for (int rep = 0; rep < 4; rep++) {
    cudaEventRecord(a);
    fp64_fma_kernel<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (rep > 0 && ms < best) best = ms;  // the first launch warms up
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (e != cudaSuccess) return SCLET_ERR_CUDA;
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return SCLET_OK;
}
