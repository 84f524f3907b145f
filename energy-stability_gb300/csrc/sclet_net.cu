// The learned coarse-step corrector: a 3-D residual convolution network
// (BF16 weights and activations, FP32 accumulation and master weights)
// trained and run by the project's own kernels (k_conv.cu, k_conv_train.cu).
//
//   x  (8 channels: the coarse ETD state and the state it started from)
//   h0 = relu(conv0 x + b0)
//   r_k = relu(conv(2k+1) h_k + b), h_{k+1} = h_k + conv(2k+2) r_k + b   (k < 4)
//   y  = (conv9 h_4 + b9) * out_scale   (4 channels: the correction)
//
// The reference has no counterpart: it is the learned part of the target's
// coarse-step form, judged after every step by the plain-ETD checks
// (sclet_learned.cu).
#include <math.h>
#include <string.h>

#include <string>
#include <vector>

#include "sclet_conv.cuh"
#include "sclet_gb300.h"
#include "sclet_internal.cuh"

using namespace sclet;

namespace {

constexpr int LAYERS = 2 + 2 * SCLET_NET_BLOCKS;
constexpr long long WPER = (long long)TAPS * CH * CH;
constexpr long long NPARAM = LAYERS * (WPER + CH);

}  // namespace

struct sclet_net {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  float out_scale = 1.0f;
  long long adam_t = 0;
  int *dev_err = nullptr;
  // FP32 master parameters: weights [LAYERS][TAPS][CH][CH] then biases
  // [LAYERS][CH]; Adam moments and the gradient in the same layout
  float *p = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;
  __nv_bfloat16 *wf = nullptr, *wt = nullptr;  // forward and adjoint BF16 copies
  bool weights_dirty = true;
  // activations for (N, batch): x, h0..h4, r0..r3; gradients: gy, ga, gh0, gh1
  int N = 0, batch = 0;
  long long act_elems = 0;
  __nv_bfloat16 *x = nullptr, *h[SCLET_NET_BLOCKS + 1] = {}, *r[SCLET_NET_BLOCKS] = {};
  __nv_bfloat16 *gy = nullptr, *ga = nullptr, *gh[2] = {nullptr, nullptr};
  float *pred = nullptr, *resid = nullptr;
  double *part = nullptr, *part_host = nullptr;
};

namespace {

constexpr int NPARTS = 152 * 4;

int fail(sclet_net *net, int code, const std::string &msg) {
  net->err = msg;
  return code;
}

#define NK(call)                                                                     \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      net->err = std::string(#call) + ": " + cudaGetErrorString(e_);                 \
      return e_ == cudaErrorMemoryAllocation ? SCLET_ERR_NOMEM : SCLET_ERR_CUDA;     \
    }                                                                                \
  } while (0)

float *wof(float *base, int l) { return base + l * WPER; }
float *bof(float *base, int l) { return base + LAYERS * WPER + l * CH; }
const __nv_bfloat16 *wl(const __nv_bfloat16 *w, int l) { return w + l * WPER; }

void free_acts(sclet_net *net) {
  cudaFree(net->x);
  for (auto &a : net->h) cudaFree(a), a = nullptr;
  for (auto &a : net->r) cudaFree(a), a = nullptr;
  cudaFree(net->gy);
  cudaFree(net->ga);
  cudaFree(net->gh[0]);
  cudaFree(net->gh[1]);
  cudaFree(net->pred);
  cudaFree(net->resid);
  net->x = net->gy = net->ga = net->gh[0] = net->gh[1] = nullptr;
  net->pred = net->resid = nullptr;
  net->N = net->batch = 0;
}

int ensure_acts(sclet_net *net, int N, int batch) {
  if (N == net->N && batch <= net->batch) return SCLET_OK;
  free_acts(net);
  // chunk-planar activations (8 BF16 channels per 16-byte unit); zeroed once,
  // so the padding slots of every chunk read as zeros
  const long long elems = conv_units(N, batch) * 8;
  const size_t bytes = sizeof(__nv_bfloat16) * elems;
  NK(cudaMalloc(&net->x, bytes));
  for (auto &a : net->h) NK(cudaMalloc(&a, bytes));
  for (auto &a : net->r) NK(cudaMalloc(&a, bytes));
  NK(cudaMalloc(&net->gy, bytes));
  NK(cudaMalloc(&net->ga, bytes));
  NK(cudaMalloc(&net->gh[0], bytes));
  NK(cudaMalloc(&net->gh[1], bytes));
  for (__nv_bfloat16 *a : {net->x, net->gy, net->ga, net->gh[0], net->gh[1]})
    NK(cudaMemsetAsync(a, 0, bytes, net->stream));
  for (auto &a : net->h) NK(cudaMemsetAsync(a, 0, bytes, net->stream));
  for (auto &a : net->r) NK(cudaMemsetAsync(a, 0, bytes, net->stream));
  const size_t outb = sizeof(float) * (size_t)SCLET_NET_OUT * N * N * N * batch;
  NK(cudaMalloc(&net->pred, outb));
  NK(cudaMalloc(&net->resid, outb));
  net->N = N;
  net->batch = batch;
  net->act_elems = elems;
  return SCLET_OK;
}

int sync_weights(sclet_net *net) {
  if (!net->weights_dirty) return SCLET_OK;
  NK(launch_conv_weights(net->p, LAYERS, net->wf, net->wt, net->stream));
  net->weights_dirty = false;
  return SCLET_OK;
}

ConvArgs conv_args(sclet_net *net, int N, int batch, int mode, int layer, const __nv_bfloat16 *aux,
                   __nv_bfloat16 *out) {
  ConvArgs a = {};
  a.N = N;
  a.batch = batch;
  a.mode = mode;
  a.bias = layer >= 0 ? bof(net->p, layer) : nullptr;
  a.aux = aux;
  a.out = out;
  a.cout = SCLET_NET_OUT;
  a.scale = net->out_scale;
  a.err = net->dev_err;
  return a;
}

// forward pass into net->pred (or out), keeping every activation
int forward(sclet_net *net, int N, int batch, const float *in, float *out, cudaStream_t s) {
  int rc = ensure_acts(net, N, batch);
  if (rc != SCLET_OK) return rc;
  if ((rc = sync_weights(net)) != SCLET_OK) return rc;
  NK(launch_conv_pack(in, SCLET_NET_IN, N, batch, net->x, s));
  NK(launch_conv(net->x, wl(net->wf, 0), conv_args(net, N, batch, CONV_RELU, 0, nullptr, net->h[0]), s));
  NK(launch_conv_halo(net->h[0], N, batch, s));
  for (int k = 0; k < SCLET_NET_BLOCKS; k++) {
    NK(launch_conv(net->h[k], wl(net->wf, 2 * k + 1),
                   conv_args(net, N, batch, CONV_RELU, 2 * k + 1, nullptr, net->r[k]), s));
    NK(launch_conv_halo(net->r[k], N, batch, s));
    NK(launch_conv(net->r[k], wl(net->wf, 2 * k + 2),
                   conv_args(net, N, batch, CONV_RESIDUAL, 2 * k + 2, net->h[k], net->h[k + 1]), s));
    NK(launch_conv_halo(net->h[k + 1], N, batch, s));
  }
  ConvArgs a = conv_args(net, N, batch, CONV_OUT_F32, LAYERS - 1, nullptr, nullptr);
  a.outf = out ? out : net->pred;
  NK(launch_conv(net->h[SCLET_NET_BLOCKS], wl(net->wf, LAYERS - 1), a, s));
  return SCLET_OK;
}

// loss = mean (pred - target)^2 and the gradient of every parameter (added to net->g)
int backward(sclet_net *net, int N, int batch, const float *target, double *loss, cudaStream_t s) {
  const long long count = (long long)SCLET_NET_OUT * N * N * N * batch;
  NK(launch_residual(net->pred, target, net->resid, count, net->part, NPARTS, s));
  NK(cudaMemcpyAsync(net->part_host, net->part, sizeof(double) * NPARTS, cudaMemcpyDeviceToHost, s));
  // dL/dy = 2 r / count; y = acc * out_scale
  NK(launch_conv_pack_grad(net->resid, SCLET_NET_OUT, (float)(2.0 / (double)count) * net->out_scale, N, batch,
                           net->gy, s));
  const int L = LAYERS - 1;
  NK(launch_conv_wgrad(net->h[SCLET_NET_BLOCKS], net->gy, N, batch, wof(net->g, L), bof(net->g, L), s));
  __nv_bfloat16 *gcur = net->gh[0], *gnext = net->gh[1];
  NK(launch_conv(net->gy, wl(net->wt, L), conv_args(net, N, batch, CONV_LINEAR, -1, nullptr, gcur), s));
  NK(launch_conv_halo(gcur, N, batch, s));
  for (int k = SCLET_NET_BLOCKS - 1; k >= 0; k--) {
    const int l1 = 2 * k + 1, l2 = 2 * k + 2;
    // h_{k+1} = h_k + conv_l2 r_k: gradient of conv_l2's weights, then of r_k
    NK(launch_conv_wgrad(net->r[k], gcur, N, batch, wof(net->g, l2), bof(net->g, l2), s));
    NK(launch_conv(gcur, wl(net->wt, l2), conv_args(net, N, batch, CONV_MASK, -1, net->r[k], net->ga), s));
    NK(launch_conv_halo(net->ga, N, batch, s));
    // r_k = relu(conv_l1 h_k): weights of conv_l1, then h_k (plus the skip path)
    NK(launch_conv_wgrad(net->h[k], net->ga, N, batch, wof(net->g, l1), bof(net->g, l1), s));
    NK(launch_conv(net->ga, wl(net->wt, l1), conv_args(net, N, batch, CONV_RESIDUAL, -1, gcur, gnext), s));
    NK(launch_conv_halo(gnext, N, batch, s));
    __nv_bfloat16 *t = gcur;
    gcur = gnext;
    gnext = t;
  }
  // h0 = relu(conv0 x)
  NK(launch_conv_relu_mask(gcur, net->h[0], N, batch, s));
  NK(launch_conv_wgrad(net->x, gcur, N, batch, wof(net->g, 0), bof(net->g, 0), s));
  NK(cudaStreamSynchronize(s));
  double acc = 0.0;
  for (int i = 0; i < NPARTS; i++) acc += net->part_host[i];
  if (loss) *loss = acc / (double)count;
  int flag = 0;
  NK(cudaMemcpy(&flag, net->dev_err, sizeof flag, cudaMemcpyDeviceToHost));
  if (flag) return fail(net, SCLET_ERR_TIMEOUT, "a bounded wait of the convolution kernel gave up");
  return SCLET_OK;
}

// deterministic initial parameters: He-normal for the ReLU layers, the
// second convolution of each block scaled by 0.1 (blocks start near the
// identity), the output layer zero (the corrector starts as no correction)
void init_params(std::vector<float> &h, unsigned long long seed) {
  h.assign(NPARAM, 0.0f);
  unsigned long long st = seed * 0x9E3779B97F4A7C15ULL + 1;
  auto next = [&]() {
    st += 0x9E3779B97F4A7C15ULL;
    unsigned long long z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l < LAYERS - 1; l++) {
    const int cin = l == 0 ? SCLET_NET_IN : CH;
    const double sd = sqrt(2.0 / (TAPS * cin)) * ((l >= 2 && l % 2 == 0) ? 0.1 : 1.0);
    for (int t = 0; t < TAPS; t++)
      for (int co = 0; co < CH; co++)
        for (int ci = 0; ci < cin; ci++) {
          const double u1 = next(), u2 = next();
          h[l * WPER + ((long long)t * CH + co) * CH + ci] = (float)(sd * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
        }
  }
}

}  // namespace

extern "C" {

long long sclet_net_param_count(void) { return NPARAM; }

int sclet_net_create(int device, unsigned long long seed, float out_scale, sclet_net **out) {
  if (!out) return SCLET_ERR_ARG;
  *out = nullptr;
  sclet_net *net = new sclet_net();
  net->device = device;
  net->out_scale = out_scale;
  auto undo = [&](int code) {
    *out = net;  // the caller reads the message, then destroys
    return code;
  };
#define NC(call)                                                                     \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      net->err = std::string(#call) + ": " + cudaGetErrorString(e_);                 \
      return undo(e_ == cudaErrorMemoryAllocation ? SCLET_ERR_NOMEM : SCLET_ERR_CUDA); \
    }                                                                                \
  } while (0)
  NC(cudaSetDevice(device));
  NC(cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking));
  const size_t pb = sizeof(float) * NPARAM;
  NC(cudaMalloc(&net->p, pb));
  NC(cudaMalloc(&net->m, pb));
  NC(cudaMalloc(&net->v, pb));
  NC(cudaMalloc(&net->g, pb));
  NC(cudaMemsetAsync(net->m, 0, pb, net->stream));
  NC(cudaMemsetAsync(net->v, 0, pb, net->stream));
  NC(cudaMemsetAsync(net->g, 0, pb, net->stream));
  NC(cudaMalloc(&net->wf, sizeof(__nv_bfloat16) * LAYERS * WPER));
  NC(cudaMalloc(&net->wt, sizeof(__nv_bfloat16) * LAYERS * WPER));
  NC(cudaMalloc(&net->dev_err, sizeof(int)));
  NC(cudaMemsetAsync(net->dev_err, 0, sizeof(int), net->stream));
  NC(cudaMalloc(&net->part, sizeof(double) * NPARTS));
  NC(cudaMallocHost(&net->part_host, sizeof(double) * NPARTS));
  std::vector<float> h;
  init_params(h, seed);
  NC(cudaMemcpy(net->p, h.data(), pb, cudaMemcpyHostToDevice));
#undef NC
  *out = net;
  return SCLET_OK;
}

void sclet_net_destroy(sclet_net *net) {
  if (!net) return;
  cudaSetDevice(net->device);
  if (net->stream) cudaStreamSynchronize(net->stream);
  free_acts(net);
  cudaFree(net->p);
  cudaFree(net->m);
  cudaFree(net->v);
  cudaFree(net->g);
  cudaFree(net->wf);
  cudaFree(net->wt);
  cudaFree(net->dev_err);
  cudaFree(net->part);
  if (net->part_host) cudaFreeHost(net->part_host);
  if (net->stream) cudaStreamDestroy(net->stream);
  delete net;
}

const char *sclet_net_last_error(const sclet_net *net) { return net ? net->err.c_str() : "null network"; }

void *sclet_net_stream(const sclet_net *net) { return net ? net->stream : nullptr; }

int sclet_net_get_params(sclet_net *net, float *host) {
  NK(cudaSetDevice(net->device));
  NK(cudaStreamSynchronize(net->stream));
  NK(cudaMemcpy(host, net->p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  return SCLET_OK;
}

int sclet_net_set_params(sclet_net *net, const float *host) {
  NK(cudaSetDevice(net->device));
  NK(cudaStreamSynchronize(net->stream));
  NK(cudaMemcpy(net->p, host, sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
  net->weights_dirty = true;
  return SCLET_OK;
}

int sclet_net_forward(sclet_net *net, int N, int batch, const float *in, float *out) {
  if (!net || !in || !out || N < 4 || batch < 1) return SCLET_ERR_ARG;
  NK(cudaSetDevice(net->device));
  int rc = forward(net, N, batch, in, out, net->stream);
  if (rc != SCLET_OK) return rc;
  return SCLET_OK;
}

int sclet_net_sync(sclet_net *net) {
  NK(cudaSetDevice(net->device));
  NK(cudaStreamSynchronize(net->stream));
  int flag = 0;
  NK(cudaMemcpy(&flag, net->dev_err, sizeof flag, cudaMemcpyDeviceToHost));
  if (flag) return fail(net, SCLET_ERR_TIMEOUT, "a bounded wait of the convolution kernel gave up");
  return SCLET_OK;
}

int sclet_net_gradient(sclet_net *net, int N, int batch, const float *in, const float *target, double *loss,
                       float *grad_host) {
  if (!net || !in || !target || N < 4 || batch < 1) return SCLET_ERR_ARG;
  NK(cudaSetDevice(net->device));
  NK(cudaMemsetAsync(net->g, 0, sizeof(float) * NPARAM, net->stream));
  int rc = forward(net, N, batch, in, nullptr, net->stream);
  if (rc != SCLET_OK) return rc;
  if ((rc = backward(net, N, batch, target, loss, net->stream)) != SCLET_OK) return rc;
  if (grad_host) NK(cudaMemcpy(grad_host, net->g, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  return SCLET_OK;
}

int sclet_net_train_step(sclet_net *net, int N, int batch, const float *in, const float *target, float lr,
                         double *loss) {
  int rc = sclet_net_gradient(net, N, batch, in, target, loss, nullptr);
  if (rc != SCLET_OK) return rc;
  net->adam_t++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = (float)(1.0 / (1.0 - pow(b1, (double)net->adam_t)));
  const float c2 = (float)(1.0 / (1.0 - pow(b2, (double)net->adam_t)));
  NK(launch_adam(net->p, net->m, net->v, net->g, NPARAM, lr, b1, b2, 1e-8f, c1, c2, net->stream));
  net->weights_dirty = true;
  return SCLET_OK;
}

int sclet_net_set_conv_runs(int runs_per_plane) { return conv_set_runs(runs_per_plane); }

}  // extern "C"

namespace sclet {
// for the learned step (sclet_learned.cu): forward on a caller's stream
int net_forward_on(sclet_net *net, int N, int batch, const float *in, float *out, cudaStream_t s) {
  return forward(net, N, batch, in, out, s);
}
int net_device(const sclet_net *net) { return net->device; }
const char *net_error(const sclet_net *net) { return net->err.c_str(); }
}  // namespace sclet
