// The batched ensemble: several contexts (each holding the runs of one block
// size side by side, sclet_create_runs) advanced together, one step of all
// of them captured as one CUDA graph whose branches (one per context, on the
// context's own stream) the GPU runs concurrently.
//
// The reference runs one simulation per process; the ensemble has no
// counterpart there.  Each run's step is the reference's time-loop body
// (source_beta_to_omega/src/ScLETD.c:84-191).
#include <string>
#include <vector>

#include "sclet_gb300.h"
#include "sclet_internal.cuh"

namespace sclet {
int ctx_capture_step(sclet_ctx *ctx);
long long ctx_steps_done(const sclet_ctx *ctx);
int ctx_device(const sclet_ctx *ctx);
int ctx_fail(sclet_ctx *ctx, int code, const char *msg);
}  // namespace sclet

using namespace sclet;

struct sclet_ensemble {
  std::vector<sclet_ctx *> ctx;
  int device = 0;
  cudaStream_t master = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::string err;
};

namespace {

int efail(sclet_ensemble *e, int code, const std::string &msg) {
  e->err = msg;
  return code;
}

#define EK(call)                                                                   \
  do {                                                                             \
    cudaError_t x_ = (call);                                                       \
    if (x_ != cudaSuccess) return efail(e, SCLET_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(x_)); \
  } while (0)

// one step of every context, each on its own stream, forked from and joined
// into the master stream (which the caller may be capturing)
int queue_all(sclet_ensemble *e) {
  EK(cudaEventRecord(e->fork, e->master));
  for (size_t i = 0; i < e->ctx.size(); i++) {
    cudaStream_t s = (cudaStream_t)sclet_stream(e->ctx[i]);
    EK(cudaStreamWaitEvent(s, e->fork, 0));
    int rc = ctx_capture_step(e->ctx[i]);
    if (rc != SCLET_OK) return efail(e, rc, sclet_last_error(e->ctx[i]));
    EK(cudaEventRecord(e->join[i], s));
    EK(cudaStreamWaitEvent(e->master, e->join[i], 0));
  }
  return SCLET_OK;
}

}  // namespace

extern "C" {

int sclet_ensemble_create(sclet_ctx *const *ctxs, int count, sclet_ensemble **out) {
  if (!out || !ctxs || count < 1) return SCLET_ERR_ARG;
  *out = nullptr;
  sclet_ensemble *e = new sclet_ensemble();
  *out = e;
  e->device = ctx_device(ctxs[0]);
  for (int i = 0; i < count; i++) {
    if (!ctxs[i] || ctx_device(ctxs[i]) != e->device) return efail(e, SCLET_ERR_ARG, "contexts on different devices");
    e->ctx.push_back(ctxs[i]);
  }
  EK(cudaSetDevice(e->device));
  EK(cudaStreamCreateWithFlags(&e->master, cudaStreamNonBlocking));
  EK(cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming));
  e->join.resize(count, nullptr);
  for (auto &j : e->join) EK(cudaEventCreateWithFlags(&j, cudaEventDisableTiming));
  return SCLET_OK;
}

void sclet_ensemble_destroy(sclet_ensemble *e) {
  if (!e) return;
  cudaSetDevice(e->device);
  if (e->master) cudaStreamSynchronize(e->master);
  if (e->exec) cudaGraphExecDestroy(e->exec);
  if (e->graph) cudaGraphDestroy(e->graph);
  for (auto j : e->join)
    if (j) cudaEventDestroy(j);
  if (e->fork) cudaEventDestroy(e->fork);
  if (e->master) cudaStreamDestroy(e->master);
  delete e;
}

const char *sclet_ensemble_last_error(const sclet_ensemble *e) { return e ? e->err.c_str() : "null ensemble"; }

int sclet_ensemble_step(sclet_ensemble *e, int nsteps) {
  EK(cudaSetDevice(e->device));
  if (nsteps <= 0) return SCLET_OK;
  // contexts that have not stepped yet take one ordinary step first (their
  // first step has its own set-up), all of them together
  bool fresh = false;
  for (auto *c : e->ctx) fresh = fresh || ctx_steps_done(c) == 0;
  if (fresh) {
    int rc = queue_all(e);
    if (rc != SCLET_OK) return rc;
    nsteps--;
  }
  if (!e->exec) {
    EK(cudaStreamBeginCapture(e->master, cudaStreamCaptureModeRelaxed));
    int rc = queue_all(e);
    cudaGraph_t g = nullptr;
    cudaError_t x = cudaStreamEndCapture(e->master, &g);
    if (rc != SCLET_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    EK(x);
    e->graph = g;
    EK(cudaGraphInstantiate(&e->exec, e->graph, 0));
  }
  for (int k = 0; k < nsteps; k++) EK(cudaGraphLaunch(e->exec, e->master));
  return SCLET_OK;
}

int sclet_ensemble_sync(sclet_ensemble *e) {
  EK(cudaSetDevice(e->device));
  EK(cudaStreamSynchronize(e->master));
  for (auto *c : e->ctx) {
    int rc = sclet_sync(c);
    if (rc != SCLET_OK) return efail(e, rc, sclet_last_error(c));
  }
  return SCLET_OK;
}

int sclet_ensemble_time_steps(sclet_ensemble *e, int nsteps, float *ms) {
  EK(cudaSetDevice(e->device));
  int rc = sclet_ensemble_sync(e);
  if (rc != SCLET_OK) return rc;
  cudaEvent_t a, b;
  EK(cudaEventCreate(&a));
  EK(cudaEventCreate(&b));
  EK(cudaEventRecord(a, e->master));
  rc = sclet_ensemble_step(e, nsteps);
  EK(cudaEventRecord(b, e->master));
  EK(cudaEventSynchronize(b));
  EK(cudaEventElapsedTime(ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc == SCLET_OK) rc = sclet_ensemble_sync(e);
  return rc;
}

}  // extern "C"
