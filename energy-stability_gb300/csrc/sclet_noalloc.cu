// Diagnostics (check_soln_new, source_beta_to_omega/src/field.c:407-678) of a
// state block the caller already holds on the device, with no allocation of
// any kind: the reduction's partial records and the gradient tensors live in a
// fixed file-scope device array.
//
// Who needs it: a caller that drives its own device memory (a pool or arena
// sized up front, an embedding runtime whose allocator must not be bypassed)
// or that runs the diagnostics between kernels it has already queued, where a
// cudaMalloc would synchronise the whole device and stall its other streams.
// sclet_check_soln needs a context, and creating one allocates the full state.
//
// Limits: at most SCLET_NOALLOC_MAX_FIELDS fields; any block edge the context
// path accepts (the reduction uses at most kMaxParts blocks whatever the size).
// The scratch array is shared by every call on a device: calls that overlap in
// time on one device (different streams, or host threads without ordering)
// race on it and give wrong results; order them on one stream.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/sclet_gb300.h"
#include "sclet_internal.cuh"
#include "sclet_physics.cuh"

namespace sclet {
namespace {

constexpr int kMaxFields = SCLET_NOALLOC_MAX_FIELDS;
constexpr int kMaxParts = 152 * 8;        // check_soln_partials() never asks for more
constexpr int kRecLen = 4 * kMaxFields + 4;  // doubles per partial record
constexpr int kLamOffset = 0;             // 36 doubles: gradient tensors of 4 fields
constexpr int kPartOffset = 64;           // partial records start 512 bytes in
constexpr int kScratchDoubles = kPartOffset + kMaxParts * kRecLen;

// Nothing here has to start at zero: each call writes the gradient tensors and
// every partial record it later reads.
__device__ __align__(256) double g_check_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_scratch_addr[kMaxDevices];  // device address of g_check_scratch, per device
CUcontext g_scratch_ctx[kMaxDevices];  // the context that address belongs to

// The current driver context, through the runtime's driver entry point (no
// link against the driver library); null when it cannot be asked.
CUcontext current_context() {
  static PFN_cuCtxGetCurrent_v4000 fn = nullptr;
  static bool looked = false;
  if (!looked) {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuCtxGetCurrent_v4000)f;
    looked = true;
  }
  CUcontext c = nullptr;
  if (fn && fn(&c) != CUDA_SUCCESS) c = nullptr;
  return c;
}

struct Lam36 {
  double v[36];
};

// The tensors travel as a kernel parameter, so no host-to-device copy is queued.
__global__ void put_lam_kernel(Lam36 lam, double *dst) {
  if (threadIdx.x < 36) dst[threadIdx.x] = lam.v[threadIdx.x];
}

void set_msg(char *msg, size_t len, const char *text) {
  if (msg && len > 0) snprintf(msg, len, "%s", text);
}

// Looks the array's address up once per device, with that device current.
// The first call on a device therefore does this set-up (it may also load the
// module); make that first call before capturing a stream.  A new context on
// the device (after cudaDeviceReset, or a context the caller made current)
// holds its own copy of the array, so the look-up is repeated for it.
int scratch_address(double **out, char *msg, size_t len) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_msg(msg, len, cudaGetErrorString(e));
    return SCLET_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    set_msg(msg, len, "device ordinal beyond the per-device table (64 devices)");
    return SCLET_ERR_ARG;
  }
  // null before the runtime's first use on this thread (the look-up below
  // makes the device's primary context current)
  const CUcontext ctx = current_context();
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev] || !ctx || g_scratch_ctx[dev] != ctx) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_check_scratch);
    if (e != cudaSuccess || !p) {
      char b[256];
      snprintf(b, sizeof b, "cudaGetSymbolAddress of the diagnostics scratch: %s", cudaGetErrorString(e));
      set_msg(msg, len, b);
      return SCLET_ERR_CUDA;
    }
    g_scratch_addr[dev] = static_cast<double *>(p);
    g_scratch_ctx[dev] = current_context();
  }
  *out = g_scratch_addr[dev];
  return SCLET_OK;
}

}  // namespace
}  // namespace sclet

using namespace sclet;

extern "C" int sclet_check_soln_noalloc(const sclet_params *p, int precision, const void *fields, int energy_form,
                                        double *out, void *stream, char *msg, size_t msg_len) {
  set_msg(msg, msg_len, "");
  if (!p || !fields || !out) {
    set_msg(msg, msg_len, "params, fields and out must not be null");
    return SCLET_ERR_ARG;
  }
  if (precision != SCLET_FP64 && precision != SCLET_MIXED) {
    set_msg(msg, msg_len, "precision must be SCLET_FP64 (double fields) or SCLET_MIXED (float fields)");
    return SCLET_ERR_ARG;
  }
  if (energy_form != 0 && energy_form != 1) {
    set_msg(msg, msg_len, "energy_form must be 0 or 1");
    return SCLET_ERR_ARG;
  }
  if (p->nx != p->ny || p->nx != p->nz || p->nx < 8 || p->nx > 1028) {
    set_msg(msg, msg_len, "block edge must be cubic (nx = ny = nz) and within [8, 1028]");
    return SCLET_ERR_ARG;
  }
  const int F = p->nac + p->nch;
  if (p->nac < 0 || p->nac > 4 || p->nch < 0 || p->nch > 1 || F < 1) {
    set_msg(msg, msg_len, "supported: 0..4 Allen-Cahn fields and 0..1 Cahn-Hilliard field");
    return SCLET_ERR_ARG;
  }
  if (F > kMaxFields) {
    char b[160];
    snprintf(b, sizeof b, "%d fields exceed the fixed scratch (at most %d fields)", F, kMaxFields);
    set_msg(msg, msg_len, b);
    return SCLET_ERR_ARG;
  }
  const int n = p->nx, N = n - 4;
  const int npart = check_soln_partials(n);
  if (npart > kMaxParts) {
    set_msg(msg, msg_len, "reduction needs more partial records than the fixed scratch holds");
    return SCLET_ERR_ARG;
  }
  double *scratch = nullptr;
  int rc = scratch_address(&scratch, msg, msg_len);
  if (rc != SCLET_OK) return rc;

  // Geometry and plugin constants as the context path sets them up
  // (init_para, vars.c:58-157; init_KL, formula.c:9-19).
  Phys ph;
  memset(&ph, 0, sizeof ph);
  ph.n = n;
  ph.nac = p->nac;
  ph.nch = p->nch;
  ph.F = F;
  ph.anisotropic = p->anisotropic;
  ph.elastic = p->elastic;
  ph.dt = p->dt;
  ph.epn2 = p->epn2;
  ph.h[0] = (p->xmax - p->xmin) / N;
  ph.h[1] = (p->ymax - p->ymin) / N;
  ph.h[2] = (p->zmax - p->zmin) / N;
  ph.kk[0] = p->kkx;
  ph.kk[1] = p->kky;
  ph.kk[2] = p->kkz;
  // the caller's blocks hold c itself (no stored offset), whatever the precision
  if (const char *why = physics_setup(p, SCLET_FP64, &ph)) {
    set_msg(msg, msg_len, why);
    return SCLET_ERR_UNSUPPORTED;
  }
  // Gradient tensor of each order parameter in the energy: the file tensor
  // when the run is anisotropic, diag(kk) otherwise.
  Lam36 lam;
  for (int m = 0; m < 4; m++)
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        lam.v[m * 9 + i * 3 + j] = p->anisotropic ? p->lambda_file[m][i * 3 + j] : (i == j ? ph.kk[i] : 0.0);

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double *d_lam = scratch + kLamOffset, *d_part = scratch + kPartOffset;
  put_lam_kernel<<<1, 64, 0, s>>>(lam, d_lam);
  launch_counter() += 1;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    if (precision == SCLET_FP64)
      e = launch_check_soln<double>(ph, static_cast<const double *>(fields), d_lam, energy_form, d_part, npart, out, s);
    else
      e = launch_check_soln<float>(ph, static_cast<const float *>(fields), d_lam, energy_form, d_part, npart, out, s);
  }
  if (e != cudaSuccess) {
    set_msg(msg, msg_len, cudaGetErrorString(e));
    return SCLET_ERR_CUDA;
  }
  return SCLET_OK;
}
