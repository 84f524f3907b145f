// Ghost exchange of field blocks on one periodic block (the reference's
// transfer(), source_beta_to_omega/src/trans.c:1939-1996, when every
// Cartesian neighbour is the rank itself).
//
// The reference packs front/back planes, then top/bottom slabs, then
// left/right slabs, all from the block as it stood before the exchange, and
// unpack() (trans.c:154-251) writes left, right, top, bottom, front, back in
// that order.  The net effect is a fixed gather: a ghost cell takes the
// pre-exchange value of its one-axis periodic image along its highest-priority
// ghost axis (z over y over x); the other two coordinates stay as they are,
// so edge and corner ghosts copy other ghost cells' previous values.
//
// Two passes (gather into a compact shell buffer, then scatter) keep the
// in-place update free of read/write races.
#include "sclet_internal.cuh"

namespace sclet {

__device__ inline long long ghost_source(int n, int z, int y, int x) {
  bool gz = z < 2 || z >= n - 2, gy = y < 2 || y >= n - 2;
  if (gz) z = wrap1(n, z);
  else if (gy) y = wrap1(n, y);
  else x = wrap1(n, x);
  return ((long long)z * n + y) * n + x;
}

template <typename T>
__global__ void ghost_gather(const T *__restrict__ u, T *__restrict__ shell, int n, long long ns, int count) {
  long long n3 = (long long)n * n * n;
  long long total = ns * count;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    int t = (int)(i / ns);
    long long s = i - (long long)t * ns;
    int z, y, x;
    shell_cell(n, s, z, y, x);
    shell[i] = u[t * n3 + ghost_source(n, z, y, x)];
  }
}

template <typename T>
__global__ void ghost_scatter(T *__restrict__ u, const T *__restrict__ shell, int n, long long ns, int count) {
  long long n3 = (long long)n * n * n;
  long long total = ns * count;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    int t = (int)(i / ns);
    long long s = i - (long long)t * ns;
    int z, y, x;
    shell_cell(n, s, z, y, x);
    u[t * n3 + ((long long)z * n + y) * n + x] = shell[i];
  }
}

static int grid_for(long long total) {
  long long b = (total + 255) / 256;
  int dev_sms = 152;
  if (b > (long long)dev_sms * 16) b = (long long)dev_sms * 16;
  return (int)(b < 1 ? 1 : b);
}

template <typename T>
cudaError_t launch_ghost_fill(T *u, int count, int n, T *shell, cudaStream_t s) {
  long long ns = shell_count(n);
  int g = grid_for(ns * count);
  ghost_gather<T><<<g, 256, 0, s>>>(u, shell, n, ns, count);
  ghost_scatter<T><<<g, 256, 0, s>>>(u, shell, n, ns, count);
  launch_counter() += 2;
  return cudaGetLastError();
}

// The elastic force is written into one shared scratch block per field p
// (elastic_calculate_ElasDri, elastic.c:617-687): interior = the field's
// result, ghosts = the exchange of that block, whose stale ghost cells still
// hold the previously exchanged field.  felas_p already carries its interior;
// `prev` is the previously exchanged block.  A ghost's source is either an
// interior cell (this field's value) or a ghost cell (prev's value).
template <typename T>
__global__ void elastic_shell_gather(const T *__restrict__ fp, const T *__restrict__ prev, T *__restrict__ shell, int n,
                                     long long ns, long long fstride, long long pstride) {
  // blockIdx.y = run
  fp += blockIdx.y * fstride;
  prev += blockIdx.y * pstride;
  shell += blockIdx.y * ns;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ns; i += (long long)gridDim.x * blockDim.x) {
    int z, y, x;
    shell_cell(n, i, z, y, x);
    bool gz = z < 2 || z >= n - 2, gy = y < 2 || y >= n - 2;
    if (gz) z = wrap1(n, z);
    else if (gy) y = wrap1(n, y);
    else x = wrap1(n, x);
    bool inner = z >= 2 && z < n - 2 && y >= 2 && y < n - 2 && x >= 2 && x < n - 2;
    long long l = ((long long)z * n + y) * n + x;
    shell[i] = inner ? fp[l] : prev[l];
  }
}

// one scatter of the shell of blockIdx.y's run (stride between runs' blocks)
template <typename T>
__global__ void shell_scatter_runs(T *__restrict__ u, const T *__restrict__ shell, int n, long long ns,
                                   long long stride) {
  u += blockIdx.y * stride;
  shell += blockIdx.y * ns;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ns; i += (long long)gridDim.x * blockDim.x) {
    int z, y, x;
    shell_cell(n, i, z, y, x);
    u[((long long)z * n + y) * n + x] = shell[i];
  }
}

template <typename T>
cudaError_t launch_elastic_shell(T *felas_p, const T *prev, int n, T *shell, cudaStream_t s, int runs,
                                 long long fstride, long long pstride) {
  long long ns = shell_count(n);
  const dim3 g(grid_for(ns), runs > 0 ? runs : 1);
  elastic_shell_gather<T><<<g, 256, 0, s>>>(felas_p, prev, shell, n, ns, fstride, pstride);
  shell_scatter_runs<T><<<g, 256, 0, s>>>(felas_p, shell, n, ns, fstride);
  launch_counter() += 2;
  return cudaGetLastError();
}

template cudaError_t launch_ghost_fill<double>(double *, int, int, double *, cudaStream_t);
template cudaError_t launch_ghost_fill<float>(float *, int, int, float *, cudaStream_t);
template cudaError_t launch_elastic_shell<double>(double *, const double *, int, double *, cudaStream_t, int,
                                                  long long, long long);
template cudaError_t launch_elastic_shell<float>(float *, const float *, int, float *, cudaStream_t, int, long long,
                                                 long long);

long long &launch_counter() {
  static long long c = 0;
  return c;
}

}  // namespace sclet
