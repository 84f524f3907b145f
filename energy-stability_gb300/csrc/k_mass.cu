// Mass of the conserved (Cahn-Hilliard) field in the mixed-precision form.
//
// The ETD step is linear in the pre-step state u and the right-hand side N:
//   u' = V3 (E . V3^-1 u + phi1 . V3^-1 N)   (ch_updateU_new, calc.c:513-535)
// so the mass the FP64 step would give, M(u') = sum over owned cells of u',
// is a fixed linear functional of (u, N):
//   M(u') = <wE, u> + <wP, N>,  wE = V3^-T (G . E),  wP = V3^-T (G . phi1),
// with G = g x g x g and g[p] = sum over owned rows i of V[i][p]; the ETD2
// corrector (correct_U_new, calc.c:569-583) adds <w2, N2 - N1>, w2 from phi2.
// The weights are computed once in FP64 from the FP64 basis.  Each mixed step
// forms the target from the stored state in FP64 (compensated sums, fixed
// reduction order), then shifts the owned cells of the new state uniformly so
// their FP64 sum meets it.  The FP32 state itself rounds that sum at the level
// of its own storage (about 1e-11 relative at 192^3).
#include "sclet_internal.cuh"

namespace sclet {

namespace {

constexpr int MB = 256;

__device__ inline void two_sum(double a, double b, double &s, double &e) {
  s = a + b;
  double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
struct Ks {
  double s, c;
  __device__ void add(double v) {
    double t, e;
    two_sum(s, v, t, e);
    s = t;
    c += e;
  }
};

// block-wide compensated reduction; thread 0 receives the pair
__device__ Ks block_reduce(Ks v) {
  __shared__ double sa[MB], sb[MB];
  sa[threadIdx.x] = v.s;
  sb[threadIdx.x] = v.c;
  __syncthreads();
  for (int w = MB / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      double s, e;
      two_sum(sa[threadIdx.x], sa[threadIdx.x + w], s, e);
      sa[threadIdx.x] = s;
      sb[threadIdx.x] = sb[threadIdx.x] + sb[threadIdx.x + w] + e;
    }
    __syncthreads();
  }
  Ks r = {sa[0], sb[0]};
  __syncthreads();
  return r;
}

// X[k][j][i] = g[i] g[j] g[k] * coefficient of CH eigen-mode (i, j, k):
// which 0: E = 1 - phi1 H, 1: phi1, 2: phi2 (same FP64 arithmetic as the
// coefficient tables of the mixed form).
__global__ void seed_kernel(double *X, const double *g, int n, int which, const double *dx, const double *dy,
                            const double *dz, double epn2, double dt, double L, double K) {
  const long long n3 = (long long)n * n * n;
  for (long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x; o < n3; o += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(o % n), j = (int)((o / n) % n), k = (int)(o / ((long long)n * n));
    const double tmp = dz[k] + dy[j] + dx[i];
    const double H = L * (tmp * tmp * epn2 - K * tmp);
    double p1, p2;
    if (fabs(H) > 1.0e-8) {
      p1 = -expm1(-dt * H) / H;
      p2 = (1.0 - p1 / dt) / H;
    } else {
      p1 = dt;
      p2 = dt / 2;
    }
    const double Hu = fabs(H) < 1.0e-8 ? 0.0 : H;
    const double c = which == 0 ? 1.0 - p1 * Hu : (which == 1 ? p1 : p2);
    X[o] = g[i] * g[j] * g[k] * c;
  }
}

// Partial target per block: sum of wa*a (or of a over owned cells when wa is
// null) plus sum of wb*(b - bsub).  Rows of x (z*n + y) are spread over the
// grid; each thread accumulates a plain FP64 sum of its cells, and the blocks
// and the final fold are compensated.
__global__ void __launch_bounds__(MB) target_kernel(const float *__restrict__ a, const double *__restrict__ wa,
                                                    const float *__restrict__ b, const float *__restrict__ bsub,
                                                    const double *__restrict__ wb, int n, double *__restrict__ part) {
  const int nrows = n * n;
  double acc = 0.0;
  for (int row = blockIdx.x; row < nrows; row += gridDim.x) {
    const int y = row % n, z = row / n;
    const bool own_row = y >= 2 && y < n - 2 && z >= 2 && z < n - 2;
    const size_t l0 = (size_t)row * n;
    for (int x = threadIdx.x; x < n; x += blockDim.x) {
      const size_t l = l0 + x;
      if (wa) acc += wa[l] * (double)a[l];
      else if (own_row && x >= 2 && x < n - 2) acc += (double)a[l];
      const double d = bsub ? (double)b[l] - (double)bsub[l] : (double)b[l];
      acc += wb[l] * d;
    }
  }
  Ks r = block_reduce(Ks{acc, 0.0});
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = r.s;
    part[2 * blockIdx.x + 1] = r.c;
  }
}

// Partial owned-cell sum of u per block.
__global__ void __launch_bounds__(MB) owned_sum_kernel(const float *__restrict__ u, int n, double *__restrict__ part) {
  double acc = 0.0;
  const int N = n - 4;
  for (int row = blockIdx.x; row < N * N; row += gridDim.x) {
    const int y = 2 + row % N, z = 2 + row / N;
    const size_t l0 = ((size_t)z * n + y) * n + 2;
    for (int x = threadIdx.x; x < N; x += blockDim.x) acc += (double)u[l0 + x];
  }
  Ks r = block_reduce(Ks{acc, 0.0});
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = r.s;
    part[2 * blockIdx.x + 1] = r.c;
  }
}

__device__ double fold(const double *part, int np) {
  Ks acc = {0.0, 0.0};
  for (int q = threadIdx.x; q < np; q += blockDim.x) {
    acc.add(part[2 * q]);
    acc.add(part[2 * q + 1]);
  }
  Ks r = block_reduce(acc);
  return r.s + r.c;
}

// Every block folds both partial sets in the same fixed order, so all blocks
// see the same shift; block 0 records (target, before, shift).
__global__ void __launch_bounds__(MB) shift_kernel(float *__restrict__ u, int n, const double *__restrict__ tpart,
                                                   const double *__restrict__ apart, int np, double *__restrict__ res) {
  __shared__ double delta;
  const double T = fold(tpart, np);
  const double A = fold(apart, np);
  if (threadIdx.x == 0) {
    const double N = n - 4;
    delta = (T - A) / (N * N * N);
    if (blockIdx.x == 0) {
      res[0] = T;
      res[1] = A;
      res[2] = delta;
    }
  }
  __syncthreads();
  const float d = (float)delta;
  const int N = n - 4;
  for (int row = blockIdx.x; row < N * N; row += gridDim.x) {
    const int y = 2 + row % N, z = 2 + row / N;
    const size_t l0 = ((size_t)z * n + y) * n + 2;
    for (int x = threadIdx.x; x < N; x += blockDim.x) u[l0 + x] += d;
  }
}

}  // namespace

int mass_partials() { return 152 * 4; }

cudaError_t mass_weight(double *w, double *tmp, const double *g, const double *viT, int n, int which, const EtdCoef &ec,
                        cudaStream_t s) {
  const long long n3 = (long long)n * n * n;
  long long b = (n3 + 255) / 256;
  seed_kernel<<<(int)(b > 152 * 16 ? 152 * 16 : b), 256, 0, s>>>(w, g, n, which, ec.dd[0], ec.dd[1], ec.dd[2], ec.epn2,
                                                                 ec.dt, ec.LCI, ec.KCI);
  launch_counter()++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // three products with V^-T return to the [k][j][i] layout
  if ((e = launch_modeprod_f64(viT, w, nullptr, tmp, nullptr, 1, n, 0, ec, n3, n3, s)) != cudaSuccess) return e;
  if ((e = launch_modeprod_f64(viT, tmp, nullptr, w, nullptr, 1, n, 0, ec, n3, n3, s)) != cudaSuccess) return e;
  if ((e = launch_modeprod_f64(viT, w, nullptr, tmp, nullptr, 1, n, 0, ec, n3, n3, s)) != cudaSuccess) return e;
  return cudaMemcpyAsync(w, tmp, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s);
}

cudaError_t mass_target(const float *a, const double *wa, const float *b, const float *bsub, const double *wb, int n,
                        double *part, cudaStream_t s) {
  target_kernel<<<mass_partials(), MB, 0, s>>>(a, wa, b, bsub, wb, n, part);
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t mass_fix(float *u, int n, const double *tpart, double *apart, double *res, cudaStream_t s) {
  owned_sum_kernel<<<mass_partials(), MB, 0, s>>>(u, n, apart);
  shift_kernel<<<mass_partials(), MB, 0, s>>>(u, n, tpart, apart, mass_partials(), res);
  launch_counter() += 2;
  return cudaGetLastError();
}

}  // namespace sclet
