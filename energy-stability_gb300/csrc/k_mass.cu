// Mass of the conserved (Cahn-Hilliard) field in the mixed-precision form.
//
// The ETD step is linear in the pre-step state u and the right-hand side N:
//   u' = V3 (E . V3^-1 u + phi1 . V3^-1 N)   (ch_updateU_new, calc.c:513-535)
// so the mass the FP64 step would give, M(u') = sum over owned cells of u',
// is a fixed linear functional of (u, N):
//   M(u') = <wE, u> + <wP, N>,  wE = V3^-T (G . E),  wP = V3^-T (G . phi1),
// with G = g x g x g and g[p] = sum over owned rows i of V[i][p]; the ETD2
// corrector (correct_U_new, calc.c:569-583) adds <w2, N2 - N1>, w2 from phi2.
// The weights are computed once in FP64 from the FP64 basis and kept as FP32
// (hi, lo) pairs.  Each mixed step forms the target from the stored state with
// error-free FP32 products and sums per thread (about 48 bits, no FP64
// instructions per cell) and compensated FP64 sums across threads in a fixed
// order, then shifts the owned cells of the new state uniformly so their sum
// meets it.  The FP32 state itself rounds that sum at the level of its own
// storage (about 1e-11 relative at 192^3).
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

// per-thread running sum as an FP32 pair (s, e): s + e carries about 48 bits
struct Fs {
  float s, e;
  __device__ void add(float v) {  // TwoSum (Knuth)
    const float t = s + v, bp = t - s;
    e += (s - (t - bp)) + (v - bp);
    s = t;
  }
  // w * x for a weight pair w (hi, lo): the hi product exactly (FMA), the small terms rounded
  __device__ void add_product(float2 w, float x) {
    const float p = w.x * x;
    add(p);
    e += fmaf(w.x, x, -p) + w.y * x;
  }
  // w * (b - c): the difference as an exact pair, then the products
  __device__ void add_product_diff(float2 w, float b, float c) {
    const float d = b - c, bp = d - b;
    const float dl = (b - (d - bp)) + (-c - bp);  // TwoSum(b, -c) error
    add_product(w, d);
    e += w.x * dl;
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
// grid; each thread accumulates an FP32 pair, and the blocks and the final
// fold are compensated FP64.
__global__ void __launch_bounds__(MB) target_kernel(const float *__restrict__ a, const float2 *__restrict__ wa,
                                                    const float *__restrict__ b, const float *__restrict__ bsub,
                                                    const float2 *__restrict__ wb, int n, double *__restrict__ part) {
  const int nrows = n * n;
  Fs acc = {0.0f, 0.0f};
  for (int row = blockIdx.x; row < nrows; row += gridDim.x) {
    const int z = row / n, y = row - z * n;
    const bool own_row = y >= 2 && y < n - 2 && z >= 2 && z < n - 2;
    const size_t l0 = (size_t)row * n;
    for (int x = threadIdx.x; x < n; x += blockDim.x) {
      const size_t l = l0 + x;
      if (wa) acc.add_product(wa[l], a[l]);
      else if (own_row && x >= 2 && x < n - 2) acc.add(a[l]);
      if (bsub) acc.add_product_diff(wb[l], b[l], bsub[l]);
      else acc.add_product(wb[l], b[l]);
    }
  }
  Ks r = block_reduce(Ks{(double)acc.s, (double)acc.e});
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = r.s;
    part[2 * blockIdx.x + 1] = r.c;
  }
}

// Partial owned-cell sum of u per block.
__global__ void __launch_bounds__(MB) owned_sum_kernel(const float *__restrict__ u, int n, double *__restrict__ part) {
  Fs acc = {0.0f, 0.0f};
  const int N = n - 4;
  for (int row = blockIdx.x; row < N * N; row += gridDim.x) {
    const int zz = row / N, y = 2 + row - zz * N, z = 2 + zz;
    const size_t l0 = ((size_t)z * n + y) * n + 2;
    for (int x = threadIdx.x; x < N; x += blockDim.x) acc.add(u[l0 + x]);
  }
  Ks r = block_reduce(Ks{(double)acc.s, (double)acc.e});
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

// One block folds both partial sets in a fixed order and records (target,
// before, shift) in res.
__global__ void __launch_bounds__(MB) fold_kernel(int n, const double *__restrict__ tpart,
                                                  const double *__restrict__ apart, int np, double *__restrict__ res) {
  const double T = fold(tpart, np);
  const double A = fold(apart, np);
  if (threadIdx.x == 0) {
    const double N = n - 4;
    res[0] = T;
    res[1] = A;
    res[2] = (T - A) / (N * N * N);
  }
}

// the uniform shift res[2] on the owned cells
__global__ void __launch_bounds__(MB) shift_kernel(float *__restrict__ u, int n, const double *__restrict__ res) {
  const float d = (float)res[2];
  const int N = n - 4;
  for (int row = blockIdx.x; row < N * N; row += gridDim.x) {
    const int zz = row / N, y = 2 + row - zz * N, z = 2 + zz;
    const size_t l0 = ((size_t)z * n + y) * n + 2;
    for (int x = threadIdx.x; x < N; x += blockDim.x) u[l0 + x] += d;
  }
}

// FP64 weights -> FP32 (hi, lo) pairs in place
__global__ void to_pairs_kernel(double *w, long long count) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
    const double v = w[i];
    const float hi = (float)v;
    reinterpret_cast<float2 *>(w)[i] = make_float2(hi, (float)(v - (double)hi));
  }
}

}  // namespace

// sixteen blocks per SM: enough loads in flight to stream the block from HBM
int mass_partials() { return 152 * 16; }

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
  if ((e = cudaMemcpyAsync(w, tmp, sizeof(double) * n3, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
  to_pairs_kernel<<<(int)(b > 152 * 16 ? 152 * 16 : b), 256, 0, s>>>(w, n3);
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t mass_target(const float *a, const double *wa, const float *b, const float *bsub, const double *wb, int n,
                        double *part, cudaStream_t s) {
  target_kernel<<<mass_partials(), MB, 0, s>>>(a, reinterpret_cast<const float2 *>(wa), b, bsub,
                                                reinterpret_cast<const float2 *>(wb), n, part);
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t mass_fix(float *u, int n, const double *tpart, double *apart, double *res, cudaStream_t s) {
  owned_sum_kernel<<<mass_partials(), MB, 0, s>>>(u, n, apart);
  fold_kernel<<<1, MB, 0, s>>>(n, tpart, apart, mass_partials(), res);
  shift_kernel<<<mass_partials(), MB, 0, s>>>(u, n, res);
  launch_counter() += 3;
  return cudaGetLastError();
}

}  // namespace sclet
