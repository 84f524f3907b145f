// Khachaturyan elastic driving force on one periodic block (the reference's
// elastic_calculate, source_beta_to_omega/src/elastic.c:617-763, with the
// distributed fftMPI transform of src/fft3d.c:98-138 replaced by a
// single-GPU mixed-radix FFT).
//
//   felas_p = Re IFFT( sum_q B_pq(k) FFT(eta_q) )       on the N^3 owned cells
//   B_pq(n) = C:e0_p:e0_q - (s0_p n) . Om(n) . (s0_q n), Om = (C n n)^-1,
//   n = k/|k| with the reference's wave-number convention (0..N/2-1, -N/2..-1),
//   n = (0,1,0) at k = 0 (elastic_calculate_BN, elastic.c:460-605).
//
// GB300 design: two real fields travel as one complex field (eta_0 + i eta_1,
// eta_2 + i eta_3), so the reference's 2 nac^2 transforms become 2 forward and
// 2 inverse complex transforms.  The reference keeps only the real part of
// each inverse transform; the contraction therefore builds the Hermitian part
// G_p(k) = (F_p(k) + conj F_p(-k)) / 2 of each product spectrum
// F_p = sum_q B_pq H_q (B is not even at the Nyquist planes), whose inverse
// transform is exactly that real part, before packing G_0 + i G_1.
// Each 1D pass keeps tiles of lines in shared memory (Stockham autosort,
// radices 4, 2, 3, 5); lines along y and z are loaded as runs of adjacent x.
#include <mutex>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

#include "sclet_internal.cuh"

namespace sclet {

template <typename T>
struct Cx;
template <>
struct Cx<double> {
  typedef double2 t;
};
template <>
struct Cx<float> {
  typedef float2 t;
};

template <typename C>
__device__ inline C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
template <typename C>
__device__ inline C cadd(C a, C b) {
  C r;
  r.x = a.x + b.x;
  r.y = a.y + b.y;
  return r;
}
template <typename C>
__device__ inline C csub(C a, C b) {
  C r;
  r.x = a.x - b.x;
  r.y = a.y - b.y;
  return r;
}
template <typename C>
__device__ inline C cconj(C a) {
  a.y = -a.y;
  return a;
}

struct Radices {
  int count;
  int r[16];
};

static Radices factor(int n) {
  Radices f;
  f.count = 0;
  while (n % 4 == 0) { f.r[f.count++] = 4; n /= 4; }
  while (n % 2 == 0) { f.r[f.count++] = 2; n /= 2; }
  while (n % 3 == 0) { f.r[f.count++] = 3; n /= 3; }
  while (n % 5 == 0) { f.r[f.count++] = 5; n /= 5; }
  if (n != 1) f.count = -1;
  return f;
}

// One batch of line FFTs over one or two grids (blockIdx.y selects data0 /
// data1).  axis 0: lines along x (contiguous); 1: along y; 2: along z.  sign
// -1 forward, +1 backward (unscaled).  tw[j] = exp(-2 pi i j / N).  A CTA
// keeps 2^ltile lines in shared memory; element-to-line maps use shifts, and
// the per-stage quotients use a float reciprocal, exact for these ranges (a
// quotient's fractional part stays >= 0.5 / divisor away from the next
// integer, far above float rounding at operands below 2^16).
struct StageDiv {
  float inv_nb[16], inv_ns[16];
};

__device__ __forceinline__ int fdiv(int e, float inv) { return __float2int_rd(((float)e + 0.5f) * inv); }

// One Stockham stage of radix R over all lines of the tile (src -> dst).
template <int R, typename C>
__device__ __forceinline__ void fft_stage(const C *__restrict__ src, C *__restrict__ dst, int tile, int N, int Ns,
                                          float inv_nb, float inv_ns, const C *__restrict__ tw, int sign) {
  const int nb = N / R;
  for (int e = threadIdx.x; e < tile * nb; e += blockDim.x) {
    const int line = fdiv(e, inv_nb), j = e - line * nb;
    const int jq = fdiv(j, inv_ns), k = j - jq * Ns;
    const C *s = src + line * N;
    C *d = dst + line * N;
    C v[R];
    // twiddle r k N / (Ns R) < N: no reduction needed
    const int tstep = k * (N / (Ns * R));
#pragma unroll
    for (int r = 0; r < R; r++) {
      v[r] = s[j + r * nb];
      if (r > 0 && k > 0) {
        C w = tw[r * tstep];
        if (sign > 0) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    C o[R];
    if (R == 2) {
      o[0] = cadd(v[0], v[1]);
      o[1] = csub(v[0], v[1]);
    } else if (R == 4) {
      C a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
      C c = cadd(v[1], v[3 % R]), d2 = csub(v[1], v[3 % R]);
      // multiply d2 by -i (forward) or +i (backward)
      C dj;
      if (sign < 0) { dj.x = d2.y; dj.y = -d2.x; }
      else { dj.x = -d2.y; dj.y = d2.x; }
      o[0] = cadd(a, c);
      o[2 % R] = csub(a, c);
      o[1] = cadd(b, dj);
      o[3 % R] = csub(b, dj);
    } else {
#pragma unroll
      for (int q = 0; q < R; q++) {
        C acc = v[0];
#pragma unroll
        for (int r = 1; r < R; r++) {
          C w = tw[((r * q) % R) * nb];
          if (sign > 0) w.y = -w.y;
          acc = cadd(acc, cmul(v[r], w));
        }
        o[q] = acc;
      }
    }
    const int idxD = jq * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) d[idxD + r * Ns] = o[r];
  }
}

template <typename T>
__global__ void __launch_bounds__(256) fft_lines_kernel(typename Cx<T>::t *data0, typename Cx<T>::t *data1, int N,
                                                        int axis, int ltile, const typename Cx<T>::t *__restrict__ tw,
                                                        int sign, Radices rad, StageDiv sd) {
  typedef typename Cx<T>::t C;
  extern __shared__ unsigned char smem_raw[];
  const int tile = 1 << ltile;
  C *buf0 = reinterpret_cast<C *>(smem_raw);
  C *buf1 = buf0 + (size_t)tile * N;
  C *data = blockIdx.y == 0 ? data0 : data1;
  const long long NN = (long long)N * N;
  // Line set of this CTA
  long long base, stride, lstride;
  if (axis == 0) {
    base = (long long)blockIdx.x * tile * N;  // lines indexed by (z*N + y)
    stride = 1;
    lstride = N;
  } else {
    const int ntx = N >> ltile;
    const int xt = blockIdx.x % ntx, w = blockIdx.x / ntx;  // w = z (axis 1) or y (axis 2)
    base = (axis == 1 ? (long long)w * NN : (long long)w * N) + (long long)xt * tile;
    stride = axis == 1 ? N : NN;
    lstride = 1;
  }
  const int total = tile * N;
  if (axis == 0) {
    for (int e = threadIdx.x; e < total; e += blockDim.x) buf0[e] = data[base + e];
  } else {
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
      const int line = e & (tile - 1), pos = e >> ltile;
      buf0[line * N + pos] = data[base + line * lstride + (long long)pos * stride];
    }
  }
  __syncthreads();
  C *src = buf0, *dst = buf1;
  int Ns = 1;
  for (int st = 0; st < rad.count; st++) {
    const int R = rad.r[st];
    const float inb = sd.inv_nb[st], ins = sd.inv_ns[st];
    switch (R) {
      case 4: fft_stage<4, C>(src, dst, tile, N, Ns, inb, ins, tw, sign); break;
      case 2: fft_stage<2, C>(src, dst, tile, N, Ns, inb, ins, tw, sign); break;
      case 3: fft_stage<3, C>(src, dst, tile, N, Ns, inb, ins, tw, sign); break;
      default: fft_stage<5, C>(src, dst, tile, N, Ns, inb, ins, tw, sign); break;
    }
    __syncthreads();
    C *t = src;
    src = dst;
    dst = t;
    Ns *= R;
  }
  if (axis == 0) {
    for (int e = threadIdx.x; e < total; e += blockDim.x) data[base + e] = src[e];
  } else {
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
      const int line = e & (tile - 1), pos = e >> ltile;
      data[base + line * lstride + (long long)pos * stride] = src[line * N + pos];
    }
  }
}

// ---- FP32 fast path: line FFTs of N = N1 * N2 points in two register passes
//
// X[k1 + N1 k2] = sum_t W_N2^(t k2) W_N^(t k1) sum_n1 x[t + N2 n1] W_N1^(n1 k1)
//
// Pass A: thread t of a line loads x[t + N2 n1] (n1 < N1), transforms them in
// registers, applies W_N^(t k1) and writes the N1 results to shared memory.
// Pass B: thread k1 reads the N2 values of its column, transforms them in
// registers and stores X[k1 + N1 k2].  Each element crosses shared memory
// once; the small transforms use constant twiddles (c_wr below).
namespace fft2 {

// exp(-2 pi i m / R) at index R (R - 1) / 2 + m, for R <= 32
__constant__ float2 c_wr[528];

template <int R, int SIGN>
__device__ __forceinline__ float2 wc(int m) {
  float2 w = c_wr[R * (R - 1) / 2 + m];
  if (SIGN > 0) w.y = -w.y;
  return w;
}

// v * (-i) for the forward sign, v * (+i) for the backward one
template <int SIGN>
__device__ __forceinline__ float2 rot(float2 v) {
  float2 r;
  if (SIGN < 0) { r.x = v.y; r.y = -v.x; }
  else { r.x = -v.y; r.y = v.x; }
  return r;
}

template <int R>
struct First {
  static constexpr int v = (R % 4 == 0 && R > 4) ? 4 : (R % 2 == 0 && R > 2) ? 2 : (R % 3 == 0 && R > 3) ? 3 : R;
};

// In-register DFT of R points, natural order in and out.  Composite R = A B:
// A-point transforms over the stride-B subsequences, twiddles W_R^(b ka),
// B-point transforms across them.
template <int R, int SIGN>
struct Dft {
  static __device__ __forceinline__ void run(float2 (&v)[R]) {
    constexpr int A = First<R>::v, B = R / A;
    static_assert(A < R, "unsupported transform length");
    float2 y[B][A];
#pragma unroll
    for (int b = 0; b < B; b++) {
      float2 u[A];
#pragma unroll
      for (int a = 0; a < A; a++) u[a] = v[b + B * a];
      Dft<A, SIGN>::run(u);
#pragma unroll
      for (int ka = 0; ka < A; ka++) y[b][ka] = (b * ka == 0) ? u[ka] : cmul(u[ka], wc<R, SIGN>(b * ka));
    }
#pragma unroll
    for (int ka = 0; ka < A; ka++) {
      float2 w[B];
#pragma unroll
      for (int b = 0; b < B; b++) w[b] = y[b][ka];
      Dft<B, SIGN>::run(w);
#pragma unroll
      for (int kb = 0; kb < B; kb++) v[ka + A * kb] = w[kb];
    }
  }
};
template <int SIGN>
struct Dft<1, SIGN> {
  static __device__ __forceinline__ void run(float2 (&)[1]) {}
};
template <int SIGN>
struct Dft<2, SIGN> {
  static __device__ __forceinline__ void run(float2 (&v)[2]) {
    const float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};
template <int SIGN>
struct Dft<3, SIGN> {
  static __device__ __forceinline__ void run(float2 (&v)[3]) {
    const float s3 = 0.86602540378443864676f;  // sin(2 pi / 3)
    const float2 t1 = cadd(v[1], v[2]);
    float2 t2, d = csub(v[1], v[2]);
    t2.x = v[0].x - 0.5f * t1.x;
    t2.y = v[0].y - 0.5f * t1.y;
    d.x *= s3;
    d.y *= s3;
    const float2 t3 = rot<SIGN>(d);
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
  }
};
template <int SIGN>
struct Dft<4, SIGN> {
  static __device__ __forceinline__ void run(float2 (&v)[4]) {
    const float2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    const float2 c = cadd(v[1], v[3]), d = rot<SIGN>(csub(v[1], v[3]));
    v[0] = cadd(a, c);
    v[2] = csub(a, c);
    v[1] = cadd(b, d);
    v[3] = csub(b, d);
  }
};
template <int SIGN>
struct Dft<5, SIGN> {
  static __device__ __forceinline__ void run(float2 (&v)[5]) {
    float2 o[5];
#pragma unroll
    for (int q = 0; q < 5; q++) {
      float2 acc = v[0];
#pragma unroll
      for (int r = 1; r < 5; r++) acc = cadd(acc, cmul(v[r], wc<5, SIGN>((r * q) % 5)));
      o[q] = acc;
    }
#pragma unroll
    for (int q = 0; q < 5; q++) v[q] = o[q];
  }
};

// Grids and blocks of one elastic call.  io 1 (first forward x-pass): lines
// are read from the order parameters (grid y = q holds eta_2q + i eta_2q+1 of
// the owned cells) instead of data; io 2 (last inverse x-pass): the real and
// imaginary parts, scaled by 1 / N^3, go to felas_2q and felas_2q+1.
struct LineIO {
  const float *u;  // order parameters, nac blocks of n^3
  float *felas;    // elastic force, nac blocks of n^3
  int n, nac;
  long long n3;
  float scale;     // 1 / N^3
  // runs side by side: run r's grids at r N^3 of data0 / data1, its order
  // parameters at u + r ustride, its force at felas + r fstride
  int runs;
  long long ustride, fstride;
};

// L lines per CTA.  axis 0: lines along x, lane order over t (pass A) and k1
// (pass B); axes 1 and 2: L adjacent x-lines, lane order over x.
template <int N1, int N2, int L, int AXIS, int SIGN, int IO>
__global__ void __launch_bounds__(L *(N1 > N2 ? N1 : N2))
    lines_kernel(float2 *data0, float2 *data1, const float2 *__restrict__ tw, LineIO io) {
  static_assert(IO == 0 || AXIS == 0, "fused packing on x-passes only");
  constexpr int N = N1 * N2;
  constexpr int RS = AXIS == 0 ? N2 + 1 : N2;  // row stride of a line's table (padded on axis 0)
  extern __shared__ float2 tab[];
  // blockIdx.y = run x (grid pair 0 or 1)
  const int per = data1 != data0 ? 2 : 1;
  const int run = blockIdx.y / per, pair = blockIdx.y - run * per;
  const long long NN = (long long)N * N;
  float2 *data = (pair == 0 ? data0 : data1) + (long long)run * NN * N;
  io.u += run * io.ustride;
  io.felas += run * io.fstride;
  const int tid = threadIdx.x;
  long long base;
  long long ps;  // element stride along the line
  if (AXIS == 0) {
    base = (long long)blockIdx.x * L * N;
    ps = 1;
  } else {
    constexpr int ntx = N / L;
    const int xt = blockIdx.x % ntx, w = blockIdx.x / ntx;  // w = z (axis 1) or y (axis 2)
    base = (AXIS == 1 ? (long long)w * NN : (long long)w * N) + (long long)xt * L;
    ps = AXIS == 1 ? N : NN;
  }
  auto at = [&](int l, int k1, int t) -> int {
    return AXIS == 0 ? (l * N1 + k1) * RS + t : (k1 * N2 + t) * L + l;
  };
  // owned-cell offset of this CTA's line l in an n^3 block (io != 0)
  auto cell0 = [&](int l) -> long long {
    const int gl = blockIdx.x * L + l, z = gl / N, y = gl - z * N;
    return ((long long)(z + 2) * io.n + (y + 2)) * io.n + 2;
  };
  const int f0 = 2 * pair;
  if (tid < L * N2) {
    const int l = AXIS == 0 ? tid / N2 : tid % L, t = AXIS == 0 ? tid % N2 : tid / L;
    float2 v[N1];
    if (IO == 1) {
      const float *re = io.u + f0 * io.n3 + cell0(l);
      const float *im = f0 + 1 < io.nac ? re + io.n3 : nullptr;
#pragma unroll
      for (int n1 = 0; n1 < N1; n1++) v[n1] = make_float2(re[t + N2 * n1], im ? im[t + N2 * n1] : 0.0f);
    } else {
      const float2 *src = data + base + (AXIS == 0 ? (long long)l * N : (long long)l);
#pragma unroll
      for (int n1 = 0; n1 < N1; n1++) v[n1] = src[(long long)(t + N2 * n1) * ps];
    }
    Dft<N1, SIGN>::run(v);
#pragma unroll
    for (int k1 = 0; k1 < N1; k1++) {
      float2 r = v[k1];
      if (k1 > 0 && t > 0) {
        float2 w = tw[t * k1];  // t k1 < N
        if (SIGN > 0) w.y = -w.y;
        r = cmul(r, w);
      }
      tab[at(l, k1, t)] = r;
    }
  }
  __syncthreads();
  if (tid < L * N1) {
    const int l = AXIS == 0 ? tid / N1 : tid % L, k1 = AXIS == 0 ? tid % N1 : tid / L;
    float2 v[N2];
#pragma unroll
    for (int t = 0; t < N2; t++) v[t] = tab[at(l, k1, t)];
    Dft<N2, SIGN>::run(v);
    if (IO == 2) {
      float *re = io.felas + f0 * io.n3 + cell0(l);
      float *im = f0 + 1 < io.nac ? re + io.n3 : nullptr;
#pragma unroll
      for (int k2 = 0; k2 < N2; k2++) {
        re[k1 + N1 * k2] = v[k2].x * io.scale;
        if (im) im[k1 + N1 * k2] = v[k2].y * io.scale;
      }
    } else {
      float2 *dst = data + base + (AXIS == 0 ? (long long)l * N : (long long)l);
#pragma unroll
      for (int k2 = 0; k2 < N2; k2++) dst[(long long)(k1 + N1 * k2) * ps] = v[k2];
    }
  }
}

// lines per CTA: 16, or 8 for lines beyond 256 points (256 threads per CTA)
template <int N1, int N2>
constexpr int lines_per_cta() {
  return N1 * N2 > 256 ? 8 : 16;
}

template <int N1, int N2>
constexpr size_t smem_bytes(int axis) {
  return sizeof(float2) * lines_per_cta<N1, N2>() * N1 * (axis == 0 ? N2 + 1 : N2);
}

template <int N1, int N2, int AXIS, int SIGN, int IO>
static cudaError_t launch_one(float2 *z0, float2 *z1, const float2 *tw, const LineIO &io, cudaStream_t s) {
  constexpr int N = N1 * N2, L = lines_per_cta<N1, N2>();
  constexpr size_t sm = smem_bytes<N1, N2>(AXIS);
  auto k = lines_kernel<N1, N2, L, AXIS, SIGN, IO>;
  if (sm > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
  }
  const int runs = io.runs > 0 ? io.runs : 1;
  const dim3 grid((unsigned)((long long)N * N / L), (z1 ? 2u : 1u) * runs);
  k<<<grid, L * (N1 > N2 ? N1 : N2), sm, s>>>(z0, z1 ? z1 : z0, tw, io);
  return cudaGetLastError();
}

// forward: x (reading the order parameters), y, z; inverse: z, y, x (writing felas)
template <int N1, int N2>
static cudaError_t launch_pass(int sign, int k, float2 *z0, float2 *z1, const float2 *tw, const LineIO &io,
                               cudaStream_t s) {
  if (sign < 0) {
    switch (k) {
      case 0: return launch_one<N1, N2, 0, -1, 1>(z0, z1, tw, io, s);
      case 1: return launch_one<N1, N2, 1, -1, 0>(z0, z1, tw, io, s);
      default: return launch_one<N1, N2, 2, -1, 0>(z0, z1, tw, io, s);
    }
  }
  switch (k) {
    case 0: return launch_one<N1, N2, 2, 1, 0>(z0, z1, tw, io, s);
    case 1: return launch_one<N1, N2, 1, 1, 0>(z0, z1, tw, io, s);
    default: return launch_one<N1, N2, 0, 1, 2>(z0, z1, tw, io, s);
  }
}

// N = 16 N1 with N1 in {2, 3, 4, 5, 6, 8, 10, 12, 16, 32}; 0 if N has no fast path
static int pass_n1(int N) {
  static const int ok[] = {2, 3, 4, 5, 6, 8, 10, 12, 16, 32};
  if (N % 16) return 0;
  for (int n1 : ok)
    if (n1 * 16 == N) return n1;
  return 0;
}

// pass k (0..2) of the forward (sign -1) or inverse (+1) 3-D transform
static cudaError_t launch(int N, int sign, int k, float2 *z0, float2 *z1, const float2 *tw, const LineIO &io,
                          cudaStream_t s) {
  switch (pass_n1(N)) {
    case 2: return launch_pass<2, 16>(sign, k, z0, z1, tw, io, s);
    case 3: return launch_pass<3, 16>(sign, k, z0, z1, tw, io, s);
    case 4: return launch_pass<4, 16>(sign, k, z0, z1, tw, io, s);
    case 5: return launch_pass<5, 16>(sign, k, z0, z1, tw, io, s);
    case 6: return launch_pass<6, 16>(sign, k, z0, z1, tw, io, s);
    case 8: return launch_pass<8, 16>(sign, k, z0, z1, tw, io, s);
    case 10: return launch_pass<10, 16>(sign, k, z0, z1, tw, io, s);
    case 12: return launch_pass<12, 16>(sign, k, z0, z1, tw, io, s);
    case 16: return launch_pass<16, 16>(sign, k, z0, z1, tw, io, s);
    default: return launch_pass<32, 16>(sign, k, z0, z1, tw, io, s);
  }
}

// fills c_wr on the current device
static cudaError_t upload_constants(cudaStream_t s) {
  std::vector<float2> h(528);
  for (int R = 1; R <= 32; R++)
    for (int m = 0; m < R; m++) {
      const double a = -2.0 * 3.14159265358979323846 * (double)m / (double)R;
      h[R * (R - 1) / 2 + m] = make_float2((float)cos(a), (float)sin(a));
    }
  cudaError_t e = cudaMemcpyToSymbolAsync(c_wr, h.data(), sizeof(float2) * 528, 0, cudaMemcpyHostToDevice, s);
  return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
}

}  // namespace fft2

// eta pairs -> complex grids (owned cells of the n^3 blocks, n = N + 4).
// The element-wise kernels below run over rows (y, z) of the grid, one CTA
// per row at a time and threads along x: no per-element index division.
template <typename T>
__global__ void pack_kernel(const T *__restrict__ u, typename Cx<T>::t *__restrict__ z01,
                            typename Cx<T>::t *__restrict__ z23, int N, int nac) {
  const int n = N + 4;
  const long long n3 = (long long)n * n * n;
  for (int row = blockIdx.x; row < N * N; row += gridDim.x)
  for (int x = threadIdx.x; x < N; x += blockDim.x) {
    const int z = row / N, y = row - z * N;
    const long long g = (long long)row * N + x;
    long long l = ((long long)(z + 2) * n + (y + 2)) * n + (x + 2);
    T v[4];
    for (int q = 0; q < 4; q++) v[q] = q < nac ? u[q * n3 + l] : (T)0;
    typename Cx<T>::t a, b;
    a.x = v[0]; a.y = v[1];
    b.x = v[2]; b.y = v[3];
    z01[g] = a;
    if (z23) z23[g] = b;
  }
}

__host__ __device__ inline int pq_slot(int p, int q) {
  if (p > q) { int t = p; p = q; q = t; }
  // (0,0)0 (0,1)1 (0,2)2 (0,3)3 (1,1)4 (1,2)5 (1,3)6 (2,2)7 (2,3)8 (3,3)9
  return p * 4 - p * (p - 1) / 2 + (q - p);
}

// Green-tensor kernel on the full grid, 10 symmetric slots (FP64, once).
struct BnConst {
  double C[81];
  double sig[4][9];
  double t0[10];
};

template <typename B>
__global__ void bn_kernel(B *__restrict__ bn, int N, BnConst bc) {
  const long long N3 = (long long)N * N * N;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < N3; g += (long long)gridDim.x * blockDim.x) {
    int x = (int)(g % N), y = (int)((g / N) % N), z = (int)(g / ((long long)N * N));
    double kx = x < N / 2 ? (double)x : -(double)(N - x);
    double ky = y < N / 2 ? (double)y : -(double)(N - y);
    double kz = z < N / 2 ? (double)z : -(double)(N - z);
    double nv[3];
    if (x == 0 && y == 0 && z == 0) {
      nv[0] = 0.0; nv[1] = 1.0; nv[2] = 0.0;
    } else {
      double r = sqrt(kx * kx + ky * ky + kz * kz);
      nv[0] = kx / r; nv[1] = ky / r; nv[2] = kz / r;
    }
    double a[9];
    for (int i = 0; i < 3; i++)
      for (int k = 0; k < 3; k++) {
        double s = 0.0;
        for (int j = 0; j < 3; j++)
          for (int l = 0; l < 3; l++) s += bc.C[((i * 3 + j) * 3 + k) * 3 + l] * nv[j] * nv[l];
        a[i * 3 + k] = s;
      }
    double det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
                 a[2] * (a[3] * a[7] - a[4] * a[6]);
    double om[9];
    om[0] = (a[4] * a[8] - a[5] * a[7]) / det;
    om[1] = -(a[3] * a[8] - a[6] * a[5]) / det;
    om[2] = (a[3] * a[7] - a[6] * a[4]) / det;
    om[3] = -(a[1] * a[8] - a[7] * a[2]) / det;
    om[4] = (a[0] * a[8] - a[2] * a[6]) / det;
    om[5] = -(a[0] * a[7] - a[6] * a[1]) / det;
    om[6] = (a[1] * a[5] - a[4] * a[2]) / det;
    om[7] = -(a[0] * a[5] - a[3] * a[2]) / det;
    om[8] = (a[0] * a[4] - a[1] * a[3]) / det;
    double v[4][3];
    for (int p = 0; p < 4; p++)
      for (int i = 0; i < 3; i++)
        v[p][i] = bc.sig[p][i * 3 + 0] * nv[0] + bc.sig[p][i * 3 + 1] * nv[1] + bc.sig[p][i * 3 + 2] * nv[2];
    for (int p = 0; p < 4; p++)
      for (int q = p; q < 4; q++) {
        double t1 = 0.0;
        for (int j = 0; j < 3; j++)
          for (int k = 0; k < 3; k++) t1 += v[p][j] * om[j * 3 + k] * v[q][k];
        bn[(long long)pq_slot(p, q) * N3 + g] = (B)(bc.t0[pq_slot(p, q)] - t1);
      }
  }
}

// Contraction on pairs {k, -k}; see the file comment.  A row (y, z) is done
// together with its mirror row (-y, -z), by the lower of the two.
template <typename T, typename B>
__global__ void contract_kernel(typename Cx<T>::t *z01, typename Cx<T>::t *z23, const B *__restrict__ bn, int N,
                                int nac) {
  typedef typename Cx<T>::t C;
  const long long N3 = (long long)N * N * N;
  // blockIdx.y = run: its grids at run N^3
  z01 += blockIdx.y * N3;
  if (z23) z23 += blockIdx.y * N3;
  for (int row = blockIdx.x; row < N * N; row += gridDim.x) {
  const int z = row / N, y = row - z * N;
  const int ym = y == 0 ? 0 : N - y, zm = z == 0 ? 0 : N - z;
  const int rowm = zm * N + ym;
  if (rowm < row) continue;
  for (int x = threadIdx.x; x < N; x += blockDim.x) {
    const int xm = x == 0 ? 0 : N - x;
    const long long g = (long long)row * N + x, gm = (long long)rowm * N + xm;
    if (gm < g) continue;  // the pair is handled by its lower index
    C H[4], Hm[4];
    C a = z01[g], am = z01[gm];
    C b, bm;
    b.x = 0; b.y = 0; bm = b;
    if (z23) { b = z23[g]; bm = z23[gm]; }
    // split Z = A + iB into the two real fields' spectra
    H[0].x = (T)0.5 * (a.x + am.x); H[0].y = (T)0.5 * (a.y - am.y);
    H[1].x = (T)0.5 * (a.y + am.y); H[1].y = (T)0.5 * (am.x - a.x);
    H[2].x = (T)0.5 * (b.x + bm.x); H[2].y = (T)0.5 * (b.y - bm.y);
    H[3].x = (T)0.5 * (b.y + bm.y); H[3].y = (T)0.5 * (bm.x - b.x);
    for (int q = 0; q < 4; q++) {
      if (q >= nac) { H[q].x = 0; H[q].y = 0; }
      Hm[q] = cconj(H[q]);
    }
    C G[4];
    for (int p = 0; p < 4; p++) {
      C f, fm;
      f.x = 0; f.y = 0; fm = f;
      for (int q = 0; q < 4; q++) {
        T bk = (T)bn[(long long)pq_slot(p, q) * N3 + g];
        T bkm = (T)bn[(long long)pq_slot(p, q) * N3 + gm];
        f.x += bk * H[q].x; f.y += bk * H[q].y;
        fm.x += bkm * Hm[q].x; fm.y += bkm * Hm[q].y;
      }
      // Hermitian part: its inverse transform is Re(IFFT(F_p))
      G[p].x = (T)0.5 * (f.x + fm.x);
      G[p].y = (T)0.5 * (f.y - fm.y);
      if (p >= nac) { G[p].x = 0; G[p].y = 0; }
    }
    C w01, w23, w01m, w23m;
    w01.x = G[0].x - G[1].y; w01.y = G[0].y + G[1].x;    // G0 + i G1
    w01m.x = G[0].x + G[1].y; w01m.y = -G[0].y + G[1].x; // conj(G0) + i conj(G1)
    w23.x = G[2].x - G[3].y; w23.y = G[2].y + G[3].x;
    w23m.x = G[2].x + G[3].y; w23m.y = -G[2].y + G[3].x;
    z01[g] = w01;
    if (gm != g) z01[gm] = w01m;
    if (z23) {
      z23[g] = w23;
      if (gm != g) z23[gm] = w23m;
    }
  }
  }
}

// Interior of felas_p from the inverse transforms, scaled by 1/N^3.
template <typename T>
__global__ void unpack_kernel(const typename Cx<T>::t *__restrict__ w01, const typename Cx<T>::t *__restrict__ w23,
                              T *__restrict__ felas, int N, int nac) {
  const int n = N + 4;
  const long long n3 = (long long)n * n * n, N3 = (long long)N * N * N;
  const double s = 1.0 / (double)N3;
  for (int row = blockIdx.x; row < N * N; row += gridDim.x)
  for (int x = threadIdx.x; x < N; x += blockDim.x) {
    const int z = row / N, y = row - z * N;
    const long long g = (long long)row * N + x;
    long long l = ((long long)(z + 2) * n + (y + 2)) * n + (x + 2);
    typename Cx<T>::t a = w01[g];
    felas[l] = (T)(a.x * s);
    if (nac > 1) felas[n3 + l] = (T)(a.y * s);
    if (nac > 2) {
      typename Cx<T>::t b = w23[g];
      felas[2 * n3 + l] = (T)(b.x * s);
      if (nac > 3) felas[3 * n3 + l] = (T)(b.y * s);
    }
  }
}

struct ElasticPlan {
  int N, nac, fp32;
  int runs;       // runs side by side (grids z01, z23 of runs N^3 each)
  Radices rad;
  void *tw;       // twiddles, complex of the working precision
  void *z01, *z23;
  void *bn;       // 10 * N^3 Green-tensor slots, double (FP64 plan) or float
  int tile, ltile;
  int fast;       // FP32 plan with a two-pass register path for N
  StageDiv sd;
  size_t smem;
  bool first;     // no previous elastic call: scratch ghosts are zero
};

static int grid1(long long total) {
  long long b = (total + 255) / 256;
  return (int)(b > 152LL * 32 ? 152LL * 32 : (b < 1 ? 1 : b));
}

cudaError_t elastic_plan_create(ElasticPlan **out, int N, int nac, const double *voigt, const double *eps, int fp32,
                                cudaStream_t s, int runs) {
  ElasticPlan *p = new ElasticPlan();
  memset(p, 0, sizeof *p);
  p->N = N;
  p->nac = nac;
  p->fp32 = fp32;
  p->runs = runs > 0 ? runs : 1;
  p->first = true;
  p->rad = factor(N);
  // several runs take the two-pass FP32 path only
  if (p->rad.count < 0 || nac < 1 || nac > 4 || (p->runs > 1 && (!fp32 || fft2::pass_n1(N) == 0))) {
    delete p;
    return cudaErrorInvalidValue;
  }
  const long long N3 = (long long)N * N * N;
  size_t csz = fp32 ? sizeof(float2) : sizeof(double2);
  cudaError_t e;
  if ((e = cudaMalloc(&p->tw, csz * N)) != cudaSuccess) goto fail;
  if ((e = cudaMalloc(&p->z01, csz * N3 * p->runs)) != cudaSuccess) goto fail;
  if (nac > 2 && (e = cudaMalloc(&p->z23, csz * N3 * p->runs)) != cudaSuccess) goto fail;
  if ((e = cudaMalloc(&p->bn, (fp32 ? sizeof(float) : sizeof(double)) * 10 * N3)) != cudaSuccess) goto fail;
  {
    std::vector<double> twd(2 * N);
    for (int j = 0; j < N; j++) {
      double a = -2.0 * 3.14159265358979323846 * (double)j / (double)N;
      twd[2 * j] = cos(a);
      twd[2 * j + 1] = sin(a);
    }
    if (fp32) {
      std::vector<float> twf(2 * N);
      for (int j = 0; j < 2 * N; j++) twf[j] = (float)twd[j];
      e = cudaMemcpyAsync(p->tw, twf.data(), sizeof(float) * 2 * N, cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      p->fast = fft2::pass_n1(N) != 0 && (p->runs > 1 || getenv("SCLET_FFT_GENERIC") == nullptr);
      if (e == cudaSuccess && p->fast) e = fft2::upload_constants(s);
    } else {
      e = cudaMemcpyAsync(p->tw, twd.data(), sizeof(double) * 2 * N, cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    if (e != cudaSuccess) goto fail;
  }
  {
    // stiffness (elastic_input, elastic.c:378-398) and s0 = C : e0
    static const int vi[3][3] = {{0, 5, 4}, {5, 1, 3}, {4, 3, 2}};
    BnConst bc;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        for (int k = 0; k < 3; k++)
          for (int l = 0; l < 3; l++) bc.C[((i * 3 + j) * 3 + k) * 3 + l] = voigt[vi[i][j] * 6 + vi[k][l]];
    for (int q = 0; q < 4; q++)
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          double acc = 0.0;
          for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++) acc += bc.C[((i * 3 + j) * 3 + k) * 3 + l] * eps[q * 9 + k * 3 + l];
          bc.sig[q][i * 3 + j] = acc;
        }
    for (int a = 0; a < 4; a++)
      for (int b = a; b < 4; b++) {
        double t0 = 0.0;
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
              for (int l = 0; l < 3; l++)
                t0 += bc.C[((i * 3 + j) * 3 + k) * 3 + l] * eps[a * 9 + i * 3 + j] * eps[b * 9 + k * 3 + l];
        bc.t0[pq_slot(a, b)] = t0;
      }
    if (fp32) bn_kernel<float><<<grid1(N3), 256, 0, s>>>((float *)p->bn, N, bc);
    else bn_kernel<double><<<grid1(N3), 256, 0, s>>>((double *)p->bn, N, bc);
    launch_counter()++;
    if ((e = cudaGetLastError()) != cudaSuccess) goto fail;
  }
  {
    // tile of lines per CTA: two ping-pong buffers within ~96 KB
    int tile = 16;
    while (tile > 1 && 2 * (size_t)tile * N * csz > 96 * 1024) tile /= 2;
    while (N % tile) tile /= 2;
    p->tile = tile;
    p->ltile = 0;
    while ((1 << p->ltile) < tile) p->ltile++;
    p->smem = 2 * (size_t)tile * N * csz;
    int ns = 1;
    for (int st = 0; st < p->rad.count; st++) {
      p->sd.inv_nb[st] = 1.0f / (float)(N / p->rad.r[st]);
      p->sd.inv_ns[st] = 1.0f / (float)ns;
      ns *= p->rad.r[st];
    }
  }
  *out = p;
  return cudaSuccess;
fail:
  elastic_plan_destroy(p);
  return e;
}

void elastic_plan_destroy(ElasticPlan *p) {
  if (!p) return;
  cudaFree(p->tw);
  cudaFree(p->z01);
  cudaFree(p->z23);
  cudaFree(p->bn);
  delete p;
}

// 3-D transform of one or two complex grids (z1 may be null) by the generic
// Stockham stages: one launch per axis, x, y, z forward and z, y, x backward.
template <typename T>
static cudaError_t fft3d(ElasticPlan *p, typename Cx<T>::t *z0, typename Cx<T>::t *z1, int sign, cudaStream_t s) {
  const int N = p->N;
  // the shared-memory attribute is per device
  constexpr int MAXDEV = 64;
  static std::mutex mu;
  static bool attr_set[MAXDEV][2] = {};
  const int which = sizeof(T) == 4 ? 1 : 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= MAXDEV) return cudaErrorInvalidDevice;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!attr_set[dev][which]) {
      e = cudaFuncSetAttribute(fft_lines_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
      if (e != cudaSuccess) return e;
      attr_set[dev][which] = true;
    }
  }
  const dim3 grid((unsigned)((long long)N * N / p->tile), z1 ? 2u : 1u);
  const typename Cx<T>::t *tw = (const typename Cx<T>::t *)p->tw;
  int order[3] = {0, 1, 2};
  if (sign > 0) { order[0] = 2; order[2] = 0; }
  for (int k = 0; k < 3; k++) {
    fft_lines_kernel<T><<<grid, 256, p->smem, s>>>(z0, z1, N, order[k], p->ltile, tw, sign, p->rad, p->sd);
    launch_counter()++;
  }
  return cudaGetLastError();
}

// launch shape of the row kernels: rows (y, z) over CTAs, x over threads
static dim3 rows_grid(int N) { return dim3((unsigned)(N * N < 152 * 16 ? N * N : 152 * 16)); }
static dim3 rows_block(int N) { return dim3((unsigned)(N >= 256 ? 256 : (N + 31) / 32 * 32)); }

template <typename T>
cudaError_t elastic_compute(ElasticPlan *p, const T *u, T *felas, int n, T *shell, cudaStream_t s, long long ustride) {
  typedef typename Cx<T>::t C;
  const int N = p->N;
  const long long n3 = (long long)n * n * n;
  C *z01 = (C *)p->z01, *z23 = (C *)p->z23;
  if (sizeof(T) == 4 && p->fast) {
    // packing and unpacking fused into the first and last x-passes
    fft2::LineIO io;
    io.u = (const float *)u;
    io.felas = (float *)felas;
    io.n = n;
    io.nac = p->nac;
    io.n3 = n3;
    io.scale = (float)(1.0 / ((double)N * N * N));
    io.runs = p->runs;
    io.ustride = ustride;
    io.fstride = (long long)p->nac * n3;
    const float2 *tw = (const float2 *)p->tw;
    for (int k = 0; k < 3; k++) {
      cudaError_t e = fft2::launch(N, -1, k, (float2 *)z01, (float2 *)z23, tw, io, s);
      launch_counter()++;
      if (e != cudaSuccess) return e;
    }
    contract_kernel<T, float><<<dim3(rows_grid(N).x, p->runs), rows_block(N), 0, s>>>(z01, z23, (const float *)p->bn,
                                                                                       N, p->nac);
    launch_counter()++;
    for (int k = 0; k < 3; k++) {
      cudaError_t e = fft2::launch(N, +1, k, (float2 *)z01, (float2 *)z23, tw, io, s);
      launch_counter()++;
      if (e != cudaSuccess) return e;
    }
  } else {
    pack_kernel<T><<<rows_grid(N), rows_block(N), 0, s>>>(u, z01, z23, N, p->nac);
    launch_counter()++;
    fft3d<T>(p, z01, z23, -1, s);
    if (p->fp32)
      contract_kernel<T, float><<<rows_grid(N), rows_block(N), 0, s>>>(z01, z23, (const float *)p->bn, N, p->nac);
    else
      contract_kernel<T, double><<<rows_grid(N), rows_block(N), 0, s>>>(z01, z23, (const double *)p->bn, N, p->nac);
    launch_counter()++;
    fft3d<T>(p, z01, z23, +1, s);
    unpack_kernel<T><<<rows_grid(N), rows_block(N), 0, s>>>(z01, z23, felas, N, p->nac);
    launch_counter()++;
  }
  // ghost cells: the shared-scratch semantics, field by field in order (all
  // runs of a field in one launch)
  const long long fstride = (long long)p->nac * n3;
  for (int q = 0; q < p->nac; q++) {
    const T *prev = felas + (long long)((q + p->nac - 1) % p->nac) * n3;
    long long pstride = fstride;
    T *gbuf = shell;
    if (p->first && q == 0) {
      // before the first call the scratch block is all zero
      cudaMemsetAsync(shell, 0, sizeof(T) * n3, s);
      prev = shell;
      pstride = 0;
      gbuf = shell + n3;
    }
    cudaError_t e = launch_elastic_shell<T>(felas + q * n3, prev, n, gbuf, s, p->runs, fstride, pstride);
    if (e != cudaSuccess) return e;
  }
  p->first = false;
  return cudaGetLastError();
}

template cudaError_t elastic_compute<double>(ElasticPlan *, const double *, double *, int, double *, cudaStream_t,
                                             long long);
template cudaError_t elastic_compute<float>(ElasticPlan *, const float *, float *, int, float *, cudaStream_t,
                                            long long);

}  // namespace sclet
