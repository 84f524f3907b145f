// Diagnostics of the state: check_soln_new (source_beta_to_omega/src/field.c:
// 407-678) as a device reduction.  Per field: max, min and vol = sum(u + 1) h^3
// over the owned cells; energy over the owned cells' corner cubes from the
// 8-corner averages and corner-difference gradients (field.c:487-511):
//   sum_m epn2/2 grad(eta_m).lambda_m.grad(eta_m)  [+ epn2/2 |grad c|^2]
//   + Landau energy of the averages.
// form 0 reproduces the reference's hard-coded 2-3-4 polynomial and its
// separate CH energy ((c^2-1)^2/4); form 1 is the plugin's total free energy
// (its F_bulk, sclet_physics.cuh, plus the gradient terms).
// Sums are compensated (TwoSum pairs) in FP64 and reduced in a fixed order,
// so the result is deterministic.
#include "sclet_internal.cuh"
#include "sclet_physics.cuh"

namespace sclet {

struct KS {
  double s, c;
};
__device__ inline void two_sum(double a, double b, double &s, double &e) {
  s = a + b;
  double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ inline void ks_add(KS &k, double v) {
  double s, e;
  two_sum(k.s, v, s, e);
  k.s = s;
  k.c += e;
}
__device__ inline KS ks_merge(KS a, KS b) {
  KS r;
  double e;
  two_sum(a.s, b.s, r.s, e);
  r.c = a.c + b.c + e;
  return r;
}

constexpr int EB = 256;  // threads per block

// Per-thread sum of T values with FP64-class accuracy.  For FP32 values the
// running sum is a float pair (s, e) updated by the error-free TwoSum (Knuth),
// about 48 bits, so a thread's few dozen terms cost FP32 instructions, not
// FP64 ones (the FP64 pipe of this GPU is 1/64 of the FP32 rate).
template <typename T>
struct Acc;
template <>
struct Acc<double> {
  double s = 0.0;
  __device__ void add(double v) { s += v; }
  __device__ double value() const { return s; }
};
template <>
struct Acc<float> {
  float s = 0.0f, e = 0.0f;
  __device__ void add(float v) {
    const float t = s + v;
    const float bp = t - s;
    e += (s - (t - bp)) + (v - bp);
    s = t;
  }
  __device__ double value() const { return (double)s + (double)e; }
  // pair sum with the partner lane at xor distance off; both lanes end with
  // the same pair (TwoSum is exact and the merge symmetric)
  __device__ void merge_lane(int off) {
    const float os = __shfl_xor_sync(0xffffffffu, s, off), oe = __shfl_xor_sync(0xffffffffu, e, off);
    const float t = s + os, bp = t - s;
    const float err = (s - (t - bp)) + (os - bp);
    e = (e + oe) + err;
    s = t;
  }
};
constexpr int MAXF = 5;

// partial record per block: for f < F: max, min, vol.s, vol.c; then
// eng_ac.s, eng_ac.c, eng_ch.s, eng_ch.c
__host__ __device__ inline int rec_len(int F) { return 4 * F + 4; }

// Reduction of the record (per field max, min, vol; two energies): warp
// butterflies, then the block's warps in lane order; fixed shape, so the
// result is deterministic.  TwoSum is exact and symmetric, so every lane of
// a butterfly holds the same pair.
__device__ __forceinline__ KS shfl_ks(KS v, int off) {
  KS o;
  o.s = __shfl_xor_sync(0xffffffffu, v.s, off);
  o.c = __shfl_xor_sync(0xffffffffu, v.c, off);
  return ks_merge(v, o);
}

// Lane 0 of every warp holds its warp's values: the block's record.
__device__ __forceinline__ void block_record_from_warps(const double (&mxd)[MAXF], const double (&mnd)[MAXF],
                                                        const KS (&vol)[MAXF], KS eac, KS ech, int F,
                                                        double *__restrict__ part) {
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int lane = tid & 31, wid = tid >> 5;
  constexpr int NW = EB / 32;
  __shared__ double wrec[NW][4 * MAXF + 4];
  if (lane == 0) {
    for (int f = 0; f < F; f++) {
      wrec[wid][4 * f] = mxd[f];
      wrec[wid][4 * f + 1] = mnd[f];
      wrec[wid][4 * f + 2] = vol[f].s;
      wrec[wid][4 * f + 3] = vol[f].c;
    }
    wrec[wid][4 * F] = eac.s;
    wrec[wid][4 * F + 1] = eac.c;
    wrec[wid][4 * F + 2] = ech.s;
    wrec[wid][4 * F + 3] = ech.c;
  }
  __syncthreads();
  if (wid == 0) {
    const int src = lane < NW ? lane : 0;  // lanes beyond the warp count repeat warp 0 (idempotent for max/min)
    double *dst = part + (long long)blockIdx.x * rec_len(F);
    for (int f = 0; f < F; f++) {
      double a = wrec[src][4 * f], b = wrec[src][4 * f + 1];
      KS v = {lane < NW ? wrec[src][4 * f + 2] : 0.0, lane < NW ? wrec[src][4 * f + 3] : 0.0};
#pragma unroll
      for (int off = NW / 2; off > 0; off >>= 1) {
        a = fmax(a, __shfl_xor_sync(0xffffffffu, a, off));
        b = fmin(b, __shfl_xor_sync(0xffffffffu, b, off));
        v = shfl_ks(v, off);
      }
      if (lane == 0) {
        dst[4 * f] = a;
        dst[4 * f + 1] = b;
        dst[4 * f + 2] = v.s;
        dst[4 * f + 3] = v.c;
      }
    }
    KS ea = {lane < NW ? wrec[src][4 * F] : 0.0, lane < NW ? wrec[src][4 * F + 1] : 0.0};
    KS eb = {lane < NW ? wrec[src][4 * F + 2] : 0.0, lane < NW ? wrec[src][4 * F + 3] : 0.0};
#pragma unroll
    for (int off = NW / 2; off > 0; off >>= 1) {
      ea = shfl_ks(ea, off);
      eb = shfl_ks(eb, off);
    }
    if (lane == 0) {
      dst[4 * F] = ea.s;
      dst[4 * F + 1] = ea.c;
      dst[4 * F + 2] = eb.s;
      dst[4 * F + 3] = eb.c;
    }
  }
}

__device__ __forceinline__ void block_record(double (&mxd)[MAXF], double (&mnd)[MAXF], KS (&vol)[MAXF], KS eac, KS ech,
                                             int F, double *__restrict__ part) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int f = 0; f < MAXF; f++) {
      mxd[f] = fmax(mxd[f], __shfl_xor_sync(0xffffffffu, mxd[f], off));
      mnd[f] = fmin(mnd[f], __shfl_xor_sync(0xffffffffu, mnd[f], off));
      vol[f] = shfl_ks(vol[f], off);
    }
    eac = shfl_ks(eac, off);
    ech = shfl_ks(ech, off);
  }
  block_record_from_warps(mxd, mnd, vol, eac, ech, F, part);
}


template <typename PL, typename T>
__global__ void __launch_bounds__(EB) energy_partial_kernel(Phys ph, const T *__restrict__ u, const double *__restrict__ elam,
                                                            int form, double *__restrict__ part) {
  // Per-cell arithmetic in the state's precision T: the cell terms of an FP32
  // state carry FP32 rounding, which is unbiased and averages out over the
  // sum; every sum (per thread, per block, over blocks) is FP64, and the
  // volume integrals add the FP32 values exactly.
  const int n = ph.n, N = n - 4, F = ph.F, nac = ph.nac;
  const long long n3 = (long long)n * n * n;
  const T i4hx = (T)(0.25 / ph.h[0]), i4hy = (T)(0.25 / ph.h[1]), i4hz = (T)(0.25 / ph.h[2]);
  const T half_epn2 = (T)(0.5 * ph.epn2);
  const double cshift = ph.cshift;
  T L[4][9];
  for (int m = 0; m < 4; m++)
    for (int k = 0; k < 9; k++) L[m][k] = (T)elam[9 * m + k];
  T Kt[16];  // plugin constants
#pragma unroll
  for (int k = 0; k < 16; k++) Kt[k] = (T)ph.K[k];
  T mx[MAXF], mn[MAXF];
  Acc<T> vsum[MAXF], eac_p, ech_p;
  long long cnt = 0;
#pragma unroll
  for (int f = 0; f < MAXF; f++) {
    mx[f] = (T)-1.0e30;
    mn[f] = (T)1.0e30;
  }
  // rows (j, k) of owned cells over the grid, x across the block: no index division per cell
  for (int row = blockIdx.x; row < N * N; row += gridDim.x) {
  const int j = 2 + row % N, k = 2 + row / N;
  for (int i = 2 + threadIdx.x; i < n - 2; i += blockDim.x) {
    const long long l = ((long long)k * n + j) * n + i;
    cnt++;
#pragma unroll
    for (int f = 0; f < MAXF; f++) {
      if (f >= F) break;
      const T t = u[f * n3 + l];
      mx[f] = t > mx[f] ? t : mx[f];
      mn[f] = t < mn[f] ? t : mn[f];
      vsum[f].add(t);
    }
    if (i >= n - 3 || j >= n - 3 || k >= n - 3) continue;
    T avg[MAXF];
    double cbar = 0.0;  // true concentration average, exact sum of the 8 values
    double cst = 0.0;   // the same of the stored values (c - cshift)
    T e_ac = (T)0, e_ch = (T)0;
#pragma unroll
    for (int f = 0; f < MAXF; f++) {
      if (f >= F) break;
      const T *q = u + f * n3;
      const T v0 = q[l], v1 = q[l + 1], v2 = q[l + n], v3 = q[l + n + 1];
      const T v4 = q[l + n * n], v5 = q[l + n * n + 1], v6 = q[l + n * n + n], v7 = q[l + n * n + n + 1];
      avg[f] = (v0 + v1 + v2 + v3 + v4 + v5 + v6 + v7) * (T)0.125;
      const T ux = ((v1 - v0) + (v3 - v2) + (v5 - v4) + (v7 - v6)) * i4hx;
      const T uy = ((v2 - v0) + (v3 - v1) + (v6 - v4) + (v7 - v5)) * i4hy;
      const T uz = ((v4 - v0) + (v5 - v1) + (v6 - v2) + (v7 - v3)) * i4hz;
      if (f < nac) {
        const T *Lm = L[f];
        const T fx = ux * Lm[0] + uy * Lm[3] + uz * Lm[6];
        const T fy = ux * Lm[1] + uy * Lm[4] + uz * Lm[7];
        const T fz = ux * Lm[2] + uy * Lm[5] + uz * Lm[8];
        e_ac += half_epn2 * (fx * ux + fy * uy + fz * uz);
      } else {
        const T gr = half_epn2 * (ux * ux + uy * uy + uz * uz);
        if (form == 0) e_ch += gr; else e_ac += gr;
        Acc<T> cs;
        cs.add(v0);
        cs.add(v1);
        cs.add(v2);
        cs.add(v3);
        cs.add(v4);
        cs.add(v5);
        cs.add(v6);
        cs.add(v7);
        cst = cs.value() * 0.125;
        cbar = cst + cshift;
      }
    }
    if (form == 0) {
      T e[4] = {0, 0, 0, 0};
#pragma unroll
      for (int f = 0; f < 4; f++)
        if (f < nac) e[f] = avg[f];
      const T s2 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2] + e[3] * e[3];
      const T s3 = e[0] * e[0] * e[0] + e[1] * e[1] * e[1] + e[2] * e[2] * e[2] + e[3] * e[3] * e[3];
      if (nac > 0)
        e_ac += (T)(2376.0 / 2372.0 / 2.0) * s2 - (T)((7128.0 + 12.0 * 2372.0) / 2372.0 / 3.0) * s3 +
                (T)((4752.0 + 12.0 * 2372.0) / 2372.0 / 4.0) * s2 * s2;
      if (ph.nch > 0) {
        const T c = (T)cbar;
        e_ch += (c * c - (T)1) * (c * c - (T)1) * (T)0.25;
      }
    } else {
      sclet_acv<T> ac[4];
      sclet_chv<T> ch[1];
#pragma unroll
      for (int m = 0; m < 4; m++) ac[m].u = m < nac ? avg[m] : (T)0;
      ch[0].c = (T)cst;
      e_ac += PL::template f_bulk<T>(ac, ch, nac, ph.nch, Kt);
    }
    eac_p.add(e_ac);
    ech_p.add(e_ch);
  }
  }
  double mxd[MAXF], mnd[MAXF];
  KS vol[MAXF], eac = {eac_p.value(), 0.0}, ech = {ech_p.value(), 0.0};
#pragma unroll
  for (int f = 0; f < MAXF; f++) {
    const double sh = f >= nac ? cshift : 0.0;
    mxd[f] = (double)mx[f] + sh;
    mnd[f] = (double)mn[f] + sh;
    // sum of (value + 1) over this thread's cells, the constant part exact
    vol[f].s = vsum[f].value();
    vol[f].c = 0.0;
    ks_add(vol[f], (double)cnt * (sh + 1.0));
  }
  block_record(mxd, mnd, vol, eac, ech, F, part);
}

// ---- FP32 states: z-marching form of the same reduction --------------------
//
// A CTA of 32 x 8 threads owns 32 x 8 owned (x, y) columns of one unit and
// walks its ZCH planes in z.  Each thread keeps the (x, y), (x, y + 1) values
// of plane z and z + 1 of every field in registers and takes the x + 1
// neighbours from the next lane, so a cell costs two loads per field instead
// of eight.  The conserved field's corner average is an exact FP32 pair sum
// finished in pair arithmetic (no FP64 instructions per cell).  Blocks loop
// over units; one partial record per block, the same layout as above.
constexpr int EZ = 8;  // planes per unit

__host__ __device__ inline int energy_units(int N) { return ((N + 31) / 32) * ((N + 7) / 8) * ((N + EZ - 1) / EZ); }

struct Pair {
  float s, e;
};
// exact running sum of floats (TwoSum, Knuth)
__device__ __forceinline__ void pair_add(Pair &p, float v) {
  const float t = p.s + v, bp = t - p.s;
  p.e += (p.s - (t - bp)) + (v - bp);
  p.s = t;
}
// (a.s + a.e) + (b.s + b.e) rounded to float
__device__ __forceinline__ float pair_sum(Pair a, Pair b) {
  const float t = a.s + b.s, bp = t - a.s;
  const float err = (a.s - (t - bp)) + (b.s - bp);
  return t + (err + a.e + b.e);
}

// FP32 constants of energy_partial_f32, rounded once on the host (kernel
// parameters: read from the constant bank, never recomputed in the loop)
struct EConst {
  float i4hx, i4hy, i4hz, half_epn2;
  float K[16];       // plugin constants, the reference composition c0 (if any) as 0
  float p2, p3, p4;  // the 2-3-4 polynomial of energy form 0
  Pair kdp, kcp;     // cshift - c0 and cshift as float pairs
};

// The plugin sees the concentration as c - c0 (exact in pair arithmetic from
// the stored c - cshift) with its c0 constant 0, where it names one.
template <typename PL>
static EConst econst(const Phys &ph) {
  EConst c;
  c.i4hx = (float)(0.25 / ph.h[0]);
  c.i4hy = (float)(0.25 / ph.h[1]);
  c.i4hz = (float)(0.25 / ph.h[2]);
  c.half_epn2 = (float)(0.5 * ph.epn2);
  for (int k = 0; k < 16; k++) c.K[k] = (float)ph.K[k];
  const double kd = PL::c0_index >= 0 ? -ph.K[PL::c0_index] : 0.0;  // ph.K holds c0 - cshift
  if (PL::c0_index >= 0) c.K[PL::c0_index] = 0.0f;
  c.kdp = Pair{(float)kd, (float)(kd - (double)(float)kd)};
  c.p2 = (float)(2376.0 / 2372.0 / 2.0);
  c.p3 = (float)((7128.0 + 12.0 * 2372.0) / 2372.0 / 3.0);
  c.p4 = (float)((4752.0 + 12.0 * 2372.0) / 2372.0 / 4.0);
  c.kcp = Pair{(float)ph.cshift, (float)(ph.cshift - (double)(float)ph.cshift)};
  return c;
}

template <typename PL, int NAC, int NCH>
__global__ void __launch_bounds__(256, 2) energy_partial_f32(Phys ph, EConst ec, const float *__restrict__ u,
                                                             const double *__restrict__ elam, int form,
                                                             double *__restrict__ part) {
  constexpr int F = NAC + NCH;
  const int n = ph.n, N = n - 4;
  const long long n3 = (long long)n * n * n;
  __shared__ float q6[4][6];  // half epn2 times the symmetrised gradient tensors: xx yy zz xy xz yz
  if (threadIdx.x < 4 * 6 && threadIdx.y == 0) {
    const int m = threadIdx.x / 6, c = threadIdx.x % 6;
    const double *L = elam + 9 * m;
    const double v = c == 0 ? L[0] : c == 1 ? L[4] : c == 2 ? L[8] : c == 3 ? L[1] + L[3] : c == 4 ? L[2] + L[6] : L[5] + L[7];
    q6[m][c] = (float)(0.5 * ph.epn2 * v);
  }
  __syncthreads();
  const float i4hx = ec.i4hx, i4hy = ec.i4hy, i4hz = ec.i4hz, half_epn2 = ec.half_epn2;
  float Kt[16];
#pragma unroll
  for (int k = 0; k < 16; k++) Kt[k] = ec.K[k];
  // blockIdx.y = run: its fields, its plugin constant 0, its partial records
  if (ph.krun) Kt[0] = (float)ph.krun[blockIdx.y];
  u += (long long)blockIdx.y * F * n3;
  part += (long long)blockIdx.y * gridDim.x * rec_len(F);
  const float p2 = ec.p2, p3 = ec.p3, p4 = ec.p4;
  const Pair kdp = ec.kdp, kcp = ec.kcp;
  float mx[F], mn[F];
  Acc<float> vsum[F], eac_p, ech_p;
  int cnt = 0;
#pragma unroll
  for (int f = 0; f < F; f++) {
    mx[f] = -1.0e30f;
    mn[f] = 1.0e30f;
  }
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int nti = (N + 31) / 32, ntj = (N + 7) / 8, units = energy_units(N);
  for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
    const int ti = unit % nti, tj = (unit / nti) % ntj, zc = unit / (nti * ntj);
    const int i = 2 + ti * 32 + tx, j = 2 + tj * 8 + ty;
    const bool own = i <= n - 3 && j <= n - 3, inner = i <= n - 4 && j <= n - 4;
    const int ic = i < n - 2 ? i : n - 2, jc = j < n - 2 ? j : n - 2;  // clamped: loads stay inside the block
    const int k0 = 2 + zc * EZ, k1 = k0 + EZ < n - 2 ? k0 + EZ : n - 2;
    float a0[F], a1[F], a2[F], a3[F];  // plane k: (i, j) (i+1, j) (i, j+1) (i+1, j+1)
    const long long row0 = ((long long)k0 * n + jc) * n + ic;
#pragma unroll
    for (int f = 0; f < F; f++) {
      const float *q = u + f * n3 + row0;
      a0[f] = q[0];
      a2[f] = q[n];
      a1[f] = __shfl_down_sync(0xffffffffu, a0[f], 1);
      a3[f] = __shfl_down_sync(0xffffffffu, a2[f], 1);
      if (tx == 31) {
        a1[f] = q[1];
        a3[f] = q[n + 1];
      }
    }
    for (int k = k0; k < k1; k++) {
      float b0[F], b1[F], b2[F], b3[F];  // plane k + 1
      const long long row = ((long long)(k + 1) * n + jc) * n + ic;
#pragma unroll
      for (int f = 0; f < F; f++) {
        const float *q = u + f * n3 + row;
        b0[f] = q[0];
        b2[f] = q[n];
        b1[f] = __shfl_down_sync(0xffffffffu, b0[f], 1);
        b3[f] = __shfl_down_sync(0xffffffffu, b2[f], 1);
        if (tx == 31) {
          b1[f] = q[1];
          b3[f] = q[n + 1];
        }
      }
      if (own) {
        cnt++;
#pragma unroll
        for (int f = 0; f < F; f++) {
          mx[f] = fmaxf(mx[f], a0[f]);
          mn[f] = fminf(mn[f], a0[f]);
          vsum[f].add(a0[f]);
        }
      }
      if (inner && k <= n - 4) {
        float avg[F > 0 ? F : 1];
        float e_ac = 0.0f, e_ch = 0.0f, cd = 0.0f, cval = 0.0f;
#pragma unroll
        for (int f = 0; f < F; f++) {
          const float v0 = a0[f], v1 = a1[f], v2 = a2[f], v3 = a3[f], v4 = b0[f], v5 = b1[f], v6 = b2[f], v7 = b3[f];
          avg[f] = (((v0 + v1) + (v2 + v3)) + ((v4 + v5) + (v6 + v7))) * 0.125f;
          const float ux = ((v1 - v0) + (v3 - v2) + (v5 - v4) + (v7 - v6)) * i4hx;
          const float uy = ((v2 - v0) + (v3 - v1) + (v6 - v4) + (v7 - v5)) * i4hy;
          const float uz = ((v4 - v0) + (v5 - v1) + (v6 - v2) + (v7 - v3)) * i4hz;
          if (f < NAC) {
            const float *qm = q6[f];
            e_ac += qm[0] * ux * ux + qm[1] * uy * uy + qm[2] * uz * uz + qm[3] * ux * uy + qm[4] * ux * uz +
                    qm[5] * uy * uz;
          } else {
            const float gr = half_epn2 * (ux * ux + uy * uy + uz * uz);
            if (form == 0) e_ch += gr;
            else e_ac += gr;
            // exact corner sum, then (sum / 8 + cshift - c0) and (sum / 8 + cshift)
            Pair cs = {v0, 0.0f};
            pair_add(cs, v1);
            pair_add(cs, v2);
            pair_add(cs, v3);
            pair_add(cs, v4);
            pair_add(cs, v5);
            pair_add(cs, v6);
            pair_add(cs, v7);
            cs.s *= 0.125f;
            cs.e *= 0.125f;
            cd = pair_sum(cs, kdp);
            cval = pair_sum(cs, kcp);
          }
        }
        if (form == 0) {
          if (NAC > 0) {
            float s2 = 0.0f, s3 = 0.0f;
#pragma unroll
            for (int f = 0; f < (NAC < 4 ? NAC : 4); f++) {
              s2 += avg[f] * avg[f];
              s3 += avg[f] * avg[f] * avg[f];
            }
            e_ac += p2 * s2 - p3 * s3 + p4 * s2 * s2;
          }
          if (NCH > 0) e_ch += (cval * cval - 1.0f) * (cval * cval - 1.0f) * 0.25f;
        } else {
          sclet_acv<float> ac[NAC > 0 ? NAC : 1];
          sclet_chv<float> ch[1];
#pragma unroll
          for (int m = 0; m < NAC; m++) ac[m].u = avg[m];
          ch[0].c = cd;
          e_ac += PL::template f_bulk<float>(ac, ch, NAC, NCH, Kt);
        }
        eac_p.add(e_ac);
        ech_p.add(e_ch);
      }
#pragma unroll
      for (int f = 0; f < F; f++) {
        a0[f] = b0[f];
        a1[f] = b1[f];
        a2[f] = b2[f];
        a3[f] = b3[f];
      }
    }
  }
  // warp butterflies in FP32 (max, min) and exact-pair arithmetic (sums),
  // then the warps' values in FP64 as in energy_partial_kernel
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int f = 0; f < F; f++) {
      mx[f] = fmaxf(mx[f], __shfl_xor_sync(0xffffffffu, mx[f], off));
      mn[f] = fminf(mn[f], __shfl_xor_sync(0xffffffffu, mn[f], off));
      vsum[f].merge_lane(off);
    }
    eac_p.merge_lane(off);
    ech_p.merge_lane(off);
    cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
  }
  double mxd[MAXF], mnd[MAXF];
  KS vol[MAXF], eac = {0.0, 0.0}, ech = {0.0, 0.0};
  if ((threadIdx.x & 31) == 0) {
    eac = KS{(double)eac_p.s, (double)eac_p.e};
    ech = KS{(double)ech_p.s, (double)ech_p.e};
#pragma unroll
    for (int f = 0; f < MAXF; f++) {
      const double sh = f >= NAC ? ph.cshift : 0.0;
      mxd[f] = f < F ? (double)mx[f < F ? f : 0] + sh : -1.0e30;
      mnd[f] = f < F ? (double)mn[f < F ? f : 0] + sh : 1.0e30;
      vol[f] = f < F ? KS{(double)vsum[f < F ? f : 0].s, (double)vsum[f < F ? f : 0].e} : KS{0.0, 0.0};
      ks_add(vol[f], (double)cnt * (sh + 1.0));
    }
  }
  block_record_from_warps(mxd, mnd, vol, eac, ech, F, part);
}

// ---- FP64 states: the same z-marching form in FP64 -------------------------
//
// The column tile and the plane walk of energy_partial_f32, with FP64 values
// and compensated FP64 (TwoSum) running sums.  Two loads per field and cell
// instead of eight.
template <typename PL, int NAC, int NCH>
__global__ void __launch_bounds__(256, 1) energy_partial_f64z(Phys ph, const double *__restrict__ u,
                                                              const double *__restrict__ elam, int form,
                                                              double *__restrict__ part) {
  constexpr int F = NAC + NCH;
  const int n = ph.n, N = n - 4;
  const long long n3 = (long long)n * n * n;
  __shared__ double q6[4][6];  // half epn2 times the symmetrised gradient tensors: xx yy zz xy xz yz
  if (threadIdx.x < 4 * 6 && threadIdx.y == 0) {
    const int m = threadIdx.x / 6, c = threadIdx.x % 6;
    const double *L = elam + 9 * m;
    const double v = c == 0 ? L[0] : c == 1 ? L[4] : c == 2 ? L[8] : c == 3 ? L[1] + L[3] : c == 4 ? L[2] + L[6] : L[5] + L[7];
    q6[m][c] = 0.5 * ph.epn2 * v;
  }
  __syncthreads();
  const double i4hx = 0.25 / ph.h[0], i4hy = 0.25 / ph.h[1], i4hz = 0.25 / ph.h[2], half_epn2 = 0.5 * ph.epn2;
  double Kt[16];
#pragma unroll
  for (int k = 0; k < 16; k++) Kt[k] = ph.K[k];
  const double p2 = 2376.0 / 2372.0 / 2.0, p3 = (7128.0 + 12.0 * 2372.0) / 2372.0 / 3.0,
               p4 = (4752.0 + 12.0 * 2372.0) / 2372.0 / 4.0;
  double mx[F], mn[F];
  KS vsum[F], eac = {0.0, 0.0}, ech = {0.0, 0.0};
  long long cnt = 0;
#pragma unroll
  for (int f = 0; f < F; f++) {
    mx[f] = -1.0e30;
    mn[f] = 1.0e30;
    vsum[f] = KS{0.0, 0.0};
  }
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int nti = (N + 31) / 32, ntj = (N + 7) / 8, units = energy_units(N);
  for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
    const int ti = unit % nti, tj = (unit / nti) % ntj, zc = unit / (nti * ntj);
    const int i = 2 + ti * 32 + tx, j = 2 + tj * 8 + ty;
    const bool own = i <= n - 3 && j <= n - 3, inner = i <= n - 4 && j <= n - 4;
    const int ic = i < n - 2 ? i : n - 2, jc = j < n - 2 ? j : n - 2;
    const int k0 = 2 + zc * EZ, k1 = k0 + EZ < n - 2 ? k0 + EZ : n - 2;
    double a0[F], a1[F], a2[F], a3[F];
    const long long row0 = ((long long)k0 * n + jc) * n + ic;
#pragma unroll
    for (int f = 0; f < F; f++) {
      const double *q = u + f * n3 + row0;
      a0[f] = q[0];
      a2[f] = q[n];
      a1[f] = __shfl_down_sync(0xffffffffu, a0[f], 1);
      a3[f] = __shfl_down_sync(0xffffffffu, a2[f], 1);
      if (tx == 31) {
        a1[f] = q[1];
        a3[f] = q[n + 1];
      }
    }
    for (int k = k0; k < k1; k++) {
      double b0[F], b1[F], b2[F], b3[F];
      const long long row = ((long long)(k + 1) * n + jc) * n + ic;
#pragma unroll
      for (int f = 0; f < F; f++) {
        const double *q = u + f * n3 + row;
        b0[f] = q[0];
        b2[f] = q[n];
        b1[f] = __shfl_down_sync(0xffffffffu, b0[f], 1);
        b3[f] = __shfl_down_sync(0xffffffffu, b2[f], 1);
        if (tx == 31) {
          b1[f] = q[1];
          b3[f] = q[n + 1];
        }
      }
      if (own) {
        cnt++;
#pragma unroll
        for (int f = 0; f < F; f++) {
          mx[f] = fmax(mx[f], a0[f]);
          mn[f] = fmin(mn[f], a0[f]);
          ks_add(vsum[f], a0[f]);
        }
      }
      if (inner && k <= n - 4) {
        double avg[F > 0 ? F : 1];
        double e_ac = 0.0, e_ch = 0.0, cbar = 0.0;
#pragma unroll
        for (int f = 0; f < F; f++) {
          const double v0 = a0[f], v1 = a1[f], v2 = a2[f], v3 = a3[f], v4 = b0[f], v5 = b1[f], v6 = b2[f],
                       v7 = b3[f];
          avg[f] = (v0 + v1 + v2 + v3 + v4 + v5 + v6 + v7) * 0.125;
          const double ux = ((v1 - v0) + (v3 - v2) + (v5 - v4) + (v7 - v6)) * i4hx;
          const double uy = ((v2 - v0) + (v3 - v1) + (v6 - v4) + (v7 - v5)) * i4hy;
          const double uz = ((v4 - v0) + (v5 - v1) + (v6 - v2) + (v7 - v3)) * i4hz;
          if (f < NAC) {
            const double *qm = q6[f];
            e_ac += qm[0] * ux * ux + qm[1] * uy * uy + qm[2] * uz * uz + qm[3] * ux * uy + qm[4] * ux * uz +
                    qm[5] * uy * uz;
          } else {
            const double gr = half_epn2 * (ux * ux + uy * uy + uz * uz);
            if (form == 0) e_ch += gr;
            else e_ac += gr;
            cbar = avg[f];
          }
        }
        if (form == 0) {
          if (NAC > 0) {
            double s2 = 0.0, s3 = 0.0;
#pragma unroll
            for (int f = 0; f < (NAC < 4 ? NAC : 4); f++) {
              s2 += avg[f] * avg[f];
              s3 += avg[f] * avg[f] * avg[f];
            }
            e_ac += p2 * s2 - p3 * s3 + p4 * s2 * s2;
          }
          if (NCH > 0) e_ch += (cbar * cbar - 1.0) * (cbar * cbar - 1.0) * 0.25;
        } else {
          sclet_acv<double> ac[NAC > 0 ? NAC : 1];
          sclet_chv<double> ch[1];
#pragma unroll
          for (int m = 0; m < NAC; m++) ac[m].u = avg[m];
          ch[0].c = cbar;
          e_ac += PL::template f_bulk<double>(ac, ch, NAC, NCH, Kt);
        }
        ks_add(eac, e_ac);
        ks_add(ech, e_ch);
      }
#pragma unroll
      for (int f = 0; f < F; f++) {
        a0[f] = b0[f];
        a1[f] = b1[f];
        a2[f] = b2[f];
        a3[f] = b3[f];
      }
    }
  }
  double mxd[MAXF], mnd[MAXF];
  KS vol[MAXF];
#pragma unroll
  for (int f = 0; f < MAXF; f++) {
    mxd[f] = f < F ? mx[f < F ? f : 0] : -1.0e30;
    mnd[f] = f < F ? mn[f < F ? f : 0] : 1.0e30;
    vol[f] = f < F ? vsum[f < F ? f : 0] : KS{0.0, 0.0};
    ks_add(vol[f], (double)cnt);  // sum of (value + 1)
  }
  block_record(mxd, mnd, vol, eac, ech, F, part);
}

// Final reduction over the block records: one warp per quantity (per field
// max, min, vol; the two energies); each lane folds a fixed strided subset of
// the records, then a butterfly (deterministic).
__global__ void energy_final_kernel(Phys ph, int form, const double *__restrict__ part, int npart,
                                    double *__restrict__ out) {
  const int F = ph.F, L = rec_len(F);
  // blockIdx.x = run
  part += (long long)blockIdx.x * npart * L;
  out += (long long)blockIdx.x * 4 * F;
  const double h3 = ph.h[0] * ph.h[1] * ph.h[2];
  __shared__ double res[4 * MAXF + 4];
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nq = 3 * F + 2;
  if (q < nq) {
    const int f = q < 3 * F ? q / 3 : -1, kind = q < 3 * F ? q % 3 : 3 + (q - 3 * F);
    double m = kind == 0 ? -1.0e30 : (kind == 1 ? 1.0e30 : 0.0);
    KS k = {0, 0};
    for (int b = lane; b < npart; b += 32) {
      const double *r = part + (long long)b * L;
      if (kind == 0) m = fmax(m, r[4 * f]);
      else if (kind == 1) m = fmin(m, r[4 * f + 1]);
      else if (kind == 2) k = ks_merge(k, KS{r[4 * f + 2], r[4 * f + 3]});
      else if (kind == 3) k = ks_merge(k, KS{r[4 * F], r[4 * F + 1]});
      else k = ks_merge(k, KS{r[4 * F + 2], r[4 * F + 3]});
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      if (kind == 0) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
      else if (kind == 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, off));
      else k = shfl_ks(k, off);
    }
    if (lane == 0) res[q] = kind < 2 ? m : k.s + k.c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int f = 0; f < F; f++) {
      out[4 * f] = res[3 * f];
      out[4 * f + 1] = res[3 * f + 1];
      out[4 * f + 2] = res[3 * f + 2] * h3;
      double e = (form == 0 && f >= ph.nac) ? res[3 * F + 1] : res[3 * F];
      out[4 * f + 3] = e * h3;
    }
  }
}

// partial records (blocks) of one reduction: four CTAs per SM at most
int check_soln_partials(int n) {
  const int u = energy_units(n - 4);
  return u > 152 * 4 ? 152 * 4 : (u < 1 ? 1 : u);
}

template <typename PL, int NAC, int NCH>
static void launch_f32(const Phys &ph, const float *u, const double *elam, int form, double *partials, int npart,
                       cudaStream_t s) {
  energy_partial_f32<PL, NAC, NCH><<<dim3(npart, ph.runs > 1 ? ph.runs : 1), dim3(32, 8), 0, s>>>(
      ph, econst<PL>(ph), u, elam, form, partials);
}

template <typename PL, typename T>
static cudaError_t check_soln_pl(const Phys &ph, const T *u, const double *elam, int form, double *partials,
                                 int npart, cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    const float *uf = u;
    switch (ph.nac * 2 + ph.nch) {
      case 1: launch_f32<PL, 0, 1>(ph, uf, elam, form, partials, npart, s); break;
      case 2: launch_f32<PL, 1, 0>(ph, uf, elam, form, partials, npart, s); break;
      case 3: launch_f32<PL, 1, 1>(ph, uf, elam, form, partials, npart, s); break;
      case 4: launch_f32<PL, 2, 0>(ph, uf, elam, form, partials, npart, s); break;
      case 5: launch_f32<PL, 2, 1>(ph, uf, elam, form, partials, npart, s); break;
      case 6: launch_f32<PL, 3, 0>(ph, uf, elam, form, partials, npart, s); break;
      case 7: launch_f32<PL, 3, 1>(ph, uf, elam, form, partials, npart, s); break;
      case 8: launch_f32<PL, 4, 0>(ph, uf, elam, form, partials, npart, s); break;
      default: launch_f32<PL, 4, 1>(ph, uf, elam, form, partials, npart, s); break;
    }
  } else {
    const double *ud = u;
    const dim3 g(npart), b(32, 8);
    switch (ph.nac * 2 + ph.nch) {
#define SCLET_F64Z(NA, NC) \
  case NA * 2 + NC: energy_partial_f64z<PL, NA, NC><<<g, b, 0, s>>>(ph, ud, elam, form, partials); break;
      SCLET_F64Z(0, 1) SCLET_F64Z(1, 0) SCLET_F64Z(1, 1) SCLET_F64Z(2, 0) SCLET_F64Z(2, 1)
      SCLET_F64Z(3, 0) SCLET_F64Z(3, 1) SCLET_F64Z(4, 0) SCLET_F64Z(4, 1)
#undef SCLET_F64Z
      default: energy_partial_kernel<PL, T><<<npart, EB, 0, s>>>(ph, u, elam, form, partials);
    }
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_check_soln(const Phys &ph, const T *u, const double *elam, int form, double *partials, int npart,
                              double *out, cudaStream_t s) {
  if (ph.F < 1 || ph.F > MAXF || ph.nac > 4 || ph.nch > 1) return cudaErrorInvalidValue;
  if (ph.runs > 1 && sizeof(T) != 4) return cudaErrorInvalidValue;  // several runs: FP32 states
  cudaError_t e = with_physics(ph.physics, [&](auto *tag) {
    using PL = std::remove_pointer_t<decltype(tag)>;
    return check_soln_pl<PL, T>(ph, u, elam, form, partials, npart, s);
  });
  if (e != cudaSuccess) return e;
  energy_final_kernel<<<ph.runs > 1 ? ph.runs : 1, 32 * (3 * MAXF + 2), 0, s>>>(ph, form, partials, npart, out);
  launch_counter() += 2;
  return cudaGetLastError();
}

template cudaError_t launch_check_soln<double>(const Phys &, const double *, const double *, int, double *, int, double *,
                                               cudaStream_t);
template cudaError_t launch_check_soln<float>(const Phys &, const float *, const double *, int, double *, int, double *,
                                              cudaStream_t);

}  // namespace sclet
