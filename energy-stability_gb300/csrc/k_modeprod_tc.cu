// Split-precision mode-n product on the 5th-generation tensor cores (tcgen05),
// the mixed-precision form of PUX / PUY / PUZ (source_beta_to_omega/src/
// calc.c:631-684).
//
// Number format: each operand is a power-of-two scale times four fixed-point
// slices of b bits, x = S * sum_p d_p 2^-b(p+1), d_0 in [-2^b, 2^b], d_p in
// [-2^(b-1), 2^(b-1)] (round to nearest at every level; 4b bits below S).
// b = 7 while the contraction length K <= 1024, else 6 (tc_slice_bits).  The
// slices are small integers held exactly in BF16.  The product keeps every
// cross term of weight w = p + q <= 3 (the split-precision scheme of Markidis
// et al. 2018 / Ootomo & Yokota 2022 carried to fixed point, as in the Ozaki
// scheme), one FP32 accumulator in tensor memory per weight class.  In classes
// 0 and 1 every partial sum is an integer below 2^24 (|sum| <= 2^(2b) per k
// times K <= 2^(24-2b)), so their accumulation is exact and unbiased; classes
// 2 and 3 sit 2^-2b and 2^-3b below the result, where accumulator rounding is
// harmless.  The matrix carries a fifth slice (its representation error would
// otherwise act on the leading data slice the same way every step); it is
// stored pre-scaled by 2^-b and its term M4 x0 joins class 3: eleven BF16 MMAs
// per k-step.  The epilogue combines the four classes with round-to-nearest
// adds.
//
// Scales: powers of two per matrix row (static) and per input row (one 1-D
// line along the contracted axis, 2^ceil(log2 max|x|) over the line, found by
// the slicing kernel), so a line holding a spectral peak or a boundary-lifting
// outlier costs precision only within itself.  The scale of an output entry
// is rank one (matrix row a' times input row r), so accumulation stays exact.
//
// Layout: input planes P[t][p][kb][r][32], k-blocked: rows r = 0 .. n*n-1 are
// 1-D lines along the contracted axis, k = 32 kb + (k % 32) < kp = roundup(n,
// 32), zero beyond n; one k-block of 128 consecutive rows is one contiguous
// 8 KB tile, so every TMA load reads whole 128-byte lines.  Matrix slices
// likewise [p][kb][a'][32].  Output FP32
// out[t][a' * n*n + r] for input row r = c * n + b, i.e. contracted index
// slowest: three products return to x-fastest order.
//
// Kernel: persistent CTAs (one per SM) looping over output tiles D[128 r x
// 128 a'] (input rows on the MMA's M side, eigen-modes a' on its N side, so
// the last a'-tile runs N = its live rows rounded up to 16 rather than a full
// 128).  A CTA takes whole groups (every a'-tile of one input tile, a'-tiles
// fastest, groups round robin, tensor fastest), so the CTAs stay balanced,
// the input slices come from HBM once (the group's later a'-tiles read them
// from L2) and the tensors of one input tile share the fused update's
// coefficient reads through L2; the matrix slices stay in L2.  Every CTA loads its own operand tiles (no
// cluster).
// A = input slices (128 r rows x 32 k, 64-byte swizzle), B = matrix slices
// (128 a' rows x 32 k), both K-major, in a three-stage mbarrier pipeline
// that runs ahead across tiles; a stage is refilled once the MMAs that read
// it have completed.
// Warp 0 issues TMA, warp 1 issues MMAs (one elected thread each) and owns the
// tensor memory (4 classes x 128 columns).  Warps 2-5 run the epilogue (TMEM
// lane quadrant warp % 4): the four classes of the tile are combined into
// registers and the tensor memory is released at once, then the scaling, the
// fused ETD update (ac_updateU_new / ch_updateU_new, calc.c:489-535) or phi2
// scaling (prepare_U2_new, calc.c:553-567) and the FP32 stores overlap the
// next tile's MMAs.  Every mbarrier wait is bounded: on timeout the CTA
// records an error, drains its copies and MMAs (bounded), frees TMEM and
// returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <stdint.h>
#include <string.h>

#include <mutex>

#include "sclet_internal.cuh"
#include "sclet_tc.cuh"

#include "sclet_tc_ptx.cuh"

namespace sclet {

namespace tc {

template <int EPI, int OUT>
__global__ void __launch_bounds__(THREADS, 1)
    modeprod_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcArgs g) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t tfull_bar[NBUF];   // accumulator set ready (MMA -> epilogue)
  __shared__ __align__(8) uint64_t tempty_bar[NBUF];  // accumulator set drained (epilogue -> MMA)
  __shared__ __align__(8) uint64_t done_bar;       // every MMA of this CTA completed
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;

  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + SMEM_ALIGN - 1) & ~(uintptr_t)(SMEM_ALIGN - 1));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long rows = (long long)g.n * g.n;
  const int a_tiles = (g.n + BN - 1) / BN;
  const int r_tiles = (int)((rows + BM - 1) / BM);
  // whole groups (every a'-tile of one input tile) per CTA, round robin
  const int groups = r_tiles * g.count;
  const int mine = (int)blockIdx.x < groups ? a_tiles * ((groups - 1 - (int)blockIdx.x) / (int)gridDim.x + 1) : 0;
  const int nkb = g.kblocks;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < NBUF; b++) {
      mbar_init(&tfull_bar[b], 1);
      mbar_init(&tempty_bar[b], EPI_WARPS);  // one arrival per epilogue warp
    }
    mbar_init(&done_bar, 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // producer: four input slices and five matrix slices per stage, the
      // k-blocks of all this CTA's tiles in one stream
      int it = 0;
      // the self-test leaves every barrier without arrivals (no copy is issued)
      for (int u = g.idle ? mine : 0; u < mine; u++) {
        const TileIdx ti = cta_tile(u, a_tiles, g.count, blockIdx.x, gridDim.x);
        for (int kb = 0; kb < nkb; kb++, it++) {
          const int s = it % STAGES;
          if (it >= STAGES && !mbar_wait(&empty_bar[s], ((it / STAGES) & 1) ^ 1)) {
            failed = 1;
            break;
          }
          if (*(volatile int *)&failed) break;
          uint8_t *st = base + s * STAGE_BYTES;
          mbar_expect_tx(&full_bar[s], STAGE_BYTES);
          // k-block kb of plane z is the contiguous block z * nkb + kb
          for (int p = 0; p < NP; p++)
            tma_load_3d(st + p * PLANE_A, &tmA, 0, ti.r_tile * BM, (ti.t * NP + p) * nkb + kb, &full_bar[s]);
          for (int p = 0; p < NPM; p++)
            tma_load_3d(st + NP * PLANE_A + p * PLANE_B, &tmB, 0, ti.a_tile * BN, p * nkb + kb, &full_bar[s]);
        }
        if (*(volatile int *)&failed) break;
      }
      if (*(volatile int *)&failed) {
        // drain: wait (bounded) for copies still in flight into this CTA
        for (int i = it - STAGES < 0 ? 0 : it - STAGES; i < it; i++) mbar_wait(&full_bar[i % STAGES], (i / STAGES) & 1);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer: 2 k-steps of 16 per stage, eleven terms each; (input
      // slice, matrix slice, class) grouped by class, small classes first; the
      // first term of each class at a tile's first k-step starts its
      // accumulator.  The last a'-tile runs N = its rows rounded up to 16.
      const int last_cols = g.n - (a_tiles - 1) * BN;
      const uint32_t idesc_full = idesc_bf16(BM, BN);
      const uint32_t idesc_last = idesc_bf16(BM, (last_cols + 15) / 16 * 16);
      const int pairA[11] = {0, 3, 2, 1, 0, 2, 1, 0, 1, 0, 0};  // input slice
      const int pairB[11] = {4, 0, 1, 2, 3, 0, 1, 2, 0, 1, 0};  // matrix slice
      const int cls[11] = {3, 3, 3, 3, 3, 2, 2, 2, 1, 1, 0};
      const bool last_two = g.n - (nkb - 1) * BK > 16;  // the last k-block needs both k-steps
      int it = 0, j = 0;
      for (int u = 0; u < mine && !*(volatile int *)&failed; u++, j++) {
        const int b = j % NBUF;
        // accumulator set b was last used by tile j - NBUF
        if (j >= NBUF && !mbar_wait(&tempty_bar[b], ((j / NBUF) & 1) ^ 1)) {
          failed = 1;
          break;
        }
        fence_after();
        const uint32_t acc = tmem + (uint32_t)(b * ACC_COLS);
        const uint32_t idesc = u % a_tiles == a_tiles - 1 ? idesc_last : idesc_full;
        bool ok = true;
        for (int kb = 0; kb < nkb; kb++, it++) {
          const int s = it % STAGES;
          if (!mbar_wait(&full_bar[s], (it / STAGES) & 1)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t sa = smem_u32(base + s * STAGE_BYTES);
          const uint32_t sb = sa + NP * PLANE_A;
#pragma unroll
          for (int ks = 0; ks < BK / 16; ks++) {
            // the last k-block's second k-step holds only zero columns when
            // n mod 32 is in 1..16: skipped (adding zero products changes no
            // accumulator)
            if (ks > 0 && kb == nkb - 1 && !last_two) continue;
            const uint32_t koff = ks * 32;
            const bool first = (kb == 0 && ks == 0);
#pragma unroll
            for (int q = 0; q < 11; q++) {
              const int pa = pairA[q], pb = pairB[q], w = cls[q];
              const bool start = first && (q == 0 || q == 5 || q == 8 || q == 10);
              uint64_t da = smem_desc(sa + pa * PLANE_A + koff);
              uint64_t db = smem_desc(sb + pb * PLANE_B + koff);
              mma_bf16(acc + (uint32_t)(w * BN), da, db, idesc, start ? 0u : 1u);
            }
          }
          mma_commit(&empty_bar[s]);
        }
        if (!ok) {
          failed = 1;
          break;
        }
        mma_commit(&tfull_bar[b]);
      }
      // every MMA issued so far must complete before the memory is freed
      mma_commit(&done_bar);
      if (!mbar_wait(&done_bar, 0)) failed = 1;
    }
  } else {
    // epilogue warps 2-9: TMEM lane quadrant q = warp % 4 holds input rows
    // q*32 .. q*32+31 of the tile, one per lane; the columns are the tile's
    // a' (eigen-mode) rows, the first half for warps 2-5, the second for
    // warps 6-9.  Each tile: combine the four classes of the warp's live
    // columns into registers, free the accumulators at once (the MMA warp
    // starts the next tile), then scale, apply the fused update and store
    // while those MMAs run.  For one a' the 32 lanes hold 32 consecutive
    // input rows, so every load and store of the warp is one contiguous
    // 128-byte run (512 bytes for the coefficient tables).
    const int q = warp & 3;
    const int c_first = ((warp - 2) >> 2) * CPW;  // the warp's first 32-column chunk
    // class weights 2^-b(w+2); exact integers combined small to large
    const float wt[NACC] = {ldexpf(1.0f, -2 * g.bits), ldexpf(1.0f, -3 * g.bits), ldexpf(1.0f, -4 * g.bits),
                            ldexpf(1.0f, -5 * g.bits)};
    int j = 0;
    for (int u = 0; u < mine; u++, j++) {
      const int b = j % NBUF;
      // one lane waits, the warp follows its verdict (tcgen05.ld below needs
      // the whole warp converged)
      int ok = 1;
      if (lane == 0) ok = mbar_wait(&tfull_bar[b], (j / NBUF) & 1) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) {
        if (lane == 0) failed = 1;
        break;
      }
      fence_after();
      const TileIdx ti = cta_tile(u, a_tiles, g.count, blockIdx.x, gridDim.x);
      const int at0 = ti.a_tile * BN;
      const int nch = (min(BN, g.n - at0) + 31) / 32;  // 32-column chunks holding live a'
      const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * ACC_COLS);
      // per live chunk two classes in flight at a time
      float acc[CPW][32];
#pragma unroll
      for (int cl = 0; cl < CPW; cl++) {
        const int c = c_first + cl;
        if (c < nch) {
          uint32_t ra[32], rb[32];
          tmem_ld32_async(ta + 3 * BN + c * 32, ra);
          tmem_ld32_async(ta + 2 * BN + c * 32, rb);
          tmem_wait_ld();
#pragma unroll
          for (int jj = 0; jj < 32; jj++)
            acc[cl][jj] = fmaf(__uint_as_float(rb[jj]), wt[2], __uint_as_float(ra[jj]) * wt[3]);
          tmem_ld32_async(ta + 1 * BN + c * 32, ra);
          tmem_ld32_async(ta + c * 32, rb);
          tmem_wait_ld();
#pragma unroll
          for (int jj = 0; jj < 32; jj++)
            acc[cl][jj] = fmaf(__uint_as_float(rb[jj]), wt[0], fmaf(__uint_as_float(ra[jj]), wt[1], acc[cl][jj]));
        }
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty_bar[b]);
      const long long r = (long long)ti.r_tile * BM + q * 32 + lane;
      const bool live = r < rows;
      const bool ch = (ti.t % g.F) >= g.nac;  // field kind: Cahn-Hilliard
      const float4 *cf = ch ? g.coef[1] : g.coef[0];
      const float2 *cf2 = ch ? g.coef2[1] : g.coef2[0];
      const long long tb = (long long)ti.t * g.n * rows;
      float *outT = g.out + tb;
      const float si = live ? g.in_scale[(long long)ti.t * rows + r] : 0.0f;
      // offsets within one tensor stay below n^3 < 2^32 (n <= 1088)
      const uint32_t urows = (uint32_t)rows;
#pragma unroll
      for (int cl = 0; cl < CPW; cl++) {
        const int c = c_first + cl;
        if (c < nch) {
          const int a0 = at0 + c * 32;
          const int lim = min(32, g.n - a0);  // live a' in the chunk
          // the chunk's 32 matrix-row scales, one per lane, broadcast below
          const float rs = lane < lim ? g.row_scale[a0 + lane] : 0.0f;
          const uint32_t o0 = (uint32_t)a0 * urows + (uint32_t)(live ? r : 0);  // eigen-mode [k][j][i] of a z-contraction
          // batches of columns: every load of a batch is issued before its
          // first store (aux and the coefficient tables are read-only here:
          // the ETD update never runs in place)
          constexpr int NB = EPI == 0 ? 8 : 4;
#pragma unroll
          for (int j0 = 0; j0 < 32; j0 += NB) {
            float uh[NB], old[NB];
            float4 c1[NB];
            float2 c2[NB];
#pragma unroll
            for (int jj = 0; jj < NB; jj++) {
              const uint32_t o = o0 + (uint32_t)(j0 + jj) * urows;
              if (j0 + jj < lim && live) {
                if (EPI == 1) {
                  uh[jj] = __ldg(g.aux + tb + o);
                  c1[jj] = __ldg(cf + o);
                } else if (EPI == 2) {
                  c2[jj] = __ldg(cf2 + o);
                }
                if (OUT == 2) old[jj] = outT[o];
              }
            }
#pragma unroll
            for (int jj = 0; jj < NB; jj++) {
              const uint32_t o = o0 + (uint32_t)(j0 + jj) * urows;
              const float sc = si * __shfl_sync(0xffffffffu, rs, j0 + jj);
              if (j0 + jj < lim && live) {
                float y = acc[cl][j0 + jj] * sc;
                if (EPI == 1) {
                  const float4 cc = c1[jj];  // (e_hi, e_lo, phi1_hi, phi1_lo)
                  y = fmaf(cc.x, uh[jj], fmaf(cc.y, uh[jj], fmaf(cc.z, y, cc.w * y)));
                } else if (EPI == 2) {
                  y = fmaf(c2[jj].x, y, c2[jj].y * y);  // (phi2_hi, phi2_lo)
                }
                if (OUT == 2) y += old[jj];
                outT[o] = y;
              }
            }
          }
        }
      }
      if (__any_sync(0xffffffffu, *(volatile int *)&failed != 0)) break;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && failed) atomicExch(g.err, 1);
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}


// FP32 rows of n (x - sub) -> slices: the row's max gives its power-of-two
// scale S; each slice is exact (the residual is scaled by 2^b and reduced by
// its nearest integer).
constexpr int SLICE_MAXC = 34;  // 32-column chunks per row: rows of up to 32 * 34 = 1088 values

// A warp takes two adjacent rows, one per half-warp (lane l: row l / 16,
// columns 2 (l % 16) + 32 c of chunk c, held in registers, C >= ceil(n / 32)).
// In the k-blocked layout the two rows' k-block c is one contiguous 128-byte
// run, so every store instruction of the warp fills whole lines.  Columns
// load as float2 when n is even.
template <int C>
__global__ void __launch_bounds__(256) slice_fields_kernel(const float *__restrict__ x, const float *__restrict__ sub,
                                                           float *__restrict__ scale, __nv_bfloat16 *__restrict__ out,
                                                           int n, int kp, int count, int bits) {
  const float step = ldexpf(1.0f, bits);
  const long long rows = (long long)n * n, total_rows = rows * count;
  const int lane = threadIdx.x & 31, h = lane >> 4, kl = 2 * (lane & 15);
  const int chunks = (n + BK - 1) / BK;
  const bool pairs = (n & 1) == 0;  // every row starts on an 8-byte boundary
  const long long warp0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long w0 = 2 * warp0; w0 < total_rows; w0 += 2 * nwarps) {
    const long long wr = w0 + h;
    const bool live = wr < total_rows;
    const long long in0 = wr * n;  // rows are contiguous lines of n
    float v0[C], v1[C];
    float m = 0.0f;
#pragma unroll
    for (int c = 0; c < C; c++) {
      v0[c] = 0.0f;
      v1[c] = 0.0f;
      const int k = kl + BK * c;
      if (live && c < chunks && k < n) {
        if (pairs) {
          float2 a = *reinterpret_cast<const float2 *>(x + in0 + k);
          if (sub) {
            const float2 b = *reinterpret_cast<const float2 *>(sub + in0 + k);
            a.x -= b.x;
            a.y -= b.y;
          }
          v0[c] = a.x;
          v1[c] = a.y;
        } else {
          v0[c] = sub ? x[in0 + k] - sub[in0 + k] : x[in0 + k];
          if (k + 1 < n) v1[c] = sub ? x[in0 + k + 1] - sub[in0 + k + 1] : x[in0 + k + 1];
        }
      }
      m = fmaxf(m, fmaxf(fabsf(v0[c]), fabsf(v1[c])));
    }
    // the row's max over its half-warp
#pragma unroll
    for (int off = 8; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if (!live) continue;
    const int t = (int)(wr / rows);
    const long long row = wr - (long long)t * rows;
    const float S = pow2_scale(m), inv = 1.0f / S;
    if (kl == 0) scale[wr] = S;
    const long long o0 = (long long)t * TC_PLANES * rows * kp + row * BK + kl;
    // stored as bf16 pairs (the pad columns n .. kp - 1 are never written:
    // they stay zero from the allocation)
#pragma unroll
    for (int c = 0; c < C; c++) {
      const int k = kl + BK * c;
      if (c < chunks && k < n) {
        float r0 = v0[c] * inv, r1 = v1[c] * inv;
#pragma unroll
        for (int p = 0; p < TC_PLANES; p++) {
          const float y0 = r0 * step, y1 = r1 * step;
          const float d0 = rintf(y0), d1 = rintf(y1);
          r0 = y0 - d0;
          r1 = y1 - d1;
          *reinterpret_cast<__nv_bfloat162 *>(out + o0 + (long long)p * rows * kp + (long long)c * rows * BK) =
              __floats2bfloat162_rn(d0, d1);
        }
      }
    }
  }
}

// FP64 matrix rows -> slices with a power-of-two scale per row.
__global__ void slice_matrix_kernel(const double *__restrict__ m, __nv_bfloat16 *__restrict__ out,
                                    float *__restrict__ row_scale, int n, int kp, int bits) {
  __shared__ double smax[128];
  const double step = ldexp(1.0, bits);
  for (int r = blockIdx.x; r < n; r += gridDim.x) {
    double mx = 0.0;
    for (int c = threadIdx.x; c < n; c += blockDim.x) mx = fmax(mx, fabs(m[(long long)r * n + c]));
    smax[threadIdx.x] = mx;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + w]);
      __syncthreads();
    }
    double S = 1.0;
    if (smax[0] > 0.0) {
      int e;
      frexp(smax[0], &e);
      S = ldexp(1.0, e);
    }
    __syncthreads();
    if (threadIdx.x == 0) row_scale[r] = (float)S;
    for (int c = threadIdx.x; c < kp; c += blockDim.x) {
      double v = c < n ? m[(long long)r * n + c] / S : 0.0;
      for (int p = 0; p < TC_PLANES_M; p++) {
        double y = v * step;
        double d = rint(y);
        v = y - d;
        // the fifth slice enters class 3, one factor 2^b below its own weight
        float q = p < TC_PLANES ? (float)d : (float)(d / step);
        out[(long long)p * n * kp + (long long)(c / BK) * n * BK + r * BK + c % BK] = __float2bfloat16_rn(q);
      }
    }
  }
}

// ETD coefficients in FP64 (the plain form's ac_init_phi / ch_init_phi and
// ac_updateU_new / ch_updateU_new arithmetic), stored as FP32 hi + lo.
__global__ void coef_kernel(float4 *coef, float2 *coef2, int n, int kind, const double *dx, const double *dy,
                            const double *dz, double kkx, double kky, double kkz, double epn2, double dt, double L,
                            double K) {
  const long long n3 = (long long)n * n * n;
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
      p1 = -expm1(-dt * H) / H;
      p2 = (1.0 - p1 / dt) / H;
    } else {
      p1 = dt;
      p2 = dt / 2;
    }
    double Hu = fabs(H) < 1.0e-8 ? 0.0 : H;
    double e = 1.0 - p1 * Hu;
    float4 c;
    c.x = (float)e;
    c.y = (float)(e - (double)c.x);
    c.z = (float)p1;
    c.w = (float)(p1 - (double)c.z);
    coef[o] = c;
    if (coef2) {
      float2 c2;
      c2.x = (float)p2;
      c2.y = (float)(p2 - (double)c2.x);
      coef2[o] = c2;
    }
  }
}

}  // namespace tc

// ---- host side ------------------------------------------------------------

int tc_kp(int n) { return (n + tc::BK - 1) / tc::BK * tc::BK; }

// Slice width: classes 0 and 1 stay exact while K 2^(2b) <= 2^24, K the
// contraction length rounded up to whole k-blocks.
int tc_slice_bits(int n) {
  const long long K = (long long)tc::BK * ((n + tc::BK - 1) / tc::BK);
  return K <= 1024 ? 7 : 6;
}

cudaError_t tc_slice_matrix(const double *m, __nv_bfloat16 *planes, float *row_scale, int n, cudaStream_t s) {
  tc::slice_matrix_kernel<<<n < 1024 ? n : 1024, 128, 0, s>>>(m, planes, row_scale, n, tc_kp(n), tc_slice_bits(n));
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t tc_slice_fields(const float *x, const float *sub, float *scale, __nv_bfloat16 *planes, int n, int count,
                            cudaStream_t s) {
  if (n > tc::BK * tc::SLICE_MAXC) return cudaErrorInvalidValue;
  long long warps = ((long long)n * n * count + 1) / 2;  // two rows per warp
  long long blocks = (warps * 32 + 255) / 256;
  int g = (int)(blocks > 152 * 32 ? 152 * 32 : blocks);
  const int chunks = (n + tc::BK - 1) / tc::BK, kp = tc_kp(n), bits = tc_slice_bits(n);
  if (chunks <= 4) tc::slice_fields_kernel<4><<<g, 256, 0, s>>>(x, sub, scale, planes, n, kp, count, bits);
  else if (chunks <= 8) tc::slice_fields_kernel<8><<<g, 256, 0, s>>>(x, sub, scale, planes, n, kp, count, bits);
  else if (chunks <= 17) tc::slice_fields_kernel<17><<<g, 256, 0, s>>>(x, sub, scale, planes, n, kp, count, bits);
  else tc::slice_fields_kernel<tc::SLICE_MAXC><<<g, 256, 0, s>>>(x, sub, scale, planes, n, kp, count, bits);
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t tc_make_coefs(float4 *coef, float2 *coef2, int n, int kind, const double *dx, const double *dy,
                          const double *dz, const double *kk, double epn2, double dt, double L, double K,
                          cudaStream_t s) {
  long long n3 = (long long)n * n * n;
  long long b = (n3 + 255) / 256;
  tc::coef_kernel<<<(int)(b > 152 * 16 ? 152 * 16 : b), 256, 0, s>>>(coef, coef2, n, kind, dx, dy, dz, kk[0], kk[1],
                                                                     kk[2], epn2, dt, L, K);
  launch_counter()++;
  return cudaGetLastError();
}

// The kernel's instances (fused update, output): (none, store), (none,
// accumulate), (ETD1, store), (phi2, store) -- the combinations the step uses.
using TcKernel = void (*)(const CUtensorMap, const CUtensorMap, TcArgs);
constexpr int TC_INSTANCES = 4;
static TcKernel tc_instance(int i) {
  static const TcKernel k[TC_INSTANCES] = {tc::modeprod_tc_kernel<0, 1>, tc::modeprod_tc_kernel<0, 2>,
                                           tc::modeprod_tc_kernel<1, 1>, tc::modeprod_tc_kernel<2, 1>};
  return k[i];
}
static TcKernel tc_kernel(int epi, int outmode) {
  if (outmode == 1 && epi >= 0 && epi <= 2) return tc_instance(epi == 0 ? 0 : epi + 1);
  if (outmode == 2 && epi == 0) return tc_instance(1);
  return nullptr;
}

// Per-device launch set-up: the dynamic shared-memory attributes (set per
// device, for every instance) and the number of CTAs that can be resident at
// once.
static int tc_setup(int *ctas) {
  constexpr int MAXDEV = 64;
  static std::mutex mu;
  static int resident[MAXDEV] = {0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= MAXDEV) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (!resident[dev]) {
    for (int i = 0; i < TC_INSTANCES; i++) {
      // all of the unified L1/shared capacity as shared memory
      e = cudaFuncSetAttribute(tc_instance(i), cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES);
      if (e != cudaSuccess) return e;
      e = cudaFuncSetAttribute(tc_instance(i), cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      if (e != cudaSuccess) return e;
    }
    int per_sm = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tc_kernel(0, 1), tc::THREADS, tc::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    resident[dev] = per_sm * sms;
  }
  *ctas = resident[dev];
  return cudaSuccess;
}

cudaError_t launch_modeprod_tc(const __nv_bfloat16 *mat, const __nv_bfloat16 *planes, int count, const TcArgs &args,
                               cudaStream_t s) {
  int ctas = 0;
  cudaError_t e = (cudaError_t)tc_setup(&ctas);
  if (e != cudaSuccess) return e;
  const TcKernel kern = tc_kernel(args.epi, args.outmode);
  if (!kern) return cudaErrorInvalidValue;
  const int n = args.n, kp = tc_kp(n);
  const int bits = tc_slice_bits(n);
  if ((long long)tc::BK * ((n + tc::BK - 1) / tc::BK) > (1LL << (24 - 2 * bits))) return cudaErrorInvalidValue;
  if ((long long)n * n * n > 0xffffffffLL) return cudaErrorInvalidValue;  // 32-bit offsets within a tensor
  CUtensorMap ma, mb;
  if ((e = make_map(&ma, planes, kp, (long long)n * n, TC_PLANES * count, tc::BM)) != cudaSuccess) return e;
  if ((e = make_map(&mb, mat, kp, n, TC_PLANES_M, tc::BN)) != cudaSuccess) return e;
  TcArgs g = args;
  g.kp = kp;
  g.kblocks = (n + tc::BK - 1) / tc::BK;
  g.bits = bits;
  const long long groups = (((long long)n * n + tc::BM - 1) / tc::BM) * count;  // input tiles
  if (groups * ((n + tc::BN - 1) / tc::BN) > 0x7fffffffLL) return cudaErrorInvalidValue;
  // persistent: as many CTAs as can be resident at once (or the tuned count)
  if (args.max_ctas > 0 && args.max_ctas < ctas) ctas = args.max_ctas;
  const int grid = (int)(groups < ctas ? groups : ctas);
  kern<<<grid, tc::THREADS, tc::SMEM_BYTES, s>>>(ma, mb, g);
  launch_counter()++;
  return cudaGetLastError();
}

}  // namespace sclet
