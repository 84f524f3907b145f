// FP32-input form of the split-BF16 tensor-core mode-n product (see
// k_modeprod_tc.cu for the number format and the slice-plane form): the
// input operand is sliced in shared memory by converter warps.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <stdint.h>
#include <string.h>

#include "sclet_internal.cuh"
#include "sclet_tc.cuh"
#include "sclet_tc_ptx.cuh"

namespace sclet {

namespace tc {

// ---- FP32-input form ---------------------------------------------------------
//
// The input operand arrives as FP32 rows (TMA, 128-byte swizzle, F_SR
// k-blocks ahead) and two converter warps (two tile rows per thread) cut it
// into the four fixed-point slices in shared memory, in the 64-byte swizzled
// K-major layout the MMAs read (the layout a TMA load of slice planes would
// produce).  The slice planes never exist in global memory.  Row scales come
// from line maxima: 2^ceil(log2 max|x|) over each input row, found by the
// epilogue that produced the rows (atomic maxima) or by tc_line_max.
//
// Rings: matrix slices (F_SA stages, full by TMA, empty when every CTA of the
// cluster has run its MMAs), raw FP32 rows (F_SR stages, full by TMA, refilled
// by the converters themselves once both warps have read a stage) and
// converted slices (F_SC stages, full when the converters have written them,
// empty when the local MMAs completed).
constexpr int F_THREADS = 256;  // producer, MMA, four epilogue, two converter warps (two per SM sub-partition)
constexpr int F_SA = 2, F_SC = 2, F_SR = 4;
constexpr int A_BYTES = NPM * PLANE_A;      // 40 KB
constexpr int C_BYTES = NP * PLANE_B;       // 32 KB
constexpr int RAW_BYTES = BN * BK * 4;      // 16 KB
constexpr int F_ALIGN = 1024;               // period of the 128-byte swizzle pattern
constexpr int F_SMEM = F_SR * RAW_BYTES + F_SA * A_BYTES + F_SC * C_BYTES + F_ALIGN;
static_assert(F_SMEM + 4096 <= 227 * 1024, "shared memory per CTA");
static_assert(BK * 4 == 128, "one FP32 row of a k-block is one 128-byte swizzle row");

// nearest integer (ties to even) of |y| < 2^22 by the 1.5 * 2^23 shift
__device__ __forceinline__ float round_int(float y) {
  return __fsub_rn(__fadd_rn(y, 12582912.0f), 12582912.0f);
}
// BF16 pair of two integer-valued floats of magnitude <= 256 (exact: their
// low 16 bits are zero), lo in the low half
__device__ __forceinline__ uint32_t pack_int_bf16x2(float lo, float hi) {
  return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

// lane 0 waits (bounded), the warp takes its verdict
__device__ __forceinline__ bool warp_wait(uint64_t *bar, uint32_t parity, int lane) {
  int ok = 1;
  if (lane == 0) ok = mbar_wait(bar, parity) ? 1 : 0;
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

template <int CA, int CR>
__global__ void __launch_bounds__(F_THREADS, 1)
    modeprod_tcf_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmX, TcArgs g) {
  constexpr int CL = CA * CR;
  constexpr uint16_t ALL = (uint16_t)((1u << CL) - 1);
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t afull[F_SA], aempty[F_SA];
  __shared__ __align__(8) uint64_t cfull[F_SC], cempty[F_SC];
  __shared__ __align__(8) uint64_t rfull[F_SR], rdone[F_SR];
  __shared__ __align__(8) uint64_t tfull_bar[NBUF], tempty_bar[NBUF];
  __shared__ __align__(8) uint64_t done_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;

  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + F_ALIGN - 1) & ~(uintptr_t)(F_ALIGN - 1));
  uint8_t *raw_base = base;                      // F_SR x 16 KB, 1024-aligned
  uint8_t *a_base = raw_base + F_SR * RAW_BYTES;  // F_SA x 40 KB
  uint8_t *c_base = a_base + F_SA * A_BYTES;      // F_SC x 32 KB
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long rows = (long long)g.n * g.n;
  const int a_tiles = (g.n + BM - 1) / BM;
  const int r_tiles = (int)((rows + BN - 1) / BN);
  const int r_groups = (r_tiles + CR - 1) / CR;
  const int a_groups = (a_tiles + CA - 1) / CA;
  const int total = a_groups * r_groups * g.count;
  const int nkb = g.kblocks;
  const int rank = (int)cluster_rank(), cid = (int)cluster_index(), ncl = (int)cluster_count();
  const int ra = rank % CA, rr = rank / CA;
  uint16_t mask_a = 0;
  for (int k = 0; k < CR; k++) mask_a |= (uint16_t)(1u << (ra + CA * k));

  if (threadIdx.x == 0) {
    for (int s = 0; s < F_SA; s++) {
      mbar_init(&afull[s], 1);
      mbar_init(&aempty[s], CL);  // the MMAs of every CTA in the cluster
    }
    for (int s = 0; s < F_SC; s++) {
      mbar_init(&cfull[s], 2);   // the local converter warps
      mbar_init(&cempty[s], 1);  // the local MMAs
    }
    for (int s = 0; s < F_SR; s++) {
      mbar_init(&rfull[s], 1);
      mbar_init(&rdone[s], 2);  // both converter warps have read the stage
    }
    for (int b = 0; b < NBUF; b++) {
      mbar_init(&tfull_bar[b], 1);
      mbar_init(&tempty_bar[b], 4);
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
  cluster_sync_all();

  if (warp == 0) {
    if (lane == 0) {
      // producer: the matrix slices of every k-block
      int it = 0;
      for (int gam = cid; gam < total; gam += ncl) {
        const TileIdx ti = tile_of<CA, CR>(gam, ra, rr, a_groups, r_groups);
        for (int kb = 0; kb < nkb; kb++, it++) {
          const int sa = it % F_SA;
          if (it >= F_SA && !mbar_wait(&aempty[sa], ((it / F_SA) & 1) ^ 1)) {
            failed = 1;
            break;
          }
          if (*(volatile int *)&failed) break;
          mbar_expect_tx(&afull[sa], A_BYTES);
          for (int p = rr; p < NPM; p += CR)
            tma_load_3d_mc(a_base + sa * A_BYTES + p * PLANE_A, &tmA, kb * BK, ti.a_tile * BM, p, &afull[sa], mask_a);
        }
        if (*(volatile int *)&failed) break;
      }
      if (*(volatile int *)&failed) {
        for (int i = it - F_SA < 0 ? 0 : it - F_SA; i < it; i++) mbar_wait(&afull[i % F_SA], (i / F_SA) & 1);
      }
      // tail: every consumption of this CTA's matrix stages by the cluster
      // has arrived, so no peer signals this CTA after it exits
      for (int s = 0; s < F_SA && s < it; s++) {
        const int last = it - 1 - ((it - 1 - s) % F_SA);
        if (!mbar_wait(&aempty[s], (last / F_SA) & 1)) failed = 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16(BM, BN);
      const int pairA[11] = {4, 0, 1, 2, 3, 0, 1, 2, 0, 1, 0};
      const int pairB[11] = {0, 3, 2, 1, 0, 2, 1, 0, 1, 0, 0};
      const int cls[11] = {3, 3, 3, 3, 3, 2, 2, 2, 1, 1, 0};
      int it = 0, j = 0;
      for (int gam = cid; gam < total && !*(volatile int *)&failed; gam += ncl, j++) {
        const int b = j % NBUF;
        if (j >= NBUF && !mbar_wait(&tempty_bar[b], ((j / NBUF) & 1) ^ 1)) {
          failed = 1;
          break;
        }
        fence_after();
        const uint32_t acc = tmem + (uint32_t)(b * ACC_COLS);
        bool ok = true;
        for (int kb = 0; kb < nkb; kb++, it++) {
          const int sa = it % F_SA, sc = it % F_SC;
          if (!mbar_wait(&afull[sa], (it / F_SA) & 1) || !mbar_wait(&cfull[sc], (it / F_SC) & 1)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t sA = smem_u32(a_base + sa * A_BYTES);
          const uint32_t sB = smem_u32(c_base + sc * C_BYTES);
#pragma unroll
          for (int ks = 0; ks < BK / 16; ks++) {
            const uint32_t koff = ks * 32;
            const bool first = (kb == 0 && ks == 0);
#pragma unroll
            for (int q = 0; q < 11; q++) {
              const int pa = pairA[q], pb = pairB[q], w = cls[q];
              const bool start = first && (q == 0 || q == 5 || q == 8 || q == 10);
              mma_bf16(acc + (uint32_t)(w * BN), smem_desc(sA + pa * PLANE_A + koff), smem_desc(sB + pb * PLANE_B + koff),
                       idesc, start ? 0u : 1u);
            }
          }
          mma_commit_mc(&aempty[sa], ALL);
          mma_commit(&cempty[sc]);
        }
        if (!ok) {
          failed = 1;
          break;
        }
        mma_commit(&tfull_bar[b]);
      }
      mma_commit(&done_bar);
      if (!mbar_wait(&done_bar, 0)) failed = 1;
    }
  } else if (warp >= 6) {
    // converters: thread i = tile rows i and i + 64; per k-block their 32
    // FP32 values -> four slice planes (16-byte granules, 64-byte swizzle).
    // Thread 192 keeps the raw ring F_SR k-blocks ahead.
    const int i = threadIdx.x - 192;
    const float step = ldexpf(1.0f, g.bits);
    const int ntiles = cid < total ? (total - cid + ncl - 1) / ncl : 0;
    const int T = ntiles * nkb;  // k-blocks of this CTA
    auto issue = [&](int j) {  // raw rows of k-block j into stage j % F_SR
      const int kb = j % nkb;
      const TileIdx ti = tile_of<CA, CR>(cid + (j / nkb) * ncl, ra, rr, a_groups, r_groups);
      uint64_t *bar = &rfull[j % F_SR];
      mbar_expect_tx(bar, RAW_BYTES);
      tma_load_3d(raw_base + (j % F_SR) * RAW_BYTES, &tmX, kb * BK, ti.r_tile * BN, ti.t, bar);
    };
    int issued = 0;
    if (i == 0)
      for (; issued < F_SR && issued < T; issued++) issue(issued);
    float mul[2] = {0.0f, 0.0f};
    bool ok = true;
    for (int it = 0; it < T && ok; it++) {
      const int kb = it % nkb, sr = it % F_SR, sc = it % F_SC;
      if (kb == 0) {  // a new tile: the rows' multipliers 2^b / S
        const TileIdx ti = tile_of<CA, CR>(cid + (it / nkb) * ncl, ra, rr, a_groups, r_groups);
#pragma unroll
        for (int hr = 0; hr < 2; hr++) {
          const long long r = (long long)ti.r_tile * BN + i + 64 * hr;
          mul[hr] = r < rows ? step / pow2_scale(__uint_as_float(g.lmax_in[(long long)ti.t * rows + r])) : 0.0f;
        }
      }
      if (!warp_wait(&rfull[sr], (it / F_SR) & 1, lane) ||
          (it >= F_SC && !warp_wait(&cempty[sc], ((it / F_SC) & 1) ^ 1, lane))) {
        ok = false;
        break;
      }
      // loops kept rolled: the kernel's four roles share the instruction cache
#pragma unroll 1
      for (int hr = 0; hr < 2; hr++) {
        const int row = i + 64 * hr;
        const uint8_t *rw = raw_base + sr * RAW_BYTES + row * 128;
        uint8_t *cw = c_base + sc * C_BYTES + row * 64;
        const float m = mul[hr];
#pragma unroll 1
        for (int h = 0; h < 4; h++) {
          const float4 lo = *reinterpret_cast<const float4 *>(rw + (((2 * h) ^ (row & 7)) << 4));
          const float4 hi = *reinterpret_cast<const float4 *>(rw + (((2 * h + 1) ^ (row & 7)) << 4));
          const float x[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
          uint32_t pk[NP][4];
#pragma unroll
          for (int e = 0; e < 8; e += 2) {
            float y0 = x[e] * m, y1 = x[e + 1] * m;
#pragma unroll
            for (int p = 0; p < NP; p++) {
              const float d0 = round_int(y0), d1 = round_int(y1);
              pk[p][e >> 1] = pack_int_bf16x2(d0, d1);
              y0 = (y0 - d0) * step;
              y1 = (y1 - d1) * step;
            }
          }
          const int off = (h ^ ((row >> 1) & 3)) << 4;
#pragma unroll
          for (int p = 0; p < NP; p++)
            *reinterpret_cast<uint4 *>(cw + p * PLANE_B + off) = make_uint4(pk[p][0], pk[p][1], pk[p][2], pk[p][3]);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(&cfull[sc]);
        mbar_arrive(&rdone[sr]);
      }
      // refill raw stage sr once both converter warps have read it
      if (i == 0 && issued < T) {
        if (mbar_wait(&rdone[sr], (it / F_SR) & 1)) issue(issued++);
        else failed = 1;
      }
      if (__any_sync(0xffffffffu, *(volatile int *)&failed != 0)) ok = false;
    }
    if (i == 0) {
      // raw copies still in flight into this CTA land before it exits (bounded)
      const int done = ok ? T : 0;
      for (int j = done > issued - F_SR ? done : (issued - F_SR < 0 ? 0 : issued - F_SR); j < issued; j++)
        mbar_wait(&rfull[j % F_SR], (j / F_SR) & 1);
    }
    if (!ok && lane == 0) failed = 1;
  } else {
    // epilogue warps 2-5, as in modeprod_tc_kernel, with the input scales
    // from the line maxima and the line maxima of the output
    __shared__ float s_isc[4][BN];
    const int q = warp & 3;
    const int row = q * 32 + lane;
    const float wt[NACC] = {ldexpf(1.0f, -2 * g.bits), ldexpf(1.0f, -3 * g.bits), ldexpf(1.0f, -4 * g.bits),
                            ldexpf(1.0f, -5 * g.bits)};
    const bool vec = (rows & 3) == 0;
    int j = 0;
    for (int gam = cid; gam < total; gam += ncl, j++) {
      const int b = j % NBUF;
      if (!warp_wait(&tfull_bar[b], (j / NBUF) & 1, lane)) {
        if (lane == 0) failed = 1;
        break;
      }
      fence_after();
      float acc[BN / 32][32];
#pragma unroll
      for (int c = 0; c < BN / 32; c++) {
        float w[32];
        const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * ACC_COLS + c * 32);
        tmem_ld32(ta + 3 * BN, acc[c]);
#pragma unroll
        for (int jj = 0; jj < 32; jj++) acc[c][jj] *= wt[3];
#pragma unroll
        for (int k = 2; k >= 0; k--) {
          tmem_ld32(ta + k * BN, w);
#pragma unroll
          for (int jj = 0; jj < 32; jj++) acc[c][jj] = fmaf(w[jj], wt[k], acc[c][jj]);
        }
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty_bar[b]);
      const TileIdx ti = tile_of<CA, CR>(gam, ra, rr, a_groups, r_groups);
      const int a = ti.a_tile * BM + row;
      const int kind = (ti.t % g.F) >= g.nac ? 1 : 0;
      const long long tb = (long long)ti.t * g.n * rows;
      const float sa = a < g.n ? g.row_scale[a] : 0.0f;
      const unsigned *lin = g.lmax_in + (long long)ti.t * rows;
      const long long rt0 = (long long)ti.r_tile * BN;
      for (int i = lane; i < BN; i += 32)
        s_isc[q][i] = rt0 + i < rows ? pow2_scale(__uint_as_float(lin[rt0 + i])) : 0.0f;
      __syncwarp();
      // output line of element (a, r): a * n + r / n, tracked as r advances
      unsigned *lout = g.lmax_out ? g.lmax_out + (long long)ti.t * rows + (long long)a * g.n : nullptr;
      long long line = rt0 / g.n, line_end = (line + 1) * g.n;
      float lm = 0.0f;
      auto track = [&](long long r, float y) {
        if (r >= line_end) {
          if (lm > 0.0f) atomicMax(lout + line, __float_as_uint(lm));
          lm = 0.0f;
          line = r / g.n;
          line_end = (line + 1) * g.n;
        }
        lm = fmaxf(lm, fabsf(y));
      };
#pragma unroll
      for (int c = 0; c < BN / 32; c++) {
        if (a < g.n) {
          const long long r0 = rt0 + c * 32;
          const long long o0 = (long long)a * rows + r0;
          const float *si = &s_isc[q][c * 32];
          if (vec && r0 + 32 <= rows) {
#pragma unroll
            for (int jj = 0; jj < 32; jj += 4) {
              float4 y = make_float4(acc[c][jj] * (si[jj] * sa), acc[c][jj + 1] * (si[jj + 1] * sa),
                                     acc[c][jj + 2] * (si[jj + 2] * sa), acc[c][jj + 3] * (si[jj + 3] * sa));
              const long long o = o0 + jj;
              if (g.epi == 1) {
                const float4 uh = *reinterpret_cast<const float4 *>(g.aux + tb + o);
                const float4 c0 = g.coef[kind][o], c1 = g.coef[kind][o + 1], c2 = g.coef[kind][o + 2],
                             c3 = g.coef[kind][o + 3];
                y.x = fmaf(c0.x, uh.x, fmaf(c0.y, uh.x, fmaf(c0.z, y.x, c0.w * y.x)));
                y.y = fmaf(c1.x, uh.y, fmaf(c1.y, uh.y, fmaf(c1.z, y.y, c1.w * y.y)));
                y.z = fmaf(c2.x, uh.z, fmaf(c2.y, uh.z, fmaf(c2.z, y.z, c2.w * y.z)));
                y.w = fmaf(c3.x, uh.w, fmaf(c3.y, uh.w, fmaf(c3.z, y.w, c3.w * y.w)));
              } else if (g.epi == 2) {
                const float2 c0 = g.coef2[kind][o], c1 = g.coef2[kind][o + 1], c2 = g.coef2[kind][o + 2],
                             c3 = g.coef2[kind][o + 3];
                y.x = fmaf(c0.x, y.x, c0.y * y.x);
                y.y = fmaf(c1.x, y.y, c1.y * y.y);
                y.z = fmaf(c2.x, y.z, c2.y * y.z);
                y.w = fmaf(c3.x, y.w, c3.y * y.w);
              }
              float4 *dst = reinterpret_cast<float4 *>(g.out + tb + o);
              if (g.outmode == 2) {
                const float4 old = *dst;
                y.x += old.x;
                y.y += old.y;
                y.z += old.z;
                y.w += old.w;
              }
              *dst = y;
              if (lout) {
                track(r0 + jj, y.x);
                track(r0 + jj + 1, y.y);
                track(r0 + jj + 2, y.z);
                track(r0 + jj + 3, y.w);
              }
            }
          } else {
#pragma unroll
            for (int jj = 0; jj < 32; jj++) {
              const long long r = r0 + jj;
              if (r < rows) {
                float y = acc[c][jj] * (si[jj] * sa);
                const long long o = o0 + jj;
                if (g.epi == 1) {
                  const float uh = g.aux[tb + o];
                  const float4 cc = g.coef[kind][o];
                  y = fmaf(cc.x, uh, fmaf(cc.y, uh, fmaf(cc.z, y, cc.w * y)));
                } else if (g.epi == 2) {
                  const float2 cc = g.coef2[kind][o];
                  y = fmaf(cc.x, y, cc.y * y);
                }
                if (g.outmode == 1) g.out[tb + o] = y;
                else y = (g.out[tb + o] += y);
                if (lout) track(r, y);
              }
            }
          }
        }
      }
      if (lout && a < g.n && lm > 0.0f) atomicMax(lout + line, __float_as_uint(lm));
      __syncwarp();
      if (__any_sync(0xffffffffu, *(volatile int *)&failed != 0)) break;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && failed) atomicExch(g.err, 1);
  cluster_sync_all();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// Line maxima of FP32 rows (x - sub, also stored to diff), one warp per row.
__global__ void line_max_kernel(const float *__restrict__ x, const float *__restrict__ sub, float *__restrict__ diff,
                                unsigned *__restrict__ lmax, int n, long long total_rows) {
  const int lane = threadIdx.x & 31;
  const long long warp0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long wr = warp0; wr < total_rows; wr += nwarps) {
    const long long in0 = wr * n;
    float m = 0.0f;
    for (int k = lane; k < n; k += 32) {
      float v = x[in0 + k];
      if (sub) {
        v -= sub[in0 + k];
        diff[in0 + k] = v;
      }
      m = fmaxf(m, fabsf(v));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if (lane == 0) lmax[wr] = __float_as_uint(m);
  }
}

}  // namespace tc

// ---- host side ------------------------------------------------------------

// FP32 rows of n values (n % 4 == 0: a 16-byte row pitch), 128-byte swizzle,
// box of 32 values x box_rows rows
static cudaError_t make_map_f32(CUtensorMap *map, const float *ptr, int n, long long rows, int depth, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  cuuint64_t dims[3] = {(cuuint64_t)n, (cuuint64_t)rows, (cuuint64_t)depth};
  cuuint64_t strides[2] = {(cuuint64_t)n * 4, (cuuint64_t)n * 4 * (cuuint64_t)rows};
  cuuint32_t box[3] = {(cuuint32_t)tc::BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(ptr), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

bool tc_fp32_input_ok(int n) { return n % 4 == 0 && n >= 8; }

cudaError_t launch_modeprod_tcf(const __nv_bfloat16 *mat, const float *x, int count, const TcArgs &args,
                                cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    for (int ca = 1; ca <= 2; ca++) {
      const void *fn =
          ca == 2 ? (const void *)tc::modeprod_tcf_kernel<2, 2> : (const void *)tc::modeprod_tcf_kernel<1, 4>;
      cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::F_SMEM);
      if (e != cudaSuccess) return e;
      e = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
      if (e != cudaSuccess) return e;
    }
    attr = true;
  }
  const int n = args.n, kp = tc_kp(n);
  if (!tc_fp32_input_ok(n) || !args.lmax_in) return cudaErrorInvalidValue;
  const int bits = tc_slice_bits(n);
  if ((long long)tc::BK * ((n + tc::BK - 1) / tc::BK) > (1LL << (24 - 2 * bits))) return cudaErrorInvalidValue;
  const int a_tiles = (n + tc::BM - 1) / tc::BM;
  const int CA = a_tiles % 2 == 0 ? 2 : 1;
  const int CR = CA == 2 ? 2 : 4;
  const int CL = CA * CR;
  CUtensorMap ma, mx;
  cudaError_t e;
  if ((e = make_map(&ma, mat, kp, n, TC_PLANES_M, tc::BM)) != cudaSuccess) return e;
  if ((e = make_map_f32(&mx, x, n, (long long)n * n, count, tc::BN)) != cudaSuccess) return e;
  TcArgs g = args;
  g.xin = x;
  g.kp = kp;
  g.kblocks = (n + tc::BK - 1) / tc::BK;
  g.bits = bits;
  const long long r_groups = (((long long)n * n + tc::BN - 1) / tc::BN + CR - 1) / CR;
  const long long groups = (long long)((a_tiles + CA - 1) / CA) * r_groups * count;
  if (groups > 0x7fffffffLL) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(tc::F_THREADS);
  cfg.dynamicSmemBytes = tc::F_SMEM;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  static int max_clusters[3] = {0, 0, 0};
  if (!max_clusters[CA]) {
    cfg.gridDim = dim3(CL * 128);
    e = CA == 2 ? cudaOccupancyMaxActiveClusters(&max_clusters[CA], tc::modeprod_tcf_kernel<2, 2>, &cfg)
                : cudaOccupancyMaxActiveClusters(&max_clusters[CA], tc::modeprod_tcf_kernel<1, 4>, &cfg);
    if (e != cudaSuccess) return e;
    if (max_clusters[CA] < 1) return cudaErrorInvalidConfiguration;
  }
  const int clusters = (int)(groups < max_clusters[CA] ? groups : max_clusters[CA]);
  cfg.gridDim = dim3(CL * clusters);
  e = CA == 2 ? cudaLaunchKernelEx(&cfg, tc::modeprod_tcf_kernel<2, 2>, ma, mx, g)
              : cudaLaunchKernelEx(&cfg, tc::modeprod_tcf_kernel<1, 4>, ma, mx, g);
  launch_counter()++;
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t tc_line_max(const float *x, const float *sub, float *diff, unsigned *lmax, int n, int count,
                        cudaStream_t s) {
  const long long rows = (long long)n * n * count;
  const long long blocks = (rows * 32 + 255) / 256;
  const int g = (int)(blocks > 152 * 32 ? 152 * 32 : blocks);
  tc::line_max_kernel<<<g, 256, 0, s>>>(x, sub, diff, lmax, n, rows);
  launch_counter()++;
  return cudaGetLastError();
}

}  // namespace sclet
