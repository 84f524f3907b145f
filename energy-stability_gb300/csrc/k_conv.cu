// Kernels of the learned coarse-step corrector: a periodic 3x3x3 convolution
// network on BF16 activations with FP32 accumulation.
//
// Activation layout (sclet_conv.cuh, conv_at): chunk-planar.  A sample is
// Np = N + 2 haloed planes (the N^3 periodic grid plus one periodic image
// layer per side); a plane holds 4 chunks of 8 channels, each chunk the
// plane's Np^2 cells (slot = yh Np + xh, 16 bytes each) padded to a multiple
// of 8 slots.
//
// conv_tc_kernel is an implicit GEMM on the 5th-generation tensor cores:
//   D[cell][co] = sum_{tap, ci} A[cell + off(tap)][ci] * W[tap][co][ci]
// with M = 128 cells, N = 32 output channels and K = 27 taps x 32 input
// channels.  A tile is 128 consecutive slots of one haloed plane.  For every
// plane dz of the stencil and every chunk, the rows all nine (dy, dx) taps
// read are one contiguous run of 128 + 2 Np + 2 slots: the producer loads
// those twelve runs (whole 128-byte lines, one TMA box each) and every tap's
// operand is a descriptor into them (no-swizzle K-major layout: rows 16 bytes
// apart, the chunks of a K step a box apart), offset by dy Np + dx rows.
// Slots in the x- or y-halo produce outputs that are dropped.  The weights
// (27 x 32 x 32 BF16, 54 KB) stay in shared memory.  Warp 0 issues TMA, warp 1
// issues the MMAs (54 per tile: two K = 16 steps per tap) into one of four
// 32-column TMEM accumulators, warps 2-5 drain them and run the fused
// epilogue (bias, ReLU, residual, ReLU-mask, FP32 planar output).  The same
// kernel computes the data gradient of a convolution with the weights
// flipped and transposed (the adjoint of a periodic convolution).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <atomic>
#include <mutex>

#include "sclet_internal.cuh"
#include "sclet_tc.cuh"
#include "sclet_tc_ptx.cuh"
#include "sclet_conv.cuh"

namespace sclet {
namespace conv {

using tc::fence_after;
using tc::fence_before;
using tc::mbar_arrive;
using tc::mbar_expect_tx;
using tc::mbar_init;
using tc::mbar_wait;
using tc::mma_bf16;
using tc::mma_commit;
using tc::smem_desc;
using tc::smem_u32;
using tc::tmem_ld32;

constexpr int ROWS = 128;                  // cells per tile (MMA M)
constexpr int MAX_STAGES = 3;              // tiles of input runs in flight
constexpr int WTILE = CH * CH * 2;         // 2 KB: one tap's 32 x 32 weights
constexpr int NACC = 4;                    // TMEM accumulators of 32 columns
constexpr int TMEM_COLS = NACC * CH;       // 128
constexpr int THREADS = 192;
constexpr int SMEM_LIMIT = 226 * 1024;  // dynamic shared memory: 227 KB per CTA less the static part

// Per-launch geometry.  ny = 1: per stencil plane and channel chunk one run
// of 128 + 2 Np + 2 slots serves all nine in-plane taps (twelve runs a tile);
// ny = 3: one run of 130 slots per stencil row dy (thirty-six runs a tile,
// fewer bytes once Np exceeds about 148).  A run is one box of box_rows lines
// of 128 bytes (8 slots), enough from any slot offset within the first line.
struct Geom {
  int ny, box_rows, box_bytes, stage_bytes, stages, smem;
};
static Geom geom_for(int N, int ny) {
  Geom g;
  g.ny = ny;
  const int R = ny == 1 ? ROWS + 2 * (N + 2) + 2 : ROWS + 2;
  g.box_rows = (R + 7 + 7) / 8;
  g.box_bytes = g.box_rows * 128;
  g.stage_bytes = 12 * ny * g.box_bytes;
  g.stages = (SMEM_LIMIT - 1024 - TAPS * WTILE) / g.stage_bytes;
  if (g.stages > MAX_STAGES) g.stages = MAX_STAGES;
  g.smem = TAPS * WTILE + (g.stages > 0 ? g.stages : 1) * g.stage_bytes + 1024;
  return g;
}
std::atomic<int> g_runs_per_plane{0};  // 0: by N; 1 or 3: forced (sclet_net_set_conv_runs)
static Geom geom_of(int N) {
  const Geom a = geom_for(N, 1), b = geom_for(N, 3);
  const int forced = g_runs_per_plane.load();
  if (forced == 1 && a.stages >= 1) return a;
  if (forced == 3) return b;
  return a.stages >= 1 && a.stage_bytes <= b.stage_bytes ? a : b;
}

// Shared-memory matrix descriptor, K-major without swizzle: 8-row core
// matrices 128 bytes apart (rows 16 bytes apart), K chunks lbo bytes apart.
__device__ __forceinline__ uint64_t smem_desc_plain(uint32_t addr, uint32_t lbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;  // leading byte offset: next K chunk
  d |= (uint64_t)(128 >> 4) << 32;              // stride byte offset: next 8 rows
  d |= (uint64_t)1 << 46;                       // descriptor version
  return d;                                     // layout type 0: no swizzle
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// tile -> (sample b, plane zh in 1..N, first slot s0 of the plane)
struct Tile {
  int b, zh, s0;
};
__device__ __forceinline__ Tile tile_of(int t, int N, int Np, int per_plane) {
  Tile x;
  const int j = t % per_plane;
  const int bz = t / per_plane;
  x.zh = 1 + bz % N;
  x.b = bz / N;
  x.s0 = Np + j * ROWS;
  return x;
}

__device__ __forceinline__ float bf(uint32_t w, int hi) {
  return __uint_as_float(hi ? (w & 0xffff0000u) : (w << 16));
}

__global__ void __launch_bounds__(THREADS, 1)
    conv_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmW, ConvArgs g,
                   int box_bytes, int stages, int ny) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[MAX_STAGES];
  __shared__ __align__(8) uint64_t empty_bar[MAX_STAGES];
  __shared__ __align__(8) uint64_t tfull_bar[NACC];
  __shared__ __align__(8) uint64_t tempty_bar[NACC];
  __shared__ __align__(8) uint64_t w_bar;
  __shared__ __align__(8) uint64_t done_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;
  __shared__ float s_bias[CH];

  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t *wsm = base;                    // 27 tap tiles of weights
  uint8_t *asm_ = base + TAPS * WTILE;    // stages x 12 ny input runs
  const int stage_bytes = 12 * ny * box_bytes;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int N = g.N, Np = N + 2;
  const int per_plane = (N * Np + ROWS - 1) / ROWS;
  const int total = g.batch * N * per_plane;

  if (threadIdx.x < CH) s_bias[threadIdx.x] = g.bias ? g.bias[threadIdx.x] : 0.0f;
  if (threadIdx.x == 0) {
    for (int s = 0; s < MAX_STAGES; s++) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < NACC; b++) {
      mbar_init(&tfull_bar[b], 1);
      mbar_init(&tempty_bar[b], 4);
    }
    mbar_init(&w_bar, 1);
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
      mbar_expect_tx(&w_bar, TAPS * WTILE);
      for (int t = 0; t < TAPS; t++) tma_load_2d(wsm + t * WTILE, &tmW, 0, t * CH, &w_bar);
      int it = 0;
      for (int tile = blockIdx.x; tile < total && !*(volatile int *)&failed; tile += gridDim.x, it++) {
        const Tile ti = tile_of(tile, N, Np, per_plane);
        const int s = it % stages;
        if (it >= stages && !mbar_wait(&empty_bar[s], ((it / stages) & 1) ^ 1)) {
          failed = 1;
          break;
        }
        // plane zh + dz - 1, chunk k: the run from slot s0 - Np - 1 (ny = 1)
        // or s0 + (dy - 1) Np - 1 (ny = 3), >= -1; a line before the buffer
        // or past its end reads as zeros
        mbar_expect_tx(&full_bar[s], stage_bytes);
        for (int dz = 0; dz < 3; dz++)
          for (int r = 0; r < ny; r++)
            for (int k = 0; k < 4; k++) {
              const long long first = (long long)ti.s0 + (ny == 1 ? -Np : (r - 1) * Np) - 1;
              const long long flat = conv_at(N, ti.b, ti.zh + dz - 1, k, first);
              tma_load_2d(asm_ + s * stage_bytes + ((dz * ny + r) * 4 + k) * box_bytes, &tmA, 0, (int)(flat >> 3),
                          &full_bar[s]);
            }
      }
      if (*(volatile int *)&failed) {
        for (int i = it - stages < 0 ? 0 : it - stages; i < it; i++) mbar_wait(&full_bar[i % stages], (i / stages) & 1);
      }
      mbar_wait(&w_bar, 0);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = tc::idesc_bf16(ROWS, CH);
      bool ok = mbar_wait(&w_bar, 0);
      if (!ok) failed = 1;
      fence_after();
      int it = 0;
      const uint32_t w0 = smem_u32(wsm), a0 = smem_u32(asm_);
      for (int tile = blockIdx.x; ok && tile < total && !*(volatile int *)&failed; tile += gridDim.x, it++) {
        const int b = it % NACC;
        if (it >= NACC && !mbar_wait(&tempty_bar[b], ((it / NACC) & 1) ^ 1)) {
          failed = 1;
          break;
        }
        const int s = it % stages;
        if (!mbar_wait(&full_bar[s], (it / stages) & 1)) {
          failed = 1;
          break;
        }
        fence_after();
        const uint32_t acc = tmem + (uint32_t)(b * CH);
        const Tile ti = tile_of(tile, N, Np, per_plane);
        // per stencil row dy: the run holding it (its offset in runs from the
        // plane's first) and the row of the tap dx = -1 within that run
        uint32_t rrun[3], rrow[3];
#pragma unroll
        for (int dy = 0; dy < 3; dy++) {
          const long long first = (long long)ti.s0 + (ny == 1 ? -Np : (dy - 1) * Np) - 1;
          rrun[dy] = ny == 1 ? 0u : (uint32_t)(dy * 4);
          rrow[dy] = (uint32_t)(first & 7) + (ny == 1 ? (uint32_t)(dy * Np) : 0u);
        }
        // descriptors of the stage's first run and of the first weight tile;
        // a tap adds its run and row offsets (16-byte units) to the address
        // field, which stays below 2^14 inside the shared memory
        const uint64_t dab = smem_desc_plain(a0 + (uint32_t)(s * stage_bytes), box_bytes);
        const uint64_t dwb = smem_desc(w0);
        const uint32_t run16 = (uint32_t)box_bytes >> 4;
#pragma unroll
        for (int tap = 0; tap < TAPS; tap++) {
          const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;  // each 0..2
#pragma unroll
          for (int ks = 0; ks < 2; ks++) {
            const uint64_t da =
                dab + (uint64_t)(((uint32_t)(dz * ny * 4 + 2 * ks) + rrun[dy]) * run16 + rrow[dy] + (uint32_t)dx);
            const uint64_t dw = dwb + (uint64_t)((tap * WTILE + ks * 32) >> 4);
            mma_bf16(acc, da, dw, idesc, (tap == 0 && ks == 0) ? 0u : 1u);
          }
        }
        mma_commit(&empty_bar[s]);
        mma_commit(&tfull_bar[b]);
      }
      mma_commit(&done_bar);
      if (!mbar_wait(&done_bar, 0)) failed = 1;
    }
  } else {
    const int q = warp & 3;
    const int row = q * 32 + lane;
    int j = 0;
    for (int tile = blockIdx.x; tile < total; tile += gridDim.x, j++) {
      const int b = j % NACC;
      int ok = 1;
      if (lane == 0) ok = mbar_wait(&tfull_bar[b], (j / NACC) & 1) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) {
        if (lane == 0) failed = 1;
        break;
      }
      fence_after();
      float acc[CH];
      tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * CH), acc);
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty_bar[b]);
      const Tile ti = tile_of(tile, N, Np, per_plane);
      const int s = ti.s0 + row;
      const int yh = s / Np, xh = s - yh * Np;
      if (yh >= 1 && yh <= N && xh >= 1 && xh <= N) {
        const long long cell0 = conv_at(N, ti.b, ti.zh, 0, s), cstride = conv_chunk_slots(N);  // chunk k: cell0 + k cstride
        if (g.mode == CONV_OUT_F32) {
          // FP32 planar output of the first `cout` channels (owned cells)
          const long long n3 = (long long)N * N * N;
          const long long own = ((long long)(ti.zh - 1) * N + (yh - 1)) * N + (xh - 1);
          float *o = g.outf + (long long)ti.b * g.cout * n3 + own;
#pragma unroll
          for (int c = 0; c < CH; c++)
            if (c < g.cout) o[c * n3] = (acc[c] + s_bias[c]) * g.scale;
        } else {
          float v[CH];
          if (g.mode == CONV_RELU) {
#pragma unroll
            for (int c = 0; c < CH; c++) v[c] = fmaxf(acc[c] + s_bias[c], 0.0f);
          } else if (g.mode == CONV_LINEAR) {
#pragma unroll
            for (int c = 0; c < CH; c++) v[c] = acc[c] + s_bias[c];
          } else {
            const uint4 *src = reinterpret_cast<const uint4 *>(g.aux);
#pragma unroll
            for (int k = 0; k < 4; k++) {
              const uint4 w = src[cell0 + k * cstride];
              const uint32_t ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
              for (int h = 0; h < 8; h++) {
                const int c = k * 8 + h;
                const float a = bf(ww[h >> 1], h & 1);
                v[c] = g.mode == CONV_RESIDUAL ? a + (acc[c] + s_bias[c]) : (a > 0.0f ? acc[c] : 0.0f);
              }
            }
          }
          uint4 *dst = reinterpret_cast<uint4 *>(g.out);
#pragma unroll
          for (int k = 0; k < 4; k++) {
            uint32_t w[4];
#pragma unroll
            for (int h = 0; h < 4; h++) {
              const __nv_bfloat162 p = __floats2bfloat162_rn(v[k * 8 + 2 * h], v[k * 8 + 2 * h + 1]);
              w[h] = *reinterpret_cast<const uint32_t *>(&p);
            }
            dst[cell0 + k * cstride] = make_uint4(w[0], w[1], w[2], w[3]);
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


// 2-D BF16 tensor map with 64-byte swizzle: rows of 32 channels (64 B),
// `rows` rows, boxes of 32 x box_rows.
static cudaError_t make_map_rows(CUtensorMap *map, const void *ptr, long long rows, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  cuuint64_t dims[2] = {(cuuint64_t)CH, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)CH * 2};
  cuuint32_t box[2] = {(cuuint32_t)CH, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// 2-D BF16 tensor map over an activation buffer as lines of 128 bytes (8 slots
// of 16 bytes), no swizzle, boxes of box_rows lines; lines outside the buffer
// read as zeros.
static cudaError_t make_map_lines(CUtensorMap *map, const void *ptr, long long lines, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  cuuint64_t dims[2] = {64, (cuuint64_t)lines};
  cuuint64_t strides[1] = {128};
  cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// per device: the shared-memory attribute and the resident CTA count
static cudaError_t conv_setup(int *ctas) {
  constexpr int MAXDEV = 64;
  static std::mutex mu;
  static int resident[MAXDEV] = {0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= MAXDEV) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (!resident[dev]) {
    e = cudaFuncSetAttribute(conv_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_LIMIT);
    if (e != cudaSuccess) return e;
    int per_sm = 0, sms = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, conv_tc_kernel, THREADS, SMEM_LIMIT);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    resident[dev] = per_sm * sms;
  }
  *ctas = resident[dev];
  return cudaSuccess;
}

}  // namespace conv

int conv_set_runs(int runs_per_plane) {
  if (runs_per_plane != 0 && runs_per_plane != 1 && runs_per_plane != 3) return -1;
  return conv::g_runs_per_plane.exchange(runs_per_plane);
}

cudaError_t launch_conv(const __nv_bfloat16 *in, const __nv_bfloat16 *w, const ConvArgs &args, cudaStream_t s) {
  int ctas = 0;
  cudaError_t e = conv::conv_setup(&ctas);
  if (e != cudaSuccess) return e;
  const int N = args.N, Np = N + 2;
  if (N < 2 || args.batch < 1) return cudaErrorInvalidValue;
  const conv::Geom gm = conv::geom_of(N);
  if (gm.stages < 1 || gm.box_rows > 256) return cudaErrorInvalidValue;
  const long long lines = conv_units(N, args.batch) / 8;
  if (lines >= 0x7fffffffLL) return cudaErrorInvalidValue;
  CUtensorMap ma, mw;
  if ((e = conv::make_map_lines(&ma, in, lines, gm.box_rows)) != cudaSuccess) return e;
  if ((e = conv::make_map_rows(&mw, w, (long long)TAPS * CH, CH)) != cudaSuccess) return e;
  const long long per_plane = ((long long)N * Np + conv::ROWS - 1) / conv::ROWS;
  const long long tiles = (long long)args.batch * N * per_plane;
  const int grid = (int)(tiles < ctas ? tiles : ctas);
  conv::conv_tc_kernel<<<grid, conv::THREADS, gm.smem, s>>>(ma, mw, args, gm.box_bytes, gm.stages, gm.ny);
  launch_counter()++;
  return cudaGetLastError();
}

}  // namespace sclet
