// Device and host helpers of the tensor-core mode-n product kernel
// (k_modeprod_tc.cu): tile constants, mbarrier / TMA / tcgen05 wrappers, the
// tile order and the tensor-map encoder.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include "sclet_tc.cuh"

namespace sclet {
namespace tc {


constexpr int BM = 128, BN = 128, BK = 32, STAGES = 3, NP = TC_PLANES, NPM = TC_PLANES_M;
constexpr int PLANE_A = BM * BK * 2;  // 8 KB: one input slice (M side, 128 input rows)
constexpr int PLANE_B = BN * BK * 2;  // 8 KB: one matrix slice (N side, 128 a' rows)
constexpr int STAGE_BYTES = NP * PLANE_A + NPM * PLANE_B;
constexpr int SMEM_ALIGN = 512;  // period of the 64-byte swizzle pattern
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + SMEM_ALIGN;
constexpr int NACC = 4;               // weight classes w = 0..3
constexpr int ACC_COLS = NACC * BN;   // one accumulator set
constexpr int NBUF = 512 / ACC_COLS;   // accumulator sets in tensor memory (1 or 2)
constexpr int TMEM_COLS = NBUF * ACC_COLS;
constexpr int EPI_WARPS = 8;          // two per TMEM lane quadrant, each half of the columns
constexpr int CPW = BN / 32 / 2;      // 32-column chunks per epilogue warp
constexpr int THREADS = 64 + 32 * EPI_WARPS;  // producer, MMA, epilogue warps
constexpr long long WAIT_LIMIT = 1LL << 22;  // polls (with backoff) before giving up
static_assert(TMEM_COLS <= 512, "tensor memory holds 512 columns");
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory per CTA");

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait; false on timeout (the caller records the error).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (long long i = 0; i < WAIT_LIMIT; i++) {
    if (mbar_try_wait(bar, parity)) return true;
    if (i > 64) __nanosleep(64);
  }
  return false;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor: K-major, 64-byte swizzle, 8-row groups
// 512 bytes apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;    // stride byte offset
  d |= (uint64_t)1 << 46;             // descriptor version
  d |= (uint64_t)4 << 61;             // 64-byte swizzle
  return d;
}

// Instruction descriptor: BF16 x BF16 -> FP32, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          dtmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; j++) v[j] = __uint_as_float(r[j]);
}

// The same load without the wait: the registers are valid after tmem_wait_ld.
__device__ __forceinline__ void tmem_ld32_async(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

struct TileIdx {
  int a_tile, r_tile, t;
};
// power-of-two scale S >= m (S = 1 for m = 0)
__device__ __forceinline__ float pow2_scale(float m) {
  if (!(m > 0.0f)) return 1.0f;
  int e;
  frexpf(m, &e);  // m = f 2^e, f in [0.5, 1)
  return ldexpf(1.0f, e);
}

// The u-th output tile of CTA `cta`: each CTA takes whole groups (every
// a'-tile of one input tile, a'-tiles fastest), groups dealt round robin with
// the tensor fastest.  Every group costs the same (the last a'-tile is
// narrower), so the CTAs stay balanced; the group's input tile, read once
// from HBM by its first a'-tile, is read again from L2 by the CTA's next
// a'-tiles; and the tensors of one input tile run side by side on
// neighbouring CTAs, so the fused update's coefficient tables (one per field
// kind) come from HBM about once per input tile.
__device__ __forceinline__ TileIdx cta_tile(int u, int a_tiles, int count, int cta, int grid) {
  TileIdx x;
  const int grp = cta + (u / a_tiles) * grid;
  x.a_tile = u % a_tiles;
  x.t = grp % count;
  x.r_tile = grp / count;
  return x;
}

}  // namespace tc

static inline PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

// k-blocked slice planes [depth][kp / BK][rows][BK] as a 3-D tensor {BK, rows,
// depth * kp / BK}: a box is one k-block of box_rows consecutive rows.
static inline cudaError_t make_map(CUtensorMap *map, const void *ptr, int kp, long long rows, int depth, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  cuuint64_t dims[3] = {(cuuint64_t)tc::BK, (cuuint64_t)rows, (cuuint64_t)depth * (cuuint64_t)(kp / tc::BK)};
  cuuint64_t strides[2] = {(cuuint64_t)tc::BK * 2, (cuuint64_t)tc::BK * 2 * (cuuint64_t)rows};
  cuuint32_t box[3] = {(cuuint32_t)tc::BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(ptr), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace sclet
