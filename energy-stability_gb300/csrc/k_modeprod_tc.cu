// Split-precision mode-n product on the 5th-generation tensor cores (tcgen05),
// the mixed-precision form of PUX / PUY / PUZ (source_beta_to_omega/src/
// calc.c:631-684).
//
// Operands travel as three BF16 planes x = x0 + x1 + x2 (x0 = bf16(x),
// x1 = bf16(x - x0), x2 = bf16(x - x0 - x1): 24 significant bits, the FP32
// state exactly).  The product keeps every cross term of order <= 2,
//   M x ~ M0 x0 + M0 x1 + M1 x0 + M0 x2 + M1 x1 + M2 x0,
// six BF16 MMAs with one FP32 accumulator in tensor memory (the 3-term split
// of Markidis et al. 2018 / Ootomo & Yokota 2022 carried to third order).
//
// Layout ("split tensor"): for each tensor t and plane p, rows r = 0 .. n*n-1
// of kp = roundup(n, 8) BF16 values, one 1-D line along the contracted axis per
// row: S[t][p][r][k].  A product contracts k and writes row (a' * n + c),
// column b for input row r = c * n + b -- the cyclic rotation that makes three
// products return to x-fastest order.
//
// Tile: D[128 a' x 128 r] in TMEM (128 lanes x 128 FP32 columns).  A = matrix
// planes (128 a' rows x 64 k, 128-byte swizzle), B = input planes (128 r rows
// x 64 k), both K-major, loaded by TMA into a two-stage mbarrier pipeline.
// Warp 0 issues TMA, warp 1 issues MMAs (one elected thread each), warp 2 owns
// the TMEM allocation, all four warps run the epilogue: TMEM -> registers ->
// shared tile -> coalesced global stores, with the ETD update (ac_updateU_new
// / ch_updateU_new, calc.c:489-535) or the phi2 scaling (prepare_U2_new,
// calc.c:553-567) fused.  Every mbarrier wait is bounded: on timeout the CTA
// records an error code, drains its copies (bounded), frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <stdint.h>
#include <string.h>

#include "sclet_internal.cuh"
#include "sclet_tc.cuh"

namespace sclet {

namespace tc {

constexpr int BM = 128, BN = 128, BK = 64, STAGES = 2;
constexpr int PLANE_A = BM * BK * 2;   // 16 KB
constexpr int PLANE_B = BN * BK * 2;   // 16 KB
constexpr int STAGE_BYTES = 3 * PLANE_A + 3 * PLANE_B;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;
constexpr int TMEM_COLS = 128;
constexpr long long WAIT_LIMIT = 1LL << 22;   // polls (with backoff) before giving up

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

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;               // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;     // stride byte offset
  d |= (uint64_t)1 << 46;               // descriptor version
  d |= (uint64_t)2 << 61;               // 128-byte swizzle
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

// Splits a float into three bf16 terms (round to nearest at each level).
__device__ __forceinline__ void split3(float x, __nv_bfloat16 &a, __nv_bfloat16 &b, __nv_bfloat16 &c) {
  a = __float2bfloat16_rn(x);
  float r = x - __bfloat162float(a);
  b = __float2bfloat16_rn(r);
  r -= __bfloat162float(b);
  c = __float2bfloat16_rn(r);
}

__device__ __forceinline__ float etd_H(const TcArgs &g, int kind, int i, int j, int k) {
  float tmp, H;
  if (kind == 0) {
    tmp = g.kk[2] * g.dd[2][k] + g.kk[1] * g.dd[1][j] + g.kk[0] * g.dd[0][i];
    H = -g.LE * (tmp * g.epn2 - g.KE);
  } else {
    tmp = g.dd[2][k] + g.dd[1][j] + g.dd[0][i];
    H = g.LCI * (tmp * tmp * g.epn2 - g.KCI * tmp);
  }
  return H;
}

// phi1 = (1 - e^{-dt H}) / H, phi2 = (1 - phi1/dt) / H (ac_init_phi, vars.c:
// 302-330), with series forms where dt H is small.
__device__ __forceinline__ void etd_phi(float H, float dt, float &phi1, float &phi2) {
  float x = dt * H;
  if (fabsf(x) < 1.0e-3f) {
    phi1 = dt * (1.0f - x * (0.5f - x * (1.0f / 6.0f)));
    phi2 = dt * (0.5f - x * (1.0f / 6.0f - x * (1.0f / 24.0f)));
  } else if (fabsf(x) < 0.1f) {
    phi1 = -expm1f(-x) / H;
    phi2 = dt * (0.5f - x * (1.0f / 6.0f - x * (1.0f / 24.0f - x * (1.0f / 120.0f - x * (1.0f / 720.0f)))));
  } else {
    phi1 = -expm1f(-x) / H;
    phi2 = (1.0f - phi1 / dt) / H;
  }
}

__global__ void __launch_bounds__(128, 1)
    modeprod_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TcArgs g) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t acc_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;

  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r_tile = blockIdx.x, a_tile = blockIdx.y, t = blockIdx.z;
  const long long rows = (long long)g.n * g.n;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&acc_bar, 1);
    failed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_slot;
  const int nkb = g.kblocks;

  if (warp == 0 && lane == 0) {
    // producer: three A planes and three B planes per stage
    int issued = 0;
    for (int kb = 0; kb < nkb; kb++) {
      const int s = kb % STAGES;
      if (kb >= STAGES && !mbar_wait(&empty_bar[s], ((kb / STAGES) & 1) ^ 1)) {
        failed = 1;
        break;
      }
      if (*(volatile int *)&failed) break;
      uint8_t *st = base + s * STAGE_BYTES;
      mbar_expect_tx(&full_bar[s], STAGE_BYTES);
      for (int p = 0; p < 3; p++) tma_load_3d(st + p * PLANE_A, &tmA, kb * BK, a_tile * BM, p, &full_bar[s]);
      for (int p = 0; p < 3; p++)
        tma_load_3d(st + 3 * PLANE_A + p * PLANE_B, &tmB, kb * BK, r_tile * BN, t * 3 + p, &full_bar[s]);
      issued = kb + 1;
    }
    if (*(volatile int *)&failed) {
      // drain: wait (bounded) for the copies still in flight into this CTA's
      // shared memory before it is reused or released
      for (int kb = issued - STAGES < 0 ? 0 : issued - STAGES; kb < issued; kb++)
        mbar_wait(&full_bar[kb % STAGES], (kb / STAGES) & 1);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: 4 k-steps of 16 per stage, six split terms each
    const uint32_t idesc = idesc_bf16(BM, BN);
    for (int kb = 0; kb < nkb; kb++) {
      const int s = kb % STAGES;
      if (!mbar_wait(&full_bar[s], (kb / STAGES) & 1)) {
        failed = 1;
        break;
      }
      fence_after();
      const uint32_t sa = smem_u32(base + s * STAGE_BYTES);
      const uint32_t sb = sa + 3 * PLANE_A;
#pragma unroll
      for (int ks = 0; ks < BK / 16; ks++) {
        const uint32_t koff = ks * 32;
        // (a plane, b plane) pairs of order <= 2; small terms first
        const int pa[6] = {2, 1, 0, 1, 0, 0};
        const int pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
        for (int q = 0; q < 6; q++) {
          uint64_t da = smem_desc(sa + pa[q] * PLANE_A + koff);
          uint64_t db = smem_desc(sb + pb[q] * PLANE_B + koff);
          mma_bf16(tmem, da, db, idesc, (kb | ks | q) != 0);
        }
      }
      mma_commit(&empty_bar[s]);
    }
    mma_commit(&acc_bar);
  }
  __syncwarp();

  // ---- epilogue ---------------------------------------------------------
  bool ok = mbar_wait(&acc_bar, 0);
  if (!ok) failed = 1;
  fence_after();
  float *tile = reinterpret_cast<float *>(base);  // [128][BN + 1] after the mainloop
  constexpr int TS = BN + 1;
  __syncthreads();
  if (!failed) {
    const int row = warp * 32 + lane;
#pragma unroll 1
    for (int c = 0; c < BN / 32; c++) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), v);
#pragma unroll
      for (int j = 0; j < 32; j++) tile[row * TS + c * 32 + j] = v[j];
    }
  }
  fence_before();
  __syncthreads();
  if (!failed) {
    const int col = threadIdx.x;
    const long long r = (long long)r_tile * BN + col;
    const int kind = (t % g.F) >= g.nac ? 1 : 0;
    if (r < rows) {
      const int cc = (int)(r / g.n), b = (int)(r % g.n);
#pragma unroll 1
      for (int rr = 0; rr < BM; rr++) {
        const int a = a_tile * BM + rr;
        if (a >= g.n) break;
        float v = tile[rr * TS + col];
        if (g.epi != 0) {
          // eigen-mode (i, j, k) = (b, c, a) of the z-contraction output
          float H = etd_H(g, kind, b, cc, a);
          float phi1, phi2;
          etd_phi(H, g.dt, phi1, phi2);
          if (fabsf(H) < 1.0e-8f) H = 0.0f;
          if (g.epi == 1) {
            const long long ao = (((long long)t * 3) * rows + (long long)a * g.n + cc) * g.kp + b;
            const long long ps = rows * g.kp;
            float uh = __bfloat162float(g.aux[ao]) + __bfloat162float(g.aux[ao + ps]) +
                       __bfloat162float(g.aux[ao + 2 * ps]);
            v = (1.0f - phi1 * H) * uh + phi1 * v;
          } else {
            v = phi2 * v;
          }
        }
        if (g.outmode == 0) {
          const long long ps = rows * g.kp;
          const long long o = (((long long)t * 3) * rows + (long long)a * g.n + cc) * g.kp + b;
          __nv_bfloat16 h0, h1, h2;
          split3(v, h0, h1, h2);
          g.out_split[o] = h0;
          g.out_split[o + ps] = h1;
          g.out_split[o + 2 * ps] = h2;
        } else {
          const long long o = (long long)t * g.n * rows + (long long)a * rows + r;
          if (g.outmode == 1) g.out_f32[o] = v;
          else g.out_f32[o] += v;
        }
      }
    }
  }
  __syncthreads();
  if (failed && threadIdx.x == 0) atomicExch(g.err, 1);
  if (warp == 2) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// FP32 field blocks (x fastest) -> split planes, rows (z, y), columns x.
__global__ void split_fields_kernel(const float *__restrict__ u, const float *__restrict__ sub,
                                    __nv_bfloat16 *__restrict__ out, int n, int kp, int count) {
  const long long n3 = (long long)n * n * n, rows = (long long)n * n;
  const long long total = n3 * count;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    int t = (int)(i / n3);
    long long l = i - (long long)t * n3;
    long long row = l / n;
    int x = (int)(l % n);
    __nv_bfloat16 a, b, c;
    split3(sub ? u[i] - sub[i] : u[i], a, b, c);
    long long o = (((long long)t * 3) * rows + row) * kp + x;
    out[o] = a;
    out[o + rows * kp] = b;
    out[o + 2 * rows * kp] = c;
  }
}

// FP64 row-major n x n matrix -> zero-padded split planes [3][n][kp].
__global__ void split_matrix_kernel(const double *__restrict__ m, __nv_bfloat16 *__restrict__ out, int n, int kp) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n * kp; i += gridDim.x * blockDim.x) {
    int r = i / kp, c = i % kp;
    // split the double itself: hi from the double, the rest from residuals
    double x = c < n ? m[(long long)r * n + c] : 0.0;
    __nv_bfloat16 a = __double2bfloat16(x);
    double rem = x - (double)__bfloat162float(a);
    __nv_bfloat16 b = __double2bfloat16(rem);
    rem -= (double)__bfloat162float(b);
    __nv_bfloat16 cc = __double2bfloat16(rem);
    out[i] = a;
    out[i + (long long)n * kp] = b;
    out[i + 2LL * n * kp] = cc;
  }
}

}  // namespace tc

// ---- host side ------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
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

static cudaError_t make_map(CUtensorMap *map, const void *ptr, int kp, long long rows, int depth, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  cuuint64_t dims[3] = {(cuuint64_t)kp, (cuuint64_t)rows, (cuuint64_t)depth};
  cuuint64_t strides[2] = {(cuuint64_t)kp * 2, (cuuint64_t)kp * 2 * (cuuint64_t)rows};
  cuuint32_t box[3] = {(cuuint32_t)tc::BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(ptr), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

int tc_kp(int n) { return (n + 7) / 8 * 8; }

cudaError_t tc_split_matrix(const double *m, __nv_bfloat16 *out, int n, cudaStream_t s) {
  tc::split_matrix_kernel<<<(n * tc_kp(n) + 255) / 256, 256, 0, s>>>(m, out, n, tc_kp(n));
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t tc_split_fields(const float *u, const float *sub, __nv_bfloat16 *out, int n, int count, cudaStream_t s) {
  long long total = (long long)n * n * n * count;
  long long b = (total + 255) / 256;
  tc::split_fields_kernel<<<(int)(b > 152 * 32 ? 152 * 32 : b), 256, 0, s>>>(u, sub, out, n, tc_kp(n), count);
  launch_counter()++;
  return cudaGetLastError();
}

cudaError_t launch_modeprod_tc(const __nv_bfloat16 *mat, const __nv_bfloat16 *in, int count, const TcArgs &args,
                               cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(tc::modeprod_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tc::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const int n = args.n, kp = tc_kp(n);
  CUtensorMap ma, mb;
  cudaError_t e;
  if ((e = make_map(&ma, mat, kp, n, 3, tc::BM)) != cudaSuccess) return e;
  if ((e = make_map(&mb, in, kp, (long long)n * n, 3 * count, tc::BN)) != cudaSuccess) return e;
  TcArgs g = args;
  g.kp = kp;
  g.kblocks = (n + tc::BK - 1) / tc::BK;
  dim3 grid((unsigned)(((long long)n * n + tc::BN - 1) / tc::BN), (unsigned)((n + tc::BM - 1) / tc::BM),
            (unsigned)count);
  tc::modeprod_tc_kernel<<<grid, 128, tc::SMEM_BYTES, s>>>(ma, mb, g);
  launch_counter()++;
  return cudaGetLastError();
}

}  // namespace sclet
