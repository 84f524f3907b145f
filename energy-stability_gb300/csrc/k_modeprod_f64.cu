// FP64 mode-n product with a cyclic layout rotation: the plain-precision form
// of PUX / PUY / PUZ (source_beta_to_omega/src/calc.c:631-684, one cblas_dgemm
// plus xyz_yzx / yzx_zxy / zxy_xyz).
//
// For each tensor t of a batch, in layout (a fastest, then b, then c):
//   out_t[a' * n*n + c*n + b] = sum_a M[a' * n + a] * in_t[(c*n + b) * n + a]
// i.e. a GEMM C[a'][r] = sum_a M[a'][a] In[r][a] over r = c*n + b, stored with r
// contiguous, so that three successive products return to the original axis
// order with every index transformed.  Epilogues fuse the ETD update
// (ac_updateU_new / ch_updateU_new, calc.c:489-535), the ETD2 phi2 scaling
// (prepare_U2_new, calc.c:553-567) and the corrector accumulation
// (correct_U_new, calc.c:569-583); the prologue fuses prepare_U1_new's
// difference (calc.c:537-551).
//
// GB300 executes FP64 at ~1.2 TFLOP/s (measured), so this kernel is bound by
// FP64 issue, not memory: 64x64 output tiles, 4x4 outputs per thread.
#include "sclet_internal.cuh"

namespace sclet {

namespace {
constexpr int BM = 64, BN = 64, BK = 16;

struct Tabs {
  const double *phi[2];  // per kind: phi1 (epilogue 1) or phi2 (epilogue 2), layout [k][j][i]
};

template <int EPI, bool SUB>
__global__ void __launch_bounds__(256) modeprod_f64_kernel(const double *__restrict__ M, const double *__restrict__ in,
                                                           const double *__restrict__ sub, double *__restrict__ out,
                                                           const double *__restrict__ aux, int n, long long in_stride,
                                                           long long out_stride, EtdCoef ec, Tabs tabs) {
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  const int t = blockIdx.z;
  const long long nn = (long long)n * n;
  const int a0 = blockIdx.y * BM;
  const long long r0 = (long long)blockIdx.x * BN;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const double *inT = in + t * in_stride;
  const double *subT = SUB ? sub + t * in_stride : nullptr;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.0;

  for (int k0 = 0; k0 < n; k0 += BK) {
    // M tile: rows a0..a0+63, cols k0..k0+15 -> As[k][a]
    for (int e = threadIdx.x; e < BM * BK; e += 256) {
      int row = e / BK, col = e % BK;
      int a = a0 + row, k = k0 + col;
      As[col][row] = (a < n && k < n) ? M[(long long)a * n + k] : 0.0;
    }
    // In tile: rows r0..r0+63, cols k0..k0+15 -> Bs[k][r]
    for (int e = threadIdx.x; e < BN * BK; e += 256) {
      int row = e / BK, col = e % BK;
      long long r = r0 + row;
      int k = k0 + col;
      double v = 0.0;
      if (r < nn && k < n) {
        v = inT[r * n + k];
        if (SUB) v -= subT[r * n + k];
      }
      Bs[col][row] = v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < BK; k++) {
      double av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; i++) av[i] = As[k][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; j++) bv[j] = Bs[k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }

  double *outT = out + t * out_stride;
  const int kind = (t % ec.F) >= ec.nac ? 1 : 0;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    int a = a0 + ty * 4 + i;
    if (a >= n) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      long long r = r0 + tx + 16 * j;
      if (r >= nn) continue;
      long long o = (long long)a * nn + r;
      double v = acc[i][j];
      if (EPI == 0) {
        outT[o] = v;
      } else if (EPI == 1) {
        // ETD1 update in eigenspace at mode (i = r % n, j = r / n, k = a)
        int ii = (int)(r % n), jj = (int)(r / n);
        double tmp, H;
        if (kind == 0) {
          tmp = ec.kk[2] * ec.dd[2][a] + ec.kk[1] * ec.dd[1][jj] + ec.kk[0] * ec.dd[0][ii];
          H = -ec.LE * (tmp * ec.epn2 - ec.KE);
        } else {
          tmp = ec.dd[2][a] + ec.dd[1][jj] + ec.dd[0][ii];
          H = ec.LCI * (tmp * tmp * ec.epn2 - ec.KCI * tmp);
        }
        if (fabs(H) < 1.0e-8) H = 0.0;
        double phi = tabs.phi[kind][o];
        double uh = aux[t * out_stride + o];
        outT[o] = (1.0 - phi * H) * uh + phi * v;
      } else if (EPI == 2) {
        outT[o] = tabs.phi[kind][o] * v;
      } else {
        outT[o] += v;
      }
    }
  }
}
}  // namespace

// Tables of phi1 / phi2 per field kind, set by the context (see sclet_api.cu).
static Tabs g_tabs[2];
void set_phi_tables(const double *phi1_ac, const double *phi1_ch, const double *phi2_ac, const double *phi2_ch) {
  g_tabs[0].phi[0] = phi1_ac;
  g_tabs[0].phi[1] = phi1_ch;
  g_tabs[1].phi[0] = phi2_ac;
  g_tabs[1].phi[1] = phi2_ch;
}

cudaError_t launch_modeprod_f64(const double *M, const double *in, const double *sub, double *out, const double *aux,
                                int count, int n, int epilogue, const EtdCoef &ec, long long in_stride,
                                long long out_stride, cudaStream_t s) {
  long long nn = (long long)n * n;
  dim3 grid((unsigned)((nn + BN - 1) / BN), (unsigned)((n + BM - 1) / BM), (unsigned)count);
  Tabs tb = epilogue == 2 ? g_tabs[1] : g_tabs[0];
  if (sub) {
    modeprod_f64_kernel<0, true><<<grid, 256, 0, s>>>(M, in, sub, out, aux, n, in_stride, out_stride, ec, tb);
  } else if (epilogue == 0) {
    modeprod_f64_kernel<0, false><<<grid, 256, 0, s>>>(M, in, sub, out, aux, n, in_stride, out_stride, ec, tb);
  } else if (epilogue == 1) {
    modeprod_f64_kernel<1, false><<<grid, 256, 0, s>>>(M, in, sub, out, aux, n, in_stride, out_stride, ec, tb);
  } else if (epilogue == 2) {
    modeprod_f64_kernel<2, false><<<grid, 256, 0, s>>>(M, in, sub, out, aux, n, in_stride, out_stride, ec, tb);
  } else {
    modeprod_f64_kernel<3, false><<<grid, 256, 0, s>>>(M, in, sub, out, aux, n, in_stride, out_stride, ec, tb);
  }
  launch_counter()++;
  return cudaGetLastError();
}

}  // namespace sclet
