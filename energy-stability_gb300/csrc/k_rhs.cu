// Nonlinear right-hand sides of the ETD step on one periodic block.
//
// Allen-Cahn (ac_calc_FU, source_beta_to_omega/src/calc.c:8-68 ->
// ac_calc_F1 / ac_calc_F2, anisotropic.c:9-628):
//   N_m = LE KE eta_m - LE AC_f(m)                 (SWTICH_AC_FIELD1)
//       + LE epn2 eta_m(outside) / h^2 on each block face (boundary lifting;
//         the outside value is the periodic image of the cell beyond the face)
//       - epn2 LE div(lambda_m grad eta_m)          (ANISOTROPIC; central
//         differences, values outside the block taken as zero)
//       - LE ElasticScale felas_m                  (ELASTIC == 1)
// Cahn-Hilliard, constant mobility (ch_calc_FU_ConstantMobility,
// calc.c:70-473):
//   t   = -LCI KCI c + LCI CH_f - LCI epn2 c(outside) / h^2 on faces
//   N_c = lap(t) (zero outside) - mu(outside) / h^2 on faces, with
//   mu = LCI (epn2 lap(c) - CH_f) at the periodic image of the outside cell
//   (ch_mu, trans.c:1433-1937).
// AC_f and CH_f come from the run's physics plugin (the drop-in form of
// formula.c:9-56, sclet_physics.cuh), a template parameter of every kernel.
#include "sclet_internal.cuh"
#include "sclet_physics.cuh"

namespace sclet {

constexpr int ZC = 32;  // default z-planes per CTA of the Allen-Cahn kernel
constexpr int PZ = 16;  // z-planes per CTA of the one-cell-per-thread CH kernels

template <typename T>
struct P {
  int n, nac, nch, F, aniso, elastic;
  T epn2, hx, hy, hz, LE, KE, LCI, KCI, es;
  T ih2x, ih2y, ih2z;   // 1 / h^2 per axis
  T i2hx, i2hy, i2hz;   // 1 / (2 h) per axis
  T K[16];              // plugin constants (reference composition shifted by cshift)
  int zc, runs;         // z-planes per CTA (AC kernel); runs side by side
  const double *krun;   // per-run plugin constant 0, or null
  // anisotropic term folded: kan[m][3 r + c] = epn2 LE (1/2h_r) lam_m[r][c] (1/2h_c),
  // the flux row r differenced along axis r
  T kan[4][9];
  T mob_m0, mob_dg;     // variable mobility M(eta0) = m0 (1 (1 - eta0) + dg eta0)
};

template <typename T>
static P<T> to_p(const Phys &ph) {
  P<T> p;
  p.n = ph.n; p.nac = ph.nac; p.nch = ph.nch; p.F = ph.F; p.aniso = ph.anisotropic; p.elastic = ph.elastic;
  p.epn2 = (T)ph.epn2; p.hx = (T)ph.h[0]; p.hy = (T)ph.h[1]; p.hz = (T)ph.h[2];
  p.ih2x = (T)(1.0 / (ph.h[0] * ph.h[0])); p.ih2y = (T)(1.0 / (ph.h[1] * ph.h[1]));
  p.ih2z = (T)(1.0 / (ph.h[2] * ph.h[2]));
  p.i2hx = (T)(0.5 / ph.h[0]); p.i2hy = (T)(0.5 / ph.h[1]); p.i2hz = (T)(0.5 / ph.h[2]);
  p.LE = (T)ph.LE; p.KE = (T)ph.KE; p.LCI = (T)ph.LCI; p.KCI = (T)ph.KCI; p.es = (T)ph.elastic_scale;
  for (int k = 0; k < 16; k++) p.K[k] = (T)ph.K[k];
  p.zc = ph.rhs_zc > 0 ? ph.rhs_zc : ZC;
  p.runs = ph.runs > 0 ? ph.runs : 1;
  p.krun = ph.krun;
  const double i2h[3] = {0.5 / ph.h[0], 0.5 / ph.h[1], 0.5 / ph.h[2]};
  for (int m = 0; m < 4; m++)
    for (int k = 0; k < 9; k++) {
      p.kan[m][k] = (T)(ph.epn2 * ph.LE * i2h[k / 3] * ph.lam[m][k] * i2h[k % 3]);
    }
  p.mob_m0 = (T)ph.mob_m0;
  p.mob_dg = (T)ph.mob_dg;
  return p;
}

// AC_f(m) / CH_f(0) of plugin PL at one cell: NAC order parameters e (known
// at compile time) and the stored concentration c.
template <typename PL, typename T, int NAC>
__device__ __forceinline__ T ac_f_n(const P<T> &p, const T *e, T c, int m) {
  sclet_acv<T> ac[NAC > 0 ? NAC : 1];
  sclet_chv<T> ch[1];
#pragma unroll
  for (int k = 0; k < NAC; k++) ac[k].u = e[k];
  ch[0].c = c;
  return PL::template ac_f<T>(ac, ch, NAC, p.nch, p.K, m);
}

template <typename PL, typename T>
__device__ __forceinline__ T ch_f(const P<T> &p, const T *e, T c) {
  sclet_acv<T> ac[4];
  sclet_chv<T> ch[1];
#pragma unroll
  for (int k = 0; k < 4; k++) ac[k].u = e[k];
  ch[0].c = c;
  return PL::template ch_f<T>(ac, ch, p.nac, 1, p.K, 0);
}

__device__ inline long long L3(int n, int z, int y, int x) { return ((long long)z * n + y) * n + x; }

// One cell per thread on a 3-D launch: threadIdx.x along x (coalesced),
// blockIdx.z = z; no index division.
constexpr int RX = 32, RY = 8;

// Allen-Cahn right-hand side, 2.5-D: a CTA owns a 32 x 8 (x, y) tile and
// marches over p.zc planes in z (ZC by default), keeping for every order parameter a ring of five
// planes (z-2 .. z+2) with a two-cell halo in x and y in shared memory (zero
// outside the block, as ac_calc_F2 reads it).  Each value comes from global
// memory about once per CTA instead of once per stencil tap.
// (ZC, the default planes per CTA, is defined at the top of the file)
constexpr int HX = RX + 4, HY = RY + 4;
constexpr int PLANE = HX * HY;     // one haloed plane

template <typename PL, typename T, int NAC, bool ANISO>
__global__ void __launch_bounds__(RX * RY, sizeof(T) == 4 ? 3 : 1) rhs_ac_kernel(P<T> p0, const T *__restrict__ u, const T *__restrict__ felas,
                                                         T *__restrict__ out) {
  extern __shared__ unsigned char smem_raw[];
  T *ring = reinterpret_cast<T *>(smem_raw);  // [nac][5][HY][HX]
  const int n = p0.n;
  const size_t n3 = (size_t)n * n * n;
  // blockIdx.z = run x z-chunks
  const int zchunks = (n + p0.zc - 1) / p0.zc;
  const int run = blockIdx.z / zchunks, zci = blockIdx.z - run * zchunks;
  P<T> p = p0;
  if (p0.krun) p.K[0] = (T)p0.krun[run];
  u += (size_t)run * p.F * n3;
  felas += (size_t)run * p.nac * n3;
  out += (size_t)run * p.F * n3;
  const int x0 = blockIdx.x * RX, y0 = blockIdx.y * RY;
  const int zb = zci * p.zc, ze = zb + p.zc < n ? zb + p.zc : n;
  const int tid = threadIdx.y * RX + threadIdx.x;
  const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
  // this thread's share of one haloed plane of every order parameter:
  // PLANE / 256 rounded up values per field
  constexpr int PER = (PLANE + RX * RY - 1) / (RX * RY);
  // this thread's cells of a haloed plane: in-plane offset, or -1 outside the block
  int poff[PER];
#pragma unroll
  for (int q = 0; q < PER; q++) {
    const int i = tid + q * RX * RY;
    const int ly = i / HX, lx = i - ly * HX;
    const int gx = x0 + lx - 2, gy = y0 + ly - 2;
    poff[q] = i < PLANE && gx >= 0 && gx < n && gy >= 0 && gy < n ? gy * n + gx : -1;
  }
  auto fetch = [&](int z, T *reg) {
    const bool zin = z >= 0 && z < n;
#pragma unroll
    for (int m = 0; m < NAC; m++) {
      const T *um = u + m * n3 + (size_t)z * n * n;
#pragma unroll
      for (int q = 0; q < PER; q++) reg[m * PER + q] = zin && poff[q] >= 0 ? um[poff[q]] : (T)0;
    }
  };
  auto store = [&](int z, const T *reg) {
#pragma unroll
    for (int m = 0; m < NAC; m++) {
      T *dst = ring + (size_t)m * 5 * PLANE + ((z + 5 * 1024) % 5) * PLANE;
#pragma unroll
      for (int q = 0; q < PER; q++) {
        const int i = tid + q * RX * RY;
        if (i < PLANE) dst[i] = reg[m * PER + q];
      }
    }
  };
  T pre[NAC * PER];
  for (int z = zb - 2; z < zb + 2; z++) {
    fetch(z, pre);
    store(z, pre);
  }
  fetch(zb + 2, pre);  // plane z + 2 of the first pass, in flight
  const int lx = threadIdx.x + 2, ly = threadIdx.y + 2;
  for (int z = zb; z < ze; z++) {
    store(z + 2, pre);
    __syncthreads();
    if (z + 3 < ze + 2) fetch(z + 3, pre);  // next plane loads overlap this plane's work
    if (x < n && y < n) {
      const size_t l = ((size_t)z * n + y) * n + x;
      // ring slots of planes z-2 .. z+2, with this thread's (ly, lx) applied
      int so[5];
      const int s0 = (z - 2 + 5 * 1024) % 5;
#pragma unroll
      for (int d = 0; d < 5; d++) so[d] = (s0 + d < 5 ? s0 + d : s0 + d - 5) * PLANE + ly * HX + lx;
      T e[NAC];
#pragma unroll
      for (int m = 0; m < NAC; m++) e[m] = ring[(size_t)m * 5 * PLANE + so[2]];
      const T c = p.nch > 0 ? u[p.nac * n3 + l] : (T)0;
      const bool face = x == 0 || x == n - 1 || y == 0 || y == n - 1 || z == 0 || z == n - 1;
#pragma unroll
      for (int m = 0; m < NAC; m++) {
        const T *um = u + m * n3;
        const T *rg = ring + (size_t)m * 5 * PLANE;
        T v = p.LE * p.KE * e[m];
        v -= p.LE * ac_f_n<PL, T, NAC>(p, e, c, m);
        if (face) {
          const int iz = img(n, z), iy = img(n, y), ix = img(n, x), lo = img(n, -1), hi = img(n, n);
          const T w = p.LE * p.epn2;
          if (x == 0) v += w * um[L3(n, iz, iy, lo)] * p.ih2x;
          if (x == n - 1) v += w * um[L3(n, iz, iy, hi)] * p.ih2x;
          if (y == 0) v += w * um[L3(n, iz, lo, ix)] * p.ih2y;
          if (y == n - 1) v += w * um[L3(n, iz, hi, ix)] * p.ih2y;
          if (z == 0) v += w * um[L3(n, lo, iy, ix)] * p.ih2z;
          if (z == n - 1) v += w * um[L3(n, hi, iy, ix)] * p.ih2z;
        }
        if (ANISO) {
          // div(lambda grad eta), ac_calc_F2 (anisotropic.c:164-628): the flux
          // component c at a neighbour q is lam[c] . (central differences at q),
          // zero when q is outside the block; y and z differences are
          // (previous - next), as the reference writes them
          auto U = [&](int dz, int dy, int dx) { return rg[so[dz + 2] + dy * HX + dx]; };
          const T c0 = U(0, 0, 0);
          const T xp2 = U(0, 0, 2), xm2 = U(0, 0, -2), yp2 = U(0, 2, 0), ym2 = U(0, -2, 0), zp2 = U(2, 0, 0),
                  zm2 = U(-2, 0, 0);
          const T xpym = U(0, -1, 1), xpyp = U(0, 1, 1), xmym = U(0, -1, -1), xmyp = U(0, 1, -1);
          const T xpzm = U(-1, 0, 1), xpzp = U(1, 0, 1), xmzm = U(-1, 0, -1), xmzp = U(1, 0, -1);
          const T ymzm = U(-1, -1, 0), ymzp = U(1, -1, 0), ypzm = U(-1, 1, 0), ypzp = U(1, 1, 0);
          // folded constants: k[3 r + c] = epn2 LE lam[r][c] / (2 h_r 2 h_c)
          const T *k = p.kan[m];
          const T ar = x < n - 1 ? k[0] * (xp2 - c0) + k[1] * (xpym - xpyp) + k[2] * (xpzm - xpzp) : (T)0;
          const T al = x > 0 ? k[0] * (c0 - xm2) + k[1] * (xmym - xmyp) + k[2] * (xmzm - xmzp) : (T)0;
          const T at = y > 0 ? k[3] * (xpym - xmym) + k[4] * (ym2 - c0) + k[5] * (ymzm - ymzp) : (T)0;
          const T ab = y < n - 1 ? k[3] * (xpyp - xmyp) + k[4] * (c0 - yp2) + k[5] * (ypzm - ypzp) : (T)0;
          const T af = z > 0 ? k[6] * (xpzm - xmzm) + k[7] * (ymzm - ypzm) + k[8] * (zm2 - c0) : (T)0;
          const T ak = z < n - 1 ? k[6] * (xpzp - xmzp) + k[7] * (ymzp - ypzp) + k[8] * (c0 - zp2) : (T)0;
          v -= ((ar - al) + (at - ab)) + (af - ak);
        }
        if (p.elastic == 1) v -= p.LE * p.es * felas[m * n3 + l];
        out[m * n3 + l] = v;
      }
    }
    __syncthreads();
  }
}

// t = -LCI KCI c + LCI CH_f, minus the face liftings (first part of
// ch_calc_FU_ConstantMobility).
template <typename PL, typename T>
__global__ void __launch_bounds__(RX * RY) rhs_ch_t_kernel(P<T> p0, const T *__restrict__ u, T *__restrict__ t) {
  const int n = p0.n;
  const int zch = (n + PZ - 1) / PZ;  // blockIdx.z = run x chunk of PZ planes
  const int run = blockIdx.z / zch, z0 = (blockIdx.z - run * zch) * PZ, z1 = z0 + PZ < n ? z0 + PZ : n;
  const int x = blockIdx.x * RX + threadIdx.x, y = blockIdx.y * RY + threadIdx.y;
  if (x >= n || y >= n) return;
  const size_t n3 = (size_t)n * n * n;
  P<T> p = p0;
  if (p0.krun) p.K[0] = (T)p0.krun[run];
  u += (size_t)run * p.F * n3;
  t += (size_t)run * n3;
  for (int z = z0; z < z1; z++) {
    const size_t l = ((size_t)z * n + y) * n + x;
    const T *cf = u + p.nac * n3;
    T e[4] = {(T)0, (T)0, (T)0, (T)0};
#pragma unroll
    for (int m = 0; m < 4; m++)
      if (m < p.nac) e[m] = u[m * n3 + l];
    const T c = cf[l];
    T v = -p.LCI * p.KCI * c;
    v += p.LCI * ch_f<PL>(p, e, c);
    if (x == 0 || x == n - 1 || y == 0 || y == n - 1 || z == 0 || z == n - 1) {
      const int iz = img(n, z), iy = img(n, y), ix = img(n, x), lo = img(n, -1), hi = img(n, n);
      const T w = p.LCI * p.epn2;
      if (x == 0) v -= w * cf[L3(n, iz, iy, lo)] * p.ih2x;
      if (x == n - 1) v -= w * cf[L3(n, iz, iy, hi)] * p.ih2x;
      if (y == 0) v -= w * cf[L3(n, iz, lo, ix)] * p.ih2y;
      if (y == n - 1) v -= w * cf[L3(n, iz, hi, ix)] * p.ih2y;
      if (z == 0) v -= w * cf[L3(n, lo, iy, ix)] * p.ih2z;
      if (z == n - 1) v -= w * cf[L3(n, hi, iy, ix)] * p.ih2z;
    }
    t[l] = v;
  }
}

// Boundary chemical potential at periodic image cell (z,y,x) (ch_mu).
template <typename PL, typename T>
__device__ inline T ch_mu_at(const P<T> &p, const T *__restrict__ u, int z, int y, int x) {
  int n = p.n;
  long long n3 = (long long)n * n * n;
  const T *cf = u + p.nac * n3;
  T cv = cf[L3(n, z, y, x)];
  T lap = (cf[L3(n, z, y, img(n, x - 1))] + (T)(-2.0) * cv + cf[L3(n, z, y, img(n, x + 1))]) * p.ih2x;
  lap += (cf[L3(n, z, img(n, y - 1), x)] + (T)(-2.0) * cv + cf[L3(n, z, img(n, y + 1), x)]) * p.ih2y;
  lap += (cf[L3(n, img(n, z - 1), y, x)] + (T)(-2.0) * cv + cf[L3(n, img(n, z + 1), y, x)]) * p.ih2z;
  T e[4] = {(T)0, (T)0, (T)0, (T)0};
  for (int m = 0; m < p.nac; m++) e[m] = u[m * n3 + L3(n, z, y, x)];
  T mu = p.LCI * p.epn2 * lap;
  mu -= p.LCI * ch_f<PL>(p, e, cv);
  return mu;
}

// N_c = lap(t) (zero outside), minus mu(outside)/h^2 on faces.
template <typename PL, typename T>
__global__ void __launch_bounds__(RX * RY) rhs_ch_lap_kernel(P<T> p0, const T *__restrict__ u, const T *__restrict__ t,
                                                             T *__restrict__ out) {
  const int n = p0.n;
  const int zch = (n + PZ - 1) / PZ;  // blockIdx.z = run x chunk of PZ planes
  const int run = blockIdx.z / zch, z0 = (blockIdx.z - run * zch) * PZ, z1 = z0 + PZ < n ? z0 + PZ : n;
  const int x = blockIdx.x * RX + threadIdx.x, y = blockIdx.y * RY + threadIdx.y;
  if (x >= n || y >= n) return;
  P<T> p = p0;
  if (p0.krun) p.K[0] = (T)p0.krun[run];
  {
    const size_t n3 = (size_t)n * n * n;
    u += (size_t)run * p.F * n3;
    t += (size_t)run * n3;
    out += (size_t)run * p.F * n3;
  }
  const size_t nn = (size_t)n * n;
  for (int z = z0; z < z1; z++) {
    const size_t l = (size_t)z * nn + (size_t)y * n + x;
    const T tc = t[l];
    const T fl = x > 0 ? t[l - 1] : (T)0, fr = x < n - 1 ? t[l + 1] : (T)0;
    const T ft = y > 0 ? t[l - n] : (T)0, fb = y < n - 1 ? t[l + n] : (T)0;
    const T ff = z > 0 ? t[l - nn] : (T)0, fk = z < n - 1 ? t[l + nn] : (T)0;
    T v = (fl + fr - (T)2 * tc) * p.ih2x;
    v += (ft + fb - (T)2 * tc) * p.ih2y;
    v += (ff + fk - (T)2 * tc) * p.ih2z;
    if (x == 0 || x == n - 1 || y == 0 || y == n - 1 || z == 0 || z == n - 1) {
      const int iz = img(n, z), iy = img(n, y), ix = img(n, x), lo = img(n, -1), hi = img(n, n);
      if (x == 0) v -= ch_mu_at<PL>(p, u, iz, iy, lo) * p.ih2x;
      if (x == n - 1) v -= ch_mu_at<PL>(p, u, iz, iy, hi) * p.ih2x;
      if (y == 0) v -= ch_mu_at<PL>(p, u, iz, lo, ix) * p.ih2y;
      if (y == n - 1) v -= ch_mu_at<PL>(p, u, iz, hi, ix) * p.ih2y;
      if (z == 0) v -= ch_mu_at<PL>(p, u, lo, iy, ix) * p.ih2z;
      if (z == n - 1) v -= ch_mu_at<PL>(p, u, hi, iy, ix) * p.ih2z;
    }
    out[l] = v;
  }
}

// ---- variable-mobility Cahn-Hilliard ---------------------------------------
// ch_calc_FU_VariableMobility (source_beta_to_omega/src/mobility.c:838-858),
// update_M_C (:860-922) run first, on the single conserved field:
//   f0 = -LCI KCI c + LCI CH_f                              (ch_calc_F0)
//   t1 = -f0 + KCI c + epn2 c_out / h^2 on faces,  f1 = -C lap0(t1) - C mu_out / h^2
//                                                           (ch_calc_F1)
//   t2 = epn2 lap0(c) - f0 + epn2 c_out / h^2 on faces,
//   f2 = -div0((M - C) grad t2)                             (ch_calc_F2,
//        ch_divergence_M_gradient :435-722: face flux (m_q + m)(a_q - a)/(2 h^2))
//   N  = LCI (f1 + f2)
// with M(eta0) the first concentration's mobility, C its largest value over
// the block, lap0 / div0 zero outside the block (values and mobility), c_out
// the periodic image outside a face and mu_out the boundary chemical potential
// there (ch_mu).  Three launches: the block maxima of M, their maximum C, then
// t1 and t2, then N.

template <typename T>
__device__ __forceinline__ T mobility(const P<T> &p, T e) {
  return p.mob_m0 * ((T)1 * ((T)1 - e) + p.mob_dg * e);
}

// per run (blockIdx.y): the largest M over the block, per CTA
template <typename T>
__global__ void __launch_bounds__(256) mob_max_kernel(P<T> p, const T *__restrict__ u, double *__restrict__ part) {
  __shared__ double sm[8];
  const size_t n3 = (size_t)p.n * p.n * p.n;
  const T *e0 = u + (size_t)blockIdx.y * p.F * n3;  // the run's first order parameter
  double mx = -1.0e30;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n3; i += (size_t)gridDim.x * blockDim.x)
    mx = fmax(mx, (double)mobility(p, e0[i]));
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) mx = fmax(mx, sm[w]);
    part[(size_t)blockIdx.y * MOB_PARTS + blockIdx.x] = mx;
  }
}

// C of every run: cmax[run] = max of its MOB_PARTS partial maxima
__global__ void __launch_bounds__(256) mob_final_kernel(const double *__restrict__ part, double *__restrict__ cmax) {
  __shared__ double sm[8];
  double mx = -1.0e30;
  for (int i = threadIdx.x; i < MOB_PARTS; i += blockDim.x) mx = fmax(mx, part[(size_t)blockIdx.x * MOB_PARTS + i]);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) mx = fmax(mx, sm[w]);
    cmax[blockIdx.x] = mx;
  }
}

// t1 and t2 of every cell (blockIdx.z = run x z)
template <typename PL, typename T>
__global__ void __launch_bounds__(RX * RY) mob_t_kernel(P<T> p0, const T *__restrict__ u, T *__restrict__ tt) {
  const int n = p0.n;
  const int zch = (n + PZ - 1) / PZ;  // blockIdx.z = run x chunk of PZ planes
  const int run = blockIdx.z / zch, z0 = (blockIdx.z - run * zch) * PZ, z1 = z0 + PZ < n ? z0 + PZ : n;
  const int x = blockIdx.x * RX + threadIdx.x, y = blockIdx.y * RY + threadIdx.y;
  if (x >= n || y >= n) return;
  const size_t n3 = (size_t)n * n * n, nn = (size_t)n * n;
  P<T> p = p0;
  if (p0.krun) p.K[0] = (T)p0.krun[run];
  u += (size_t)run * p.F * n3;
  T *t1 = tt + (size_t)run * 2 * n3, *t2 = t1 + n3;
  for (int z = z0; z < z1; z++) {
    const size_t l = (size_t)z * nn + (size_t)y * n + x;
    const T *cf = u + p.nac * n3;
    T e[4] = {(T)0, (T)0, (T)0, (T)0};
#pragma unroll
    for (int m = 0; m < 4; m++)
      if (m < p.nac) e[m] = u[m * n3 + l];
    const T c = cf[l];
    T f0 = -p.LCI * p.KCI * c;
    f0 += p.LCI * ch_f<PL>(p, e, c);
    const T cl = x > 0 ? cf[l - 1] : (T)0, cr = x < n - 1 ? cf[l + 1] : (T)0;
    const T ct = y > 0 ? cf[l - n] : (T)0, cb = y < n - 1 ? cf[l + n] : (T)0;
    const T cz = z > 0 ? cf[l - nn] : (T)0, ck = z < n - 1 ? cf[l + nn] : (T)0;
    T la = (cl + cr - (T)2 * c) * p.ih2x;
    la += (ct + cb - (T)2 * c) * p.ih2y;
    la += (cz + ck - (T)2 * c) * p.ih2z;
    T a = -f0 + p.KCI * c;
    T b = p.epn2 * la - f0;
    if (x == 0 || x == n - 1 || y == 0 || y == n - 1 || z == 0 || z == n - 1) {
      const int iz = img(n, z), iy = img(n, y), ix = img(n, x), lo = img(n, -1), hi = img(n, n);
      T w;
      if (x == 0) { w = p.epn2 * cf[L3(n, iz, iy, lo)] * p.ih2x; a += w; b += w; }
      if (x == n - 1) { w = p.epn2 * cf[L3(n, iz, iy, hi)] * p.ih2x; a += w; b += w; }
      if (y == 0) { w = p.epn2 * cf[L3(n, iz, lo, ix)] * p.ih2y; a += w; b += w; }
      if (y == n - 1) { w = p.epn2 * cf[L3(n, iz, hi, ix)] * p.ih2y; a += w; b += w; }
      if (z == 0) { w = p.epn2 * cf[L3(n, lo, iy, ix)] * p.ih2z; a += w; b += w; }
      if (z == n - 1) { w = p.epn2 * cf[L3(n, hi, iy, ix)] * p.ih2z; a += w; b += w; }
    }
    t1[l] = a;
    t2[l] = b;
  }
}

// N = LCI (f1 + f2) of every cell (blockIdx.z = run x z)
template <typename PL, typename T>
__global__ void __launch_bounds__(RX * RY) mob_n_kernel(P<T> p0, const T *__restrict__ u, const T *__restrict__ tt,
                                                        const double *__restrict__ cmax, T *__restrict__ out) {
  const int n = p0.n;
  const int zch = (n + PZ - 1) / PZ;  // blockIdx.z = run x chunk of PZ planes
  const int run = blockIdx.z / zch, z0 = (blockIdx.z - run * zch) * PZ, z1 = z0 + PZ < n ? z0 + PZ : n;
  const int x = blockIdx.x * RX + threadIdx.x, y = blockIdx.y * RY + threadIdx.y;
  if (x >= n || y >= n) return;
  const size_t n3 = (size_t)n * n * n, nn = (size_t)n * n;
  P<T> p = p0;
  if (p0.krun) p.K[0] = (T)p0.krun[run];
  u += (size_t)run * p.F * n3;
  out += (size_t)run * p.F * n3;
  const T *t1 = tt + (size_t)run * 2 * n3, *t2 = t1 + n3;
  const T C = (T)cmax[run];
  for (int z = z0; z < z1; z++) {
    const size_t l = (size_t)z * nn + (size_t)y * n + x;
    // f1 = -C lap0(t1) - C mu_out / h^2
    const T tc = t1[l];
    const T al = x > 0 ? t1[l - 1] : (T)0, ar = x < n - 1 ? t1[l + 1] : (T)0;
    const T at = y > 0 ? t1[l - n] : (T)0, ab = y < n - 1 ? t1[l + n] : (T)0;
    const T af = z > 0 ? t1[l - nn] : (T)0, ak = z < n - 1 ? t1[l + nn] : (T)0;
    T la = (al + ar - (T)2 * tc) * p.ih2x;
    la += (at + ab - (T)2 * tc) * p.ih2y;
    la += (af + ak - (T)2 * tc) * p.ih2z;
    T f1 = -C * la;
    if (x == 0 || x == n - 1 || y == 0 || y == n - 1 || z == 0 || z == n - 1) {
      const int iz = img(n, z), iy = img(n, y), ix = img(n, x), lo = img(n, -1), hi = img(n, n);
      if (x == 0) f1 -= C * ch_mu_at<PL>(p, u, iz, iy, lo) * p.ih2x;
      if (x == n - 1) f1 -= C * ch_mu_at<PL>(p, u, iz, iy, hi) * p.ih2x;
      if (y == 0) f1 -= C * ch_mu_at<PL>(p, u, iz, lo, ix) * p.ih2y;
      if (y == n - 1) f1 -= C * ch_mu_at<PL>(p, u, iz, hi, ix) * p.ih2y;
      if (z == 0) f1 -= C * ch_mu_at<PL>(p, u, lo, iy, ix) * p.ih2z;
      if (z == n - 1) f1 -= C * ch_mu_at<PL>(p, u, hi, iy, ix) * p.ih2z;
    }
    // f2 = -div0((M - C) grad t2), M - C and t2 zero outside the block
    const T *e0 = u;
    const T bc = t2[l], mc = mobility(p, e0[l]) - C;
    auto nb = [&](bool in, size_t q, T &bq, T &mq) {
      bq = in ? t2[q] : (T)0;
      mq = in ? mobility(p, e0[q]) - C : (T)0;
    };
    T bq, mq, d;
    const T hx = (T)0.5 * p.ih2x, hy = (T)0.5 * p.ih2y, hz = (T)0.5 * p.ih2z;
    nb(x > 0, l - 1, bq, mq);
    d = (mq + mc) * (bq - bc) * hx;
    nb(x < n - 1, l + 1, bq, mq);
    d += (mq + mc) * (bq - bc) * hx;
    nb(y > 0, l - n, bq, mq);
    d += (mq + mc) * (bq - bc) * hy;
    nb(y < n - 1, l + n, bq, mq);
    d += (mq + mc) * (bq - bc) * hy;
    nb(z > 0, l - nn, bq, mq);
    d += (mq + mc) * (bq - bc) * hz;
    nb(z < n - 1, l + nn, bq, mq);
    d += (mq + mc) * (bq - bc) * hz;
    out[(size_t)p.nac * n3 + l] = p.LCI * (f1 - d);
  }
}

template <typename PL, typename T>
static cudaError_t launch_rhs_pl(const Phys &ph, const T *u, const T *felas, T *out, T *scratch, cudaStream_t s) {
  P<T> p = to_p<T>(ph);
  long long n3 = (long long)ph.n * ph.n * ph.n;
  const dim3 blk(RX, RY), grd((ph.n + RX - 1) / RX, (ph.n + RY - 1) / RY, ((ph.n + PZ - 1) / PZ) * p.runs);
  if (ph.nac > 0) {
    const size_t smem = sizeof(T) * ph.nac * 5 * PLANE;
    const dim3 gac((ph.n + RX - 1) / RX, (ph.n + RY - 1) / RY, ((ph.n + p.zc - 1) / p.zc) * p.runs);
    cudaError_t e = cudaSuccess;
    switch (ph.nac * 2 + (ph.anisotropic ? 1 : 0)) {
#define SCLET_RHS_AC(NAC, AN)                                                                                  \
  case NAC * 2 + AN:                                                                                           \
    e = cudaFuncSetAttribute(rhs_ac_kernel<PL, T, NAC, AN>, cudaFuncAttributeMaxDynamicSharedMemorySize,        \
                             (int)smem);                                                                       \
    if (e == cudaSuccess) rhs_ac_kernel<PL, T, NAC, AN><<<gac, blk, smem, s>>>(p, u, felas, out);               \
    break;
      SCLET_RHS_AC(1, 0) SCLET_RHS_AC(1, 1) SCLET_RHS_AC(2, 0) SCLET_RHS_AC(2, 1)
      SCLET_RHS_AC(3, 0) SCLET_RHS_AC(3, 1) SCLET_RHS_AC(4, 0) SCLET_RHS_AC(4, 1)
#undef SCLET_RHS_AC
      default: e = cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    launch_counter()++;
  }
  if (PL::max_nch > 0 && ph.varmob && ph.nch == 1) {
    if (!ph.mob_t || !ph.mob_part) return cudaErrorInvalidValue;
    T *tt = static_cast<T *>(ph.mob_t);
    double *cmax = ph.mob_part + (size_t)MOB_PARTS * p.runs;
    mob_max_kernel<T><<<dim3(MOB_PARTS, p.runs), 256, 0, s>>>(p, u, ph.mob_part);
    mob_final_kernel<<<p.runs, 256, 0, s>>>(ph.mob_part, cmax);
    mob_t_kernel<PL, T><<<grd, blk, 0, s>>>(p, u, tt);
    mob_n_kernel<PL, T><<<grd, blk, 0, s>>>(p, u, tt, cmax, out);
    launch_counter() += 4;
  } else if (PL::max_nch > 0) {
    for (int m = 0; m < ph.nch; m++) {
      // one conserved field (the plugins' CH_f is defined for c_0 only)
      rhs_ch_t_kernel<PL, T><<<grd, blk, 0, s>>>(p, u, scratch);
      rhs_ch_lap_kernel<PL, T><<<grd, blk, 0, s>>>(p, u, scratch, out + (long long)ph.nac * n3);  // per run: + r F n^3
      launch_counter() += 2;
    }
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_rhs(const Phys &ph, const T *u, const T *felas, T *out, T *scratch, cudaStream_t s) {
  return with_physics(ph.physics, [&](auto *tag) {
    using PL = std::remove_pointer_t<decltype(tag)>;
    return launch_rhs_pl<PL, T>(ph, u, felas, out, scratch, s);
  });
}

template cudaError_t launch_rhs<double>(const Phys &, const double *, const double *, double *, double *, cudaStream_t);
template cudaError_t launch_rhs<float>(const Phys &, const float *, const float *, float *, float *, cudaStream_t);

}  // namespace sclet
