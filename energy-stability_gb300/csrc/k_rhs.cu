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
// The physics plugin is the Landau 2-4-6 form with a cross term and a c-eta
// coupling (the drop-in replacement of formula.c:9-56).
#include "sclet_internal.cuh"

namespace sclet {

template <typename T>
struct P {
  int n, nac, nch, F, aniso, elastic;
  T epn2, hx, hy, hz, LE, KE, LCI, KCI, es;
  T ih2x, ih2y, ih2z;   // 1 / h^2 per axis
  T i2hx, i2hy, i2hz;   // 1 / (2 h) per axis
  T a2, a4, a6, g, th, c0, A;
  T lam[4][9];
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
  p.a2 = (T)ph.a2; p.a4 = (T)ph.a4; p.a6 = (T)ph.a6; p.g = (T)ph.g; p.th = (T)ph.th; p.c0 = (T)(ph.c0 - ph.cshift); p.A = (T)ph.A;
  for (int m = 0; m < 4; m++)
    for (int k = 0; k < 9; k++) p.lam[m][k] = (T)ph.lam[m][k];
  return p;
}

// dF/deta_m of the plugin (AC_f).
template <typename T>
__device__ inline T ac_f(const P<T> &p, const T *e, T c, int m) {
  T u = e[m], u2 = u * u, others = (T)0;
  for (int k = 0; k < p.nac; k++)
    if (k != m) others += e[k] * e[k];
  T f = p.a2 * u + p.a4 * u2 * u + p.a6 * u2 * u2 * u + (T)2 * p.g * u * others;
  if (p.nch > 0) f -= (T)2 * p.th * (c - p.c0) * u;
  return f;
}

// dF/dc of the plugin (CH_f).
template <typename T>
__device__ inline T ch_f(const P<T> &p, const T *e, T c) {
  T s = (T)0;
  for (int k = 0; k < p.nac; k++) s += e[k] * e[k];
  return p.A * (c - p.c0) - p.th * s;
}

__device__ inline long long L3(int n, int z, int y, int x) { return ((long long)z * n + y) * n + x; }

// lambda . (central differences) at cell (z,y,x), component `comp`, with
// values outside the block read as zero (ac_calc_F2 first loop).
template <typename T>
__device__ inline T grad_comp(const P<T> &p, const T *__restrict__ u, const T *lam, int z, int y, int x, int comp) {
  int n = p.n;
  T al = x > 0 ? u[L3(n, z, y, x - 1)] : (T)0, ar = x < n - 1 ? u[L3(n, z, y, x + 1)] : (T)0;
  T at = y > 0 ? u[L3(n, z, y - 1, x)] : (T)0, ab = y < n - 1 ? u[L3(n, z, y + 1, x)] : (T)0;
  T af = z > 0 ? u[L3(n, z - 1, y, x)] : (T)0, ak = z < n - 1 ? u[L3(n, z + 1, y, x)] : (T)0;
  T gx = (ar - al) * p.i2hx, gy = (at - ab) * p.i2hy, gz = (af - ak) * p.i2hz;
  return lam[comp * 3 + 0] * gx + lam[comp * 3 + 1] * gy + lam[comp * 3 + 2] * gz;
}

// div of the above (ac_calc_F2 second loop).
template <typename T>
__device__ inline T aniso_f2(const P<T> &p, const T *__restrict__ u, const T *lam, int z, int y, int x) {
  int n = p.n;
  T ar = x < n - 1 ? grad_comp(p, u, lam, z, y, x + 1, 0) : (T)0;
  T al = x > 0 ? grad_comp(p, u, lam, z, y, x - 1, 0) : (T)0;
  T at = y > 0 ? grad_comp(p, u, lam, z, y - 1, x, 1) : (T)0;
  T ab = y < n - 1 ? grad_comp(p, u, lam, z, y + 1, x, 1) : (T)0;
  T af = z > 0 ? grad_comp(p, u, lam, z - 1, y, x, 2) : (T)0;
  T ak = z < n - 1 ? grad_comp(p, u, lam, z + 1, y, x, 2) : (T)0;
  T t = (T)0;
  t += (ar - al) * p.i2hx;
  t += (at - ab) * p.i2hy;
  t += (af - ak) * p.i2hz;
  return t;
}

template <typename T>
__global__ void __launch_bounds__(256) rhs_ac_kernel(P<T> p, const T *__restrict__ u, const T *__restrict__ felas,
                                                     T *__restrict__ out) {
  int n = p.n;
  long long n3 = (long long)n * n * n;
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < n3; l += (long long)gridDim.x * blockDim.x) {
    int x = (int)(l % n), y = (int)((l / n) % n), z = (int)(l / ((long long)n * n));
    T e[4];
    for (int m = 0; m < p.nac; m++) e[m] = u[m * n3 + l];
    T c = p.nch > 0 ? u[p.nac * n3 + l] : (T)0;
    bool face = x == 0 || x == n - 1 || y == 0 || y == n - 1 || z == 0 || z == n - 1;
    int iz = img(n, z), iy = img(n, y), ix = img(n, x), lo = img(n, -1), hi = img(n, n);
    for (int m = 0; m < p.nac; m++) {
      const T *um = u + m * n3;
      T v = p.LE * p.KE * e[m];
      v -= p.LE * ac_f(p, e, c, m);
      if (face) {
        T w = p.LE * p.epn2;
        if (x == 0) v += w * um[L3(n, iz, iy, lo)] * p.ih2x;
        if (x == n - 1) v += w * um[L3(n, iz, iy, hi)] * p.ih2x;
        if (y == 0) v += w * um[L3(n, iz, lo, ix)] * p.ih2y;
        if (y == n - 1) v += w * um[L3(n, iz, hi, ix)] * p.ih2y;
        if (z == 0) v += w * um[L3(n, lo, iy, ix)] * p.ih2z;
        if (z == n - 1) v += w * um[L3(n, hi, iy, ix)] * p.ih2z;
      }
      if (p.aniso) v -= p.epn2 * p.LE * aniso_f2(p, um, p.lam[m], z, y, x);
      if (p.elastic == 1) v -= p.LE * p.es * felas[m * n3 + l];
      out[m * n3 + l] = v;
    }
  }
}

// t = -LCI KCI c + LCI CH_f, minus the face liftings (first part of
// ch_calc_FU_ConstantMobility).
template <typename T>
__global__ void __launch_bounds__(256) rhs_ch_t_kernel(P<T> p, const T *__restrict__ u, T *__restrict__ t) {
  int n = p.n;
  long long n3 = (long long)n * n * n;
  const T *cf = u + p.nac * n3;
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < n3; l += (long long)gridDim.x * blockDim.x) {
    int x = (int)(l % n), y = (int)((l / n) % n), z = (int)(l / ((long long)n * n));
    T e[4];
    for (int m = 0; m < p.nac; m++) e[m] = u[m * n3 + l];
    T c = cf[l];
    T v = -p.LCI * p.KCI * c;
    v += p.LCI * ch_f(p, e, c);
    if (x == 0 || x == n - 1 || y == 0 || y == n - 1 || z == 0 || z == n - 1) {
      int iz = img(n, z), iy = img(n, y), ix = img(n, x), lo = img(n, -1), hi = img(n, n);
      T w = p.LCI * p.epn2;
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
template <typename T>
__device__ inline T ch_mu_at(const P<T> &p, const T *__restrict__ u, int z, int y, int x) {
  int n = p.n;
  long long n3 = (long long)n * n * n;
  const T *cf = u + p.nac * n3;
  T cv = cf[L3(n, z, y, x)];
  T lap = (cf[L3(n, z, y, img(n, x - 1))] + (T)(-2.0) * cv + cf[L3(n, z, y, img(n, x + 1))]) * p.ih2x;
  lap += (cf[L3(n, z, img(n, y - 1), x)] + (T)(-2.0) * cv + cf[L3(n, z, img(n, y + 1), x)]) * p.ih2y;
  lap += (cf[L3(n, img(n, z - 1), y, x)] + (T)(-2.0) * cv + cf[L3(n, img(n, z + 1), y, x)]) * p.ih2z;
  T e[4];
  for (int m = 0; m < p.nac; m++) e[m] = u[m * n3 + L3(n, z, y, x)];
  T mu = p.LCI * p.epn2 * lap;
  mu -= p.LCI * ch_f(p, e, cv);
  return mu;
}

// N_c = lap(t) with zero outside, minus mu(outside)/h^2 on faces.
template <typename T>
__global__ void __launch_bounds__(256) rhs_ch_lap_kernel(P<T> p, const T *__restrict__ u, const T *__restrict__ t,
                                                         T *__restrict__ out) {
  int n = p.n;
  long long n3 = (long long)n * n * n, nn = (long long)n * n;
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < n3; l += (long long)gridDim.x * blockDim.x) {
    int x = (int)(l % n), y = (int)((l / n) % n), z = (int)(l / nn);
    T tc = t[l];
    T fl = x > 0 ? t[l - 1] : (T)0, fr = x < n - 1 ? t[l + 1] : (T)0;
    T ft = y > 0 ? t[l - n] : (T)0, fb = y < n - 1 ? t[l + n] : (T)0;
    T ff = z > 0 ? t[l - nn] : (T)0, fk = z < n - 1 ? t[l + nn] : (T)0;
    T v = (fl + fr - (T)2 * tc) * p.ih2x;
    v += (ft + fb - (T)2 * tc) * p.ih2y;
    v += (ff + fk - (T)2 * tc) * p.ih2z;
    if (x == 0 || x == n - 1 || y == 0 || y == n - 1 || z == 0 || z == n - 1) {
      int iz = img(n, z), iy = img(n, y), ix = img(n, x), lo = img(n, -1), hi = img(n, n);
      if (x == 0) v -= ch_mu_at(p, u, iz, iy, lo) * p.ih2x;
      if (x == n - 1) v -= ch_mu_at(p, u, iz, iy, hi) * p.ih2x;
      if (y == 0) v -= ch_mu_at(p, u, iz, lo, ix) * p.ih2y;
      if (y == n - 1) v -= ch_mu_at(p, u, iz, hi, ix) * p.ih2y;
      if (z == 0) v -= ch_mu_at(p, u, lo, iy, ix) * p.ih2z;
      if (z == n - 1) v -= ch_mu_at(p, u, hi, iy, ix) * p.ih2z;
    }
    out[l] = v;
  }
}

template <typename T>
cudaError_t launch_rhs(const Phys &ph, const T *u, const T *felas, T *out, T *scratch, cudaStream_t s) {
  P<T> p = to_p<T>(ph);
  long long n3 = (long long)ph.n * ph.n * ph.n;
  long long blocks = (n3 + 255) / 256;
  int g = (int)(blocks > 152LL * 32 ? 152LL * 32 : blocks);
  if (ph.nac > 0) {
    rhs_ac_kernel<T><<<g, 256, 0, s>>>(p, u, felas, out);
    launch_counter()++;
  }
  for (int m = 0; m < ph.nch; m++) {
    // one conserved field (the plugin's CH_f is defined for c_0 only)
    rhs_ch_t_kernel<T><<<g, 256, 0, s>>>(p, u, scratch);
    rhs_ch_lap_kernel<T><<<g, 256, 0, s>>>(p, u, scratch, out + (long long)ph.nac * n3);
    launch_counter() += 2;
  }
  return cudaGetLastError();
}

template cudaError_t launch_rhs<double>(const Phys &, const double *, const double *, double *, double *, cudaStream_t);
template cudaError_t launch_rhs<float>(const Phys &, const float *, const float *, float *, float *, cudaStream_t);

}  // namespace sclet
