// Internal declarations shared by the CUDA translation units of sclet_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sclet_gb300.h"

namespace sclet {

// Physics-plugin constants and per-run scalars passed by value to kernels.
struct Phys {
  int n, nac, nch, F;
  int anisotropic, elastic;
  double dt, epn2;
  double h[3];
  double kk[3];
  double lam[4][9];      // F2 tensors: diag(kk) - file tensor, row-major
  double elastic_scale;
  // physics plugin (SCLET_PHYSICS_*) and its constants as the kernels see
  // them (the reference composition shifted by cshift, see below); LE, KE,
  // LCI, KCI from the plugin's init_KL
  int physics;
  double K[16];
  double LE, KE, LCI, KCI;
  // Offset of the stored conserved field: the device holds c - cshift.  The
  // mixed form stores c - c0 (cshift = c0), which keeps FP32 storage and the
  // transforms at the scale of the fluctuations; the scheme is linear in c
  // and the constant state c0 is a fixed point, so this changes nothing in
  // exact arithmetic.  It needs a plugin whose c enters only as c - c0
  // (SCLET_C0_INDEX); 0 otherwise and in the FP64 form.
  double cshift;
  // runs of the same block size held side by side (the batched ensemble):
  // run r's fields are the F blocks at r F n^3; krun (device, runs values,
  // or null) replaces plugin constant 0 per run (the Landau a2)
  int runs;
  const double *krun;
  // launch shape chosen by the autotuner (0: the default)
  int rhs_zc;       // z-planes per CTA of the Allen-Cahn right-hand side
  int tc_ctas;      // persistent CTAs of the tensor-core products
  // variable-mobility Cahn-Hilliard (VariableMobility = 1): M(eta0) =
  // mob_m0 (1 - eta0 + mob_dg eta0) (mobility_constants); device scratch of
  // two blocks per run (mob_t, the precision's type) and of the block maxima
  // of M (mob_part: MOB_PARTS per run, then one C per run)
  int varmob;
  double mob_m0, mob_dg;
  void *mob_t;
  double *mob_part;
};

constexpr int MOB_PARTS = 512;  // partial maxima of M per run
void mobility_constants(double *m0, double *dg);

// Geometry helpers (owned cells are 2 .. n-3 per axis, period N = n - 4).
__host__ __device__ inline int img(int n, int v) {
  int N = n - 4;
  int r = (v - 2) % N;
  if (r < 0) r += N;
  return 2 + r;
}
__host__ __device__ inline int wrap1(int n, int v) {
  int N = n - 4;
  return v < 2 ? v + N : (v >= n - 2 ? v - N : v);
}

// Number of ghost cells of an n^3 block: 4 z-planes, 4 y-slabs of the inner
// z range, 4 x-columns of the inner z,y range.
__host__ __device__ inline long long shell_count(int n) {
  long long N = n - 4;
  return 4LL * n * n + 4LL * N * n + 4LL * N * N;
}
// Maps a shell index to its cell.
__device__ inline void shell_cell(int n, long long s, int &z, int &y, int &x) {
  long long N = n - 4;
  long long nz = 4LL * n * n;
  if (s < nz) {
    int p = (int)(s / ((long long)n * n));
    long long r = s - (long long)p * n * n;
    z = p < 2 ? p : n - 4 + p;
    y = (int)(r / n);
    x = (int)(r % n);
    return;
  }
  s -= nz;
  long long ny = 4LL * N * n;
  if (s < ny) {
    int zz = (int)(s / (4LL * n));
    long long r = s - (long long)zz * 4 * n;
    int p = (int)(r / n);
    z = 2 + zz;
    y = p < 2 ? p : n - 4 + p;
    x = (int)(r % n);
    return;
  }
  s -= ny;
  {
    int zz = (int)(s / (4LL * N));
    long long r = s - (long long)zz * 4 * N;
    int yy = (int)(r / 4);
    int p = (int)(r % 4);
    z = 2 + zz;
    y = 2 + yy;
    x = p < 2 ? p : n - 4 + p;
  }
}

// ---- kernel launchers (each returns the launch's cudaError_t) -------------
// Ghost fill of `count` blocks (stride n^3) in place; shell: scratch of
// count * shell_count(n) elements.
template <typename T>
cudaError_t launch_ghost_fill(T *u, int count, int n, T *shell, cudaStream_t s);
// Elastic scratch semantics: felas_p (p in order) gets its ghost cells from
// the fill of the shared scratch block (see k_halo.cu).  `prev` is the block
// that was last filled (felas_{p-1}, or the last field of the previous call).
// runs: blocks side by side, felas_p's at fstride and prev's at pstride
// apart (0: one prev for all); shell holds runs * shell_count(n) values.
template <typename T>
cudaError_t launch_elastic_shell(T *felas_p, const T *prev, int n, T *shell, cudaStream_t s, int runs = 1,
                                 long long fstride = 0, long long pstride = 0);

// Right-hand sides of all fields into out (F blocks).  felas: nac blocks.
template <typename T>
cudaError_t launch_rhs(const Phys &ph, const T *u, const T *felas, T *out, T *scratch, cudaStream_t s);

// Mode-n product with rotation, FP64: for `count` tensors,
// out_t[a'*n*n + r] = sum_a M[a'*n + a] in_t[r*n + a]  (M row-major).
// Epilogues: 0 store; 1 ETD1 update out = (1 - phi H) uhat + phi * acc with
// uhat = aux_t (read) ; 2 out = phi2 * acc ; 3 out += acc.  Prologue `sub`:
// in_t - sub_t.  kinds: per-tensor field kind selector (t % F >= nac -> CH).
struct EtdCoef {
  const double *dd[3];   // eigenvalues / h^2 per axis (device)
  double kk[3];
  double epn2, dt, LE, KE, LCI, KCI;
  int nac, F;
};
cudaError_t launch_modeprod_f64(const double *M, const double *in, const double *sub, double *out,
                                const double *aux, int count, int n, int epilogue, const EtdCoef &ec,
                                long long in_stride, long long out_stride, cudaStream_t s);

// Elastic force (FFT based) -- see k_fft.cu.
struct ElasticPlan;
cudaError_t elastic_plan_create(ElasticPlan **plan, int big_n, int nac, const double *voigt,
                                const double *eps, int fp32, cudaStream_t s, int runs = 1);
void elastic_plan_destroy(ElasticPlan *plan);
// felas (nac blocks of n^3) from the AC fields u (first nac blocks).
// runs (the plan's): run r's order parameters at u + r ustride, its force at
// felas + r nac n^3; shell holds n^3 + runs * shell_count(n) values
template <typename T>
cudaError_t elastic_compute(ElasticPlan *plan, const T *u, T *felas, int n, T *shell, cudaStream_t s,
                            long long ustride = 0);

// Diagnostics: out (F*4 doubles, device) per field max, min, vol, energy.
template <typename T>
cudaError_t launch_check_soln(const Phys &ph, const T *u, const double *elam, int form, double *partials,
                              int npart, double *out, cudaStream_t s);
int check_soln_partials(int n);

// Conserved-field mass of the mixed form (see k_mass.cu).  Weight `which`
// (0 E, 1 phi1, 2 phi2) into w (n^3 slots of 8 bytes: computed in FP64, then
// stored as FP32 (hi, lo) pairs) using tmp (n^3 doubles); g (n) and viT
// (n x n row-major) on the device.
cudaError_t mass_weight(double *w, double *tmp, const double *g, const double *viT, int n, int which,
                        const EtdCoef &ec, cudaStream_t s);
int mass_partials();
// part (2 * mass_partials()) = partial sums of wa.a (owned sum of a if wa is
// null) + wb.(b - bsub); wa, wb hold the weight pairs of mass_weight
cudaError_t mass_target(const float *a, const double *wa, const float *b, const float *bsub, const double *wb, int n,
                        double *part, cudaStream_t s);
// shifts the owned cells of u so that their sum meets the target partials
cudaError_t mass_fix(float *u, int n, const double *tpart, double *apart, double *res, cudaStream_t s);

// 16-bit codes of one field block (see k_codec.cu); kind 0 AC, 1 CH; the
// stored values plus shift are the field's values.
template <typename T>
cudaError_t launch_field_u16(const T *u, int kind, double shift, long long cells, unsigned short *out, cudaStream_t s);

// Counts kernel launches issued by this library (per process).
long long &launch_counter();

}  // namespace sclet
