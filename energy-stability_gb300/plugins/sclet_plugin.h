/*
 * Physics-plugin shim: one plugin source compiled twice, as plain C for the
 * host (the CPU oracle) and as CUDA C++ for the device kernels.
 *
 * The reference's extension point is formula.c
 * (source_beta_to_omega/src/formula.c:9-56): init_KL() sets the linear
 * operator constants LE, KE (Allen-Cahn) and LCI, KCI (Cahn-Hilliard);
 * AC_f(n) and CH_f(n) return the derivative of the bulk free energy with
 * respect to order parameter n and concentration n.  They read the cell's
 * values from the globals ac[m].u and ch[m].c, which the macros
 * SWTICH_AC_FIELD1 / SWITCH_CH_FIELD1 / SWITCH_CH_FIELDMU (ScLETD.h:108-158)
 * load before every call.
 *
 * A plugin here is written the same way -- ac[m].u, ch[m].c, nac, nch and the
 * field index n -- but ac and ch are the cell's values passed in (registers
 * on the device, with nac and nch compile-time constants there, so the loops
 * over fields unroll), and the plugin's numeric constants are K(0), K(1), ...
 * (the numbers of landau_input.txt).  A plugin file defines, with the macros
 * below:
 *   SCLET_MAX_NCH(v)     concentrations it supports (0 or 1)
 *   SCLET_C0_INDEX(i)    index of its reference composition c0 when c enters
 *                        only as (c - K(i)); -1 otherwise.  Where the state
 *                        stores c - c0 (the mixed form), the library passes
 *                        the stored value as ch[0].c and K(i) - c0 as K(i).
 *   SCLET_DEFAULTS = {...};   default constants
 *   SCLET_INIT_KL { ... }     sets kl->LE, kl->KE, kl->LCI, kl->KCI (host)
 *   SCLET_AC_F { ... }        returns AC_f(n)
 *   SCLET_CH_F { ... }        returns CH_f(n)
 *   SCLET_F_BULK { ... }      returns the bulk free-energy density (the part
 *                             of the energy that AC_f and CH_f derive from;
 *                             the diagnostics add the gradient terms)
 * The arithmetic type is `real` (double on the host, the state's precision on
 * the device).
 *
 * The including file names the plugin: in C it defines
 * SCLET_PLUGIN_NS(x) as a prefixed name (e.g. landau246_##x); in C++ it
 * includes the plugin inside a namespace and defines SCLET_PLUGIN_NS(x) as x.
 * After its plugins it #undefs K (and, in C, real).
 */
#ifndef SCLET_PLUGIN_H
#define SCLET_PLUGIN_H

#define SCLET_PLUGIN_NK 16 /* constants per plugin */

typedef struct sclet_kl {
  double LE, KE, LCI, KCI;
} sclet_kl;

#ifdef __CUDACC__

template <typename real>
struct sclet_acv {
  real u;
};
template <typename real>
struct sclet_chv {
  real c;
};

#define SCLET_PLUGIN_FN template <typename real> __host__ __device__ __forceinline__ real
#define SCLET_AC_F                                                                                         \
  SCLET_PLUGIN_FN SCLET_PLUGIN_NS(AC_f)(const sclet_acv<real> *ac, const sclet_chv<real> *ch, const int nac, \
                                        const int nch, const real *Kp, const int n)
#define SCLET_CH_F                                                                                         \
  SCLET_PLUGIN_FN SCLET_PLUGIN_NS(CH_f)(const sclet_acv<real> *ac, const sclet_chv<real> *ch, const int nac, \
                                        const int nch, const real *Kp, const int n)
#define SCLET_F_BULK                                                                                          \
  SCLET_PLUGIN_FN SCLET_PLUGIN_NS(F_bulk)(const sclet_acv<real> *ac, const sclet_chv<real> *ch, const int nac, \
                                          const int nch, const real *Kp)
#define SCLET_INIT_KL static inline void SCLET_PLUGIN_NS(init_KL)(const double *Kp, sclet_kl *kl)

#else /* C, host */

typedef struct sclet_acv {
  double u;
} sclet_acv;
typedef struct sclet_chv {
  double c;
} sclet_chv;

#define SCLET_AC_F                                                                                             \
  static inline double SCLET_PLUGIN_NS(AC_f)(const sclet_acv *ac, const sclet_chv *ch, const int nac, const int nch, \
                                             const double *Kp, const int n)
#define SCLET_CH_F                                                                                             \
  static inline double SCLET_PLUGIN_NS(CH_f)(const sclet_acv *ac, const sclet_chv *ch, const int nac, const int nch, \
                                             const double *Kp, const int n)
#define SCLET_F_BULK                                                                                             \
  static inline double SCLET_PLUGIN_NS(F_bulk)(const sclet_acv *ac, const sclet_chv *ch, const int nac, const int nch, \
                                               const double *Kp)
#define SCLET_INIT_KL static inline void SCLET_PLUGIN_NS(init_KL)(const double *Kp, sclet_kl *kl)

#endif

#define SCLET_MAX_NCH(v) enum { SCLET_PLUGIN_NS(max_nch) = (v) };
#define SCLET_C0_INDEX(i) enum { SCLET_PLUGIN_NS(c0_index) = (i) };
#define SCLET_DEFAULTS static const double SCLET_PLUGIN_NS(defaults)[SCLET_PLUGIN_NK]

#endif

/* redefined at every inclusion: the includer #undefs them after its plugins */
#define K(i) (Kp[i])
#ifndef __CUDACC__
#define real double
#endif
