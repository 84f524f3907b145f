// The physics plugins (energy-stability_gb300/plugins/*.h) compiled for the
// device, and the host-side set-up of a run's plugin constants.  A plugin is
// the drop-in form of the reference's formula.c (init_KL, AC_f, CH_f,
// source_beta_to_omega/src/formula.c:9-56); the same plugin file is compiled
// into the CPU oracle as C.
#pragma once

#include "sclet_internal.cuh"

#include "../plugins/sclet_plugin.h"

namespace sclet {
namespace physics {

namespace landau246 {
#define SCLET_PLUGIN_NS(x) x
#include "../plugins/landau246.h"
#undef SCLET_PLUGIN_NS
}  // namespace landau246

namespace formula234 {
#define SCLET_PLUGIN_NS(x) x
#include "../plugins/formula234.h"
#undef SCLET_PLUGIN_NS
}  // namespace formula234

#undef K

// One plugin as a type: the kernels take it as a template parameter, so its
// functions inline into the stencils with the field counts known.
#define SCLET_PLUGIN_TRAITS(Name, ns)                                                                         \
  struct Name {                                                                                               \
    static constexpr int max_nch = ns::max_nch, c0_index = ns::c0_index;                                      \
    template <typename T>                                                                                     \
    __host__ __device__ __forceinline__ static T ac_f(const sclet_acv<T> *ac, const sclet_chv<T> *ch, int nac, \
                                                      int nch, const T *k, int n) {                           \
      return ns::AC_f<T>(ac, ch, nac, nch, k, n);                                                             \
    }                                                                                                         \
    template <typename T>                                                                                     \
    __host__ __device__ __forceinline__ static T ch_f(const sclet_acv<T> *ac, const sclet_chv<T> *ch, int nac, \
                                                      int nch, const T *k, int n) {                           \
      return ns::CH_f<T>(ac, ch, nac, nch, k, n);                                                             \
    }                                                                                                         \
    template <typename T>                                                                                     \
    __host__ __device__ __forceinline__ static T f_bulk(const sclet_acv<T> *ac, const sclet_chv<T> *ch,        \
                                                        int nac, int nch, const T *k) {                       \
      return ns::F_bulk<T>(ac, ch, nac, nch, k);                                                              \
    }                                                                                                         \
    static void init_kl(const double *k, sclet_kl *kl) { ns::init_KL(k, kl); }                                \
    static const double *defaults() { return ns::defaults; }                                                  \
  };

SCLET_PLUGIN_TRAITS(Landau246, landau246)
SCLET_PLUGIN_TRAITS(Formula234, formula234)
#undef SCLET_PLUGIN_TRAITS

}  // namespace physics

// Calls body with the plugin type of `id` as PL (a generic lambda taking a
// PL* tag); returns cudaErrorInvalidValue for an unknown id.
template <typename F>
inline cudaError_t with_physics(int id, F &&body) {
  switch (id) {
    case SCLET_PHYSICS_LANDAU246: return body((physics::Landau246 *)nullptr);
    case SCLET_PHYSICS_FORMULA234: return body((physics::Formula234 *)nullptr);
    default: return cudaErrorInvalidValue;
  }
}

// Plugin part of Phys from the run's parameters: the linear-operator
// constants from the plugin's init_KL, the stored-offset cshift of the
// conserved field and the constants as the device kernels see them.
// Returns 0, or a message naming what the plugin cannot run.
const char *physics_setup(const sclet_params *p, int precision, Phys *ph);

}  // namespace sclet
