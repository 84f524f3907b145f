// Host-side set-up of the physics plugin of a run (see sclet_physics.cuh).
#include <string.h>

#include "sclet_physics.cuh"

namespace sclet {

const char *physics_setup(const sclet_params *p, int precision, Phys *ph) {
  const char *msg = nullptr;
  cudaError_t e = with_physics(p->physics, [&](auto *tag) -> cudaError_t {
    using PL = std::remove_pointer_t<decltype(tag)>;
    if (p->nch > PL::max_nch) {
      msg = PL::max_nch == 0 ? "the physics plugin takes no conserved concentration (nch must be 0)"
                             : "the physics plugin takes at most one conserved concentration";
      return cudaErrorInvalidValue;
    }
    // the plugin's constants: landau_input.txt's numbers where the plugin
    // reads them (the Landau plugin), its defaults beyond
    double k[16];
    memcpy(k, PL::defaults(), sizeof k);
    if (p->physics == SCLET_PHYSICS_LANDAU246) memcpy(k, p->landau, sizeof p->landau);
    sclet_kl kl;
    PL::init_kl(k, &kl);
    ph->physics = p->physics;
    ph->LE = kl.LE;
    ph->KE = kl.KE;
    ph->LCI = kl.LCI;
    ph->KCI = kl.KCI;
    // the mixed form stores c - c0 where the plugin's c enters as c - K(c0)
    ph->cshift = (precision == SCLET_MIXED && p->nch > 0 && PL::c0_index >= 0) ? k[PL::c0_index] : 0.0;
    if (PL::c0_index >= 0) k[PL::c0_index] -= ph->cshift;
    memcpy(ph->K, k, sizeof k);
    return cudaSuccess;
  });
  if (e != cudaSuccess && !msg) msg = "unknown physics plugin (sclet_params.physics)";
  return e == cudaSuccess ? nullptr : msg;
}

}  // namespace sclet
