// Host-side set-up of the physics plugin of a run (see sclet_physics.cuh).
#include <math.h>
#include <string.h>

#include "sclet_physics.cuh"

namespace sclet {

// update_M_C (source_beta_to_omega/src/mobility.c:860-922): the mobility of
// the first concentration (Cu) as a function of the first order parameter,
// M = cu0 (1 - cu0) (DA (1 - eta0) + DG eta0), DA = 1 and DG the ratio of the
// two phases' Arrhenius diffusivities D0 exp(-Q / RT) at T = 823 K.
void mobility_constants(double *m0, double *dg) {
  const double rt = 8.314472 * 823.0, cu0 = 0.15;
  const double da = 4.7e-5 * exp(-2.44e5 / rt);
  *dg = (4.3e-5 * exp(-2.80e5 / rt)) / da;
  *m0 = cu0 * (1.0 - cu0);
}

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
    // the mixed form stores c - c0 where the plugin's c enters as c - K(c0);
    // not with variable mobility, whose right-hand side is not invariant
    // under that shift (its f1 carries KCI c beside LCI KCI c)
    ph->cshift = (precision == SCLET_MIXED && p->nch > 0 && PL::c0_index >= 0 && !p->variable_mobility)
                     ? k[PL::c0_index]
                     : 0.0;
    if (PL::c0_index >= 0) k[PL::c0_index] -= ph->cshift;
    memcpy(ph->K, k, sizeof k);
    return cudaSuccess;
  });
  if (e != cudaSuccess && !msg) msg = "unknown physics plugin (sclet_params.physics)";
  ph->varmob = p->variable_mobility;
  mobility_constants(&ph->mob_m0, &ph->mob_dg);
  return e == cudaSuccess ? nullptr : msg;
}

}  // namespace sclet
