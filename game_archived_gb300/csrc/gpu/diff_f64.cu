/*
 * Diffusion branch, FP64 path: the kernels of diff.cuh with R = double,
 * compiled with --fmad=false so that every expression rounds as the
 * reference's C.
 */
#include "diff.cuh"

namespace game {

void launch_diffusion_momentum(Context *c, const StepParams &p, const SView<double> &sv)
{
    diffusion_momentum<double>(c, p, c->hg64, c->dg64, sv);
}

void launch_diffusion_scalar(Context *c, const StepParams &p, const SView<double> &sv)
{
    diffusion_scalar<double>(c, p, c->hg64, c->dg64, sv, c->cp_ice, c->cp_water);
}

}  // namespace game
