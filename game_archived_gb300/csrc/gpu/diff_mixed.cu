/*
 * Diffusion branch, mixed path: the kernels of diff.cuh with R = float on
 * the FP32 tables and the FP32 shadow of state_new; the divergences of the
 * diffusive fluxes are summed as double-word pairs and stored in double.
 */
#include "diff.cuh"

namespace game {

void launch_diffusion_momentum(Context *c, const StepParams &p, const SView<float> &sv)
{
    diffusion_momentum<float>(c, p, c->hg32, c->dg32, sv);
}

void launch_diffusion_scalar(Context *c, const StepParams &p, const SView<float> &sv)
{
    diffusion_scalar<float>(c, p, c->hg32, c->dg32, sv, c->cp32_ice, c->cp32_water);
}

}  // namespace game
