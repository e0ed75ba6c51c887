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

void launch_held_suarez_radiation(Context *c, const DState &so)
{
    ProfScope ps(c, "kd_hs_rad");
    kd_hs_rad<<<dnb(c->ns), 256, 0, c->stream>>>(c->ns, c->nc, c->n_cond, c->dg64.lat, c->dg64.rad_cov, c->temperature,
                                                  so, c->dbuf->rad);
    c->kernel_launches++;
}

}  // namespace game
