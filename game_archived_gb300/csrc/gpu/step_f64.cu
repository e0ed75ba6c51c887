/* FP64 instantiation of the step (compiled with --fmad=false: every product
 * and sum is rounded separately, as in the reference built with
 * -ffp-contract=off) */
#include "step.cuh"

namespace game {

int launch_step_f64(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st)
{
    launch_step<double>(c, p, so, sn, st);
    return 0;
}

int launch_damping_table(Context *c, const StepParams &p)
{
    if (c->nl < 2) return 0;
    if (c->damp_key[0] == p.damping_start_height && c->damp_key[1] == p.damping_coeff_max && c->damp_key[2] == p.dt)
        return 0;
    const long long n = (long long)(c->nl - 1) * c->nc;
    k_damping_table<<<nblocks(n, 256), 256, 0, c->stream>>>(c->vg, p.damping_start_height, p.damping_coeff_max, p.dt,
                                                            c->damp_dc, c->damp_inv, c->damp_inv_df);
    CK(cudaGetLastError());
    c->kernel_launches++;
    c->damp_key[0] = p.damping_start_height;
    c->damp_key[1] = p.damping_coeff_max;
    c->damp_key[2] = p.dt;
    return 0;
}

}  // namespace game
