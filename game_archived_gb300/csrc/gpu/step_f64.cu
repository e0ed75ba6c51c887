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

}  // namespace game
