/* Mixed-precision instantiation of the step: horizontal operators, their
 * tables and intermediates in FP32; prognostic state, divergence
 * accumulation, thermodynamics and the vertical implicit solves in FP64. */
#include "step.cuh"

namespace game {

int launch_step_mixed(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st)
{
    launch_step<float>(c, p, so, sn, st);
    return 0;
}

}  // namespace game
