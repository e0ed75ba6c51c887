/*
 * Diffusion branch of the RKHEVI step (diff_f64.cu), run at the first RK
 * substep when a diffusion switch is on.
 */
#pragma once

#include "context.h"

namespace game {

/* momentum part (vector_tendencies_expl.c:41-69): Brunt-Vaisala frequency and
 * TKE update, horizontal and vertical momentum diffusion into the friction
 * acceleration, dissipation rate.  Reads state_new before the wind update. */
void launch_diffusion_momentum(Context *c, const StepParams &p, const DState &sn);

/* scalar part (scalar_tendencies_expl.c:44-88): diffusion coefficients,
 * temperature and mass diffusion into temperature_diffusion_heating and
 * mass_diff_tendency */
void launch_diffusion_scalar(Context *c, const StepParams &p, const DState &sn);

}  // namespace game
