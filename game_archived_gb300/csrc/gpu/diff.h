/*
 * Diffusion branch of the RKHEVI step (kernels in diff.cuh), run at the
 * first RK substep when a diffusion switch is on: FP64 instantiation in
 * diff_f64.cu, FP32 (mixed path) in diff_mixed.cu.
 */
#pragma once

#include "context.h"

namespace game {

/* momentum part (vector_tendencies_expl.c:41-69): Brunt-Vaisala frequency and
 * TKE update, horizontal and vertical momentum diffusion into the friction
 * acceleration, dissipation rate.  sv: state_new (FP64) or its FP32 shadow,
 * read before the wind update. */
void launch_diffusion_momentum(Context *c, const StepParams &p, const SView<double> &sv);
void launch_diffusion_momentum(Context *c, const StepParams &p, const SView<float> &sv);

/* scalar part (scalar_tendencies_expl.c:44-88): diffusion coefficients,
 * temperature and mass diffusion into temperature_diffusion_heating and
 * mass_diff_tendency */
void launch_diffusion_scalar(Context *c, const StepParams &p, const SView<double> &sv);
void launch_diffusion_scalar(Context *c, const StepParams &p, const SView<float> &sv);

/* Held-Suarez radiative forcing (rad_on = 2) into radiation_tendency, from
 * state_old and its temperature, at the first RK substep of a step with
 * rad_update = 1 (manage_rkhevi.c:80-84); FP64 on both paths */
void launch_held_suarez_radiation(Context *c, const DState &so);

}  // namespace game
