/* adjoint and tangent-linear windows of the RKHEVI step, dry and moist builds
 * (adj_f64.cu) */
#pragma once

#include "context.h"

namespace game {

/* state blocks: [rho C S][rho theta_v S][theta_v' S][Pi' S][w (L+1) Nc][u L Ne],
 * the prefix of a State mirror (C constituents) */
long long adj_block_len(Context *c);
/* forward window from init->dev over n_steps; aux_* are the lagged fields of
 * the previous step (device vector layout; read only when p.first_step is 0),
 * fv_bounds the vertical mass flux at levels 0 and L ([L+1][Nc]), aux_sed
 * (moist build, always read) the sedimentation heat the first substage
 * reads ([L][Nc]); the end state is written to final_out->dev when given */
int adj_window_forward(Context *c, StateMirror *init, const StepParams &p, int n_steps, const double *aux_P,
                       const double *aux_pvt, const double *aux_v2g, const double *fv_bounds, const double *aux_sed,
                       StateMirror *final_out);
/* tangent-linear of the last forward window: init_dot -> final_dot (blocks) */
int adj_window_tl(Context *c, const double *init_dot, double *final_dot);
/* adjoint of the last forward window: final_bar -> init_bar (blocks) */
int adj_window_backward(Context *c, const double *final_bar, double *init_bar);
/* J = sum_i w_i p_sfc,i^2 of a state (moist: with the vapour's gas constant
 * and temperature) and, when bar_blk is given, dJ/dstate */
int adj_objective(Context *c, StateMirror *s, const double *w_dev, double *J, double *bar_blk);
/* y += x on the device (n doubles) */
void adj_add_into(Context *c, double *y, const double *x, long long n);
/* device buffer of Nc column weights for adj_objective */
double *adj_obj_weights(Context *c);

}  // namespace game
