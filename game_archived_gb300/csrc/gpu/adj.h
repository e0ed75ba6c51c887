/* adjoint and tangent-linear windows of the dry RKHEVI step (adj_f64.cu) */
#pragma once

#include "context.h"

namespace game {

/* state blocks: [rho S][rho theta_v S][theta_v' S][Pi' S][w (L+1) Nc][u L Ne],
 * the prefix of a dry State mirror */
long long adj_block_len(Context *c);
/* forward window from init->dev over n_steps; aux_* are the lagged fields of
 * the previous step (device vector layout; read only when p.first_step is 0),
 * fv_bounds the vertical mass flux at levels 0 and L ([L+1][Nc]); the end
 * state is written to final_out->dev when final_out is given */
int adj_window_forward(Context *c, StateMirror *init, const StepParams &p, int n_steps, const double *aux_P,
                       const double *aux_pvt, const double *aux_v2g, const double *fv_bounds, StateMirror *final_out);
/* tangent-linear of the last forward window: init_dot -> final_dot (blocks) */
int adj_window_tl(Context *c, const double *init_dot, double *final_dot);
/* adjoint of the last forward window: final_bar -> init_bar (blocks) */
int adj_window_backward(Context *c, const double *final_bar, double *init_bar);
/* J = sum_i w_i p_sfc,i^2 of a dry state and, when bar_blk is given, dJ/dstate */
int adj_objective(Context *c, StateMirror *s, const double *w_dev, double *J, double *bar_blk);
/* y += x on the device (n doubles) */
void adj_add_into(Context *c, double *y, const double *x, long long n);
/* device buffer of Nc column weights for adj_objective */
double *adj_obj_weights(Context *c);

}  // namespace game
