/* launchers of the single-operator kernels (ops_f64.cu) and of the step */
#pragma once

#include "context.h"

namespace game {

enum { OP_GRAD_H = 1, OP_GRAD_V = 2, OP_GRAD_CON = 4 };
enum { OP_STV_H = 1, OP_STV_V = 2, OP_STV_UPSTREAM = 4 };

void op_grad(Context *c, const double *f, double *vec, int parts);
void op_cov_to_con(Context *c, double *vec);
void op_scalar_times_vector(Context *c, const double *s, const double *vec, double *out, int parts);
void op_divv(Context *c, const double *vec, const double *density, const double *wind, double *out, int tracer);
void op_inner_product(Context *c, const double *a, const double *b, double *out);
void op_rel_vort(Context *c, const double *wind, double *tri, double *curl);
void op_pot_vort(Context *c, const double *rel, const double *rho, double *pv);
void op_vorticity_flux(Context *c, const double *flux, const double *pv, double *out);
void op_mul(Context *c, long long n, const double *a, const double *b, double *out);
void op_add_vertical_divv(Context *c, const double *vec, double *out);
void op_linear_combine(Context *c, StateMirror *a, StateMirror *b, StateMirror *o, double c0, double c1);

int launch_step_f64(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st);
int launch_step_mixed(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st);
/* recomputes the damping table when the damping parameters changed (not
 * inside a stream capture) */
int launch_damping_table(Context *c, const StepParams &p);

const char *last_error();

}  // namespace game
