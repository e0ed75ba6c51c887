/* the sub-steps of manage_rkhevi on device buffers (substeps_f64.cu) */
#pragma once

#include "context.h"

namespace game {

/* manage_pressure_gradient: p_nl, p_l hold the previous nonlinear / linear
 * gradients on entry (pgrad_acc_old is formed from them unless this is the
 * first step) and the new ones on return; decel = rho_gas / rho_total */
void sub_pressure_gradient(Context *c, const StepParams &p, StateMirror *s, double *p_nl, double *p_l, double *pg_old,
                           double *decel);
/* calc_pressure_grad_condensates_v: decel = rho_gas / rho_total - 1 and the
 * vertical condensate term at the inner interfaces of cond_v */
void sub_condensates_v(Context *c, StateMirror *s, double *decel, double *cond_v);
/* the tendency assembly of vector_tendencies_expl */
void sub_vector_tendency(Context *c, const StepParams &p, int rk, double *tend_wind, const double *pg_old,
                         const double *p_nl, const double *p_l, const double *pvt, const double *v2g,
                         const double *friction, const double *cond_v);
void sub_cp_tables(Context *c, const double *temperature, double *cp_ice, double *cp_water);
void sub_scalar_tendencies(Context *c, const StepParams &p, StateMirror *sn, StateMirror *st, int rk, double *theta,
                           const double *cp_ice, const double *cp_water, const double *pt_rates,
                           const double *pt_heat, const double *sed_heat);
int sub_ver_waves(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st, int rk);
void sub_gen_densities(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st, int rk,
                       const double *temperature, const double *cp_ice, const double *cp_water, double *sed_heat);

}  // namespace game
