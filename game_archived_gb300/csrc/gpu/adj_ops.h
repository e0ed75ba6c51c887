/* adjoints of the single operators on device-layout fields (adj_ops_f64.cu)
 * and of the sound-wave column solver (adj_f64.cu); bars of a forward's
 * inputs are accumulated */
#pragma once

#include "context.h"

namespace game {

void op_grad_adj(Context *c, const double *out_b, double *in_b);
void op_divv_adj(Context *c, const double *out_b, double *in_b);
void op_stv_adj(Context *c, const double *s, const double *v, const double *out_b, double *s_b, double *v_b);
void op_inner_adj(Context *c, const double *a, const double *b, const double *out_b, double *a_b, double *b_b);
void op_vflux_adj(Context *c, const double *flux, const double *pv, const double *out_b, double *flux_b, double *pv_b);
/* divv_h_tracer: bars of the flux field (horizontal part), the density and
 * the wind (horizontal part, through the terrain correction) */
void op_divv_tracer_adj(Context *c, const double *density, const double *wind, const double *out_b, double *in_b,
                        double *dens_b, double *wind_b);
/* pv is the forward's potential vorticity; zero_u a zeroed [L][Ne] buffer;
 * tri_b a zeroed [L][Nt] work buffer */
void op_pot_vort_adj(Context *c, const double *wind, const double *rho, const double *pv, const double *pv_b,
                     const double *zero_u, double *wind_b, double *rho_b, double *tri_b);
/* three_band_solver_gen_densities: sn_b holds the bar of the solver's output
 * on entry (the tracers' new densities, zeroed on return); so_b (tracer
 * densities, w), st_b (tracer densities), sn_b (w) and t_b (temperature) are
 * accumulated; sed_b, the bar of the sedimentation heat, is read and zeroed
 * at rk 0.  Layer counts up to 256. */
int adj_gen_densities(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st,
                      const double *temperature, int rk, double *sed_b, StateMirror *so_b, StateMirror *sn_b,
                      StateMirror *st_b, double *t_b);
/* three_band_solver_ver_waves of the dry build: sn_bar holds the bar of the
 * solver's output state on entry and the bar of its input state on return;
 * so_bar and st_bar (rho, rho theta_v, w) are accumulated */
int adj_waves_backward(Context *c, StateMirror *so, StateMirror *sn, StateMirror *st, const StepParams &p, int rk,
                       StateMirror *so_bar, StateMirror *sn_bar, StateMirror *st_bar);

}  // namespace game
