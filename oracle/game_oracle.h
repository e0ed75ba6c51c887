/*
 * ORACLE -- test infrastructure only.  Never linked into, loaded by or called
 * from the product path (libgame_gb300.so); only tests/, the smoke check and
 * the CPU-baseline arm of bench.py use it, as the checker.
 *
 * A CPU restatement, in plain C99 with run-time grid sizes, of GAME's RKHEVI
 * step (MHBalsmeier/GAME_archived, src/time_stepping/manage_rkhevi.c:20-100)
 * and of every operator it calls.  Each function cites the reference lines it
 * follows and keeps the reference's order of floating-point operations, so
 * that, compiled with -ffp-contract=off, it reproduces the reference's own
 * results bit for bit (pinned by tests/test_oracle_vs_reference.py against the
 * reference compiled from its sources, and by the fixtures in tests/golden/).
 *
 * Arrays use the reference layout: Scalar_field [layer][cell], Vector_field
 * level blocks of (NO_OF_SCALARS_H vertical | NO_OF_VECTORS_H horizontal),
 * Curl_field level blocks of (edges | rhombi), Dual_vector_field level blocks
 * of (edges | triangles).
 */
#ifndef GAME_ORACLE_H
#define GAME_ORACLE_H

typedef struct orc_grid {
    int nc, ne, nt, nl, n_oro, moisture_on, n_const, n_cond;
    double radius;
    const double *normal_distance, *volume, *area, *z_scalar, *z_vector, *gravity_m, *slope;
    const double *theta_v_bg, *exner_bg, *exner_bg_grad, *ipw, *trsk_weights, *rhombi_weights;
    const int *trsk_indices, *trsk_mci, *from, *to, *adj, *adj_sign, *rhombi_idx, *is_land;
    const double *dual_area, *dual_z_vector, *f_vec;
    const int *dual_from, *dual_to, *vort_idx, *vort_sign;
    const double *gravity_potential; /* only the output metrics use it */
    /* diffusion branch */
    const double *layer_thickness, *dual_normal_distance;
    double eff_hor_res, mean_velocity_area;
    /* Held-Suarez forcing */
    const double *latitude_scalar;
    /* output diagnostics (src/io/write_output.c, src/io/spatial_ops_for_output.c) */
    const double *direction, *roughness_length, *sfc_albedo, *latlon_weights;
    const int *latlon_indices;
    long n_latlon;
} orc_grid;

typedef struct orc_state {
    double *rho, *rhotheta_v, *theta_v_pert, *exner_pert, *wind;
} orc_state;

/* pointers into one Diagnostics struct laid out as the reference's: the
 * diffusion branch reproduces out-of-range accesses of the reference that land
 * in the members following n_squared and vector_field_placeholder */
typedef struct orc_diag {
    double *flux_density, *flux_density_divv, *rel_vort_on_triangles, *rel_vort, *pot_vort;
    double *temperature, *v_squared, *scalar_field_placeholder;
    /* diffusion branch */
    double *wind_divv, *curl_of_vorticity, *vector_field_placeholder, *n_squared, *dv_hdz;
    /* output diagnostics */
    double *u_at_edge, *v_at_edge, *u_at_cell, *v_at_cell, *monin_obukhov_length, *roughness_velocity;
} orc_diag;

typedef struct orc_forcings {
    double *pgrad_acc_old, *pgrad_nl, *pgrad_l, *pgrad_condensates_v, *v_squared_grad, *pot_vort_tend;
    double *radiation_tendency;
    double *sfc_sw_in, *sfc_lw_out; /* Held-Suarez forcing: written as zero */
} orc_forcings;

typedef struct orc_irrev {
    double *temperature_diffusion_heating, *friction_acc, *heating_diss, *pressure_gradient_decel_factor;
    double *condensates_sediment_heat, *mass_diff_tendency, *phase_trans_rates, *phase_trans_heating_rate;
    /* diffusion branch */
    double *molecular_diffusion_coeff, *mass_diffusion_coeff_numerical_h, *mass_diffusion_coeff_numerical_v;
    double *temp_diffusion_coeff_numerical_h, *temp_diffusion_coeff_numerical_v, *viscosity, *viscosity_rhombi;
    double *viscosity_triangles, *vert_hor_viscosity, *tke;
} orc_irrev;

typedef struct orc_config {
    int totally_first_step_bool, temperature_diff_h, temperature_diff_v, momentum_diff_h, momentum_diff_v;
    int mass_diff_h, mass_diff_v, rad_on, prog_soil_temp, sfc_phase_trans, sfc_sensible_heat_flux;
    int rad_update, time_to_next_analysis, pbl_scheme, total_run_span;
    double damping_start_height_over_toa, damping_coeff_max, impl_thermo_weight;
    double cloud_droplets_velocity, rain_velocity, snow_velocity, radiation_delta_t;
} orc_config;

/* operators (same argument meaning as the reference functions) */
int orc_grad_hor_cov(const orc_grid *g, const double *in, double *out);
int orc_grad_vert_cov(const orc_grid *g, const double *in, double *out);
int orc_grad_cov(const orc_grid *g, const double *in, double *out);
int orc_grad(const orc_grid *g, const double *in, double *out);
int orc_grad_hor(const orc_grid *g, const double *in, double *out);
int orc_vector_field_hor_cov_to_con(const orc_grid *g, double *f);
int orc_divv_h(const orc_grid *g, const double *in, double *out);
int orc_divv_h_tracer(const orc_grid *g, const double *in, const double *density, const double *wind, double *out);
int orc_scalar_times_vector(const orc_grid *g, const double *s, const double *v, double *out);
int orc_scalar_times_vector_h(const orc_grid *g, const double *s, const double *v, double *out);
int orc_scalar_times_vector_h_upstream(const orc_grid *g, const double *s, const double *v, double *out);
int orc_scalar_times_vector_v(const orc_grid *g, const double *s, const double *v, double *out);
int orc_inner_product(const orc_grid *g, const double *a, const double *b, double *out);
int orc_calc_rel_vort_on_triangles(const orc_grid *g, const double *wind, double *out);
int orc_calc_rel_vort(const orc_grid *g, const double *wind, orc_diag *d);
int orc_add_f_to_rel_vort(const orc_grid *g, const double *rel, double *out);
int orc_calc_pot_vort(const orc_grid *g, const double *wind, const double *density, orc_diag *d);
int orc_vorticity_flux(const orc_grid *g, const double *flux, const double *pot_vort, double *out);
int orc_linear_combine_two_states(const orc_grid *g, const orc_state *s0, const orc_state *s1, orc_state *out,
                                  double c0, double c1);
int orc_temperature_diagnostics(const orc_grid *g, const orc_state *s, orc_diag *d);
int orc_calc_h2otracers_source_rates(const orc_grid *g, const orc_state *s, orc_diag *d, const orc_config *c,
                                     orc_irrev *ir, double dt);
int orc_manage_pressure_gradient(const orc_grid *g, const orc_state *s, orc_diag *d, orc_forcings *f,
                                 orc_irrev *ir, const orc_config *c);
int orc_calc_pressure_grad_condensates_v(const orc_grid *g, const orc_state *s, orc_forcings *f, orc_irrev *ir);
/* diffusion branch (src/subgrid_scale, src/spatial_operators/momentum_diff_diss.c) */
int orc_add_vertical_divv(const orc_grid *g, const double *in, double *out);
int orc_update_n_squared(const orc_grid *g, const orc_state *s, orc_diag *d);
int orc_tke_update(const orc_grid *g, orc_irrev *ir, double dt, const orc_state *s, orc_diag *d);
int orc_hor_viscosity(const orc_grid *g, const orc_state *s, orc_irrev *ir, const orc_diag *d);
int orc_hor_momentum_diffusion(const orc_grid *g, const orc_state *s, orc_diag *d, orc_irrev *ir);
int orc_vert_momentum_diffusion(const orc_grid *g, const orc_state *s, orc_diag *d, orc_irrev *ir);
int orc_simple_dissipation_rate(const orc_grid *g, const orc_state *s, orc_irrev *ir);
int orc_scalar_diffusion_coeffs(const orc_grid *g, const orc_state *s, const orc_config *c, orc_irrev *ir,
                                orc_diag *d);
/* Held-Suarez forcing (src/radiation/held_suar.c, planetary_boundary_layer.c) */
int orc_held_suarez_radiation(const orc_grid *g, const orc_state *s, const orc_diag *d, orc_forcings *f);
int orc_pbl_held_suarez(const orc_grid *g, const orc_state *s, const orc_diag *d, orc_irrev *ir);
int orc_vector_tendencies_expl(const orc_grid *g, const orc_state *s, orc_state *tend, orc_diag *d,
                               orc_forcings *f, orc_irrev *ir, const orc_config *c, int rk_step, double dt);
int orc_scalar_tendencies_expl(const orc_grid *g, const orc_state *s_old, const orc_state *s, orc_state *tend,
                               double dt, orc_diag *d, orc_forcings *f, orc_irrev *ir, const orc_config *c,
                               int rk_step);
int orc_three_band_solver_ver_waves(const orc_grid *g, const orc_state *s_old, orc_state *s_new,
                                    const orc_state *tend, const orc_config *c, double dt, int rk_step);
int orc_three_band_solver_gen_densities(const orc_grid *g, const orc_state *s_old, orc_state *s_new,
                                        const orc_state *tend, const orc_diag *d, orc_irrev *ir,
                                        const orc_config *c, double dt, int rk_step);
int orc_manage_rkhevi(const orc_grid *g, const orc_state *s_old, orc_state *s_new, orc_state *tend,
                      orc_diag *d, orc_forcings *f, orc_irrev *ir, const orc_config *c, double dt, double t);

/* output metrics (src/io/write_output.c:105-121, 1515-1668) */
double orc_global_scalar_integrator(const orc_grid *g, const double *field);
/* mslp may be NULL */
int orc_surface_pressure(const orc_grid *g, const orc_state *s, const double *temperature, double *p_sfc,
                         double *mslp);

/* output diagnostics: the operators only output uses (src/io/io.h:14-16,
 * src/spatial_operators/spatial_operators.h:27-30) */
int orc_calc_uv_at_edge(const orc_grid *g, const double *in, double *u, double *v);
int orc_curl_field_to_cells(const orc_grid *g, const double *in, double *out);
int orc_edges_to_cells(const orc_grid *g, const double *in, double *out);
int orc_edges_to_cells_lowest_layer(const orc_grid *g, const double *in, double *out);
int orc_inner_product_tangential(const orc_grid *g, const double *in0, const double *in1, double *out);
/* writes state->theta_v_pert of the top layer back as (x + bg) - bg, as the
 * reference does */
int orc_epv_diagnostics(const orc_grid *g, const double *pot_vort, orc_state *s, double *epv);
int orc_interpolate_to_ll(const orc_grid *g, const double *in, double *out);

/* the fields write_out computes (src/io/write_output.c:51-1513), without the
 * writers */
#define ORC_N_PRESSURE_LEVELS 6
typedef struct orc_output {
    /* surface, [Nc] each (write_output.c:90-351) */
    double *mslp, *surface_p, *t2, *tcdc, *rprate, *sprate, *cape, *sfc_sw_down, *u10, *v10, *gusts;
    /* model layers, [S] each (:718-749) */
    double *pressure, *rh, *rel_vort, *divv_h, *epv;
    /* pressure levels, [Nc][6] each (:751-826) */
    double *geopotential_height, *t_pl, *rh_pl, *epv_pl, *u_pl, *v_pl, *rel_vort_pl;
} orc_output;
int orc_write_out_fields(const orc_grid *g, orc_state *s, const double *temperature_soil, const double *wind_lowest,
                         int n_wind_steps, orc_diag *d, const double *sfc_sw_in, const orc_config *c, orc_output *o);

#endif
