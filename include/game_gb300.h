/*
 * game_gb300 -- GB300-native RKHEVI dynamical-core step of GAME
 * (MHBalsmeier/GAME_archived) behind the reference's own C entry points.
 *
 * Drop-in boundary.  The functions in section 2 have exactly the names,
 * argument lists and argument meaning of the reference routines they replace;
 * a reference build links this library in place of its
 * src/spatial_operators/*.o and src/time_stepping/*.o.  The reference's
 * array typedefs (Scalar_field, Vector_field, Curl_field, Dual_vector_field)
 * decay to double* in a parameter list and are written as double* here; the
 * struct arguments are the reference's own structs (src/game_types.h:70-238),
 * passed by pointer and never dereferenced by the caller's side of this
 * header.  Their layout depends on the reference's compile-time enums
 * RES_ID, NO_OF_LAYERS and MOISTURE_ON, which the caller hands to
 * game_gpu_init once; the library computes every member offset at run time.
 *
 * Return values: 0 on success, nonzero on a CUDA or validation error
 * (game_gpu_last_error() describes it).  The reference returns 0 and calls
 * exit(1) on errors; this library never exits the process.
 *
 * Residency.  By default (resident = 0) every call reads its inputs from host
 * memory and writes its results back to host memory before returning, as the
 * reference does.  With game_gpu_set_resident(1), manage_rkhevi and
 * linear_combine_two_states work on device mirrors of the State structs and
 * touch host memory only through game_gpu_sync_to_device/_to_host.  The
 * per-operator entry points (grad, divv_h, ...) always work host-in/host-out:
 * the reference calls them on host arrays outside the time step.
 *
 * Threading: one context per process, not re-entrant; calls are synchronous.
 */
#ifndef GAME_GB300_H
#define GAME_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

struct grid;
struct dualgrid;
struct state;
struct diagnostics;
struct forcings;
struct irreversible_quantities;
struct config;
struct config_io;

/* ------------------------------------------------------------------------
 * 1. library control (no counterpart in the reference)
 * ---------------------------------------------------------------------- */
enum { GAME_GPU_FP64 = 0, GAME_GPU_MIXED = 1 };

/* Uploads and renumbers the grid tables once, after the reference's
 * set_grid_properties (src/io/set_grid_properties.c:21-255) has filled grid
 * and dualgrid.  res_id, no_of_layers and moisture_on are the reference's
 * RES_ID, NO_OF_LAYERS and MOISTURE_ON (src/game_types.h:12-20). */
int game_gpu_init(int res_id, int no_of_layers, int moisture_on, struct grid *grid, struct dualgrid *dualgrid);
int game_gpu_finalize(void);
/* GAME_GPU_FP64: every operator in FP64 (results equal the reference's to
 * rounding); GAME_GPU_MIXED: horizontal operators in FP32, vertical solves,
 * density and mass-flux accumulation in FP64.  Set before the first step. */
int game_gpu_set_precision(int precision);
int game_gpu_set_resident(int resident);
int game_gpu_set_graphs(int on);
/* the vertical column solvers (any layer count up to 256): 0 (default) by
 * layer count, batch size and precision -- per-thread Thomas sweeps (the
 * reference's elimination order, column_solvers.c:641-669) held in registers
 * for 26 layers and in local memory otherwise, except that the mixed path
 * solves a batch of fewer than 6144 columns (the sound-wave solve: one
 * system per column; the tracer solve: one per constituent and column) of
 * another layer count with the warp-cooperative parallel cyclic reduction;
 * 1 per-thread Thomas sweeps; 2 warp cyclic reduction in both precisions (a
 * different elimination order: the FP64 results move by rounding) */
int game_gpu_set_column_solver(int mode);
/* arithmetic of the mixed path's vertical eliminations (the sound-wave and
 * tracer column solves, column_solvers.c): 1 (default) double-float, two
 * FP32 numbers per value carrying 48 significand bits, which runs on the
 * FP32 pipe (GB300 executes FP64 at 1/64 of its FP32 rate); 0 FP64.  The
 * state, the tendencies and the mass-flux accumulation stay FP64 either way;
 * the FP64 path never uses double-float. */
int game_gpu_set_double_float(int on);
int game_gpu_sync_to_device(struct state *state);
int game_gpu_sync_to_host(struct state *state);
/* writes the library's copies of the lagged step fields back into the host
 * structs: forcings->pressure_gradient_acc_neg_nl holds the decelerated sum
 * nl + l and pressure_gradient_acc_neg_l holds 0 (their sum, the only form
 * in which the step reads them, is exact); pot_vort_tend, v_squared_grad,
 * diagnostics->temperature, irrev->phase_trans_rates, phase_trans_heating_rate,
 * condensates_sediment_heat. */
int game_gpu_sync_aux_to_host(struct diagnostics *diagnostics, struct forcings *forcings,
                              struct irreversible_quantities *irrev);
int game_gpu_synchronize(void);
const char *game_gpu_last_error(void);
int game_gpu_host_alloc(void **ptr, size_t bytes);
int game_gpu_host_free(void *ptr);
long long game_gpu_kernel_launches(int reset);
/* selects the CUDA device (one process per GPU); call before game_gpu_init */
int game_gpu_set_device(int device);
/* timing on the library's own stream: record event `slot`, elapsed a -> b */
int game_gpu_event_record(int slot);
int game_gpu_event_elapsed(int a, int b, float *ms);
/* per-kernel timing: while on, every step kernel is bracketed by events
 * (CUDA graphs are bypassed); entries are (kernel name, total ms, launches) */
int game_gpu_profile(int on);
int game_gpu_profile_count(void);
int game_gpu_profile_get(int i, const char **name, double *ms, long long *launches);
/* the mixed path's numeric primitives beside the CUDA operations they stand
 * for, over n host values (for tests; no context needed): op 0 / 1 the
 * Newton-refined FP64 reciprocal with 1 / 2 steps, 2 IEEE 1.0 / x, 3 / 4
 * double -> float by integer operations / by the conversion instruction,
 * 5 / 6 float -> double likewise, 7 the double-float split and join of x,
 * 8 the double-float reciprocal, 9 / 10 double-float product / sum of in[i]
 * and in[n + i]; in and out are double arrays except the float side of ops
 * 3 to 6 */
int game_gpu_numerics(int op, const void *in, void *out, long long n);
/* ---- health check and checkpoints (no counterpart in the reference's
 * library interface; see each) ---- */
enum { GAME_GPU_UNHEALTHY = 2 };
struct game_gpu_health {
    long long nonfinite;              /* NaN or +-Inf values anywhere in the State */
    long long negative_density;       /* negative values among the constituent densities */
    long long first_nonfinite;        /* position of the first, in doubles from the start of the State, or -1 */
    long long first_negative_density; /* likewise */
};
/* Counts non-finite values and negative densities of a State on the device
 * (its device copy in resident mode, else the host struct uploaded first).
 * Returns 0 when there are none, GAME_GPU_UNHEALTHY (message in
 * game_gpu_last_error) when there are, -1 on a CUDA error.  The reference
 * aborts on negative densities when it reads a state
 * (src/io/set_initial_state.c:318-328) and clips its tracer solutions at zero
 * (src/time_stepping/column_solvers.c:621-627), so either count being nonzero
 * after a step means the run has broken down. */
int game_gpu_check_state(struct state *state, struct game_gpu_health *report);
/* every > 0: manage_rkhevi checks state_new after every every-th call and
 * returns GAME_GPU_UNHEALTHY if the check fails (the step's results are still
 * written); 0 (default) switches the check off */
int game_gpu_set_health_check(int every);
/* A checkpoint for a bit-identical resume: the State the next step starts
 * from (state_new after a step) with the whole Diagnostics, Forcings,
 * Irreversible_quantities and Config structs, after the library's device
 * copies of the lagged step fields are written back into them.  The
 * reference's restart reads a State only (src/io/set_initial_state.c:244-336)
 * and so starts from recomputed lagged fields; a run resumed from this
 * checkpoint -- read into the host structs by game_gpu_read_checkpoint, in
 * this process or in a new one with the same grid -- continues the
 * uninterrupted run bit for bit.  read_checkpoint refuses a file written for
 * another RES_ID, layer count or moisture build, or whose digest does not
 * match; in resident mode it also uploads the State. */
int game_gpu_write_checkpoint(const char *path, struct state *state, struct diagnostics *diagnostics,
                              struct forcings *forcings, struct irreversible_quantities *irrev, struct config *config);
int game_gpu_read_checkpoint(const char *path, struct state *state, struct diagnostics *diagnostics,
                             struct forcings *forcings, struct irreversible_quantities *irrev, struct config *config);

/* bytes copied host->device and device->host by the library */
int game_gpu_transfer_bytes(long long *h2d, long long *d2h, int reset);

/* ------------------------------------------------------------------------
 * 2. drop-in entry points (reference signatures)
 * ---------------------------------------------------------------------- */
/* src/time_stepping/time_stepping.h:6 -> src/time_stepping/manage_rkhevi.c:20 */
int manage_rkhevi(struct state *state_old, struct state *state_new, struct grid *grid, struct dualgrid *dualgrid,
                  struct state *state_tendency, struct diagnostics *diagnostics, struct forcings *forcings,
                  struct irreversible_quantities *irrev, struct config *config, double delta_t,
                  double time_coordinate);
/* src/spatial_operators/spatial_operators.h:24 -> linear_combine_two_states.c:14 */
int linear_combine_two_states(struct state *state_0, struct state *state_1, struct state *state_out,
                              double coeff_0, double coeff_1, struct grid *grid);

/* The sub-steps of manage_rkhevi (time_stepping.h:7-12), for drivers that call
 * them one by one.  FP64, host-in/host-out in every residency mode, on private
 * device buffers (they never touch the device mirrors of a resident run).
 * They write the reference's output members; Diagnostics members the
 * reference uses as scratch (scalar_field_placeholder, flux_density_divv,
 * and flux_density inside scalar_tendencies_expl) are left alone.  Like
 * manage_rkhevi they return an error when a diffusion, radiation, PBL, soil
 * or surface-flux switch is on. */
/* time_stepping.h:7 -> src/time_stepping/manage_pressure_gradient.c:17 */
int manage_pressure_gradient(struct state *state, struct grid *grid, struct dualgrid *dualgrid,
                             struct diagnostics *diagnostics, struct forcings *forcings,
                             struct irreversible_quantities *irrev, struct config *config);
/* time_stepping.h:8 -> manage_pressure_gradient.c:74 */
int calc_pressure_grad_condensates_v(struct state *state, struct grid *grid, struct forcings *forcings,
                                     struct irreversible_quantities *irrev);
/* time_stepping.h:9 -> src/time_stepping/vector_tendencies_expl.c:18 */
int vector_tendencies_expl(struct state *state, struct state *state_tendency, struct grid *grid,
                           struct dualgrid *dualgrid, struct diagnostics *diagnostics, struct forcings *forcings,
                           struct irreversible_quantities *irrev, struct config *config, int rk_step, double delta_t);
/* time_stepping.h:10 -> src/time_stepping/scalar_tendencies_expl.c:17 */
int scalar_tendencies_expl(struct state *state_old, struct state *state, struct state *state_tendency,
                           struct grid *grid, struct dualgrid *dualgrid, double delta_t,
                           struct diagnostics *diagnostics, struct forcings *forcings,
                           struct irreversible_quantities *irrev, struct config *config, int rk_step);
/* time_stepping.h:11 -> src/time_stepping/column_solvers.c:19 */
int three_band_solver_ver_waves(struct state *state_old, struct state *state_new, struct state *state_tendency,
                                struct diagnostics *diagnostics, struct forcings *forcings, struct config *config,
                                double delta_t, struct grid *grid, int rk_step);
/* time_stepping.h:12 -> column_solvers.c:385 */
int three_band_solver_gen_densities(struct state *state_old, struct state *state_new, struct state *state_tendency,
                                    struct diagnostics *diagnostics, struct irreversible_quantities *irrev,
                                    struct config *config, double delta_t, int rk_step, struct grid *grid);
/* spatial_operators.h:6-11 -> gradient_operators.c:14,35,56,66,76 */
int grad_hor_cov(double *in_field, double *out_field, struct grid *grid);
int grad_vert_cov(double *in_field, double *out_field, struct grid *grid);
int vector_field_hor_cov_to_con(double *cov_to_con_field, struct grid *grid);
int grad_cov(double *in_field, double *out_field, struct grid *grid);
int grad(double *in_field, double *out_field, struct grid *grid);
int grad_hor(double *in_field, double *out_field, struct grid *grid);
/* spatial_operators.h:12-14 -> vorticities.c:18,87,104 */
int calc_pot_vort(double *velocity_field, double *density_field, struct diagnostics *diagnostics, struct grid *grid,
                  struct dualgrid *dualgrid);
int add_f_to_rel_vort(double *rel_vort, double *out_field, struct dualgrid *dualgrid);
int calc_rel_vort(double *velocity_field, struct diagnostics *diagnostics, struct grid *grid,
                  struct dualgrid *dualgrid);
/* spatial_operators.h:15 -> vorticity_flux.c:16 (pot_vorticity is a Curl_field) */
int vorticity_flux(double *mass_flux_density, double *pot_vorticity, double *out_field, struct grid *grid,
                   struct dualgrid *dualgrid);
/* spatial_operators.h:16-17 -> divergences.c:14,66 */
int divv_h(double *in_field, double *out_field, struct grid *grid);
int divv_h_tracer(double *in_field, double *density_field, double *wind_field, double *out_field, struct grid *grid);
/* spatial_operators.h:20-23 -> multiplications.c:35,45,68,98 */
int scalar_times_vector(double *scalar_field, double *vector_field, double *out_field, struct grid *grid);
int scalar_times_vector_h(double *in_field_h, double *vector_field, double *out_field, struct grid *grid);
int scalar_times_vector_h_upstream(double *in_field_h, double *vector_field, double *out_field, struct grid *grid);
int scalar_times_vector_v(double *in_field_v, double *vector_field, double *out_field, struct grid *grid);
/* spatial_operators.h:25 -> inner_product.c:13 */
int inner_product(double *in_field_0, double *in_field_1, double *out_field, struct grid *grid);
/* spatial_operators.h:19,24 -> multiplications.c:15,25: pointwise products of
 * two Scalar_fields / Vector_fields */
int scalar_times_scalar(double *in_field_0, double *in_field_1, double *out_field);
int vector_times_vector(double *in_field_0, double *in_field_1, double *out_field);
/* spatial_operators.h:18 -> divergences.c:150: adds the divergence of the
 * vertical part of in_field to out_field */
int add_vertical_divv(double *in_field, double *out_field, struct grid *grid);
/* Not exported: the per-point helpers tangential_wind,
 * vertical_contravariant_corr, remap_verpri2horpri_vector and
 * horizontal_covariant (spatial_operators.h:27-31), which only the operators
 * this library replaces call, and the diffusion sub-steps
 * hor_momentum_diffusion, vert_momentum_diffusion and simple_dissipation_rate
 * (:34-36), which run inside manage_rkhevi. */

/* ---- 3. integrals and surface pressure (the model's monitoring output) ---- */

/* src/io/write_output.c:28 -> :1659-1668: sum of density_gen * volume over all
 * grid boxes.  Summed on the device with compensated (double-word)
 * accumulation of the exact products, so the result is the exact sum
 * rounded once, where the reference's serial loop carries up to
 * NO_OF_SCALARS roundings.  Returns NaN on error (game_gpu_last_error). */
double global_scalar_integrator(double *density_gen, struct grid *grid);

/* The values write_out_integral (src/io/write_output.c:1515-1596) appends to
 * its files, without the file: integral_id 0 -> result[NO_OF_CONSTITUENTS],
 * the mass of every constituent; 1 -> result[0], the integral of
 * rho*theta_v; 2 -> result[0..2] = 0.5 * kinetic, potential and
 * C_D_V * internal energy of the gas phase.  The temperature of id 2 is the
 * one the reference's diagnostics hold at that point: T(state_old) of the
 * last manage_rkhevi call, or T(state) before the first step
 * (coordinator.c:250 and :280-284).  Reads the device mirror in resident
 * mode, else uploads state first.  No counterpart function in the reference
 * (write_out_integral also writes files). */
int game_gpu_write_out_integral(struct state *state, int integral_id, double *result);

/* Surface pressure and mean-sea-level pressure of every column
 * (src/io/write_output.c:105-121, with temperature_diagnostics of state as
 * write_out computes it at :83): surface_p[NO_OF_SCALARS_H] and, when mslp
 * is not NULL, mslp[NO_OF_SCALARS_H], in the reference's column order.
 * No counterpart function in the reference (the loop is inside write_out). */
int game_gpu_surface_pressure(struct state *state, double *surface_p, double *mslp);

/* ---- 4. adjoint and tangent-linear models of the step ----
 *
 * A window of n_steps RKHEVI steps, with hand-written adjoint kernels for
 * every operator of the step (pressure gradient, vorticities, vorticity
 * flux, kinetic energy and its gradient, momentum tendencies, flux
 * divergences, the sound-wave rows, the tridiagonal solve and its
 * back-substitution; on the moist build also the temperature and phase
 * transitions of every step, the moist scalar tendencies, the tracer column
 * solve with its sedimentation heat and the condensate terms of the
 * momentum).  No counterpart in the reference.
 *
 * The forward of record runs in the library's precision
 * (game_gpu_set_precision): GAME_GPU_FP64, the FP64 step; GAME_GPU_MIXED,
 * the fused mixed step itself, so that state_final is what a mixed run
 * produces.  The tangent-linear and adjoint models are FP64 in both cases,
 * linearised about the forward's checkpointed trajectory.  A mixed window
 * leaves the lagged step fields of a device-resident run as it found them.
 *
 * rkhevi_window_forward runs the window from state_init as the reference's
 * time loop would (src/coordinator.c:302-324: each step starts with
 * linear_combine_two_states(new -> old) and calls manage_rkhevi), stores one
 * checkpoint per step on the device and writes the end state to state_final.
 * With config->totally_first_step_bool = 1 the window depends on state_init
 * only; otherwise the lagged fields of forcings (pressure gradient, vorticity
 * flux, kinetic-energy gradient) and the flux_density boundary values of
 * diagnostics enter as fixed inputs.  The control variables are rho,
 * rhotheta_v, exner_pert and wind of state_init; theta_v_pert is rediagnosed
 * from rhotheta_v / rho at every step start, so its derivative is 0.
 *
 * rkhevi_window_tl: the tangent-linear model of the last forward window,
 * d(state_final) for a perturbation state_init_dot (State structs holding
 * perturbations).  rkhevi_window_backward: its adjoint, the gradient with
 * respect to state_init of <state_final_bar, state_final> (State structs
 * holding bars); each step is recomputed from its checkpoint, keeping both
 * RK stage states, then differentiated in reverse.
 *
 * game_gpu_sfc_pressure_objective: J = sum_i weights[i] p_sfc,i^2 over the
 * columns (surface pressure of src/io/write_output.c:105-121, reference
 * column order) and, when state_bar is not NULL, dJ/dstate written to
 * state_bar (nonzero on the lowest layer's rho, theta_v_pert, exner_pert;
 * moist build: the gas constant of the moist air and the temperature of
 * temperature_diagnostics, so also the vapour density).
 *
 * The dry build and the moist build of six constituents; the diffusion
 * switches and the Held-Suarez forcing must be off (an error otherwise). */
/* Adjoints of the single operators, the reverse half of each forward/backward
 * pair.  Host arrays in the reference layouts of the forward call.  Bars of
 * the forward's inputs are accumulated (in_bar += (d out / d in)^T out_bar),
 * the bar of its output is read; operators that are not linear also take the
 * forward's inputs, the point of linearisation.  Entries of an output the
 * forward does not write (the TOA and surface w of grad and
 * scalar_times_vector) carry no bar.  No counterpart in the reference. */
/* gradient_operators.c:66 (grad) */
int grad_adj(double *out_field_bar, double *in_field_bar, struct grid *grid);
/* divergences.c:14 (divv_h) */
int divv_h_adj(double *out_field_bar, double *in_field_bar, struct grid *grid);
/* divergences.c:66 (divv_h_tracer): bars of the flux field (its horizontal
 * part), of the density and of the wind (its horizontal part, which enters
 * through the terrain-following correction in the orography layers); the
 * upstream density pick is held fixed */
int divv_h_tracer_adj(double *in_field, double *density_field, double *wind_field, double *out_field_bar,
                      double *in_field_bar, double *density_field_bar, double *wind_field_bar, struct grid *grid);
/* multiplications.c:35 (scalar_times_vector) */
int scalar_times_vector_adj(double *scalar_field, double *vector_field, double *out_field_bar,
                            double *scalar_field_bar, double *vector_field_bar, struct grid *grid);
/* inner_product.c:13 (inner_product; with both inputs the wind it is the kinetic energy) */
int inner_product_adj(double *in_field_0, double *in_field_1, double *out_field_bar, double *in_field_0_bar,
                      double *in_field_1_bar, struct grid *grid);
/* vorticities.c:18 (calc_pot_vort): bar of diagnostics->pot_vort (curl layout) */
int calc_pot_vort_adj(double *velocity_field, double *density_field, double *pot_vort_bar,
                      double *velocity_field_bar, double *density_field_bar, struct grid *grid,
                      struct dualgrid *dualgrid);
/* vorticity_flux.c:16 (vorticity_flux) */
int vorticity_flux_adj(double *mass_flux_density, double *pot_vorticity, double *out_field_bar,
                       double *mass_flux_density_bar, double *pot_vorticity_bar, struct grid *grid,
                       struct dualgrid *dualgrid);
/* column_solvers.c:19 (three_band_solver_ver_waves, dry build): the adjoint
 * of the column solve with its tridiagonal elimination.  state_new_bar holds
 * on entry the bar of the state_new the forward returns and on return the bar
 * of the state_new it receives (fields the solver does not write pass their
 * bars through); state_old_bar and state_tendency_bar are accumulated. */
int three_band_solver_ver_waves_adj(struct state *state_old, struct state *state_new, struct state *state_tendency,
                                    struct diagnostics *diagnostics, struct forcings *forcings, struct config *config,
                                    double delta_t, struct grid *grid, int rk_step, struct state *state_old_bar,
                                    struct state *state_new_bar, struct state *state_tendency_bar);
/* column_solvers.c:385 (three_band_solver_gen_densities, moist build): the
 * adjoint of the tracers' implicit vertical advection and sedimentation with
 * its tridiagonal elimination.  state_new_bar holds on entry the bar of the
 * new tracer densities the forward writes (zero on return: the forward
 * overwrites them) and accumulates the bar of the new vertical wind;
 * state_old_bar (tracer densities, vertical wind), state_tendency_bar
 * (tracer densities) and diagnostics_bar->temperature are accumulated.  At
 * rk_step 0 irrev_bar->condensates_sediment_heat is read as the bar of the
 * sedimentation heat the forward writes and zeroed.  Upwind picks and
 * flux-sign branches are held fixed; clipped (negative) solutions carry no
 * derivative.  Up to 256 layers. */
int three_band_solver_gen_densities_adj(struct state *state_old, struct state *state_new,
                                        struct state *state_tendency, struct diagnostics *diagnostics,
                                        struct irreversible_quantities *irrev, struct config *config, double delta_t,
                                        int rk_step, struct grid *grid, struct state *state_old_bar,
                                        struct state *state_new_bar, struct state *state_tendency_bar,
                                        struct diagnostics *diagnostics_bar,
                                        struct irreversible_quantities *irrev_bar);

/* time_stepping.h:6 (manage_rkhevi, dry build): the adjoint of one step,
 * the reference's arguments followed by the bars.  state_new_bar is the bar
 * of the state_new the step returns; state_old_bar receives the bar of
 * state_old (written, not accumulated).  As in the reference's time loop
 * (src/coordinator.c:305), state_new equals state_old on entry, so the step
 * is a function of state_old alone; the lagged fields of forcings (the
 * previous step's pressure gradient, vorticity flux and kinetic-energy
 * gradient) are constants of the call unless config->totally_first_step_bool
 * is set.  Equal to a one-step window (rkhevi_window_forward with n_steps =
 * 1, then rkhevi_window_backward), which it replaces for a caller that
 * differentiates one step at a time. */
int manage_rkhevi_adj(struct state *state_old, struct state *state_new, struct grid *grid, struct dualgrid *dualgrid,
                      struct state *state_tendency, struct diagnostics *diagnostics, struct forcings *forcings,
                      struct irreversible_quantities *irrev, struct config *config, double delta_t,
                      double time_coordinate, struct state *state_new_bar, struct state *state_old_bar);
int rkhevi_window_forward(struct state *state_init, struct state *state_final, struct grid *grid,
                          struct dualgrid *dualgrid, struct diagnostics *diagnostics, struct forcings *forcings,
                          struct irreversible_quantities *irrev, struct config *config, double delta_t, int n_steps);
int rkhevi_window_tl(struct state *state_init_dot, struct state *state_final_dot);
/* checkpoints of the windows that follow: every-th step start (default 1:
 * all) and the window's end are stored; the backward sweep recomputes any
 * other step start in FP64 from the checkpoint before it (every - 1 extra
 * steps at most per backward step), and the tangent-linear model
 * re-linearises only at stored starts, so the two stay exact transposes.
 * Device memory of the checkpoints falls by about that factor. */
int game_gpu_set_checkpoint_stride(int every);
int rkhevi_window_backward(struct state *state_final_bar, struct state *state_init_bar);
int game_gpu_sfc_pressure_objective(struct state *state, const double *weights, double *objective,
                                    struct state *state_bar);

/* ---- 5. the weighted-sum reduction without any allocation ---- */

/* sums[k] = sum over i < n of fields[k*n + i] * weights[i], for k < n_fields,
 * with the compensated accumulation of global_scalar_integrator.  All four
 * arrays are DEVICE pointers; sums is written on the device in stream order
 * (stream: a cudaStream_t, NULL for the default stream), and the call returns
 * without waiting for it.  No game_gpu_init is needed.
 *
 * Allocates nothing: no cudaMalloc, no cudaFree, no library routine that
 * allocates.  Its scratch is a fixed 77,856-byte device array inside the
 * library, which limits n_fields to 1..8 (larger counts are rejected with an
 * error); n is unlimited.  For callers that cannot allocate device memory at
 * the point of the call: hosts that keep several streams busy and cannot take
 * the device-wide synchronisation of cudaMalloc/cudaFree, and hosts that have
 * given all device memory to their own pool.
 *
 * The first call on each device (with that device current) looks up the
 * scratch array's device address and keeps it; make it before any stream
 * capture begins, and do not call this entry point on a device reset
 * (cudaDeviceReset) since its first call.  The scratch's counters start at
 * zero when the device code loads and every call leaves them at zero, so the
 * host never clears them.  Calls on one device share the scratch: calls whose
 * kernels may overlap (different streams without ordering, several host
 * threads) race and return wrong sums; keep them in one stream.
 *
 * No counterpart in the reference. */
int game_gpu_weighted_sums_noalloc(const double *fields, int n_fields, long long n, const double *weights,
                                   double *sums, void *stream);

/* ---- 6. output diagnostics ----
 *
 * The operators only the reference's output code uses, with its signatures
 * (host-in/host-out, like section 2's operators): */
/* src/io/io.h:15 -> src/io/spatial_ops_for_output.c:168: one [NO_OF_SCALARS_H]
 * field to the [NO_OF_LATLON_IO_POINTS] lat-lon grid with the grid's
 * latlon_interpol_indices / _weights */
int interpolate_to_ll(double in_field[], double out_field[], struct grid *grid);
/* io.h:16 -> spatial_ops_for_output.c:199: [NO_OF_VECTORS_H] -> [NO_OF_SCALARS_H] */
int edges_to_cells_lowest_layer(double in_field[], double out_field[], struct grid *grid);
/* io.h:14 -> spatial_ops_for_output.c:17: Ertel's potential vorticity from
 * the Curl_field pot_vort (as calc_pot_vort leaves it); also writes state's
 * theta_v_pert of the top layer back as (x + theta_v_bg) - theta_v_bg, as the
 * reference does */
int epv_diagnostics(double *pot_vort, struct state *state, double *epv, struct grid *grid,
                    struct dualgrid *dualgrid);
/* spatial_ops_for_output.c:137 (declared in that file) */
int inner_product_tangential(double *in_field_0, double *in_field_1, double *out_field, struct grid *grid,
                             struct dualgrid *dualgrid);
/* src/spatial_operators/spatial_operators.h:27-30 -> averaging.c:152,176,206:
 * calc_uv_at_edge writes the horizontal entries of out_field_u/_v only */
int calc_uv_at_edge(double *in_field, double *out_field_u, double *out_field_v, struct grid *grid);
int curl_field_to_cells(double *in_field, double *out_field, struct grid *grid);
int edges_to_cells(double *in_field, double *out_field, struct grid *grid);

/* The fields write_out (src/io/write_output.c:51-1513) computes for its
 * surface, pressure-level and model-level files, without the writers: the
 * caller passes them to its netCDF / GRIB code.  Every pointer may be NULL
 * (field not wanted).  Native-grid layout (argument native):
 *   surface fields            [NO_OF_SCALARS_H]
 *   model layers              [NO_OF_SCALARS] (Scalar_field order)
 *   pressure levels           [NO_OF_SCALARS_H][6], levels 200, 300, 500,
 *                             700, 850, 925 hPa (the reference's arrays)
 *   w                         unused
 * Lat-lon layout (argument latlon), interpolate_to_ll of every horizontal
 * slice, as the GRIB path writes them:
 *   surface fields            [NO_OF_LATLON_IO_POINTS]
 *   model layers              [NO_OF_LAYERS][NO_OF_LATLON_IO_POINTS]
 *   pressure levels           [6][NO_OF_LATLON_IO_POINTS]
 *   w                         [NO_OF_LEVELS][NO_OF_LATLON_IO_POINTS],
 *                             the vertical wind at the levels
 * Missing values (pressure levels below the lowest layer) are 9999, and so
 * is every lat-lon point next to one. */
struct game_gpu_output_fields {
    /* surface: write_output.c:100-350 */
    double *mslp, *surface_p, *t2, *tcdc, *rprate, *sprate, *cape, *sfc_sw_down, *u10, *v10, *gusts;
    /* model layers: temperature, pressure, relative humidity (%), eastward
     * and northward wind, relative vorticity, horizontal divergence, Ertel's
     * potential vorticity (:718-749) */
    double *temperature, *pressure, *rh, *u, *v, *rel_vort, *divv_h, *epv;
    /* pressure levels (:751-826) */
    double *geopotential_height, *t_pl, *rh_pl, *epv_pl, *u_pl, *v_pl, *rel_vort_pl;
    double *w;
};

/* Computes the fields from state_write_out: its device mirror in resident
 * mode, else the host struct, uploaded.  wind_h_lowest_layer_array holds the
 * lowest layer's horizontal wind at min_no_of_output_steps time steps,
 * [min_no_of_output_steps][NO_OF_VECTORS_H] as the reference's driver fills
 * it (src/coordinator.c:350-358); NULL takes the slots recorded on the device
 * by game_gpu_record_wind_lowest instead.  Reads diagnostics'
 * monin_obukhov_length, roughness_velocity and v_squared only when the
 * config switches the gusts' boundary-layer branch on (sfc_sensible_heat_flux,
 * sfc_phase_trans or pbl_scheme == 1), forcings' sfc_sw_in, and
 * state_write_out's temperature_soil only with prog_soil_temp == 1.
 * Like write_out it rounds the top layer of state_write_out's theta_v_pert as
 * (x + theta_v_bg) - theta_v_bg (on the mirror in resident mode, else on the
 * host struct); unlike write_out it leaves the Diagnostics work arrays
 * (temperature, rel_vort, pot_vort, u/v_at_edge, u/v_at_cell,
 * scalar_field_placeholder) alone.  The gust diagnostics follow write_out run
 * on one thread: the reference's loop shares a work array between its
 * OpenMP threads.  No counterpart function in the reference (the loops are
 * inside write_out). */
int game_gpu_write_out_fields(struct state *state_write_out, double wind_h_lowest_layer_array[],
                              int min_no_of_output_steps, struct diagnostics *diagnostics,
                              struct forcings *forcings, struct grid *grid, struct config *config,
                              struct game_gpu_output_fields *native, struct game_gpu_output_fields *latlon);

/* src/io/io.h:10 -> src/io/write_output.c:51: the fields computed on the GPU
 * (as game_gpu_write_out_fields does) and the reference's netCDF files
 * written in the working directory: <run_id>+<t>s_surface.nc,
 * <run_id>+<t>s_pressure_levels.nc and <run_id>+<t>s.nc, t = (int)(t_write -
 * t_init), with the reference's dimensions, variables, units and order, under
 * the reference's switches.  GRIB output (grib_output_switch = 1) is not
 * available and returns an error.  config_io is the reference's Config_io. */
int write_out(struct state *state_write_out, double wind_h_lowest_layer_array[], int min_no_of_output_steps,
              double t_init, double t_write, struct diagnostics *diagnostics, struct forcings *forcings,
              struct grid *grid, struct dualgrid *dualgrid, struct config_io *config_io, struct config *config,
              struct irreversible_quantities *irrev);
/* io.h:12 -> write_output.c:1670: linear_combine_two_states with the
 * weights of t_write between t_0 and t_p1 */
int interpolation_t(struct state *state_0, struct state *state_p1, struct state *state_write, double t_0,
                    double t_p1, double t_write, struct grid *grid);
/* io.h:11 -> write_output.c:1515: the integral of integral_id (as
 * game_gpu_write_out_integral computes it) appended to the reference's text
 * file in the working directory ("masses", "potential_temperature_density"
 * or "energy") in its format */
int write_out_integral(struct state *state_write_out, double time_since_init, struct grid *grid,
                       struct dualgrid *dualgrid, struct diagnostics *diagnostics, int integral_id);

/* Copies the lowest layer's horizontal wind of state (its device mirror in
 * resident mode, else the host struct) into device slot `slot`
 * (0 <= slot < 4096), the device-side counterpart of the driver's
 * wind_h_lowest_layer bookkeeping (src/coordinator.c:350-358). */
int game_gpu_record_wind_lowest(struct state *state, int slot);

#ifdef __cplusplus
}
#endif
#endif
