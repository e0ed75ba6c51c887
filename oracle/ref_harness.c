/*
 * Test-infrastructure harness linked into the reference build (oracle/_ref).
 *
 * Compiled against the reference's own game_types.h (with the enums of one
 * configuration), it exports the compiler's sizeof/offsetof for every member
 * of the reference structs (src/game_types.h:70-238), so that the run-time
 * layout used by the GPU library can be checked member by member.  The
 * reference's functions themselves (manage_rkhevi, grad, divv_h, ...) are
 * called directly from Python through this shared library.
 */
#include <stddef.h>
#include <string.h>
#include "game_types.h"

#define GRID_MEMBERS(X) X(no_of_oro_layers) X(normal_distance) X(volume) X(area) X(z_scalar) X(z_vector) \
    X(gravity_potential) X(gravity_m) X(slope) X(theta_v_bg) X(exner_bg) X(exner_bg_grad) X(layer_thickness) \
    X(trsk_indices) X(trsk_modified_curl_indices) X(from_index) X(to_index) X(adjacent_vector_indices_h) \
    X(adjacent_signs_h) X(density_to_rhombi_indices) X(latitude_scalar) X(longitude_scalar) \
    X(inner_product_weights) X(direction) X(density_to_rhombi_weights) X(trsk_weights) X(sfc_albedo) \
    X(sfc_rho_c) X(t_conduc_soil) X(roughness_length) X(is_land) X(latlon_interpol_indices) \
    X(latlon_interpol_weights) X(z_soil_interface) X(z_soil_center) X(mean_velocity_area) X(t_const_soil) \
    X(z_t_const) X(toa) X(oro_id) X(stretching_parameter) X(radius) X(eff_hor_res)
#define DUALGRID_MEMBERS(X) X(area) X(z_vector) X(normal_distance) X(from_index) X(to_index) \
    X(vorticity_indices_triangles) X(vorticity_signs_triangles) X(f_vec)
#define STATE_MEMBERS(X) X(rho) X(rhotheta_v) X(theta_v_pert) X(exner_pert) X(wind) X(temperature_soil)
#define DIAG_MEMBERS(X) X(flux_density) X(flux_density_divv) X(rel_vort_on_triangles) X(rel_vort) X(pot_vort) \
    X(temperature) X(c_g_p_field) X(v_squared) X(wind_divv) X(curl_of_vorticity) X(scalar_field_placeholder) \
    X(vector_field_placeholder) X(u_at_edge) X(v_at_edge) X(u_at_cell) X(v_at_cell) X(n_squared) X(dv_hdz) \
    X(scalar_flux_resistance) X(power_flux_density_sensible) X(power_flux_density_latent) \
    X(roughness_velocity) X(monin_obukhov_length)
#define FORC_MEMBERS(X) X(pgrad_acc_old) X(pressure_gradient_acc_neg_nl) X(pressure_gradient_acc_neg_l) \
    X(pressure_grad_condensates_v) X(v_squared_grad) X(pot_vort_tend) X(sfc_sw_in) X(sfc_lw_out) \
    X(radiation_tendency)
#define IRREV_MEMBERS(X) X(temperature_diffusion_heating) X(friction_acc) X(heating_diss) \
    X(molecular_diffusion_coeff) X(mass_diffusion_coeff_numerical_h) X(mass_diffusion_coeff_numerical_v) \
    X(temp_diffusion_coeff_numerical_h) X(temp_diffusion_coeff_numerical_v) X(pressure_gradient_decel_factor) \
    X(condensates_sediment_heat) X(mass_diff_tendency) X(phase_trans_rates) X(phase_trans_heating_rate) \
    X(viscosity) X(viscosity_rhombi) X(viscosity_triangles) X(vert_hor_viscosity) X(tke)
#define CONFIG_MEMBERS(X) X(totally_first_step_bool) X(temperature_diff_h) X(temperature_diff_v) \
    X(momentum_diff_h) X(momentum_diff_v) X(mass_diff_h) X(mass_diff_v) X(rad_on) X(prog_soil_temp) \
    X(sfc_phase_trans) X(sfc_sensible_heat_flux) X(rad_update) X(time_to_next_analysis) X(pbl_scheme) \
    X(total_run_span) X(damping_start_height_over_toa) X(damping_coeff_max) X(impl_thermo_weight) \
    X(cloud_droplets_velocity) X(rain_velocity) X(snow_velocity) X(radiation_delta_t)

#define CASE(TYPE, m) if (strcmp(name, #m) == 0) return (long)offsetof(TYPE, m);

long ref_offsetof(int sid, const char *name)
{
#define G(m) CASE(Grid, m)
#define DG(m) CASE(Dualgrid, m)
#define ST(m) CASE(State, m)
#define DI(m) CASE(Diagnostics, m)
#define FO(m) CASE(Forcings, m)
#define IR(m) CASE(Irreversible_quantities, m)
#define CO(m) CASE(Config, m)
    switch (sid) {
    case 0: GRID_MEMBERS(G) break;
    case 1: DUALGRID_MEMBERS(DG) break;
    case 2: STATE_MEMBERS(ST) break;
    case 3: DIAG_MEMBERS(DI) break;
    case 4: FORC_MEMBERS(FO) break;
    case 5: IRREV_MEMBERS(IR) break;
    case 6: CONFIG_MEMBERS(CO) break;
    }
    return -1;
}

long ref_sizeof(int sid)
{
    switch (sid) {
    case 0: return (long)sizeof(Grid);
    case 1: return (long)sizeof(Dualgrid);
    case 2: return (long)sizeof(State);
    case 3: return (long)sizeof(Diagnostics);
    case 4: return (long)sizeof(Forcings);
    case 5: return (long)sizeof(Irreversible_quantities);
    case 6: return (long)sizeof(Config);
    }
    return -1;
}

void ref_dims(long out[8])
{
    out[0] = RES_ID; out[1] = NO_OF_LAYERS; out[2] = MOISTURE_ON; out[3] = NO_OF_SCALARS_H;
    out[4] = NO_OF_VECTORS_H; out[5] = NO_OF_DUAL_SCALARS_H; out[6] = NO_OF_CONSTITUENTS; out[7] = NO_OF_VECTORS;
}

/* OpenMP thread count of the reference's parallel loops.  The gust loop of
 * write_out (src/io/write_output.c:298-346) shares its work array
 * vector_to_minimize between threads, so its result depends on the thread
 * schedule unless it runs on one thread. */
#include <omp.h>
void ref_set_num_threads(int n) { omp_set_num_threads(n); }
int ref_get_max_threads(void) { return omp_get_max_threads(); }

/* offsets of the members of the reference's Config_io */
#define CONFIG_IO_MEMBERS(X) X(grib_output_switch) X(netcdf_output_switch) X(pressure_level_output_switch) \
    X(model_level_output_switch) X(surface_output_switch) X(write_out_interval) X(write_out_integrals) X(year) \
    X(month) X(day) X(hour) X(run_id) X(month_string) X(day_string) X(hour_string) X(ideal_input_id)
long ref_config_io_offsetof(const char *name)
{
#define CIO(m) if (strcmp(name, #m) == 0) return (long)offsetof(Config_io, m);
    CONFIG_IO_MEMBERS(CIO)
#undef CIO
    return -1;
}
long ref_config_io_sizeof(void) { return (long)sizeof(Config_io); }
