/*
 * Run-time byte layout of GAME's structs (see layout.h).  The member lists
 * below restate the declarations in src/game_types.h:62-238 in declaration
 * order; every member is either int or double.
 */
#include "layout.h"

#include <string.h>

/* element-count kinds */
enum {
    K_ONE, K_S, K_VT, K_CURL, K_DV, K_NE, K_NC, K_NT, K_SOIL, K_SOIL1, K_LL,
    K_LNT, K_HV_PLUS, K_CS, K_PT, K_SOILNC
};

typedef struct { const char *name; int is_int; int kind; int mult; } mdesc;

#define D(n, k, m) {n, 0, k, m}
#define I(n, k, m) {n, 1, k, m}

/* src/game_types.h:70-114 */
static const mdesc GRID[] = {
    I("no_of_oro_layers", K_ONE, 1),
    D("normal_distance", K_VT, 1), D("volume", K_S, 1), D("area", K_VT, 1), D("z_scalar", K_S, 1),
    D("z_vector", K_VT, 1), D("gravity_potential", K_S, 1), D("gravity_m", K_VT, 1), D("slope", K_VT, 1),
    D("theta_v_bg", K_S, 1), D("exner_bg", K_S, 1), D("exner_bg_grad", K_VT, 1), D("layer_thickness", K_S, 1),
    I("trsk_indices", K_NE, 10), I("trsk_modified_curl_indices", K_NE, 10), I("from_index", K_NE, 1),
    I("to_index", K_NE, 1), I("adjacent_vector_indices_h", K_NC, 6), I("adjacent_signs_h", K_NC, 6),
    I("density_to_rhombi_indices", K_NE, 4), D("latitude_scalar", K_NC, 1), D("longitude_scalar", K_NC, 1),
    D("inner_product_weights", K_S, 8), D("direction", K_NE, 1), D("density_to_rhombi_weights", K_NE, 4),
    D("trsk_weights", K_NE, 10), D("sfc_albedo", K_NC, 1), D("sfc_rho_c", K_NC, 1), D("t_conduc_soil", K_NC, 1),
    D("roughness_length", K_NC, 1), I("is_land", K_NC, 1), I("latlon_interpol_indices", K_LL, 5),
    D("latlon_interpol_weights", K_LL, 5), D("z_soil_interface", K_SOIL1, 1), D("z_soil_center", K_SOIL, 1),
    D("mean_velocity_area", K_ONE, 1), D("t_const_soil", K_NC, 1), D("z_t_const", K_ONE, 1), D("toa", K_ONE, 1),
    I("oro_id", K_ONE, 1), D("stretching_parameter", K_ONE, 1), D("radius", K_ONE, 1), D("eff_hor_res", K_ONE, 1),
};

/* src/game_types.h:117-126 */
static const mdesc DUALGRID[] = {
    D("area", K_CURL, 1), D("z_vector", K_DV, 1), D("normal_distance", K_DV, 1), I("from_index", K_NE, 1),
    I("to_index", K_NE, 1), I("vorticity_indices_triangles", K_NT, 3), I("vorticity_signs_triangles", K_NT, 3),
    D("f_vec", K_NE, 2),
};

/* src/game_types.h:128-135 */
static const mdesc STATE[] = {
    D("rho", K_CS, 1), D("rhotheta_v", K_S, 1), D("theta_v_pert", K_S, 1), D("exner_pert", K_S, 1),
    D("wind", K_VT, 1), D("temperature_soil", K_SOILNC, 1),
};

/* src/game_types.h:138-162 */
static const mdesc DIAGNOSTICS[] = {
    D("flux_density", K_VT, 1), D("flux_density_divv", K_S, 1), D("rel_vort_on_triangles", K_LNT, 1),
    D("rel_vort", K_CURL, 1), D("pot_vort", K_CURL, 1), D("temperature", K_S, 1), D("c_g_p_field", K_S, 1),
    D("v_squared", K_S, 1), D("wind_divv", K_S, 1), D("curl_of_vorticity", K_VT, 1),
    D("scalar_field_placeholder", K_S, 1), D("vector_field_placeholder", K_VT, 1), D("u_at_edge", K_VT, 1),
    D("v_at_edge", K_VT, 1), D("u_at_cell", K_S, 1), D("v_at_cell", K_S, 1), D("n_squared", K_S, 1),
    D("dv_hdz", K_HV_PLUS, 1), D("scalar_flux_resistance", K_NC, 1), D("power_flux_density_sensible", K_NC, 1),
    D("power_flux_density_latent", K_NC, 1), D("roughness_velocity", K_NC, 1), D("monin_obukhov_length", K_NC, 1),
};

/* src/game_types.h:180-190 */
static const mdesc FORCINGS[] = {
    D("pgrad_acc_old", K_VT, 1), D("pressure_gradient_acc_neg_nl", K_VT, 1),
    D("pressure_gradient_acc_neg_l", K_VT, 1), D("pressure_grad_condensates_v", K_VT, 1),
    D("v_squared_grad", K_VT, 1), D("pot_vort_tend", K_VT, 1), D("sfc_sw_in", K_NC, 1), D("sfc_lw_out", K_NC, 1),
    D("radiation_tendency", K_S, 1),
};

/* src/game_types.h:219-238 */
static const mdesc IRREV[] = {
    D("temperature_diffusion_heating", K_S, 1), D("friction_acc", K_VT, 1), D("heating_diss", K_S, 1),
    D("molecular_diffusion_coeff", K_S, 1), D("mass_diffusion_coeff_numerical_h", K_S, 1),
    D("mass_diffusion_coeff_numerical_v", K_S, 1), D("temp_diffusion_coeff_numerical_h", K_S, 1),
    D("temp_diffusion_coeff_numerical_v", K_S, 1), D("pressure_gradient_decel_factor", K_S, 1),
    D("condensates_sediment_heat", K_S, 1), D("mass_diff_tendency", K_CS, 1), D("phase_trans_rates", K_PT, 1),
    D("phase_trans_heating_rate", K_S, 1), D("viscosity", K_S, 1), D("viscosity_rhombi", K_VT, 1),
    D("viscosity_triangles", K_LNT, 1), D("vert_hor_viscosity", K_HV_PLUS, 1), D("tke", K_S, 1),
};

/* src/game_types.h:193-216 */
static const mdesc CONFIG[] = {
    I("totally_first_step_bool", K_ONE, 1), I("temperature_diff_h", K_ONE, 1), I("temperature_diff_v", K_ONE, 1),
    I("momentum_diff_h", K_ONE, 1), I("momentum_diff_v", K_ONE, 1), I("mass_diff_h", K_ONE, 1),
    I("mass_diff_v", K_ONE, 1), I("rad_on", K_ONE, 1), I("prog_soil_temp", K_ONE, 1), I("sfc_phase_trans", K_ONE, 1),
    I("sfc_sensible_heat_flux", K_ONE, 1), I("rad_update", K_ONE, 1), I("time_to_next_analysis", K_ONE, 1),
    I("pbl_scheme", K_ONE, 1), I("total_run_span", K_ONE, 1), D("damping_start_height_over_toa", K_ONE, 1),
    D("damping_coeff_max", K_ONE, 1), D("impl_thermo_weight", K_ONE, 1), D("cloud_droplets_velocity", K_ONE, 1),
    D("rain_velocity", K_ONE, 1), D("snow_velocity", K_ONE, 1), D("radiation_delta_t", K_ONE, 1),
};

static const mdesc *TABLES[GAME_N_STRUCTS] = {GRID, DUALGRID, STATE, DIAGNOSTICS, FORCINGS, IRREV, CONFIG};
static const int COUNTS[GAME_N_STRUCTS] = {
    (int)(sizeof GRID / sizeof GRID[0]), (int)(sizeof DUALGRID / sizeof DUALGRID[0]),
    (int)(sizeof STATE / sizeof STATE[0]), (int)(sizeof DIAGNOSTICS / sizeof DIAGNOSTICS[0]),
    (int)(sizeof FORCINGS / sizeof FORCINGS[0]), (int)(sizeof IRREV / sizeof IRREV[0]),
    (int)(sizeof CONFIG / sizeof CONFIG[0]),
};

int game_dims_init(game_dims *d, int res_id, int n_layers, int moisture_on)
{
    if (res_id < 0 || res_id > 9 || n_layers < 2 || (moisture_on != 0 && moisture_on != 1)) return -1;
    long p4 = 1L << (2 * res_id);
    d->res_id = res_id;
    d->n_layers = n_layers;
    d->moisture_on = moisture_on;
    d->n_cells = 10 * p4 + 2;
    d->n_edges = 30 * p4;
    d->n_triangles = 20 * p4;
    d->vpl = d->n_cells + d->n_edges;
    d->dpl = d->n_edges + d->n_triangles;
    d->n_scalars = d->n_cells * n_layers;
    d->n_vectors = (long)n_layers * d->n_edges + (long)(n_layers + 1) * d->n_cells;
    d->n_dual_vectors = (long)(n_layers + 1) * d->n_edges + (long)n_layers * d->n_triangles;
    d->n_curl = (long)n_layers * 2 * d->n_edges + d->n_edges;
    d->n_condensed = 4 * moisture_on;
    d->n_constituents = 1 + moisture_on + d->n_condensed;
    d->n_soil = 5;
    d->n_latlon = (4L << res_id) * (2L << res_id);
    return 0;
}

static long kind_count(const game_dims *d, int kind)
{
    switch (kind) {
    case K_ONE: return 1;
    case K_S: return d->n_scalars;
    case K_VT: return d->n_vectors;
    case K_CURL: return d->n_curl;
    case K_DV: return d->n_dual_vectors;
    case K_NE: return d->n_edges;
    case K_NC: return d->n_cells;
    case K_NT: return d->n_triangles;
    case K_SOIL: return d->n_soil;
    case K_SOIL1: return d->n_soil + 1;
    case K_LL: return d->n_latlon;
    case K_LNT: return (long)d->n_layers * d->n_triangles;
    case K_HV_PLUS: return (long)d->n_layers * d->n_edges + d->n_edges;
    case K_CS: return (long)d->n_constituents * d->n_scalars;
    case K_PT: return (long)(d->n_condensed + 1) * d->n_scalars;
    case K_SOILNC: return (long)d->n_soil * d->n_cells;
    }
    return 0;
}

int game_layout_count(int sid)
{
    if (sid < 0 || sid >= GAME_N_STRUCTS) return -1;
    return COUNTS[sid];
}

/* walks the member list up to member i (or to the end when i == count) */
static size_t walk(const game_dims *d, int sid, int upto, game_member *m)
{
    size_t off = 0;
    const mdesc *t = TABLES[sid];
    for (int i = 0; i < COUNTS[sid]; ++i) {
        size_t al = t[i].is_int ? sizeof(int) : sizeof(double);
        off = (off + al - 1) / al * al;
        long cnt = kind_count(d, t[i].kind) * t[i].mult;
        if (i == upto) {
            m->name = t[i].name;
            m->is_int = t[i].is_int;
            m->count = cnt;
            m->offset = off;
            return off;
        }
        off += (size_t)cnt * al;
    }
    /* struct size: rounded up to the largest member alignment */
    return (off + sizeof(double) - 1) / sizeof(double) * sizeof(double);
}

int game_layout_member(const game_dims *d, int sid, int i, game_member *m)
{
    if (sid < 0 || sid >= GAME_N_STRUCTS || i < 0 || i >= COUNTS[sid]) return -1;
    walk(d, sid, i, m);
    return 0;
}

size_t game_layout_offset(const game_dims *d, int sid, const char *name)
{
    if (sid < 0 || sid >= GAME_N_STRUCTS) return (size_t)-1;
    for (int i = 0; i < COUNTS[sid]; ++i)
        if (strcmp(TABLES[sid][i].name, name) == 0) {
            game_member m;
            walk(d, sid, i, &m);
            return m.offset;
        }
    return (size_t)-1;
}

size_t game_layout_sizeof(const game_dims *d, int sid)
{
    if (sid < 0 || sid >= GAME_N_STRUCTS) return 0;
    game_member m;
    return walk(d, sid, COUNTS[sid], &m);
}
