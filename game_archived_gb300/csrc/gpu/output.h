/* output diagnostics on the device mirrors (output_f64.cu): the fields
 * write_out computes (src/io/write_output.c:51-1513) and the operators only
 * output uses (src/io/spatial_ops_for_output.c, src/spatial_operators/
 * averaging.c:135-234) */
#pragma once

#include "context.h"
#include "game_gb300.h"

namespace game {

constexpr int N_PRESSURE_LEVELS = 6;

/* switches of one output pass */
struct OutParams {
    int n_cond, moist, n_const;
    int prog_soil_temp;
    int gust_turbulence;  /* the gust diagnostics' boundary-layer branch (write_output.c:302) */
    int n_wind_steps;
    double snow_velocity, rain_velocity;
};

/* device arrays of one output pass; every field in device order */
struct OutFields {
    /* surface [Nc] */
    double *mslp, *surface_p, *t2, *tcdc, *rprate, *sprate, *cape, *sfc_sw_down, *u10, *v10, *gusts;
    /* model layers [L][Nc] */
    double *temperature, *pressure, *rh, *u, *v, *rel_vort, *divv_h, *epv;
    /* pressure levels [6][Nc] */
    double *geopotential_height, *t_pl, *rh_pl, *epv_pl, *u_pl, *v_pl, *rel_vort_pl;
};

/* inputs the caller supplies from host memory, uploaded in device order */
struct OutInputs {
    const double *sfc_sw_in;            /* [Nc] */
    const double *temperature_soil;     /* [Nc], only with prog_soil_temp */
    const double *monin_obukhov_length; /* [Nc], only with gust_turbulence */
    const double *roughness_velocity;   /* [Nc], only with gust_turbulence */
    const double *v_squared;            /* [L][Nc], only with gust_turbulence */
    const double *wind_lowest;          /* [n_wind_steps][Ne] */
};

/* computes every field of f from the state mirror s; rounds the top layer
 * of s's theta_v_pert as (x + bg) - bg, as write_out does */
int output_fields(Context *c, StateMirror *s, const OutParams &p, const OutInputs &in, const OutFields &f);

/* host inputs of one output pass, reference order (NULL where not needed) */
struct OutHost {
    const double *sfc_sw_in;            /* [Nc] */
    const double *temperature_soil;     /* [Nc] */
    const double *monin_obukhov_length; /* [Nc] */
    const double *roughness_velocity;   /* [Nc] */
    const double *v_squared;            /* [L][Nc] */
    const double *wind_lowest;          /* [n_wind_steps][Ne], NULL: the recorded device slots */
};

/* uploads the host inputs, runs output_fields on the mirror s and writes the
 * requested native-grid and lat-lon fields to host memory (either set of
 * pointers may be NULL) */
int output_run(Context *c, StateMirror *s, const OutParams &p, const OutHost &h,
               const struct game_gpu_output_fields *native, const struct game_gpu_output_fields *latlon);

/* copies the lowest layer's horizontal wind of s into device slot `slot` */
int output_record_wind(Context *c, StateMirror *s, int slot);
constexpr int MAX_WIND_SLOTS = 4096;

/* host [n_slices][Ne] (reference order) -> device [n_slices][Ne] */
int output_upload_edges(Context *c, const double *host, int n_slices, double *dev);
/* interpolate_to_ll of one device [Nc] field into host_out [N_ll] */
int output_latlon_host(Context *c, const double *dev_field, double *host_out);

/* dst[k][N_ll] = interpolate_to_ll(src[k]) for k < n_fields; src is a device
 * array of n_fields device pointers to [Nc] fields in device order */
int output_latlon(Context *c, const double *const *src, int n_fields, double *dst);

/* the single operators (device layout): calc_uv_at_edge on the horizontal
 * wind u [L][Ne] -> ue, ve [L][Ne]; edges_to_cells [L][Ne] -> [L][Nc];
 * curl_field_to_cells of a curl field's rhombus part [L][Ne] -> [L][Nc];
 * edges_to_cells_lowest_layer [Ne] -> [Nc]; inner_product_tangential of two
 * vector fields -> [L][Nc]; epv_diagnostics of a curl field */
void op_uv_at_edge(Context *c, const double *u, double *ue, double *ve);
void op_edges_to_cells(Context *c, const double *ue, double *out);
void op_curl_to_cells(Context *c, const double *zv, double *out);
void op_edges_to_cells_lowest(Context *c, const double *ue, double *out);
void op_inner_product_tangential(Context *c, const double *a, const double *b, double *out);
int op_epv(Context *c, const double *pot_vort, DState s, double *epv);

/* scatter of [k][Nc] device-order slices to reference order [k][Nc] and of
 * the pressure-level fields [6][Nc] to the reference's [Nc][6], into dst
 * (device memory) */
void output_to_reference_cells(Context *c, const double *src, int n_slices, double *dst);
void output_to_reference_levels(Context *c, const double *src, double *dst);
/* dst[k][n] (device order) <- src[k][n] (reference order) for cells
 * (edges = 0) or edges (edges = 1) */
void output_from_reference(Context *c, const double *src, int n_slices, int edges, double *dst);

}  // namespace game
