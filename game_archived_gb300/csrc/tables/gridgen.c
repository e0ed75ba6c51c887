/*
 * Icosahedral-hexagonal C-grid table builder (see gridgen.h).
 *
 * Compile with -ffp-contract=off so that x86_64 and aarch64 hosts round every
 * product and sum the same way.
 */
#include "gridgen.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* physical constants of GAME (src/game_constants.h:10-27) */
#define RADIUS_EARTH 6371000.789927
#define OMEGA_EARTH (7.292115e-5)
#define G_MEAN_SFC_ABS 9.80616
#define P_0 100000.0
#define C_D_P 1005.0
#define R_D 287.057811
#define N_PENT 12
#define EPS_SECURITY (1e-10)
#define ORTH_CRITERION_DEG 89.99

static char g_err[256];
const char *gt_last_error(void) { return g_err; }
#define FAIL(...) do { snprintf(g_err, sizeof g_err, __VA_ARGS__); goto fail; } while (0)

/* ---------------------------------------------------------------- vectors */
typedef struct { double x, y, z; } v3;
static inline v3 v3_add(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static inline v3 v3_sub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline v3 v3_scale(v3 a, double s) { v3 r = {a.x * s, a.y * s, a.z * s}; return r; }
static inline double v3_dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 v3_cross(v3 a, v3 b)
{
    v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}
static inline double v3_norm(v3 a) { return sqrt(v3_dot(a, a)); }
static inline v3 v3_unit(v3 a) { return v3_scale(a, 1.0 / v3_norm(a)); }
static inline v3 v3_from_geo(double lat, double lon)
{
    v3 r = {cos(lat) * cos(lon), cos(lat) * sin(lon), sin(lat)};
    return r;
}
static inline void v3_to_geo(v3 a, double *lat, double *lon)
{
    *lat = asin(a.z / v3_norm(a));
    *lon = atan2(a.y, a.x);
}

/* area of the spherical triangle (a, b, c) on the unit sphere, a, b, c unit
 * vectors (Van Oosterom & Strackee 1983). */
static inline double sph_tri_area(v3 a, v3 b, v3 c)
{
    double num = fabs(v3_dot(a, v3_cross(b, c)));
    double den = 1.0 + v3_dot(a, b) + v3_dot(b, c) + v3_dot(c, a);
    return 2.0 * atan2(num, den);
}

/* central angle between two unit vectors */
static inline double central_angle(v3 a, v3 b)
{
    return 2.0 * asin(0.5 * v3_norm(v3_sub(a, b)));
}

/* direction (radians, counter-clockwise from east) of the chord a->b seen at
 * the point p (geodetic direction, geodesy.c:find_geodetic_direction) */
static double chord_direction(v3 a, v3 b, v3 p)
{
    double lat, lon;
    v3_to_geo(p, &lat, &lon);
    v3 rel = v3_sub(b, a);
    v3 east = {-sin(lon), cos(lon), 0.0};
    v3 north = {-sin(lat) * cos(lon), -sin(lat) * sin(lon), cos(lat)};
    return atan2(v3_dot(north, rel), v3_dot(east, rel));
}

static double turn_angle(double a0, double a1)
{
    double r = a1 - a0;
    if (r > M_PI) r -= 2.0 * M_PI;
    if (r < -M_PI) r += 2.0 * M_PI;
    return r;
}

/* ------------------------------------------- dual-vector directions
 * The reference's generator gives a dual vector the direction of the great
 * circle through its two dual points, evaluated at the point of that circle
 * nearest to the primal vector point, where "nearest" is the first minimum
 * of the chord distance over the 1001 sample parameters t_i = i / 1002
 * (horizontal_generation.c:519-576 with geodesy.c:15-92 and 369-387).  The
 * samples, distances and directions below are computed from geographical
 * coordinates with the same formulas, so the sampled parameter and the
 * direction are the reference's.  Only the window of samples searched
 * differs: the distance along the circle has a single minimum, at the
 * angle t* = atan2(p.q, p.a) / theta (a, q an orthonormal pair spanning the
 * circle's plane, a the first point), so the first minimum over all samples
 * lies within a sample of t* and a window of +-DUAL_WINDOW samples around it
 * holds it. */
#define DUAL_SAMPLES 1001
#define DUAL_WINDOW 4

static double chord_geo(double lat_1, double lon_1, double lat_2, double lon_2)
{
    if (lat_1 == lat_2 && lon_1 == lon_2) return 0;
    const double x_1 = cos(lat_1) * cos(lon_1), y_1 = cos(lat_1) * sin(lon_1), z_1 = sin(lat_1);
    const double x_2 = cos(lat_2) * cos(lon_2), y_2 = cos(lat_2) * sin(lon_2), z_2 = sin(lat_2);
    return sqrt(pow(x_2 - x_1, 2) + pow(y_2 - y_1, 2) + pow(z_2 - z_1, 2));
}

/* the point at parameter t of the great circle from 1 to 2, uniform in angle */
static void geodetic_point(double lat_1, double lon_1, double lat_2, double lon_2, double t, double *lat,
                           double *lon)
{
    const double d = chord_geo(lat_1, lon_1, lat_2, lon_2);
    const double theta = 2.0 * asin(d / 2.0);
    const double tau = 0.5 + sqrt(1.0 / pow(d, 2) - 0.25) * tan(theta * (t - 0.5));
    const double z = tau * sin(lat_2) + (1.0 - tau) * sin(lat_1);
    const double x = tau * cos(lat_2) * cos(lon_2) + (1.0 - tau) * cos(lat_1) * cos(lon_1);
    const double y = tau * cos(lat_2) * sin(lon_2) + (1.0 - tau) * cos(lat_1) * sin(lon_1);
    *lat = asin(z / sqrt(pow(x, 2) + pow(y, 2) + pow(z, 2)));
    *lon = atan2(y, x);
}

/* direction (counter-clockwise from east) of the chord 1 -> 2 in the local
 * frame of the circle's point at parameter t */
static double geodetic_direction(double lat_1, double lon_1, double lat_2, double lon_2, double t)
{
    const double rx = cos(lat_2) * cos(lon_2) - cos(lat_1) * cos(lon_1);
    const double ry = cos(lat_2) * sin(lon_2) - cos(lat_1) * sin(lon_1);
    const double rz = sin(lat_2) - sin(lat_1);
    double lat, lon;
    geodetic_point(lat_1, lon_1, lat_2, lon_2, t, &lat, &lon);
    const double x_comp = -sin(lon) * rx + cos(lon) * ry + 0 * rz;
    const double y_comp = -sin(lat) * cos(lon) * rx + -sin(lat) * sin(lon) * ry + cos(lat) * rz;
    return atan2(y_comp, x_comp);
}

/* the sampled parameter of the point of the circle 1 -> 2 nearest to p */
static double nearest_sample(double lat_1, double lon_1, double lat_2, double lon_2, double lat_p, double lon_p)
{
    const v3 a = v3_from_geo(lat_1, lon_1), b = v3_from_geo(lat_2, lon_2), p = v3_from_geo(lat_p, lon_p);
    const v3 q = v3_unit(v3_sub(b, v3_scale(a, v3_dot(a, b))));
    const double theta = atan2(v3_dot(b, q), v3_dot(b, a));
    const double t_star = atan2(v3_dot(p, q), v3_dot(p, a)) / theta;
    int i_0 = (int)floor(t_star * (DUAL_SAMPLES + 1.0)) - DUAL_WINDOW, i_1 = i_0 + 2 * DUAL_WINDOW + 1;
    if (i_0 < 0) i_0 = 0;
    if (i_1 > DUAL_SAMPLES - 1) i_1 = DUAL_SAMPLES - 1;
    int best = -1;
    double best_d = 0;
    for (int i = i_0; i <= i_1; ++i) {
        double lat, lon;
        geodetic_point(lat_1, lon_1, lat_2, lon_2, (i + 0.0) / (DUAL_SAMPLES + 1.0), &lat, &lon);
        const double d = chord_geo(lat_p, lon_p, lat, lon);
        if (best < 0 || d < best_d) {
            best = i;
            best_d = d;
        }
    }
    return (best + 0.0) / (DUAL_SAMPLES + 1.0);
}

/* ----------------------------------------------------------- pair hashing */
typedef struct { int64_t *keys; int *vals; long cap; } pairmap;

static int pm_init(pairmap *m, long n)
{
    long cap = 16;
    while (cap < 2 * n) cap <<= 1;
    m->cap = cap;
    m->keys = malloc(cap * sizeof(int64_t));
    m->vals = malloc(cap * sizeof(int));
    if (!m->keys || !m->vals) return -1;
    for (long i = 0; i < cap; ++i) m->keys[i] = -1;
    return 0;
}
static void pm_free(pairmap *m) { free(m->keys); free(m->vals); }
static inline int64_t pm_key(int a, int b)
{
    int lo = a < b ? a : b, hi = a < b ? b : a;
    return ((int64_t)lo << 32) | (int64_t)(uint32_t)hi;
}
/* returns the stored value, or inserts val and returns -1 */
static int pm_get_or_put(pairmap *m, int a, int b, int val)
{
    int64_t k = pm_key(a, b);
    uint64_t h = (uint64_t)k * 0x9E3779B97F4A7C15ull;
    long i = (long)(h >> 20) & (m->cap - 1);
    while (m->keys[i] != -1) {
        if (m->keys[i] == k) return m->vals[i];
        i = (i + 1) & (m->cap - 1);
    }
    m->keys[i] = k;
    m->vals[i] = val;
    return -1;
}
static int pm_get(const pairmap *m, int a, int b)
{
    int64_t k = pm_key(a, b);
    uint64_t h = (uint64_t)k * 0x9E3779B97F4A7C15ull;
    long i = (long)(h >> 20) & (m->cap - 1);
    while (m->keys[i] != -1) {
        if (m->keys[i] == k) return m->vals[i];
        i = (i + 1) & (m->cap - 1);
    }
    return -1;
}

/* ----------------------------------------------------------- table export */
static void *add_array(game_tables *t, const char *name, int type, long n)
{
    if (t->n_arrays >= GT_MAX_ARRAYS) return NULL;
    gt_array *a = &t->arrays[t->n_arrays];
    snprintf(a->name, sizeof a->name, "%s", name);
    a->type = type;
    a->n = n;
    a->ptr = calloc(n > 0 ? n : 1, type == GT_DOUBLE ? sizeof(double) : sizeof(int));
    if (!a->ptr) return NULL;
    t->n_arrays++;
    return a->ptr;
}

void *gt_get(const game_tables *t, const char *name, long *n)
{
    for (int i = 0; i < t->n_arrays; ++i)
        if (strcmp(t->arrays[i].name, name) == 0) {
            if (n) *n = t->arrays[i].n;
            return t->arrays[i].ptr;
        }
    return NULL;
}

int gt_count(const game_tables *t) { return t->n_arrays; }

int gt_info(const game_tables *t, int i, const char **name, int *type, long *n, void **ptr)
{
    if (i < 0 || i >= t->n_arrays) return -1;
    *name = t->arrays[i].name;
    *type = t->arrays[i].type;
    *n = t->arrays[i].n;
    *ptr = t->arrays[i].ptr;
    return 0;
}

int gt_dims(const game_tables *t, int *o)
{
    o[0] = t->res_id; o[1] = t->n_layers; o[2] = t->n_oro_layers; o[3] = t->n_cells;
    o[4] = t->n_edges; o[5] = t->n_triangles; o[6] = t->n_lloyd; o[7] = 0;
    return 0;
}

void gt_free(game_tables *t)
{
    if (!t) return;
    for (int i = 0; i < t->n_arrays; ++i) free(t->arrays[i].ptr);
    free(t);
}

/* ------------------------------------------------- ICAO standard atmosphere
 * (grid_generator/src/vertical_grid.c:20-25, 350-392) */
static const double T_SFC = 273.15 + 15;
static const double TEMP_GRADIENT = -0.65 / 100;
static const double P_0_STANDARD = 101325;
static const double TROPO_HEIGHT_STANDARD = 11e3;
static const double INVERSE_HEIGHT_STANDARD = 20e3;
static const double TEMP_GRADIENT_INV_STANDARD = 0.1 / 100;

double gt_standard_temp(double z)
{
    const double tropo_temp = T_SFC + TROPO_HEIGHT_STANDARD * TEMP_GRADIENT;
    if (z < TROPO_HEIGHT_STANDARD) return T_SFC + z * TEMP_GRADIENT;
    if (z < INVERSE_HEIGHT_STANDARD) return tropo_temp;
    return tropo_temp + TEMP_GRADIENT_INV_STANDARD * (z - INVERSE_HEIGHT_STANDARD);
}

double gt_standard_pres(double z)
{
    const double tropo_temp = T_SFC + TROPO_HEIGHT_STANDARD * TEMP_GRADIENT;
    const double expo = -G_MEAN_SFC_ABS / (R_D * TEMP_GRADIENT);
    if (z < TROPO_HEIGHT_STANDARD)
        return P_0_STANDARD * pow(1 + TEMP_GRADIENT * z / T_SFC, expo);
    if (z < INVERSE_HEIGHT_STANDARD)
        return P_0_STANDARD * pow(1 + TEMP_GRADIENT * TROPO_HEIGHT_STANDARD / T_SFC, expo)
               * exp(-G_MEAN_SFC_ABS * (z - TROPO_HEIGHT_STANDARD) / (R_D * tropo_temp));
    double p_inv = P_0_STANDARD * pow(1 + TEMP_GRADIENT * TROPO_HEIGHT_STANDARD / T_SFC, expo)
                   * exp(-G_MEAN_SFC_ABS * (INVERSE_HEIGHT_STANDARD - TROPO_HEIGHT_STANDARD) / (R_D * tropo_temp));
    return p_inv * pow(1 + TEMP_GRADIENT * (z - INVERSE_HEIGHT_STANDARD) / T_SFC, expo);
}

/* -------------------------------------------------- gradient (host version)
 * used for the derived tables slope, gravity_m and exner_bg_grad, as the
 * reference derives them when loading the grid
 * (src/io/set_grid_properties.c:217-221). */
typedef struct {
    int nc, ne, nl, n_oro;
    const int *from, *to;
    const double *nd, *ipw, *slope;
} grad_ctx;

static void grad_hor_cov_h(const grad_ctx *g, const double *in, double *out)
{
    /* src/spatial_operators/gradient_operators.c:14-33 */
    long vpl = g->nc + g->ne;
    for (int e = 0; e < g->ne; ++e)
        for (int l = 0; l < g->nl; ++l) {
            long vi = g->nc + l * vpl + e;
            out[vi] = (in[g->to[e] + (long)l * g->nc] - in[g->from[e] + (long)l * g->nc]) / g->nd[vi];
        }
}

static void grad_vert_cov_h(const grad_ctx *g, const double *in, double *out)
{
    /* src/spatial_operators/gradient_operators.c:35-54 */
    long vpl = g->nc + g->ne;
    for (long i = g->nc; i < (long)(g->nl + 1) * g->nc - g->nc; ++i) {
        long layer = i / g->nc, h = i - layer * g->nc;
        long lower = h + layer * g->nc, upper = h + (layer - 1) * g->nc;
        long vi = h + layer * vpl;
        out[vi] = (in[upper] - in[lower]) / g->nd[vi];
    }
}

static double remap_verpri2horpri_h(const grad_ctx *g, const double *f, int layer, int e)
{
    /* src/spatial_operators/averaging.c:14-39 */
    long vpl = g->nc + g->ne;
    int fr = g->from[e], to = g->to[e];
    double c = g->ipw[8 * ((long)layer * g->nc + fr) + 6] * f[layer * vpl + fr];
    c += g->ipw[8 * ((long)layer * g->nc + to) + 6] * f[layer * vpl + to];
    if (layer < g->nl - 1) {
        c += g->ipw[8 * ((long)layer * g->nc + fr) + 7] * f[(layer + 1) * vpl + fr];
        c += g->ipw[8 * ((long)layer * g->nc + to) + 7] * f[(layer + 1) * vpl + to];
    }
    return 0.5 * c;
}

static void hor_cov_to_con_h(const grad_ctx *g, double *f)
{
    /* src/spatial_operators/averaging.c:113-133 */
    long vpl = g->nc + g->ne;
    for (long i = 0; i < (long)g->n_oro * g->ne; ++i) {
        int li = (int)(i / g->ne), e = (int)(i - (long)li * g->ne);
        double vg = remap_verpri2horpri_h(g, f, li + (g->nl - g->n_oro), e);
        long vi = g->nc + (long)(g->nl - g->n_oro + li) * vpl + e;
        f[vi] += -g->slope[vi] * vg;
    }
}

/* ------------------------------------------------------------------ build */
/* ------------------------------------------------ lat-lon output tables
 * Interpolation of the cell fields to the regular lat-lon output grid
 * (grid_generator/src/interpolate_ll.c:16-85): for every lat-lon point the
 * five cells nearest by the reference's geodetic distance
 * (geodesy.c:calculate_distance_h), weights 1 / (d^(2 + eps) + eps)
 * normalised to sum one.  The reference scans every cell for every point; here
 * the cells are bucketed on a 3-D grid and each point scans the buckets inside
 * a chord radius that grows until it provably holds the five nearest, then
 * applies the reference's selection rule to those candidates, so the
 * indices and weights are the ones the reference's scan gives.  That rule
 * (index_helpers.c:find_min_index_exclude) starts every search from cell 0,
 * chosen or not, and takes a later cell only if it is strictly nearer and
 * not chosen yet: cell 0 is therefore always a candidate, ties go to the
 * lowest index, and near cell 0 the same index can be chosen more than
 * once. */
#define LL_EPS 1e-10

static double ll_distance(double lat_a, double lon_a, double lat_b, double lon_b)
{
    return 2.0 * 1.0 * asin(sqrt(0.5 - 0.5 * (cos(lat_a) * cos(lat_b) * cos(lon_b - lon_a) + sin(lat_a) * sin(lat_b))));
}

static int cmp_int(const void *a, const void *b)
{
    const int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

static int latlon_tables(game_tables *T, int res_id, const double *lat_c, const double *lon_c, int Nc)
{
    const int n_lat = (int)(2 * pow(2, res_id)), n_lon = (int)(4 * pow(2, res_id));
    const long n_ll = (long)n_lat * n_lon;
    int *idx = add_array(T, "latlon_interpol_indices", GT_INT, 5 * n_ll);
    double *wts = add_array(T, "latlon_interpol_weights", GT_DOUBLE, 5 * n_ll);
    if (!idx || !wts) return -1;
    /* buckets: a B^3 grid over [-1, 1]^3 with about one cell spacing per edge */
    int B = (int)ceil(2.0 / sqrt(4.0 * M_PI / Nc));
    if (B < 1) B = 1;
    const double h = 2.0 / B;
    const long nb = (long)B * B * B;
    int *start = calloc((size_t)nb + 1, sizeof(int)), *fill = malloc((size_t)nb * sizeof(int));
    int *order = malloc((size_t)Nc * sizeof(int)), *bucket = malloc((size_t)Nc * sizeof(int));
    v3 *P = malloc((size_t)Nc * sizeof(v3));
    int err = !start || !fill || !order || !bucket || !P;
    if (!err) {
        for (int c = 0; c < Nc; ++c) {
            P[c] = v3_from_geo(lat_c[c], lon_c[c]);
            int ix = (int)((P[c].x + 1.0) / h), iy = (int)((P[c].y + 1.0) / h), iz = (int)((P[c].z + 1.0) / h);
            ix = ix < 0 ? 0 : (ix >= B ? B - 1 : ix);
            iy = iy < 0 ? 0 : (iy >= B ? B - 1 : iy);
            iz = iz < 0 ? 0 : (iz >= B ? B - 1 : iz);
            bucket[c] = (ix * B + iy) * B + iz;
            start[bucket[c] + 1]++;
        }
        for (long b = 0; b < nb; ++b) start[b + 1] += start[b];
        for (long b = 0; b < nb; ++b) fill[b] = start[b];
        for (int c = 0; c < Nc; ++c) order[fill[bucket[c]]++] = c;
    }
    const double d_lat = M_PI / n_lat, d_lon = 2 * M_PI / n_lon;
    const long n_run = err ? 0 : n_ll;
    #pragma omp parallel for schedule(dynamic, 64) reduction(|:err)
    for (long i = 0; i < n_run; ++i) {
        const int lat_index = (int)(i / n_lon), lon_index = (int)(i - (long)lat_index * n_lon);
        const double lat_value = M_PI / 2 - 0.5 * d_lat - lat_index * d_lat, lon_value = lon_index * d_lon;
        const v3 q = v3_from_geo(lat_value, lon_value);
        int *cand = NULL, n_cand = 0, cap = 0, oom = 0;
        /* grow a chord radius until the fifth-nearest cell inside it lies
         * well within it: then no cell outside can be among the five nearest
         * whatever the rounding of either distance formula */
        for (double r = 2.0 * h;; r *= 2.0) {
            const int whole = r >= 2.0;
            n_cand = 0;
            int lo[3], hi[3];
            const double qc[3] = {q.x, q.y, q.z};
            for (int a = 0; a < 3; ++a) {
                lo[a] = whole ? 0 : (int)floor((qc[a] - r + 1.0) / h);
                hi[a] = whole ? B - 1 : (int)floor((qc[a] + r + 1.0) / h);
                if (lo[a] < 0) lo[a] = 0;
                if (hi[a] > B - 1) hi[a] = B - 1;
            }
            for (int ix = lo[0]; ix <= hi[0]; ++ix)
                for (int iy = lo[1]; iy <= hi[1]; ++iy)
                    for (int iz = lo[2]; iz <= hi[2]; ++iz) {
                        const long b = ((long)ix * B + iy) * B + iz;
                        for (int k = start[b]; k < start[b + 1]; ++k) {
                            const int c = order[k];
                            const v3 dv = v3_sub(P[c], q);
                            if (!whole && v3_dot(dv, dv) > r * r) continue;
                            if (n_cand == cap) {
                                /* one slot more than cap stays free for cell 0 */
                                int *grown = oom ? NULL : realloc(cand, (size_t)(2 * cap + 65) * sizeof(int));
                                if (!grown) {
                                    oom = 1;
                                    continue;
                                }
                                cand = grown;
                                cap = 2 * cap + 64;
                            }
                            cand[n_cand++] = c;
                        }
                    }
            if (oom || whole) break;
            if (n_cand >= 5) {
                double best[5] = {1e300, 1e300, 1e300, 1e300, 1e300};
                for (int k = 0; k < n_cand; ++k) {
                    const v3 dv = v3_sub(P[cand[k]], q);
                    double d2 = v3_dot(dv, dv);
                    for (int m = 0; m < 5; ++m)
                        if (d2 < best[m]) {
                            const double t = best[m];
                            best[m] = d2;
                            d2 = t;
                        }
                }
                if (sqrt(best[4]) < 0.8 * r) break;
            }
        }
        if (oom || n_cand < 5) {
            free(cand);
            err = 1;
            continue;
        }
        /* cell 0 takes part in every search (the scan starts from it) */
        int has0 = 0;
        for (int k = 0; k < n_cand; ++k) has0 |= cand[k] == 0;
        if (!has0) cand[n_cand++] = 0; /* room for one more is always kept */
        qsort(cand, (size_t)n_cand, sizeof(int), cmp_int);
        double *dist = malloc((size_t)n_cand * sizeof(double));
        if (!dist) {
            free(cand);
            err = 1;
            continue;
        }
        for (int k = 0; k < n_cand; ++k) dist[k] = ll_distance(lat_value, lon_value, lat_c[cand[k]], lon_c[cand[k]]);
        int chosen[5] = {-1, -1, -1, -1, -1};
        double w[5], w_sum = 0;
        for (int j = 0; j < 5; ++j) {
            int result = 0;
            double current = dist[0]; /* cand[0] == 0 */
            for (int k = 1; k < n_cand; ++k) {
                if (dist[k] < current) {
                    int excluded = 0;
                    for (int m = 0; m < 5; ++m) excluded |= chosen[m] == cand[k];
                    if (!excluded) {
                        current = dist[k];
                        result = cand[k];
                    }
                }
            }
            chosen[j] = result;
            w[j] = 1 / (pow(ll_distance(lat_value, lon_value, lat_c[result], lon_c[result]), 2 + LL_EPS) + LL_EPS);
            w_sum += w[j];
        }
        for (int j = 0; j < 5; ++j) {
            idx[5 * i + j] = chosen[j];
            wts[5 * i + j] = w[j] / w_sum;
        }
        free(cand);
        free(dist);
    }
    free(start);
    free(fill);
    free(order);
    free(bucket);
    free(P);
    return err ? -1 : 0;
}

game_tables *gt_build(int res_id, int n_layers, int n_oro_layers, double toa,
                      double stretching, double radius_rescale, int n_lloyd,
                      int oro_kind, const double *oro_params, int n_threads)
{
    game_tables *T = NULL;
    v3 *X = NULL, *circ = NULL, *mid = NULL;
    int *tri = NULL, *ring_tri = NULL, *ring_edge = NULL, *ring_n = NULL;
    int *e_tri = NULL;
    pairmap pm = {0};
    g_err[0] = 0;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    if (res_id < 0 || res_id > 8) FAIL("res_id out of range");
    if (n_layers < 2) FAIL("n_layers must be >= 2");
    if (n_oro_layers < 0 || n_oro_layers >= n_layers) FAIL("0 <= n_oro_layers < n_layers required");
    if (stretching < 1.0) FAIL("stretching_parameter must be >= 1");

    const long pow4 = 1L << (2 * res_id);
    const int Nc = (int)(10 * pow4 + 2), Ne = (int)(30 * pow4), Nt = (int)(20 * pow4);
    const int L = n_layers;
    const long VPL = Nc + Ne, DPL = Ne + Nt;
    const long S = (long)L * Nc, Vt = (long)L * VPL + Nc, Dv = (long)L * DPL + Ne;
    const double radius = radius_rescale * RADIUS_EARTH;

    T = calloc(1, sizeof(game_tables));
    if (!T) FAIL("out of memory");
    T->res_id = res_id; T->n_layers = L; T->n_oro_layers = n_oro_layers; T->n_lloyd = n_lloyd;
    T->n_cells = Nc; T->n_edges = Ne; T->n_triangles = Nt;
    T->toa = toa; T->stretching = stretching; T->radius = radius; T->radius_rescale = radius_rescale;

    /* ---- icosahedron (discrete_coordinate_trafos.c:507-535 orientation) */
    X = malloc((size_t)Nc * sizeof(v3));
    tri = malloc((size_t)3 * Nt * sizeof(int));
    if (!X || !tri) FAIL("out of memory");
    {
        double lat[12], lon[12];
        lat[0] = M_PI / 2; lon[0] = 0;
        for (int i = 1; i <= 5; ++i) { lat[i] = atan(0.5); lon[i] = (i - 1) * 2 * M_PI / 5; }
        for (int i = 6; i <= 10; ++i) { lat[i] = -atan(0.5); lon[i] = 2 * M_PI / 10 + (i - 6) * 2 * M_PI / 5; }
        lat[11] = -M_PI / 2; lon[11] = 0;
        for (int i = 0; i < 12; ++i) X[i] = v3_from_geo(lat[i], lon[i]);
        /* faces: all vertex triples whose pairwise chords have the edge length */
        double edge_len = 1e9;
        for (int i = 0; i < 12; ++i)
            for (int j = i + 1; j < 12; ++j) {
                double d = v3_norm(v3_sub(X[i], X[j]));
                if (d < edge_len) edge_len = d;
            }
        int nf = 0;
        for (int i = 0; i < 12; ++i)
            for (int j = i + 1; j < 12; ++j)
                for (int k = j + 1; k < 12; ++k) {
                    double a = v3_norm(v3_sub(X[i], X[j])), b = v3_norm(v3_sub(X[j], X[k])),
                           c = v3_norm(v3_sub(X[k], X[i]));
                    if (fabs(a - edge_len) < 1e-6 && fabs(b - edge_len) < 1e-6 && fabs(c - edge_len) < 1e-6) {
                        int p = i, q = j, r = k;
                        if (v3_dot(X[p], v3_cross(X[q], X[r])) < 0) { int s = q; q = r; r = s; }
                        tri[3 * nf] = p; tri[3 * nf + 1] = q; tri[3 * nf + 2] = r;
                        ++nf;
                    }
                }
        if (nf != 20) FAIL("icosahedron construction found %d faces", nf);
    }

    /* ---- recursive bisection (geodesic midpoints) */
    {
        int nv = 12, nt = 20;
        int *tri2 = malloc((size_t)3 * Nt * sizeof(int));
        if (!tri2) FAIL("out of memory");
        for (int lev = 0; lev < res_id; ++lev) {
            pairmap mp;
            if (pm_init(&mp, 3L * nt)) { free(tri2); FAIL("out of memory"); }
            int nt2 = 0;
            for (int t = 0; t < nt; ++t) {
                int v[3] = {tri[3 * t], tri[3 * t + 1], tri[3 * t + 2]}, m[3];
                for (int j = 0; j < 3; ++j) {
                    int a = v[j], b = v[(j + 1) % 3];
                    int got = pm_get_or_put(&mp, a, b, nv);
                    if (got < 0) {
                        X[nv] = v3_unit(v3_scale(v3_add(X[a], X[b]), 0.5));
                        m[j] = nv++;
                    } else {
                        m[j] = got;
                    }
                }
                /* children, all counter-clockwise: corners first, centre last */
                int ch[4][3] = {{v[0], m[0], m[2]}, {m[0], v[1], m[1]}, {m[2], m[1], v[2]}, {m[0], m[1], m[2]}};
                for (int c = 0; c < 4; ++c) {
                    tri2[3 * nt2] = ch[c][0]; tri2[3 * nt2 + 1] = ch[c][1]; tri2[3 * nt2 + 2] = ch[c][2];
                    ++nt2;
                }
            }
            pm_free(&mp);
            memcpy(tri, tri2, (size_t)3 * nt2 * sizeof(int));
            nt = nt2;
        }
        free(tri2);
        if (nv != Nc || nt != Nt) FAIL("subdivision produced %d cells / %d triangles", nv, nt);
    }

    /* ---- edges: numbered in order of first appearance, oriented as first traversed */
    int *from = add_array(T, "from_index", GT_INT, Ne);
    int *to = add_array(T, "to_index", GT_INT, Ne);
    int *vort_idx = add_array(T, "vorticity_indices_triangles", GT_INT, 3L * Nt);
    int *vort_sign = add_array(T, "vorticity_signs_triangles", GT_INT, 3L * Nt);
    int *from_dual = add_array(T, "from_index_dual", GT_INT, Ne);
    int *to_dual = add_array(T, "to_index_dual", GT_INT, Ne);
    int *adj = add_array(T, "adjacent_vector_indices_h", GT_INT, 6L * Nc);
    int *adj_sign = add_array(T, "adjacent_signs_h", GT_INT, 6L * Nc);
    if (!from || !to || !vort_idx || !vort_sign || !from_dual || !to_dual || !adj || !adj_sign) FAIL("out of memory");
    e_tri = malloc((size_t)2 * Ne * sizeof(int));
    if (!e_tri || pm_init(&pm, 3L * Nt)) FAIL("out of memory");
    {
        int ne = 0;
        for (int t = 0; t < Nt; ++t)
            for (int j = 0; j < 3; ++j) {
                int a = tri[3 * t + j], b = tri[3 * t + (j + 1) % 3];
                int e = pm_get_or_put(&pm, a, b, ne);
                if (e < 0) {
                    from[ne] = a; to[ne] = b;
                    e_tri[2 * ne] = t; e_tri[2 * ne + 1] = -1;
                    ++ne;
                } else {
                    e_tri[2 * e + 1] = t;
                }
            }
        if (ne != Ne) FAIL("edge count %d != %d", ne, Ne);
        for (int e = 0; e < Ne; ++e)
            if (e_tri[2 * e + 1] < 0) FAIL("open edge %d", e);
    }
    /* adjacency (index.c:18-62): ascending edge index, +1 where the cell is
     * the edge's from cell; pentagons get a sixth slot of 0 / sign 0, as the
     * reference maps -1 to 0 on loading (set_grid_properties.c:196-203). */
    {
        int *cnt = calloc(Nc, sizeof(int));
        if (!cnt) FAIL("out of memory");
        for (int e = 0; e < Ne; ++e) {
            int f = from[e], g = to[e];
            if (cnt[f] >= 6 || cnt[g] >= 6) { free(cnt); FAIL("cell with more than six edges"); }
            adj[6 * f + cnt[f]] = e; adj_sign[6 * f + cnt[f]] = 1; cnt[f]++;
            adj[6 * g + cnt[g]] = e; adj_sign[6 * g + cnt[g]] = -1; cnt[g]++;
        }
        for (int c = 0; c < Nc; ++c) {
            int want = c < N_PENT ? 5 : 6;
            if (cnt[c] != want) { int got = cnt[c]; free(cnt); FAIL("cell %d has %d edges", c, got); }
            if (c < N_PENT) { adj[6 * c + 5] = 0; adj_sign[6 * c + 5] = 0; }
        }
        free(cnt);
    }
    /* triangle edges, ascending (miscellaneous.c:40-84) */
    {
        for (int t = 0; t < Nt; ++t) {
            int ev[3];
            for (int j = 0; j < 3; ++j) ev[j] = pm_get(&pm, tri[3 * t + j], tri[3 * t + (j + 1) % 3]);
            for (int a = 0; a < 3; ++a)
                for (int b = a + 1; b < 3; ++b)
                    if (ev[b] < ev[a]) { int s = ev[a]; ev[a] = ev[b]; ev[b] = s; }
            for (int j = 0; j < 3; ++j) vort_idx[3 * t + j] = ev[j];
        }
    }
    /* cell rings: triangles around each cell in counter-clockwise order and the
     * edge between ring triangle l and l+1 */
    ring_tri = malloc((size_t)6 * Nc * sizeof(int));
    ring_edge = malloc((size_t)6 * Nc * sizeof(int));
    ring_n = calloc(Nc, sizeof(int));
    if (!ring_tri || !ring_edge || !ring_n) FAIL("out of memory");
    {
        /* for each cell, store (x, y, t) of each incident triangle rotated to (c, x, y) */
        int *inc_x = malloc((size_t)6 * Nc * sizeof(int)), *inc_y = malloc((size_t)6 * Nc * sizeof(int));
        int *inc_t = malloc((size_t)6 * Nc * sizeof(int)), *inc_n = calloc(Nc, sizeof(int));
        if (!inc_x || !inc_y || !inc_t || !inc_n) { free(inc_x); free(inc_y); free(inc_t); free(inc_n); FAIL("out of memory"); }
        int bad = 0;
        for (int t = 0; t < Nt; ++t)
            for (int j = 0; j < 3; ++j) {
                int c = tri[3 * t + j], x = tri[3 * t + (j + 1) % 3], y = tri[3 * t + (j + 2) % 3];
                if (inc_n[c] >= 6) { bad = 1; continue; }
                inc_x[6 * c + inc_n[c]] = x; inc_y[6 * c + inc_n[c]] = y; inc_t[6 * c + inc_n[c]] = t;
                inc_n[c]++;
            }
        for (int c = 0; c < Nc && !bad; ++c) {
            int n = inc_n[c];
            if (n != (c < N_PENT ? 5 : 6)) { bad = 2; break; }
            int cur = 0;
            for (int l = 0; l < n; ++l) {
                ring_tri[6 * c + l] = inc_t[6 * c + cur];
                int y = inc_y[6 * c + cur];
                ring_edge[6 * c + l] = pm_get(&pm, c, y);
                int nxt = -1;
                for (int k = 0; k < n; ++k) if (inc_x[6 * c + k] == y) nxt = k;
                if (nxt < 0) { bad = 3; break; }
                cur = nxt;
            }
            if (cur != 0) bad = 4;
            ring_n[c] = n;
        }
        free(inc_x); free(inc_y); free(inc_t); free(inc_n);
        if (bad) FAIL("cell ring construction failed (%d)", bad);
    }

    /* ---- Lloyd iterations towards an SCVT (optimize.c:17-118) */
    circ = malloc((size_t)Nt * sizeof(v3));
    if (!circ) FAIL("out of memory");
    for (int it = 0; it <= n_lloyd; ++it) {
        #pragma omp parallel for schedule(static)
        for (int t = 0; t < Nt; ++t) {
            v3 a = X[tri[3 * t]], b = X[tri[3 * t + 1]], c = X[tri[3 * t + 2]];
            circ[t] = v3_unit(v3_cross(v3_sub(b, a), v3_sub(c, a)));
        }
        if (it == n_lloyd) break;
        #pragma omp parallel for schedule(static)
        for (int c = 0; c < Nc; ++c) {
            int n = ring_n[c];
            v3 acc = {0, 0, 0};
            for (int l = 0; l < n; ++l) {
                v3 p1 = circ[ring_tri[6 * c + l]], p2 = circ[ring_tri[6 * c + (l + 1) % n]];
                double w = sph_tri_area(X[c], p1, p2);
                acc = v3_add(acc, v3_scale(v3_add(v3_add(X[c], p1), p2), w));
            }
            X[c] = v3_unit(acc);
        }
    }

    /* ---- horizontal geometry */
    double *lat_c = add_array(T, "latitude_scalar", GT_DOUBLE, Nc);
    double *lon_c = add_array(T, "longitude_scalar", GT_DOUBLE, Nc);
    double *lat_e = add_array(T, "latitude_vector", GT_DOUBLE, Ne);
    double *lon_e = add_array(T, "longitude_vector", GT_DOUBLE, Ne);
    double *lat_t = add_array(T, "latitude_scalar_dual", GT_DOUBLE, Nt);
    double *lon_t = add_array(T, "longitude_scalar_dual", GT_DOUBLE, Nt);
    double *direction = add_array(T, "direction", GT_DOUBLE, Ne);
    double *direction_dual = add_array(T, "direction_dual", GT_DOUBLE, Ne);
    double *f_vec = add_array(T, "f_vec", GT_DOUBLE, 2L * Ne);
    double *cell_unit = add_array(T, "pent_hex_face_unity_sphere", GT_DOUBLE, Nc);
    double *tri_unit = add_array(T, "triangle_face_unit_sphere", GT_DOUBLE, Nt);
    double *oro = add_array(T, "oro", GT_DOUBLE, Nc);
    mid = malloc((size_t)Ne * sizeof(v3));
    if (!lat_c || !lon_c || !lat_e || !lon_e || !lat_t || !lon_t || !direction || !direction_dual || !f_vec
        || !cell_unit || !tri_unit || !oro || !mid) FAIL("out of memory");
    for (int c = 0; c < Nc; ++c) v3_to_geo(X[c], &lat_c[c], &lon_c[c]);
    if (latlon_tables(T, res_id, lat_c, lon_c, Nc)) FAIL("lat-lon interpolation tables: out of memory");
    for (int t = 0; t < Nt; ++t) v3_to_geo(circ[t], &lat_t[t], &lon_t[t]);
    int orth_bad = 0;
    for (int e = 0; e < Ne; ++e) {
        /* midpoint of the chord between the two cell centres (set_vector_h_doubles) */
        v3 m = v3_scale(v3_add(X[from[e]], X[to[e]]), 0.5);
        v3_to_geo(m, &lat_e[e], &lon_e[e]);
        mid[e] = v3_unit(m);
        direction[e] = chord_direction(X[from[e]], X[to[e]], mid[e]);
        /* dual orientation so that the dual direction is the normal turned
         * counter-clockwise by 90 degrees (direct_tangential_unity) */
        int ta = e_tri[2 * e], tb = e_tri[2 * e + 1];
        double rel = nearest_sample(lat_t[ta], lon_t[ta], lat_t[tb], lon_t[tb], lat_e[e], lon_e[e]);
        double dd = geodetic_direction(lat_t[ta], lon_t[ta], lat_t[tb], lon_t[tb], rel);
        if (turn_angle(direction[e], dd) * 180.0 / M_PI < -ORTH_CRITERION_DEG) {
            int s = ta; ta = tb; tb = s;
            rel = 1 - rel;
            dd = geodetic_direction(lat_t[ta], lon_t[ta], lat_t[tb], lon_t[tb], rel);
        }
        double ang = fabs(turn_angle(direction[e], dd) * 180.0 / M_PI);
        if (ang < ORTH_CRITERION_DEG || ang > 90 + (90 - ORTH_CRITERION_DEG)) orth_bad++;
        from_dual[e] = ta; to_dual[e] = tb;
        direction_dual[e] = dd;
        /* Coriolis vector (miscellaneous.c:18-38) */
        f_vec[e] = 2 * OMEGA_EARTH / radius_rescale * cos(lat_e[e]) * sin(direction_dual[e]);
        f_vec[Ne + e] = 2 * OMEGA_EARTH / radius_rescale * sin(lat_e[e]);
    }
    if (orth_bad) FAIL("grid non-orthogonal at %d edges", orth_bad);
    /* vorticity signs (miscellaneous.c:40-84): -1 where the triangle is the dual from point */
    for (int t = 0; t < Nt; ++t)
        for (int j = 0; j < 3; ++j) {
            int e = vort_idx[3 * t + j];
            if (from_dual[e] != t && to_dual[e] != t) FAIL("triangle/edge incidence broken");
            double chg = turn_angle(direction_dual[e], direction[e]) * 180.0 / M_PI;
            int sign = 1;
            if (from_dual[e] == t && chg < -ORTH_CRITERION_DEG) sign = -1;
            if (to_dual[e] == t && chg > ORTH_CRITERION_DEG) sign = -1;
            vort_sign[3 * t + j] = sign;
        }
    /* unit-sphere areas of triangles and cells, with the reference's sanity checks
     * (horizontal_generation.c:100-236) */
    {
        double sum_t = 0, sum_c = 0;
        for (int t = 0; t < Nt; ++t) {
            tri_unit[t] = sph_tri_area(X[tri[3 * t]], X[tri[3 * t + 1]], X[tri[3 * t + 2]]);
            sum_t += tri_unit[t];
        }
        for (int c = 0; c < Nc; ++c) {
            int n = ring_n[c];
            double a = 0;
            for (int l = 0; l < n; ++l)
                a += sph_tri_area(X[c], circ[ring_tri[6 * c + l]], circ[ring_tri[6 * c + (l + 1) % n]]);
            cell_unit[c] = a;
            sum_c += a;
        }
        if (fabs(sum_t / (4 * M_PI) - 1) > EPS_SECURITY) FAIL("triangle areas do not sum to the sphere");
        if (fabs(sum_c / (4 * M_PI) - 1) > EPS_SECURITY) FAIL("cell areas do not sum to the sphere");
        double ideal_c = 4 * M_PI / Nc, ideal_t = 4 * M_PI / Nt;
        for (int c = 0; c < Nc; ++c)
            if (cell_unit[c] <= 0 || fabs(cell_unit[c] / ideal_c - 1) > 0.4) FAIL("irregular cell area at %d", c);
        for (int t = 0; t < Nt; ++t)
            if (tri_unit[t] <= 0 || fabs(tri_unit[t] / ideal_t - 1) > 0.4) FAIL("irregular triangle area at %d", t);
    }

    /* ---- orography */
    if (oro_kind == 1) {
        double h0 = oro_params[0], hw = oro_params[1];
        v3 c0 = v3_from_geo(oro_params[2], oro_params[3]);
        for (int c = 0; c < Nc; ++c) {
            double d = radius * central_angle(X[c], c0);
            oro[c] = h0 * exp(-(d / hw) * (d / hw) * log(2.0));
        }
    }

    /* ---- vertical grid (vertical_grid.c:27-76) */
    double *z_scalar = add_array(T, "z_scalar", GT_DOUBLE, S);
    double *z_vector = add_array(T, "z_vector", GT_DOUBLE, Vt);
    double *nd = add_array(T, "normal_distance", GT_DOUBLE, Vt);
    double *area = add_array(T, "area", GT_DOUBLE, Vt);
    double *volume = add_array(T, "volume", GT_DOUBLE, S);
    double *z_scalar_dual = add_array(T, "z_scalar_dual", GT_DOUBLE, (long)(L + 1) * Nt);
    double *z_vector_dual = add_array(T, "z_vector_dual", GT_DOUBLE, Dv);
    double *nd_dual = add_array(T, "normal_distance_dual", GT_DOUBLE, Dv);
    double *area_dual = add_array(T, "area_dual", GT_DOUBLE, Dv);
    double *gravity_potential = add_array(T, "gravity_potential", GT_DOUBLE, S);
    double *theta_v_bg = add_array(T, "theta_v_bg", GT_DOUBLE, S);
    double *exner_bg = add_array(T, "exner_bg", GT_DOUBLE, S);
    double *ipw = add_array(T, "inner_product_weights", GT_DOUBLE, 8 * S);
    if (!z_scalar || !z_vector || !nd || !area || !volume || !z_scalar_dual || !z_vector_dual || !nd_dual
        || !area_dual || !gravity_potential || !theta_v_bg || !exner_bg || !ipw) FAIL("out of memory");
    {
        double max_oro = 0;
        for (int c = 0; c < Nc; ++c) if (oro[c] > max_oro) max_oro = oro[c];
        double *zpre = malloc((size_t)(L + 1) * sizeof(double));
        if (!zpre) FAIL("out of memory");
        for (int h = 0; h < Nc; ++h) {
            for (int j = 0; j < L + 1; ++j) {
                double z_rel = 1 - (j + 0.0) / L;
                double sigma_z = pow(z_rel, stretching);
                double A = sigma_z * toa, B;
                if (j >= L - n_oro_layers) B = (j - (L - n_oro_layers) + 0.0) / n_oro_layers;
                else B = 0;
                zpre[j] = A + B * oro[h];
            }
            if (h == 0 && max_oro >= zpre[L - n_oro_layers]) { free(zpre); FAIL("orography reaches the lowest flat level"); }
            for (int l = 0; l < L; ++l) z_scalar[(long)l * Nc + h] = 0.5 * (zpre[l] + zpre[l + 1]);
        }
        free(zpre);
    }
    /* z_vector and normal distances (vertical_grid.c:78-140) */
    for (long i = 0; i < Vt; ++i) {
        long layer = i / VPL, h = i - layer * VPL;
        if (h >= Nc) {
            int e = (int)(h - Nc);
            z_vector[i] = 0.5 * (z_scalar[layer * Nc + from[e]] + z_scalar[layer * Nc + to[e]]);
            nd[i] = (radius + z_vector[i]) * central_angle(X[from[e]], X[to[e]]);
        } else {
            long upper = h + (layer - 1) * Nc, lower = h + layer * Nc;
            if (layer == 0) {
                z_vector[i] = toa;
                nd[i] = toa - z_scalar[lower];
            } else if (layer == L) {
                z_vector[i] = oro[h];
                nd[i] = z_scalar[upper] - z_vector[i];
            } else {
                nd[i] = z_scalar[upper] - z_scalar[lower];
                z_vector[i] = z_scalar[lower] + 0.5 * nd[i];
            }
        }
    }
    /* dual z (vertical_grid.c:142-165, 240-281) */
    for (long i = 0; i < (long)(L + 1) * Nt; ++i) {
        long layer = i / Nt, h = i - layer * Nt;
        const int *vi = &vort_idx[3 * h];
        z_scalar_dual[i] = 1.0 / 6 * (z_vector[layer * VPL + from[vi[0]]] + z_vector[layer * VPL + from[vi[1]]]
                                      + z_vector[layer * VPL + from[vi[2]]] + z_vector[layer * VPL + to[vi[0]]]
                                      + z_vector[layer * VPL + to[vi[1]]] + z_vector[layer * VPL + to[vi[2]]]);
    }
    for (long i = 0; i < Dv; ++i) {
        long layer = i / DPL, h = i - layer * DPL;
        if (h >= Ne) {
            long t = h - Ne;
            long upper = t + layer * Nt, lower = t + (layer + 1) * Nt;
            nd_dual[i] = z_scalar_dual[upper] - z_scalar_dual[lower];
            const int *vi = &vort_idx[3 * t];
            z_vector_dual[i] = 1.0 / 3 * (z_vector[Nc + layer * VPL + vi[0]] + z_vector[Nc + layer * VPL + vi[1]]
                                          + z_vector[Nc + layer * VPL + vi[2]]);
        } else {
            int e = (int)h;
            if (layer == 0) z_vector_dual[i] = toa;
            else if (layer == L) z_vector_dual[i] = 0.5 * (z_vector[L * VPL + from[e]] + z_vector[L * VPL + to[e]]);
            else z_vector_dual[i] = 0.5 * (z_vector[Nc + e + (layer - 1) * VPL] + z_vector[Nc + e + layer * VPL]);
            nd_dual[i] = (radius + z_vector_dual[i]) * central_angle(circ[from_dual[e]], circ[to_dual[e]]);
        }
    }
    /* areas (vertical_grid.c:238-262 set_area, :200-236 set_area_dual) */
    for (long i = 0; i < Vt; ++i) {
        long layer = i / VPL, h = i - layer * VPL;
        if (h < Nc) {
            area[i] = cell_unit[h] * (radius + z_vector[i]) * (radius + z_vector[i]);
        } else {
            long dvi = (layer + 1) * DPL + h - Nc;
            double r0 = radius + z_vector_dual[dvi], r1 = radius + z_vector_dual[dvi - DPL];
            area[i] = nd_dual[dvi] * (0.5 * r1 * r1 / r0 - 0.5 * r0);
        }
    }
    for (long i = 0; i < Dv; ++i) {
        long layer = i / DPL, h = i - layer * DPL;
        if (h >= Ne) {
            area_dual[i] = (radius + z_vector_dual[i]) * (radius + z_vector_dual[i]) * tri_unit[h - Ne];
        } else {
            double r0, r1, base;
            if (layer == 0) {
                long p = Nc + h;
                r0 = radius + z_vector[p]; r1 = radius + toa; base = nd[p];
            } else if (layer == L) {
                long p = Nc + (long)(L - 1) * VPL + h;
                r0 = radius + 0.5 * (z_vector[(long)L * VPL + from[h]] + z_vector[(long)L * VPL + to[h]]);
                r1 = radius + z_vector[p];
                base = nd[p] * r0 / r1;
            } else {
                long p = Nc + layer * VPL + h;
                r0 = radius + z_vector[p]; r1 = radius + z_vector[p - VPL]; base = nd[p];
            }
            area_dual[i] = base * (0.5 * r1 * r1 / r0 - 0.5 * r0);
        }
    }
    /* volumes (vertical_grid.c:167-187) */
    for (long i = 0; i < S; ++i) {
        long layer = i / Nc, h = i - layer * Nc;
        double base_area = area[h + (layer + 1) * VPL];
        double r0 = radius + z_vector[h + (layer + 1) * VPL], r1 = radius + z_vector[h + layer * VPL];
        volume[i] = base_area / (3.0 * r0 * r0) * (r1 * r1 * r1 - r0 * r0 * r0);
    }
    /* gravity potential (gravity_potential.c:13-25) and background state
     * (vertical_grid.c:311-348) */
    for (long i = 0; i < S; ++i)
        gravity_potential[i] = -G_MEAN_SFC_ABS * (radius * radius / (radius + z_scalar[i]) - radius);
    for (int h = 0; h < Nc; ++h)
        for (int l = L - 1; l >= 0; --l) {
            long si = (long)l * Nc + h;
            double temperature = gt_standard_temp(z_scalar[si]);
            if (l == L - 1) {
                double pressure = gt_standard_pres(z_scalar[si]);
                exner_bg[si] = pow(pressure / P_0, R_D / C_D_P);
            } else {
                double t_below = gt_standard_temp(z_scalar[si + Nc]);
                double b = -0.5 * exner_bg[si + Nc] / t_below
                           * (temperature - t_below + 2.0 / C_D_P * (gravity_potential[si] - gravity_potential[si + Nc]));
                double c = exner_bg[si + Nc] * exner_bg[si + Nc] * temperature / t_below;
                exner_bg[si] = b + sqrt(b * b + c);
            }
            theta_v_bg[si] = temperature / exner_bg[si];
        }
    /* inner-product weights (inner_product.c:15-60) */
    for (long i = 0; i < S; ++i) {
        long layer = i / Nc, h = i - layer * Nc;
        for (int j = 0; j < 6; ++j) {
            if (j < 5 || h >= N_PENT) {
                long vi = Nc + layer * VPL + adj[6 * h + j];
                ipw[8 * i + j] = area[vi];
                ipw[8 * i + j] = ipw[8 * i + j] * nd[vi];
                ipw[8 * i + j] = ipw[8 * i + j] / (2 * volume[i]);
            } else {
                ipw[8 * i + j] = 0;
            }
        }
        double dz;
        if (layer == 0) dz = 2 * (z_vector[h] - z_scalar[i]);
        else dz = z_scalar[i - Nc] - z_scalar[i];
        ipw[8 * i + 6] = area[h + layer * VPL] * dz / (2 * volume[i]);
        if (layer == L - 1) dz = 2 * (z_scalar[i] - z_vector[(long)L * VPL + h]);
        else dz = z_scalar[i] - z_scalar[i + Nc];
        ipw[8 * i + 7] = area[h + (layer + 1) * VPL] * dz / (2 * volume[i]);
    }

    /* ---- rhombus interpolation (rhombus_averaging.c:16-273) */
    int *rho_idx = add_array(T, "density_to_rhombi_indices", GT_INT, 4L * Ne);
    double *rho_w = add_array(T, "density_to_rhombi_weights", GT_DOUBLE, 4L * Ne);
    if (!rho_idx || !rho_w) FAIL("out of memory");
    {
        int err = 0;
        const double rz2 = (radius + z_vector[Nc]) * (radius + z_vector[Nc]);
        #pragma omp parallel for schedule(static) reduction(|:err)
        for (int i = 0; i < Ne; ++i) {
            int pre[6], vir[4], dbl0 = -1, dbl1 = -1, cnt = 0;
            for (int j = 0; j < 3; ++j) pre[j] = vort_idx[3 * to_dual[i] + j];
            for (int j = 0; j < 3; ++j) pre[3 + j] = vort_idx[3 * from_dual[i] + j];
            for (int j = 0; j < 6; ++j)
                for (int k = j + 1; k < 6; ++k)
                    if (pre[j] == pre[k]) { dbl0 = j; dbl1 = k; }
            for (int j = 0; j < 6; ++j)
                if (j != dbl0 && j != dbl1 && cnt < 4) vir[cnt++] = pre[j];
            if (cnt != 4) { err |= 1; continue; }
            int di[4] = {-1, -1, -1, -1}, nd_ = 0;
            for (int j = 0; j < 4; ++j) {
                int cand[2] = {from[vir[j]], to[vir[j]]};
                for (int q = 0; q < 2; ++q) {
                    int found = 0;
                    for (int m = 0; m < 4; ++m) if (di[m] == cand[q]) found = 1;
                    if (!found && nd_ < 4) di[nd_++] = cand[q];
                }
            }
            if (nd_ != 4) { err |= 2; continue; }
            double rhombus_area = area_dual[Ne + from_dual[i]] + area_dual[Ne + to_dual[i]];
            int first_case = 0, second_case = 0;
            double check = 0;
            for (int j = 0; j < 4; ++j) {
                int d = di[j];
                rho_idx[4 * i + j] = d;
                /* first rhombus edge touching d, and the rhombus-interior dual point on it */
                int k0 = 0;
                while (k0 < 4 && from[vir[k0]] != d && to[vir[k0]] != d) ++k0;
                if (k0 == 4) { err |= 4; break; }
                int v0 = vir[k0];
                int dual0 = from_dual[v0], keep = 0;
                for (int l = 0; l < 4; ++l)
                    if (l != k0 && (from_dual[vir[l]] == dual0 || to_dual[vir[l]] == dual0)) keep = 1;
                if (!keep) dual0 = to_dual[v0];
                int k1 = 0;
                while (k1 < 4 && !((from[vir[k1]] == d || to[vir[k1]] == d) && vir[k1] != v0)) ++k1;
                if (k1 == 4) { err |= 8; break; }
                int v1 = vir[k1];
                double w;
                if (d == from[i] || d == to[i]) {
                    first_case++;
                    int dual1 = from_dual[v1];
                    keep = 0;
                    for (int l = 0; l < 4; ++l)
                        if (l != k1 && (from_dual[vir[l]] == dual1 || to_dual[vir[l]] == dual1)) keep = 1;
                    if (!keep) dual1 = to_dual[v1];
                    double t0 = sph_tri_area(X[d], circ[dual0], mid[v0]);
                    double t1 = sph_tri_area(X[d], circ[dual0], mid[i]);
                    double t2 = sph_tri_area(X[d], circ[dual1], mid[i]);
                    double t3 = sph_tri_area(X[d], circ[dual1], mid[v1]);
                    w = rz2 * (t0 + t1 + t2 + t3) / rhombus_area;
                } else {
                    second_case++;
                    double t0 = sph_tri_area(X[d], circ[dual0], mid[v0]);
                    double t1 = sph_tri_area(X[d], circ[dual0], mid[v1]);
                    w = rz2 * (t0 + t1) / rhombus_area;
                }
                rho_w[4 * i + j] = w;
                if (w <= 0 || w >= 1) err |= 16;
                check += w;
            }
            if (first_case != 2 || second_case != 2) err |= 32;
            if (fabs(check - 1) > EPS_SECURITY) err |= 64;
        }
        if (err) FAIL("rhombus interpolation failed (flags %d)", err);
    }

    /* ---- modified TRSK weights (coriolis.c:16-440) */
    int *trsk_idx = add_array(T, "trsk_indices", GT_INT, 10L * Ne);
    int *trsk_mci = add_array(T, "trsk_modified_curl_indices", GT_INT, 10L * Ne);
    double *trsk_w = add_array(T, "trsk_weights", GT_DOUBLE, 10L * Ne);
    if (!trsk_idx || !trsk_mci || !trsk_w) FAIL("out of memory");
    {
        const double rescale_1d = (radius + z_scalar[0]) / (radius + z_vector[0]);
        const double rescale_2d = rescale_1d * rescale_1d;
        int err = 0;
        #pragma omp parallel for schedule(static) reduction(|:err)
        for (int i = 0; i < Ne; ++i) {
            int offset = 0;
            for (int k = 0; k < 10; ++k) {
                if (k == 0 || k == 5) offset = 0;
                int index_offset = k < 5 ? 0 : 5;
                int sign_0 = k < 5 ? -1 : 1;
                int c = k < 5 ? from[i] : to[i];
                int ncell = c < N_PENT ? 5 : 6;
                int slot = k - index_offset;
                if (slot < 6 && slot < ncell && adj[6 * c + slot] == i) offset += 1;
                if (offset > 1) { err |= 1; break; }
                int pos = slot + offset;
                int e2 = (pos < ncell) ? adj[6 * c + pos] : -1;
                trsk_idx[10 * i + k] = e2;
                if (e2 == -1) { trsk_w[10 * i + k] = 0; continue; }
                int sign_1 = from[e2] == c ? 1 : -1;
                /* kites of cell c per vertex, counter-clockwise */
                double kite[6], check = 0;
                int last = -1, first = -1;
                const double rz2 = (radius + z_vector[Nc + i]) * (radius + z_vector[Nc + i]);
                for (int l = 0; l < ncell; ++l) {
                    v3 vl = circ[ring_tri[6 * c + l]];
                    int eprev = ring_edge[6 * c + (l + ncell - 1) % ncell], ecur = ring_edge[6 * c + l];
                    double a0 = sph_tri_area(X[c], vl, mid[eprev]);
                    double a1 = sph_tri_area(X[c], vl, mid[ecur]);
                    kite[l] = rz2 * (a0 + a1);
                    check += kite[l];
                }
                double cell_area = rescale_2d * area[c];
                if (fabs(check / cell_area - 1) > EPS_SECURITY) { err |= 2; break; }
                for (int l = 0; l < ncell; ++l) {
                    if (ring_edge[6 * c + l] == i) last = l;
                    if (ring_edge[6 * c + l] == e2) first = (l + 1) % ncell;
                }
                double sum = 0.0;
                if (first <= last) {
                    for (int l = first; l <= last; ++l) sum += kite[l];
                } else {
                    for (int l = first; l < ncell; ++l) sum += kite[l];
                    for (int l = 0; l <= last; ++l) sum += kite[l];
                }
                sum = sum / cell_area;
                if (sum < 0 || sum > 1) { err |= 4; break; }
                double w = sign_0 * (sum - 0.5) * sign_1;
                trsk_w[10 * i + k] = -rescale_1d * nd_dual[e2] / nd[Nc + i] * w;
            }
            if (err) continue;
            /* Gassmann (2018) re-sorting: walk the vertices of each cell starting
             * at the dual point on the far side of edge i */
            int pre_i[10];
            double pre_w[10];
            for (int j = 0; j < 10; ++j) { pre_i[j] = trsk_idx[10 * i + j]; pre_w[j] = trsk_w[10 * i + j]; }
            for (int side = 0; side < 2; ++side) {
                int c = side == 0 ? from[i] : to[i];
                int n = c < N_PENT ? 5 : 6;
                int base = side == 0 ? 0 : 5;
                int next_v = side == 0 ? to_dual[i] : from_dual[i];
                int used[6] = {0, 0, 0, 0, 0, 0}, n_used = 0;
                for (int j = 0; j < n - 1; ++j) {
                    int written = 0;
                    for (int k = 0; k < n - 1; ++k) {
                        int e2 = pre_i[base + k];
                        if (!written && !used[k] && (from_dual[e2] == next_v || to_dual[e2] == next_v)) {
                            trsk_idx[10 * i + base + j] = e2;
                            trsk_w[10 * i + base + j] = pre_w[base + k];
                            used[k] = 1; n_used++; written = 1;
                        }
                    }
                    int cur = trsk_idx[10 * i + base + j];
                    next_v = (to_dual[cur] == next_v) ? from_dual[cur] : to_dual[cur];
                }
                if (n_used != n - 1) err |= 8;
            }
            if (err) continue;
            int *mci = &trsk_mci[10 * i];
            const int *ti = &trsk_idx[10 * i];
            mci[0] = to[i] < N_PENT ? ti[8] : ti[9];
            mci[1] = ti[0];
            if (from[i] < N_PENT) {
                mci[2] = ti[3]; mci[3] = ti[5]; mci[4] = 0;
                if (trsk_w[10 * i + 4] != 0) err |= 16;
            } else {
                mci[2] = ti[2]; mci[3] = ti[4]; mci[4] = ti[5];
            }
            mci[5] = from[i] < N_PENT ? ti[3] : ti[4];
            mci[6] = ti[5];
            if (to[i] < N_PENT) {
                mci[7] = ti[8]; mci[8] = ti[0]; mci[9] = 0;
                if (trsk_w[10 * i + 9] != 0) err |= 32;
            } else {
                mci[7] = ti[7]; mci[8] = ti[9]; mci[9] = ti[0];
            }
        }
        if (err) FAIL("TRSK construction failed (flags %d)", err);
        /* energy-conservation check, Eq. (39) of Thuburn et al. (2009) (coriolis.c:405-430) */
        int bad = 0;
        for (int i = 0; i < Ne && !bad; ++i)
            for (int j = 0; j < 10; ++j) {
                int f = trsk_idx[10 * i + j];
                if (f == -1) continue;
                double v0 = nd[Nc + i] / (rescale_1d * nd_dual[f]) * trsk_w[10 * i + j];
                int second = -1;
                for (int k = 0; k < 10; ++k) if (trsk_idx[10 * f + k] == i) second = 10 * f + k;
                if (second == -1) { bad = 1; break; }
                double v1 = nd[Nc + f] / (rescale_1d * nd_dual[i]) * trsk_w[second];
                if (fabs(v0 + v1) > EPS_SECURITY) { bad = 2; break; }
            }
        if (bad) FAIL("TRSK antisymmetry check failed (%d)", bad);
        for (long i = 0; i < 10L * Ne; ++i) if (trsk_idx[i] == -1) trsk_idx[i] = 0;
    }

    /* ---- quantities the model derives on loading (set_grid_properties.c:205-252) */
    double *layer_thickness = add_array(T, "layer_thickness", GT_DOUBLE, S);
    double *slope = add_array(T, "slope", GT_DOUBLE, Vt);
    double *gravity_m = add_array(T, "gravity_m", GT_DOUBLE, Vt);
    double *exner_bg_grad = add_array(T, "exner_bg_grad", GT_DOUBLE, Vt);
    if (!layer_thickness || !slope || !gravity_m || !exner_bg_grad) FAIL("out of memory");
    for (long i = 0; i < S; ++i) {
        long layer = i / Nc, h = i - layer * Nc;
        layer_thickness[i] = z_vector[h + layer * VPL] - z_vector[h + (layer + 1) * VPL];
    }
    {
        grad_ctx g = {Nc, Ne, L, n_oro_layers, from, to, nd, ipw, slope};
        grad_hor_cov_h(&g, z_scalar, slope);
        grad_hor_cov_h(&g, gravity_potential, gravity_m);
        grad_vert_cov_h(&g, gravity_potential, gravity_m);
        hor_cov_to_con_h(&g, gravity_m);
        grad_hor_cov_h(&g, exner_bg, exner_bg_grad);
        grad_vert_cov_h(&g, exner_bg, exner_bg_grad);
        hor_cov_to_con_h(&g, exner_bg_grad);
    }

    free(X); free(circ); free(mid); free(tri); free(ring_tri); free(ring_edge); free(ring_n); free(e_tri);
    pm_free(&pm);
    return T;
fail:
    free(X); free(circ); free(mid); free(tri); free(ring_tri); free(ring_edge); free(ring_n); free(e_tri);
    if (pm.keys) pm_free(&pm);
    gt_free(T);
    return NULL;
}
