/*
 * Output diagnostics on the device mirrors: the fields write_out computes
 * (src/io/write_output.c:51-1513) and the operators only output uses
 * (src/io/spatial_ops_for_output.c, src/spatial_operators/averaging.c:
 * 135-234).  FP64, compiled with --fmad=false, every sum in the reference's
 * order; the transcendental functions (pow, log, exp, sin, cos) are CUDA's.
 *
 * Kernels of one output pass (all on the context's stream):
 *   k_out_cells       per grid box: temperature, pressure, relative humidity
 *   k_out_surface     per column: MSLP, surface pressure, 2 m temperature,
 *                     CAPE, short-wave down flux, cloud cover, precipitation
 *   k_out_wind10_e    per edge: mean lowest-layer wind over the output
 *                     interval, turned to u/v, extrapolated to 10 m
 *   k_out_wind10_c    per column: 10 m wind at the cell, gusts
 *   divv_h, calc_rel_vort, calc_pot_vort (the step's operator kernels)
 *   k_curl_to_cells, k_uv_at_edge, k_edges_to_cells   model-layer winds and
 *                     vorticity at the cells
 *   k_epv_theta, grad, k_epv_pv, k_inner_tangential, k_epv_round   EPV
 *   k_out_plevels     per column: the six pressure levels
 * and k_latlon for the lat-lon interpolation of any set of [Nc] fields.
 */
#include <algorithm>
#include <utility>
#include <vector>

#include "kernels.cuh"
#include "ops.h"
#include "output.h"

namespace game {

/* work arrays of the output pass, allocated on the first call */
struct OutBufs {
    double *t, *p, *rh, *epv, *relv, *divv, *uc, *vc;  /* [L][Nc] */
    double *ue, *ve;                                  /* [L][Ne] */
    double *rel, *pv;                                 /* curl fields */
    double *tri;                                      /* [L][Nt] */
    double *theta, *grad, *pvmod;                     /* [L][Nc], vector fields */
    double *surface;                                  /* 11 x [Nc] */
    double *plevels;                                  /* 7 x [6][Nc] */
    double *u10e, *v10e;                              /* [Ne] */
    double *in_sw, *in_tsoil, *in_mol, *in_rv, *in_v2; /* uploaded inputs */
    double *wind_lowest;                              /* [slots][Ne] */
    int wind_slots;
    double *ll_out;                                   /* lat-lon results */
    long long ll_cap;
    const double **ll_src;                            /* device array of field pointers */
    int ll_src_cap;
    double *ref_stage;                                /* reference-order staging, max(8 S, NV) */
    std::vector<void *> owned;
};

namespace {

using G = HGrid<double>;
constexpr double LAPSE = 0.0065;
constexpr double Z_TROPOPAUSE = 12e3;
constexpr double EPS_SEC = 1e-10;
constexpr double G_MEAN_SFC_ABS = 9.80616;

__device__ __forceinline__ double temperature_of(const VGrid &vg, const DState &s, int n_cond, int moist,
                                                 long long ns, long long i)
{
    /* temperature_diagnostics (src/constituents/derived_quantities.c:15-40) */
    double t = (vg.theta_v_bg[i] + s.theta_v_pert[i]) * (vg.exner_bg[i] + s.exner_pert[i]);
    if (moist) t = t / (1.0 + s.rho[(n_cond + 1) * ns + i] / s.rho[n_cond * ns + i] * (M_D / M_V - 1.0));
    return t;
}

__device__ __forceinline__ double gas_constant_of(const DState &s, int n_cond, int moist, long long ns, long long i)
{
    /* gas_constant_diagnostics (derived_quantities.c:42-61) */
    if (!moist) return R_D;
    double r = (s.rho[n_cond * ns + i] - s.rho[(n_cond + 1) * ns + i]) * R_D + s.rho[(n_cond + 1) * ns + i] * R_V;
    return r / s.rho[n_cond * ns + i];
}

__device__ __forceinline__ double rel_humidity(double abs_humidity, double temperature)
{
    /* derived_quantities.c:63-81 (water above T_0, ice at and below) */
    const double vapour_pressure = abs_humidity * R_V * temperature;
    double saturation_pressure = 0.0;
    if (temperature > T_0) saturation_pressure = sat_pressure_water(temperature);
    if (temperature <= T_0) saturation_pressure = sat_pressure_ice(temperature);
    return vapour_pressure / saturation_pressure;
}

__device__ __forceinline__ void passive_turn(double u_in, double v_in, double turn_angle, double *u_out,
                                             double *v_out)
{
    /* geodesy.c:206-223: the active turn by -turn_angle */
    const double a = -turn_angle;
    *u_out = cos(a) * u_in - sin(a) * v_in;
    *v_out = sin(a) * u_in + cos(a) * v_in;
}

/* tangential component at edge e of an edge field u of one layer
 * (averaging.c:135-150, TRSK weights in table order) */
__device__ __forceinline__ double tangential(const G &g, const double *u_layer, int e)
{
    double r = 0;
    for (int k = 0; k < 10; ++k) r += g.trsk_w[(long long)k * g.ne + e] * u_layer[g.trsk_i[(long long)k * g.ne + e]];
    return r;
}

/* per grid box: temperature, pressure, relative humidity in percent
 * (write_output.c:83, :732-741) */
__global__ void k_out_cells(VGrid vg, DState s, OutParams p, double *t, double *pr, double *rh)
{
    const long long ns = (long long)vg.nl * vg.nc, i = gtid();
    if (i >= ns) return;
    const double T = temperature_of(vg, s, p.n_cond, p.moist, ns, i);
    t[i] = T;
    rh[i] = p.n_const >= 4 ? 100.0 * rel_humidity(s.rho[(p.n_cond + 1) * ns + i], T) : 0.0;
    pr[i] = s.rho[p.n_cond * ns + i] * gas_constant_of(s, p.n_cond, p.moist, ns, i) * T;
}

/* pseudopotential temperature of the lowest layer (write_output.c:1680-1736,
 * Bolton 1980 in the moist case) */
__device__ double pseudopotential(const VGrid &vg, const DState &s, const OutParams &p, const double *t,
                                  long long ns, long long i)
{
    if (!p.moist) return vg.theta_v_bg[i] + s.theta_v_pert[i];
    const int nc_ = p.n_cond;
    const double T = t[i];
    const double rv = s.rho[(nc_ + 1) * ns + i];
    const double r = rv / (s.rho[nc_ * ns + i] - rv);
    const double alpha_1 = 0.2854 * (1.0 - 0.28e-3 * r);
    const double alpha_3 = r * (1.0 + 0.81e-3 * r);
    const double pressure = P_0 * pow(vg.exner_bg[i] + s.exner_pert[i], C_D_P / R_D);
    double saturation_pressure;
    if (T >= T_0) saturation_pressure = sat_pressure_water(T);
    else saturation_pressure = sat_pressure_ice(T);
    const double vapour_pressure = rv * R_V * T;
    const double rel_hum = vapour_pressure / saturation_pressure;
    const double t_lcl = 1.0 / (1.0 / (T - 55.0) - log(rel_hum) / 2840.0) + 55.0;
    const double alpha_2 = 3.376 / t_lcl - 0.00254;
    return T * pow(P_0 / pressure, alpha_1) * exp(alpha_2 * alpha_3);
}

struct SurfOut {
    double *mslp, *surface_p, *t2, *tcdc, *rprate, *sprate, *cape, *sfc_sw_down;
};

/* per column (write_output.c:100-211) */
__global__ void k_out_surface(G g, VGrid vg, OutGrid og, const double *layer_thickness, DState s, OutParams p,
                              const double *t, const double *sfc_sw_in, const double *t_soil, SurfOut o)
{
    const int nc = vg.nc, nl = vg.nl;
    const int i = (int)gtid();
    if (i >= nc) return;
    const long long ns = (long long)nl * nc, lo = (long long)(nl - 1) * nc + i;
    const double *zs = vg.z_scalar, *zv = vg.z_v;
    const double t_low = t[lo];
    const double rgas = gas_constant_of(s, p.n_cond, p.moist, ns, lo);
    const double pv = s.rho[p.n_cond * ns + lo] * rgas * t_low;
    const double gm = g.gravity_m_v[lo];
    const double t_mslp = t_low + LAPSE * zs[lo];
    o.mslp[i] = pv / pow(1 - (t_mslp - t_low) / t_mslp, gm / (rgas * LAPSE));
    const double z_sfc = zv[(long long)nl * nc + i];
    const double t_sfc = t_low + LAPSE * (zs[lo] - z_sfc);
    o.surface_p[i] = pv / pow(1.0 - (t_sfc - t_low) / t_sfc, gm / (rgas * LAPSE));
    /* 2 m temperature: the layer nearest to 2 m above the surface (first
     * index of the minimum) and its neighbour */
    int closest = 0;
    double best = fabs(z_sfc + 2 - zs[i]);
    for (int j = 1; j < nl; ++j) {
        const double d = fabs(z_sfc + 2 - zs[(long long)j * nc + i]);
        if (d < best) {
            best = d;
            closest = j;
        }
    }
    const double z_c = zs[(long long)closest * nc + i];
    const double temp_closest = t[(long long)closest * nc + i];
    const double delta_z_temp = z_sfc + 2 - z_c;
    double gradient;
    if (p.prog_soil_temp == 1) {
        gradient = (temp_closest - t_soil[i]) / (z_c - z_sfc);
    } else {
        int second = closest - 1;
        if (z_c > z_sfc + 2 && closest < nl - 1) second = closest + 1;
        gradient = (temp_closest - t[(long long)second * nc + i]) / (z_c - zs[(long long)second * nc + i]);
    }
    o.t2[i] = temp_closest + delta_z_temp * gradient;
    /* CAPE from the lowest layer up to the tropopause (stops at the top
     * layer where the reference would read above the model top) */
    double cape = 0.0;
    int layer = nl - 1;
    double z_height = zs[(long long)layer * nc + i];
    const double theta_e = pseudopotential(vg, s, p, t, ns, lo);
    while (z_height < Z_TROPOPAUSE) {
        const long long li = (long long)layer * nc + i;
        const double theta_v = vg.theta_v_bg[li] + s.theta_v_pert[li];
        const double delta_z = layer_thickness[li];
        const double integrand = g.gravity_m_v[li] * (theta_e - theta_v) / theta_v;
        if (integrand > 0.0) cape += integrand * delta_z;
        --layer;
        if (layer < 0) break;
        z_height = zs[(long long)layer * nc + i];
    }
    o.cape[i] = cape;
    o.sfc_sw_down[i] = sfc_sw_in[i] / (1.0 - og.sfc_albedo[i] + EPS_SEC);
    const double min_precip_rate = 0.01 / (1000.0 * 3600.0 / 1024.0);
    double tcdc = 0.0, sprate = 0.0, rprate = 0.0;
    if (p.n_cond == 4) {
        double cwc = 0.0;
        for (int k = 0; k < nl; ++k) {
            const long long ki = (long long)k * nc + i;
            if (zs[ki] < Z_TROPOPAUSE) cwc += (s.rho[2 * ns + ki] + s.rho[3 * ns + ki]) * (zv[ki] - zv[ki + nc]);
        }
        tcdc = fmin(10.0 * cwc, 1.0);
        tcdc = 100.0 * tcdc;
        if (tcdc < 0.5) tcdc = 0.0;
        sprate = p.snow_velocity * s.rho[lo];
        rprate = p.rain_velocity * s.rho[ns + lo];
    }
    if (rprate < min_precip_rate) rprate = 0.0;
    if (sprate < min_precip_rate) sprate = 0.0;
    o.tcdc[i] = tcdc;
    o.sprate[i] = sprate;
    o.rprate[i] = rprate;
}

/* per edge: the lowest-layer wind averaged over the output interval, turned
 * to eastward / northward and extrapolated to 10 m (write_output.c:213-285) */
__global__ void k_out_wind10_e(G g, VGrid vg, OutGrid og, const double *wl, int n_steps, double *u, double *v)
{
    const int ne = g.ne, nc = g.nc, nl = g.nl;
    const int h = (int)gtid();
    if (h >= ne) return;
    double mu = 0.0, mv = 0.0;
    for (int t = 0; t < n_steps; ++t) {
        const double *w = wl + (long long)t * ne;
        const double wt = tangential(g, w, h);
        mu += 1.0 / n_steps * w[h];
        mv += 1.0 / n_steps * wt;
    }
    double uu, vv;
    passive_turn(mu, mv, -og.direction[h], &uu, &vv);
    const int f = g.from[h], to = g.to[h];
    const double actual = 0.5 * (og.roughness_length[f] + og.roughness_length[to]);
    double extrapolation = 0.02;
    if (og.is_land[f] == 0) extrapolation = actual;
    const double z_sfc = 0.5 * (vg.z_v[(long long)nl * nc + f] + vg.z_v[(long long)nl * nc + to]);
    const double z_agl = g.z_h[(long long)(nl - 1) * ne + h] - z_sfc;
    const double rescale = log(10.0 / extrapolation) / log(z_agl / actual);
    u[h] = rescale * uu;
    v[h] = rescale * vv;
}

/* speed at a height above the surface from sqrt(v_squared) of the two layers
 * nearest to it (write_output.c:310-340) */
__device__ double speed_at(const VGrid &vg, const double *v2, int i, double height)
{
    const int nc = vg.nc, nl = vg.nl;
    const double *zs = vg.z_scalar;
    const double z_sfc = vg.z_v[(long long)nl * nc + i];
    int closest = 0;
    double best = fabs(zs[i] - (z_sfc + height));
    for (int j = 1; j < nl; ++j) {
        const double d = fabs(zs[(long long)j * nc + i] - (z_sfc + height));
        if (d < best) {
            best = d;
            closest = j;
        }
    }
    int second = closest - 1;
    const double z_c = zs[(long long)closest * nc + i];
    if (closest < nl - 1 && z_c - z_sfc > height) second = closest + 1;
    const double s_c = pow(v2[(long long)closest * nc + i], 0.5);
    return s_c + (s_c - pow(v2[(long long)second * nc + i], 0.5)) / (z_c - zs[(long long)second * nc + i])
                     * (z_sfc + height - z_c);
}

/* per column: 10 m wind at the cell (edges_to_cells_lowest_layer,
 * spatial_ops_for_output.c:199-225) and gusts (write_output.c:294-350) */
__global__ void k_out_wind10_c(G g, VGrid vg, OutParams p, const double *ue, const double *ve, const double *mol,
                               const double *rv, const double *v2, double *u10, double *v10, double *gusts)
{
    const int nc = g.nc, nl = g.nl;
    const int i = (int)gtid();
    if (i >= nc) return;
    const int n_edges = i < N_PENT ? 5 : 6;
    double u = 0, v = 0;
    for (int j = 0; j < n_edges; ++j) u += 0.5 * ipw_at(g, j, nl - 1, i) * ue[g.adj[(long long)j * nc + i]];
    for (int j = 0; j < n_edges; ++j) v += 0.5 * ipw_at(g, j, nl - 1, i) * ve[g.adj[(long long)j * nc + i]];
    u10[i] = u;
    v10[i] = v;
    const double speed = pow(pow(u, 2.0) + pow(v, 2.0), 0.5);
    if (p.gust_turbulence && fabs(mol[i]) > EPS_SEC) {
        double gust = speed + 7.71 * rv[i] * pow(fmax(1.0 - 0.5 / 12.0 * 1000.0 / mol[i], 0.0), 1.0 / 3.0);
        const double h850 = 8000.0 * log(1000.0 / 850.0), h950 = 8000.0 * log(1000.0 / 950.0);
        const double u850 = speed_at(vg, v2, i, h850), u950 = speed_at(vg, v2, i, h950);
        gust += 0.6 * fmax(0.0, u850 - u950);
        gusts[i] = fmin(gust, 3.0 * speed);
    } else {
        gusts[i] = 1.67 * speed;
    }
}

/* curl_field_to_cells (averaging.c:176-204) of the rhombus part zv [L][Ne] */
__global__ void k_curl_to_cells(G g, const double *zv, double *out)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const int n_edges = c < N_PENT ? 5 : 6;
    double r = 0;
    for (int j = 0; j < n_edges; ++j) r += 0.5 * ipw_at(g, j, l, c) * zv[(long long)l * g.ne + g.adj[(long long)j * g.nc + c]];
    out[i] = r;
}

/* edges_to_cells (averaging.c:206-234) of an edge field [L][Ne] */
__global__ void k_edges_to_cells(G g, const double *ue, double *out)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const int n_edges = c < N_PENT ? 5 : 6;
    double r = 0;
    for (int j = 0; j < n_edges; ++j) r += 0.5 * ipw_at(g, j, l, c) * ue[(long long)l * g.ne + g.adj[(long long)j * g.nc + c]];
    out[i] = r;
}

/* edges_to_cells_lowest_layer (spatial_ops_for_output.c:199-225) */
__global__ void k_edges_to_cells_lowest(G g, const double *ue, double *out)
{
    const int i = (int)gtid();
    if (i >= g.nc) return;
    const int n_edges = i < N_PENT ? 5 : 6;
    double r = 0;
    for (int j = 0; j < n_edges; ++j) r += 0.5 * ipw_at(g, j, g.nl - 1, i) * ue[g.adj[(long long)j * g.nc + i]];
    out[i] = r;
}

/* calc_uv_at_edge (averaging.c:152-174) of the horizontal wind u [L][Ne] */
__global__ void k_uv_at_edge(G g, OutGrid og, const double *u, double *ue, double *ve)
{
    const long long n = (long long)g.nl * g.ne, i = gtid();
    if (i >= n) return;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    const double w0 = u[i];
    const double w1 = tangential(g, u + (long long)l * g.ne, e);
    passive_turn(w0, w1, -og.direction[e], &ue[i], &ve[i]);
}

/* theta_v' with the background added in the top layer only, the field whose
 * gradient epv_diagnostics takes (spatial_ops_for_output.c:113-118) */
__global__ void k_epv_theta(VGrid vg, DState s, double *f)
{
    const long long ns = (long long)vg.nl * vg.nc, i = gtid();
    if (i >= ns) return;
    f[i] = i < vg.nc ? s.theta_v_pert[i] + vg.theta_v_bg[i] : s.theta_v_pert[i];
}

/* the state's theta_v' of the top layer as the reference leaves it:
 * (x + bg) - bg (spatial_ops_for_output.c:119-122) */
__global__ void k_epv_round(VGrid vg, DState s, const double *f)
{
    const int i = (int)gtid();
    if (i < vg.nc) s.theta_v_pert[i] = f[i] - vg.theta_v_bg[i];
}

/* the potential vorticity as a modified vector field: horizontal vorticity
 * interpolated to the horizontal vector points, vertical vorticity averaged
 * to the vertical vector points (spatial_ops_for_output.c:26-111); pv is a
 * curl field (tangential [L+1][Ne], rhombus [L][Ne]), out a vector field */
__global__ void k_epv_pv(G g, VGrid vg, const double *pzh, const double *pzv, double *out)
{
    const int nc = g.nc, ne = g.ne, nl = g.nl;
    const long long nw = (long long)(nl + 1) * nc, n = nw + (long long)nl * ne, i = gtid();
    if (i >= n) return;
    const double *zv = vg.z_v;
    if (i >= nw) {
        const long long ih = i - nw;
        const int l = (int)(ih / ne), e = (int)(ih - (long long)l * ne);
        const int f = g.from[e], t = g.to[e];
        const long long a = (long long)l * nc, b = (long long)(l + 1) * nc;
        const double zi = g.z_h[ih];
        const double lt = 0.5 * (zv[a + f] + zv[a + t]) - 0.5 * (zv[b + f] + zv[b + t]);
        double upper, lower;
        if (l == 0) upper = (0.5 * (zv[a + f] + zv[a + t]) - zi) / lt;
        else upper = 0.5 * (g.z_h[ih - ne] - zi) / lt;
        if (l == nl - 1) lower = (zi - 0.5 * (zv[b + f] + zv[b + t])) / lt;
        else lower = 0.5 * (zi - g.z_h[ih + ne]) / lt;
        out[i] = upper * pzh[(long long)l * ne + e] + lower * pzh[(long long)(l + 1) * ne + e];
    } else {
        const int k = (int)(i / nc), c = (int)(i - (long long)k * nc);
        double r = 0;
        if (k == 0) {
            for (int j = 0; j < 6; ++j) r += 0.5 * ipw_at(g, j, 0, c) * pzv[g.adj[(long long)j * nc + c]];
        } else if (k == nl) {
            const double *z = pzv + (long long)(nl - 1) * ne;
            for (int j = 0; j < 6; ++j) r += 0.5 * ipw_at(g, j, nl - 1, c) * z[g.adj[(long long)j * nc + c]];
        } else {
            const double *zu = pzv + (long long)(k - 1) * ne, *zl = pzv + (long long)k * ne;
            for (int j = 0; j < 6; ++j) r += 0.25 * ipw_at(g, j, k - 1, c) * zu[g.adj[(long long)j * nc + c]];
            for (int j = 0; j < 6; ++j) r += 0.25 * ipw_at(g, j, k, c) * zl[g.adj[(long long)j * nc + c]];
        }
        out[i] = r;
    }
}

/* inner_product_tangential (spatial_ops_for_output.c:137-166): a given in
 * tangential components, all six edge slots (weight 0 in a pentagon's
 * sixth) */
__global__ void k_inner_tangential(G g, const double *aw, const double *au, const double *bw, const double *bu,
                                   double *out)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const double *bl = bu + (long long)l * g.ne, *al = au + (long long)l * g.ne;
    double r = 0;
    for (int j = 0; j < 6; ++j) {
        const int a = g.adj[(long long)j * g.nc + c];
        const double tw = tangential(g, bl, a);
        r += ipw_at(g, j, l, c) * al[a] * tw;
    }
    r += ipw_at(g, 6, l, c) * aw[i] * bw[i];
    r += ipw_at(g, 7, l, c) * aw[i + g.nc] * bw[i + g.nc];
    out[i] = r;
}

struct PlOut {
    double *gh, *t, *rh, *epv, *u, *v, *relv;
};
struct PlIn {
    const double *p, *gpot, *t, *rh, *epv, *u, *v, *relv;
};

/* per column: vertical interpolation to the six pressure levels in ln p
 * between the layer nearest to the level and its neighbour, 9999 below the
 * lowest layer (write_output.c:766-825); out [6][Nc] */
__global__ void k_out_plevels(int nc, int nl, PlIn in, PlOut o)
{
    const int i = (int)gtid();
    if (i >= nc) return;
    const double levels[N_PRESSURE_LEVELS] = {20000, 30000, 50000, 70000, 85000, 92500};
    for (int j = 0; j < N_PRESSURE_LEVELS; ++j) {
        const double pl = levels[j];
        int closest = 0;
        double best = fabs(log(pl / in.p[i]));
        for (int k = 1; k < nl; ++k) {
            const double d = fabs(log(pl / in.p[(long long)k * nc + i]));
            if (d < best) {
                best = d;
                closest = k;
            }
        }
        int second = closest + 1;
        if (pl < in.p[(long long)closest * nc + i]) second = closest - 1;
        const long long oi = (long long)j * nc + i;
        if ((closest == nl - 1 && second == nl) || second < 0) {
            o.gh[oi] = o.t[oi] = o.rh[oi] = o.epv[oi] = o.relv[oi] = o.u[oi] = o.v[oi] = 9999;
        } else {
            const long long a = (long long)closest * nc + i, b = (long long)second * nc + i;
            const double w = 1 - best / (fabs(log(in.p[a] / in.p[b])) + EPS_SEC);
            o.gh[oi] = (w * in.gpot[a] + (1 - w) * in.gpot[b]) / G_MEAN_SFC_ABS;
            o.t[oi] = w * in.t[a] + (1 - w) * in.t[b];
            o.rh[oi] = w * in.rh[a] + (1 - w) * in.rh[b];
            o.epv[oi] = w * in.epv[a] + (1 - w) * in.epv[b];
            o.relv[oi] = w * in.relv[a] + (1 - w) * in.relv[b];
            o.u[oi] = w * in.u[a] + (1 - w) * in.u[b];
            o.v[oi] = w * in.v[a] + (1 - w) * in.v[b];
        }
    }
}

/* interpolate_to_ll (spatial_ops_for_output.c:168-197) of field
 * blockIdx.y: inverse-distance weights of the five nearest cells; a 9999
 * (missing) among them makes the point missing */
__global__ void k_latlon(OutGrid og, const double *const *src, double *dst)
{
    const long long n = og.n_ll, i = gtid();
    if (i >= n) return;
    const double *in = src[blockIdx.y];
    double r = 0;
    for (int j = 0; j < 5; ++j) {
        const double v = in[og.ll_idx[(long long)j * n + i]];
        if (v != 9999) {
            r += og.ll_w[(long long)j * n + i] * v;
        } else {
            r = 9999;
            break;
        }
    }
    dst[(long long)blockIdx.y * n + i] = r;
}

/* reference order <-> device order */
__global__ void k_cells_to_ref(const int *c_n2o, int nc, long long n, const double *src, double *dst)
{
    const long long i = gtid();
    if (i >= n) return;
    const long long k = i / nc;
    const int c = (int)(i - k * nc);
    dst[k * nc + c_n2o[c]] = src[i];
}

__global__ void k_levels_to_ref(const int *c_n2o, int nc, const double *src, double *dst)
{
    const long long i = gtid();
    if (i >= (long long)N_PRESSURE_LEVELS * nc) return;
    const int j = (int)(i / nc), c = (int)(i - (long long)j * nc);
    dst[(long long)c_n2o[c] * N_PRESSURE_LEVELS + j] = src[i];
}

__global__ void k_from_ref(const int *n2o, int n1, long long n, const double *src, double *dst)
{
    const long long i = gtid();
    if (i >= n) return;
    const long long k = i / n1;
    const int x = (int)(i - k * n1);
    dst[i] = src[k * n1 + n2o[x]];
}

inline unsigned nb(long long n, int bs = 256) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

/* ----------------------------------------------------------- buffers */
static void release_obuf(Context *c)
{
    if (!c->obuf) return;
    for (void *p : c->obuf->owned) cudaFree(p);
    delete c->obuf;
    c->obuf = nullptr;
}

template <typename T>
static T *oalloc(OutBufs *b, long long n)
{
    void *p = nullptr;
    if (cudaMalloc(&p, (size_t)(n > 0 ? n : 1) * sizeof(T)) != cudaSuccess) return nullptr;
    b->owned.push_back(p);
    return (T *)p;
}

static OutBufs *ensure_obuf(Context *c)
{
    if (c->obuf) return c->obuf;
    OutBufs *b = new OutBufs{};
    c->obuf = b;
    c->obuf_release = release_obuf;
    const long long S = c->ns, E = (long long)c->nl * c->ne, NC = c->nc;
    bool ok = true;
    auto A = [&](double *&p, long long n) {
        p = oalloc<double>(b, n);
        ok = ok && p;
    };
    A(b->t, S); A(b->p, S); A(b->rh, S); A(b->epv, S); A(b->relv, S); A(b->divv, S); A(b->uc, S); A(b->vc, S);
    A(b->ue, E); A(b->ve, E);
    A(b->rel, c->ncurl); A(b->pv, c->ncurl); A(b->tri, (long long)c->nl * c->nt);
    A(b->theta, S); A(b->grad, c->nv); A(b->pvmod, c->nv);
    A(b->surface, 11 * NC); A(b->plevels, 7LL * N_PRESSURE_LEVELS * NC);
    A(b->u10e, c->ne); A(b->v10e, c->ne);
    A(b->in_sw, NC); A(b->in_tsoil, NC); A(b->in_mol, NC); A(b->in_rv, NC); A(b->in_v2, S);
    A(b->ref_stage, std::max<long long>(8 * S, c->nv));
    if (!ok) {
        release_obuf(c);
        fail("output diagnostics: out of device memory");
        return nullptr;
    }
    return b;
}

/* ----------------------------------------------------------- operators */
void op_uv_at_edge(Context *c, const double *u, double *ue, double *ve)
{
    k_uv_at_edge<<<nb((long long)c->nl * c->ne), 256, 0, c->stream>>>(c->hg64, c->og, u, ue, ve);
    c->kernel_launches++;
}

void op_edges_to_cells(Context *c, const double *ue, double *out)
{
    k_edges_to_cells<<<nb(c->ns), 256, 0, c->stream>>>(c->hg64, ue, out);
    c->kernel_launches++;
}

void op_curl_to_cells(Context *c, const double *zv, double *out)
{
    k_curl_to_cells<<<nb(c->ns), 256, 0, c->stream>>>(c->hg64, zv, out);
    c->kernel_launches++;
}

void op_edges_to_cells_lowest(Context *c, const double *ue, double *out)
{
    k_edges_to_cells_lowest<<<nb(c->nc, 128), 128, 0, c->stream>>>(c->hg64, ue, out);
    c->kernel_launches++;
}

void op_inner_product_tangential(Context *c, const double *a, const double *b, double *out)
{
    const long long off = (long long)(c->nl + 1) * c->nc;
    k_inner_tangential<<<nb(c->ns), 256, 0, c->stream>>>(c->hg64, a, a + off, b, b + off, out);
    c->kernel_launches++;
}

int op_epv(Context *c, const double *pot_vort, DState s, double *epv)
{
    OutBufs *b = ensure_obuf(c);
    if (!b) return -1;
    const long long coff = (long long)(c->nl + 1) * c->ne;
    k_epv_pv<<<nb(c->nv), 256, 0, c->stream>>>(c->hg64, c->vg, pot_vort, pot_vort + coff, b->pvmod);
    k_epv_theta<<<nb(c->ns), 256, 0, c->stream>>>(c->vg, s, b->theta);
    /* the gradient leaves the top and surface levels untouched: zero, as
     * the reference's calloc'd work array */
    CK(cudaMemsetAsync(b->grad, 0, (size_t)c->nv * sizeof(double), c->stream));
    op_grad(c, b->theta, b->grad, OP_GRAD_H | OP_GRAD_V | OP_GRAD_CON);
    op_inner_product_tangential(c, b->pvmod, b->grad, epv);
    k_epv_round<<<nb(c->nc, 128), 128, 0, c->stream>>>(c->vg, s, b->theta);
    c->kernel_launches += 3;
    CK(cudaGetLastError());
    return 0;
}

/* ------------------------------------------------------- the output pass */
int output_fields(Context *c, StateMirror *sm, const OutParams &p, const OutInputs &in, const OutFields &f)
{
    OutBufs *b = ensure_obuf(c);
    if (!b) return -1;
    const DState s = sm->ds;
    const long long S = c->ns;
    cudaStream_t st = c->stream;
    double *T = f.temperature, *P = f.pressure, *RH = f.rh;
    {
        ProfScope ps(c, "out_cells");
        k_out_cells<<<nb(S), 256, 0, st>>>(c->vg, s, p, T, P, RH);
    }
    SurfOut so{f.mslp, f.surface_p, f.t2, f.tcdc, f.rprate, f.sprate, f.cape, f.sfc_sw_down};
    {
        ProfScope ps(c, "out_surface");
        k_out_surface<<<nb(c->nc, 128), 128, 0, st>>>(c->hg64, c->vg, c->og, c->dg64.layer_thickness, s, p, T,
                                                       in.sfc_sw_in, in.temperature_soil, so);
    }
    {
        ProfScope ps(c, "out_wind10");
        k_out_wind10_e<<<nb(c->ne), 256, 0, st>>>(c->hg64, c->vg, c->og, in.wind_lowest, p.n_wind_steps, b->u10e,
                                                  b->v10e);
        k_out_wind10_c<<<nb(c->nc, 128), 128, 0, st>>>(c->hg64, c->vg, p, b->u10e, b->v10e, in.monin_obukhov_length,
                                                        in.roughness_velocity, in.v_squared, f.u10, f.v10, f.gusts);
    }
    c->kernel_launches += 4;
    /* model layers: divergence, relative vorticity, winds at the cells */
    {
        ProfScope ps(c, "out_divv_vort");
        op_divv(c, s.w, nullptr, nullptr, f.divv_h, 0);
        op_rel_vort(c, s.w, b->tri, b->rel);
        op_curl_to_cells(c, b->rel + (long long)(c->nl + 1) * c->ne, f.rel_vort);
    }
    {
        ProfScope ps(c, "out_uv");
        op_uv_at_edge(c, s.u, b->ue, b->ve);
        op_edges_to_cells(c, b->ue, f.u);
        op_edges_to_cells(c, b->ve, f.v);
    }
    /* Ertel's potential vorticity from the potential vorticity of the dry
     * air density */
    {
        ProfScope ps(c, "out_epv");
        op_pot_vort(c, b->rel, s.rho + (long long)p.n_cond * S, b->pv);
        if (op_epv(c, b->pv, s, f.epv)) return -1;
    }
    PlIn pi{P, c->gravity_potential, T, RH, f.epv, f.u, f.v, f.rel_vort};
    PlOut po{f.geopotential_height, f.t_pl, f.rh_pl, f.epv_pl, f.u_pl, f.v_pl, f.rel_vort_pl};
    {
        ProfScope ps(c, "out_plevels");
        k_out_plevels<<<nb(c->nc, 128), 128, 0, st>>>(c->nc, c->nl, pi, po);
    }
    c->kernel_launches++;
    CK(cudaGetLastError());
    return 0;
}

int output_latlon(Context *c, const double *const *src, int n_fields, double *dst)
{
    if (!c->og.ll_ok) return fail("lat-lon output: the grid's latlon_interpol_indices are out of range");
    if (n_fields < 1 || n_fields > 65535) return fail("lat-lon output: field count out of range");
    dim3 grid(nb(c->og.n_ll), (unsigned)n_fields);
    ProfScope ps(c, "out_latlon");
    k_latlon<<<grid, 256, 0, c->stream>>>(c->og, src, dst);
    c->kernel_launches++;
    CK(cudaGetLastError());
    return 0;
}

void output_to_reference_cells(Context *c, const double *src, int n_slices, double *dst)
{
    const long long n = (long long)n_slices * c->nc;
    k_cells_to_ref<<<nb(n), 256, 0, c->stream>>>(c->og.c_n2o, c->nc, n, src, dst);
    c->kernel_launches++;
}

void output_to_reference_levels(Context *c, const double *src, double *dst)
{
    k_levels_to_ref<<<nb((long long)N_PRESSURE_LEVELS * c->nc), 256, 0, c->stream>>>(c->og.c_n2o, c->nc, src, dst);
    c->kernel_launches++;
}

void output_from_reference(Context *c, const double *src, int n_slices, int edges, double *dst)
{
    const int n1 = edges ? c->ne : c->nc;
    const long long n = (long long)n_slices * n1;
    k_from_ref<<<nb(n), 256, 0, c->stream>>>(edges ? c->og.e_n2o : c->og.c_n2o, n1, n, src, dst);
    c->kernel_launches++;
}


/* ------------------------------------------------- host orchestration */
/* uploads n_slices reference-order slices of cells or edges into dst
 * (device order) through the reference-order staging array */
static int upload_slices(Context *c, OutBufs *b, const double *host, int n_slices, int edges, double *dst)
{
    const long long n = (long long)n_slices * (edges ? c->ne : c->nc);
    if (n > std::max<long long>(8 * c->ns, c->nv)) return fail("output diagnostics: input larger than staging");
    CK(cudaMemcpyAsync(b->ref_stage, host, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    c->h2d_bytes += n * (long long)sizeof(double);
    output_from_reference(c, b->ref_stage, n_slices, edges, dst);
    return 0;
}

static int ensure_wind_slots(Context *c, OutBufs *b, int n)
{
    if (n <= b->wind_slots) return 0;
    int want = std::max(n, std::min(2 * b->wind_slots, MAX_WIND_SLOTS));
    double *p = oalloc<double>(b, (long long)want * c->ne);
    if (!p) return fail("output diagnostics: out of device memory (wind slots)");
    if (b->wind_slots)
        CK(cudaMemcpyAsync(p, b->wind_lowest, (size_t)b->wind_slots * c->ne * sizeof(double),
                           cudaMemcpyDeviceToDevice, c->stream));
    b->wind_lowest = p;  /* the old array stays owned until release */
    b->wind_slots = want;
    return 0;
}

int output_record_wind(Context *c, StateMirror *s, int slot)
{
    if (slot < 0 || slot >= MAX_WIND_SLOTS) return fail("wind slot out of range (0..4095)");
    OutBufs *b = ensure_obuf(c);
    if (!b) return -1;
    if (ensure_wind_slots(c, b, slot + 1)) return -1;
    CK(cudaMemcpyAsync(b->wind_lowest + (long long)slot * c->ne, s->ds.u + (long long)(c->nl - 1) * c->ne,
                       (size_t)c->ne * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    return 0;
}

namespace {
/* the 27 field pointers of game_gpu_output_fields in declaration order, and
 * where each lives: 0 surface [Nc], 1 model layers [L][Nc], 2 pressure
 * levels [6][Nc], 3 vertical wind [L+1][Nc] (lat-lon only) */
constexpr int N_OUT = 27;
constexpr int OUT_KIND[N_OUT] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 2, 3};
void out_ptrs(const struct game_gpu_output_fields *o, double *p[N_OUT])
{
    double *const src[N_OUT] = {o->mslp, o->surface_p, o->t2, o->tcdc, o->rprate, o->sprate, o->cape, o->sfc_sw_down,
                                o->u10, o->v10, o->gusts, o->temperature, o->pressure, o->rh, o->u, o->v,
                                o->rel_vort, o->divv_h, o->epv, o->geopotential_height, o->t_pl, o->rh_pl,
                                o->epv_pl, o->u_pl, o->v_pl, o->rel_vort_pl, o->w};
    for (int k = 0; k < N_OUT; ++k) p[k] = src[k];
}
}  // namespace

int output_run(Context *c, StateMirror *sm, const OutParams &p, const OutHost &h,
               const struct game_gpu_output_fields *native, const struct game_gpu_output_fields *latlon)
{
    OutBufs *b = ensure_obuf(c);
    if (!b) return -1;
    const long long NC = c->nc, S = c->ns, NLL = c->og.n_ll;
    const int nl = c->nl;
    /* inputs */
    if (upload_slices(c, b, h.sfc_sw_in, 1, 0, b->in_sw)) return -1;
    if (p.prog_soil_temp && upload_slices(c, b, h.temperature_soil, 1, 0, b->in_tsoil)) return -1;
    if (p.gust_turbulence) {
        if (upload_slices(c, b, h.monin_obukhov_length, 1, 0, b->in_mol)) return -1;
        if (upload_slices(c, b, h.roughness_velocity, 1, 0, b->in_rv)) return -1;
        if (upload_slices(c, b, h.v_squared, nl, 0, b->in_v2)) return -1;
    }
    if (p.n_wind_steps < 1) return fail("min_no_of_output_steps must be at least 1");
    if (h.wind_lowest) {
        if (p.n_wind_steps > MAX_WIND_SLOTS) return fail("min_no_of_output_steps above 4096");
        if (ensure_wind_slots(c, b, p.n_wind_steps)) return -1;
        for (int t0 = 0; t0 < p.n_wind_steps; t0 += 8) {
            const int n = std::min(8, p.n_wind_steps - t0);
            if (upload_slices(c, b, h.wind_lowest + (long long)t0 * c->ne, n, 1, b->wind_lowest + (long long)t0 * c->ne))
                return -1;
        }
    } else if (p.n_wind_steps > b->wind_slots) {
        return fail("wind_h_lowest_layer_array is NULL and fewer wind slots were recorded than min_no_of_output_steps");
    }
    /* the fields, device order */
    OutFields f;
    double *sf = b->surface, *pl = b->plevels;
    f.mslp = sf; f.surface_p = sf + NC; f.t2 = sf + 2 * NC; f.tcdc = sf + 3 * NC; f.rprate = sf + 4 * NC;
    f.sprate = sf + 5 * NC; f.cape = sf + 6 * NC; f.sfc_sw_down = sf + 7 * NC; f.u10 = sf + 8 * NC;
    f.v10 = sf + 9 * NC; f.gusts = sf + 10 * NC;
    f.temperature = b->t; f.pressure = b->p; f.rh = b->rh; f.u = b->uc; f.v = b->vc; f.rel_vort = b->relv;
    f.divv_h = b->divv; f.epv = b->epv;
    const long long PL = (long long)N_PRESSURE_LEVELS * NC;
    f.geopotential_height = pl; f.t_pl = pl + PL; f.rh_pl = pl + 2 * PL; f.epv_pl = pl + 3 * PL;
    f.u_pl = pl + 4 * PL; f.v_pl = pl + 5 * PL; f.rel_vort_pl = pl + 6 * PL;
    OutInputs in{b->in_sw, b->in_tsoil, b->in_mol, b->in_rv, b->in_v2, b->wind_lowest};
    if (output_fields(c, sm, p, in, f)) return -1;
    const double *dev[N_OUT] = {f.mslp, f.surface_p, f.t2, f.tcdc, f.rprate, f.sprate, f.cape, f.sfc_sw_down,
                                f.u10, f.v10, f.gusts, f.temperature, f.pressure, f.rh, f.u, f.v, f.rel_vort,
                                f.divv_h, f.epv, f.geopotential_height, f.t_pl, f.rh_pl, f.epv_pl, f.u_pl,
                                f.v_pl, f.rel_vort_pl, sm->ds.w};
    /* native grid: reference order through the staging array */
    if (native) {
        double *hp[N_OUT];
        out_ptrs(native, hp);
        for (int k = 0; k < N_OUT; ++k) {
            if (!hp[k] || OUT_KIND[k] == 3) continue;
            long long n;
            if (OUT_KIND[k] == 2) {
                output_to_reference_levels(c, dev[k], b->ref_stage);
                n = PL;
            } else {
                const int slices = OUT_KIND[k] == 1 ? nl : 1;
                output_to_reference_cells(c, dev[k], slices, b->ref_stage);
                n = slices * NC;
            }
            CK(cudaMemcpyAsync(hp[k], b->ref_stage, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
            c->d2h_bytes += n * (long long)sizeof(double);
        }
        (void)S;
    }
    /* lat-lon: one launch over every requested horizontal slice */
    if (latlon) {
        double *hp[N_OUT];
        out_ptrs(latlon, hp);
        std::vector<const double *> src;
        std::vector<std::pair<double *, long long>> dst; /* host array, slices */
        for (int k = 0; k < N_OUT; ++k) {
            if (!hp[k]) continue;
            const int kind = OUT_KIND[k];
            const int slices = kind == 0 ? 1 : kind == 1 ? nl : kind == 2 ? N_PRESSURE_LEVELS : nl + 1;
            for (int j = 0; j < slices; ++j) src.push_back(dev[k] + (long long)j * NC);
            dst.push_back({hp[k], slices});
        }
        const int n_fields = (int)src.size();
        if (n_fields > 0) {
            if ((long long)n_fields * NLL > b->ll_cap) {
                double *o = oalloc<double>(b, (long long)n_fields * NLL);
                if (!o) return fail("output diagnostics: out of device memory (lat-lon fields)");
                b->ll_out = o;
                b->ll_cap = (long long)n_fields * NLL;
            }
            if (n_fields > b->ll_src_cap) {
                const double **q = oalloc<const double *>(b, n_fields);
                if (!q) return fail("output diagnostics: out of device memory (lat-lon field table)");
                b->ll_src = q;
                b->ll_src_cap = n_fields;
            }
            CK(cudaMemcpyAsync(b->ll_src, src.data(), src.size() * sizeof(const double *), cudaMemcpyHostToDevice,
                               c->stream));
            if (output_latlon(c, b->ll_src, n_fields, b->ll_out)) return -1;
            long long at = 0;
            for (auto &d : dst) {
                const long long n = d.second * NLL;
                CK(cudaMemcpyAsync(d.first, b->ll_out + at, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost,
                                   c->stream));
                c->d2h_bytes += n * (long long)sizeof(double);
                at += n;
            }
        }
    }
    return 0;
}


int output_upload_edges(Context *c, const double *host, int n_slices, double *dev)
{
    OutBufs *b = ensure_obuf(c);
    if (!b) return -1;
    return upload_slices(c, b, host, n_slices, 1, dev);
}

int output_latlon_host(Context *c, const double *dev_field, double *host_out)
{
    OutBufs *b = ensure_obuf(c);
    if (!b) return -1;
    if (b->ll_cap < c->og.n_ll) {
        double *o = oalloc<double>(b, c->og.n_ll);
        if (!o) return fail("output diagnostics: out of device memory (lat-lon field)");
        b->ll_out = o;
        b->ll_cap = c->og.n_ll;
    }
    if (b->ll_src_cap < 1) {
        const double **q = oalloc<const double *>(b, 1);
        if (!q) return fail("output diagnostics: out of device memory (lat-lon field table)");
        b->ll_src = q;
        b->ll_src_cap = 1;
    }
    CK(cudaMemcpyAsync(b->ll_src, &dev_field, sizeof(const double *), cudaMemcpyHostToDevice, c->stream));
    if (output_latlon(c, b->ll_src, 1, b->ll_out)) return -1;
    CK(cudaMemcpyAsync(host_out, b->ll_out, (size_t)c->og.n_ll * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    c->d2h_bytes += c->og.n_ll * (long long)sizeof(double);
    return 0;
}

}  // namespace game
