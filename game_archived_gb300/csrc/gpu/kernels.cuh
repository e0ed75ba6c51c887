/*
 * RKHEVI step kernels.
 *
 * Every device function restates one reference operator at one point and
 * keeps the reference's order of floating-point operations, so that the FP64
 * instantiation (compiled with --fmad=false) rounds like the reference C.
 * Horizontal operators are templated on R: double on the FP64 path, float on
 * the mixed path, where the prognostic state, the vertical solves and the
 * density/mass-flux divergence accumulation stay in double.
 *
 * Kernels of one RK substage (src/time_stepping/manage_rkhevi.c:48-97):
 *   k_cell_prepare      T, theta_v, moist phase-transition rates (once per step)
 *   k_tri_vort          vertical relative vorticity on triangles        (rk 1)
 *   k_edge_vort         rhombus / tangential potential vorticity, mass flux (rk 1)
 *   k_cell_kinetic      kinetic energy, vertical mass flux               (rk 1)
 *   k_momentum_h        pressure gradient + vorticity flux + KE gradient
 *                       -> horizontal tendency and wind update
 *   k_momentum_v        the same for w at the interfaces
 *   k_scalar_tend       mass / rho*theta_v flux divergences -> tendencies
 * The implicit vertical column solves (sound waves, tracer advection and
 * sedimentation) are in solvers.cuh.
 */
#pragma once

#include <cuda_runtime.h>

#include "devgrid.cuh"
#include "dfloat.cuh"
#include "numeric.cuh"

namespace game {
/* internal linkage: the FP64 and the mixed translation unit each compile
 * their own copy with their own contraction flags */
namespace {

template <typename R>
__device__ __forceinline__ R ipw_at(const HGrid<R> &g, int j, int l, int c)
{
    return g.ipw[((long long)j * g.nl + l) * g.nc + c];
}

/* vertical covariant gradient of a cell field at an inner interface k
 * (src/spatial_operators/gradient_operators.c:35-54) */
template <typename R, typename F>
__device__ __forceinline__ R grad_v(const HGrid<R> &g, const F *f, int k, int c)
{
    return (R(f[(long long)(k - 1) * g.nc + c]) - R(f[(long long)k * g.nc + c])) / g.nd_v[(long long)k * g.nc + c];
}

/* horizontal gradient at edge e of layer l, with the terrain-following
 * covariant -> contravariant correction in the orography layers
 * (gradient_operators.c:14-33, averaging.c:14-39 and :113-133) */
template <typename R, typename F>
__device__ __forceinline__ R grad_h(const HGrid<R> &g, const F *f, int l, int e)
{
    const int fr = g.from[e], to = g.to[e];
    const long long le = (long long)l * g.ne + e;
    R out = (R(f[(long long)l * g.nc + to]) - R(f[(long long)l * g.nc + fr])) / g.nd_h[le];
    if (l >= g.nl - g.n_oro) {
        /* a zero slope adds -0: the mixed path skips it */
        if (sizeof(R) == sizeof(float) && g.slope_h[le] == R(0)) return out;
        R c = ipw_at(g, 6, l, fr) * grad_v(g, f, l, fr);
        c += ipw_at(g, 6, l, to) * grad_v(g, f, l, to);
        if (l < g.nl - 1) {
            c += ipw_at(g, 7, l, fr) * grad_v(g, f, l + 1, fr);
            c += ipw_at(g, 7, l, to) * grad_v(g, f, l + 1, to);
        }
        c = R(0.5) * c;
        out += -g.slope_h[le] * c;
    }
    return out;
}

/* horizontal covariant wind component (averaging.c:97-111) */
template <typename R, typename F>
__device__ __forceinline__ R hor_covariant(const HGrid<R> &g, const F *u, const F *w, int l, int e)
{
    const long long le = (long long)l * g.ne + e;
    R r = R(u[le]);
    if (l >= g.nl - g.n_oro) {
        const R slope = g.slope_h[le];
        /* a zero slope adds 0: the mixed path skips it */
        if (sizeof(R) == sizeof(float) && slope == R(0)) return r;
        const int fr = g.from[e], to = g.to[e];
        R c = ipw_at(g, 6, l, fr) * R(w[(long long)l * g.nc + fr]);
        c += ipw_at(g, 6, l, to) * R(w[(long long)l * g.nc + to]);
        if (l < g.nl - 1) {
            c += ipw_at(g, 7, l, fr) * R(w[(long long)(l + 1) * g.nc + fr]);
            c += ipw_at(g, 7, l, to) * R(w[(long long)(l + 1) * g.nc + to]);
        }
        c = R(0.5) * c;
        r += slope * c;
    }
    return r;
}

/* sum of all constituent densities (src/constituents/derived_quantities.c:83-95) */
__device__ __forceinline__ double density_total(const double *rho, int n_const, long long ns, long long i)
{
    double r = 0.0;
    for (int k = 0; k < n_const; ++k) r += rho[k * ns + i];
    return r;
}

/* ------------------------------------------------------ thermodynamics
 * src/constituents/dictionary.c (FP64 on both paths) */
__device__ __forceinline__ double c_p_ice(double t)
{
    if (t > T_0) t = T_0;
    if (t < 20.0) t = 20.0;
    double q = t / 125.1;
    double r = -2.0572 + 0.14644 * t + 0.06163 * t * exp(-(q * q));
    return r / M_V;
}

__device__ __forceinline__ double c_p_water(double t)
{
    double tc = t - T_0, r;
    if (tc >= 0.0) {
        if (tc > 35.0) tc = 35.0;
        double a = tc - 35.0;
        r = 0.9979 + 3.1e-6 * (a * a) + 3.8e-9 * pow(a, 4.0);
    } else {
        if (tc < -37.0) tc = -37.0;
        r = 1.000938 - 2.7052e-3 * tc - 2.3235e-5 * (tc * tc) + 4.3778e-6 * pow(tc, 3.0) + 2.7136e-7 * pow(tc, 4.0);
    }
    return 4186.8 * r;
}

__device__ __forceinline__ double c_p_cond(int id, double t) { return (id % 2 == 0) ? c_p_ice(t) : c_p_water(t); }

__device__ __forceinline__ double enthalpy_evaporation(double t)
{
    double r;
    if (t < T_0) {
        if (t < 30.0) t = 30.0;
        r = 56579.0 - 42.212 * t + exp(0.1149 * (281.6 - t));
        r = r / M_V;
    } else {
        if (t > T_0 + 100.0) t = T_0 + 100.0;
        r = 3151378.0 - 2386.0 * t;
    }
    return r;
}

__device__ __forceinline__ double enthalpy_sublimation(double t)
{
    if (t < 30.0) t = 30.0;
    if (t > T_0) t = T_0;
    double q = t / 123.75;
    double r = 46782.5 + 35.8925 * t - 0.07414 * (t * t) + 541.5 * exp(-(q * q));
    return r / M_V;
}

__device__ __forceinline__ double sat_pressure_water(double t)
{
    double tc = t - T_0, r;
    if (tc > 100.0) tc = 100.0;
    if (tc > 0.0) {
        r = exp(34.494 - 4924.99 / (tc + 237.1)) / pow(tc + 105.0, 1.57);
    } else {
        if (tc < -50.0) tc = -50.0;
        r = 6.107799961 + 4.436518521e-1 * tc + 1.428945805e-2 * (tc * tc) + 2.650648471e-4 * pow(tc, 3.0)
            + 3.031240396e-6 * pow(tc, 4.0) + 2.034080948e-8 * pow(tc, 5.0) + 6.136820929e-11 * pow(tc, 6.0);
        r = 100.0 * r;
    }
    return r;
}

__device__ __forceinline__ double dsat_pressure_water_dT(double t)
{
    double tc = t - T_0;
    if (tc > 100.0) tc = 100.0;
    if (tc < 0.0) tc = 0.0;
    double a = tc + 237.1;
    return sat_pressure_water(t) * (4924.99 / (a * a) - 1.57 / (tc + 105.0));
}

__device__ __forceinline__ double sat_pressure_ice(double t)
{
    double tc = t - T_0;
    if (tc < -80.0) tc = -80.0;
    if (tc > 0.0) tc = 0.0;
    double a = tc + 868.0;
    return exp(43.494 - 6545.8 / (tc + 278.0)) / (a * a);
}

__device__ __forceinline__ double dsat_pressure_ice_dT(double t)
{
    double tc = t - T_0;
    if (tc < -80.0) tc = -80.0;
    if (tc > 0.0) tc = 0.0;
    double a = tc + 278.0;
    return sat_pressure_ice(t) * (6545.8 / (a * a) - 2.0 / (tc + 868.0));
}

/* mass-weighted c_v (derived_quantities.c:97-115); cp_ice / cp_water are
 * c_p_cond of the even (ice) and odd (liquid) condensates at the cell's
 * temperature, evaluated once per step */
__device__ __forceinline__ double c_v_mass_weighted(const double *rho, int n_cond, int moist, long long ns,
                                                    long long i, double cp_ice, double cp_water)
{
    double r = 0.0;
    for (int k = 0; k < n_cond; ++k) r += rho[k * ns + i] * ((k % 2 == 0) ? cp_ice : cp_water);
    r += rho[n_cond * ns + i] * C_D_V;
    if (moist) r += rho[(n_cond + 1) * ns + i] * C_V_V;
    return r;
}

/* --------------------------------------------------- k_cell_prepare
 * temperature (derived_quantities.c:15-40) from state_old and, for the moist
 * build, phase-transition rates and heating (phase_trans.c:16-311) */
__global__ void k_cell_prepare(VGrid vg, StepParams p, DState so, double *temperature, double *pt_rates,
                               double *pt_heat, double *cp_ice_out, double *cp_water_out)
{
    const long long ns = (long long)vg.nl * vg.nc;
    const long long i = gtid();
    if (i >= ns) return;
    const int cond = p.n_cond;
    double T;
    if (!p.moist) {
        T = (vg.theta_v_bg[i] + so.theta_v_pert[i]) * (vg.exner_bg[i] + so.exner_pert[i]);
        temperature[i] = T;
        return;
    }
    const double *rho = so.rho;
    T = (vg.theta_v_bg[i] + so.theta_v_pert[i]) * (vg.exner_bg[i] + so.exner_pert[i])
        / (1.0 + rho[(cond + 1) * ns + i] / rho[cond * ns + i] * (M_D / M_V - 1.0));
    temperature[i] = T;
    const double cpi = c_p_ice(T), cpw = c_p_water(T);
    cp_ice_out[i] = cpi;
    cp_water_out[i] = cpw;
    const double dt = p.dt;
    const double max_cloud_water = 0.2e-3;
    /* each transcendental evaluated once; reused values are the same numbers
     * the reference recomputes */
    const double sat0 = T >= T_0 ? sat_pressure_water(T) : sat_pressure_ice(T);
    double wvp = rho[(cond + 1) * ns + i] * R_V * T;
    double dry = (rho[cond * ns + i] - rho[(cond + 1) * ns + i]) * R_D * T;
    double air = dry + wvp;
    double ef = T >= T_0 ? 1.00071 * exp(0.000000045 * air) : 0.99882 * exp(0.00000008 * air);
    double sat = ef * sat0;
    int dir = T >= T_0 ? 0 : 1;
    double dsat;
    if (dir == 0) {
        double tc = T - T_0;
        if (tc > 100.0) tc = 100.0;
        if (tc < 0.0) tc = 0.0;
        const double q0 = tc + 237.1;
        dsat = sat0 * (4924.99 / (q0 * q0) - 1.57 / (tc + 105.0));
    } else {
        double tc = T - T_0;
        if (tc < -80.0) tc = -80.0;
        if (tc > 0.0) tc = 0.0;
        const double q0 = tc + 278.0;
        dsat = sat0 * (6545.8 / (q0 * q0) - 2.0 / (tc + 868.0));
    }
    const double h_evap = enthalpy_evaporation(T), h_subl = enthalpy_sublimation(T);
    const double h_melt = h_subl - h_evap;
    double cv = c_v_mass_weighted(rho, cond, 1, ns, i, cpi, cpw);
    double pth = dir == 0 ? h_evap : h_subl;
    double a = -R_V * pth / cv;
    double b = R_V * T - R_V * rho[(cond + 1) * ns + i] * pth / cv + ef * dsat * pth / cv;
    double cc = wvp - sat;
    double pp = b / a;
    double q = cc / a;
    double diff = -0.5 * pp - sqrt(0.25 * (pp * pp) - q);
    double r0, r1, r2, r3, r4, heat;
    if (sat >= wvp) {
        if (T >= T_0) {
            r2 = -rho[2 * ns + i] / dt;
            double ptd = fmin(rho[3 * ns + i], diff);
            r4 = ptd / dt;
            r3 = rho[2 * ns + i] / dt - ptd / dt;
            heat = r2 * h_melt - ptd * h_evap / dt;
        } else {
            r3 = -rho[3 * ns + i] / dt;
            double ptd = fmin(rho[2 * ns + i], diff);
            r4 = ptd / dt;
            r2 = rho[3 * ns + i] / dt - ptd / dt;
            heat = -r3 * h_melt - ptd * h_subl / dt;
        }
    } else {
        if (T >= T_0) {
            r2 = -rho[2 * ns + i] / dt;
            r4 = diff / dt;
            r3 = rho[2 * ns + i] / dt - diff / dt;
            heat = r2 * h_melt - diff * h_evap / dt;
        } else {
            r3 = -rho[3 * ns + i] / dt;
            r4 = diff / dt;
            r2 = rho[3 * ns + i] / dt - diff / dt;
            heat = -r3 * h_melt - diff * h_subl / dt;
        }
    }
    r0 = 0.0;
    r1 = 0.0;
    if (T < T_0) {
        r0 = fmax(rho[2 * ns + i] - max_cloud_water * rho[4 * ns + i], 0.0) / 1000.0;
        r2 -= r0;
    } else if (T >= T_0) {
        r1 = fmax(rho[3 * ns + i] - max_cloud_water * rho[4 * ns + i], 0.0) / 1000.0;
        r3 -= r1;
    }
    if (T >= T_0 && rho[i] > 0.0) {
        r0 = -rho[i] / dt;
        r1 -= r0;
        heat += r0 * h_melt;
    }
    if (T < T_0 && rho[ns + i] > 0.0) {
        r1 = -rho[ns + i] / dt;
        r0 -= r1;
        heat += -r1 * h_melt;
    }
    pt_rates[i] = r0;
    pt_rates[ns + i] = r1;
    pt_rates[2 * ns + i] = r2;
    pt_rates[3 * ns + i] = r3;
    pt_rates[4 * ns + i] = r4;
    pt_heat[i] = heat;
}

/* ------------------------------------------------ k_cell_prepare_f32
 * the same diagnostics and phase-transition rates in FP32 (mixed path).  The
 * condensation quadratic's root -p/2 - sqrt(p^2/4 - q) is evaluated as
 * q / (-p/2 + sqrt(p^2/4 - q)) when p < 0, the algebraically identical form
 * without cancellation, which FP32 needs. */
__device__ __forceinline__ float c_p_ice_f(float t)
{
    if (t > float(T_0)) t = float(T_0);
    if (t < 20.f) t = 20.f;
    const float q = t / 125.1f;
    return (-2.0572f + 0.14644f * t + 0.06163f * t * expf(-(q * q))) / float(M_V);
}
__device__ __forceinline__ float c_p_water_f(float t)
{
    float tc = t - float(T_0), r;
    if (tc >= 0.f) {
        if (tc > 35.f) tc = 35.f;
        const float a = tc - 35.f, a2 = a * a;
        r = 0.9979f + 3.1e-6f * a2 + 3.8e-9f * (a2 * a2);
    } else {
        if (tc < -37.f) tc = -37.f;
        const float t2 = tc * tc;
        r = 1.000938f - 2.7052e-3f * tc - 2.3235e-5f * t2 + 4.3778e-6f * (t2 * tc) + 2.7136e-7f * (t2 * t2);
    }
    return 4186.8f * r;
}
__device__ __forceinline__ float enthalpy_evaporation_f(float t)
{
    if (t < float(T_0)) {
        if (t < 30.f) t = 30.f;
        return (56579.0f - 42.212f * t + expf(0.1149f * (281.6f - t))) / float(M_V);
    }
    if (t > float(T_0) + 100.f) t = float(T_0) + 100.f;
    return 3151378.0f - 2386.0f * t;
}
__device__ __forceinline__ float enthalpy_sublimation_f(float t)
{
    if (t < 30.f) t = 30.f;
    if (t > float(T_0)) t = float(T_0);
    const float q = t / 123.75f;
    return (46782.5f + 35.8925f * t - 0.07414f * (t * t) + 541.5f * expf(-(q * q))) / float(M_V);
}

__global__ void k_cell_prepare_f32(VGrid vg, StepParams p, DState so, double *temperature, double *pt_rates,
                                   double *pt_heat, double *cp_ice_out, double *cp_water_out, float *cp32_ice,
                                   float *cp32_water)
{
    const long long ns = (long long)vg.nl * vg.nc;
    const long long i = gtid();
    if (i >= ns) return;
    const int cond = p.n_cond;
    const double *rho = so.rho;
    const float th = to_float(vg.theta_v_bg[i] + so.theta_v_pert[i]), pi = to_float(vg.exner_bg[i] + so.exner_pert[i]);
    if (!p.moist) {
        temperature[i] = to_double(th) * to_double(pi);
        return;
    }
    float r[6];
    for (int k = 0; k < 6; ++k) r[k] = to_float(rho[k * ns + i]);
    const float rv = r[cond + 1], rg = r[cond];
    const float T = th * pi / (1.f + rv / rg * float(M_D / M_V - 1.0));
    temperature[i] = to_double(T);
    const float cpi = c_p_ice_f(T), cpw = c_p_water_f(T);
    cp_ice_out[i] = to_double(cpi);
    cp_water_out[i] = to_double(cpw);
    cp32_ice[i] = cpi;
    cp32_water[i] = cpw;
    const float dt = float(p.dt), T0 = float(T_0);
    const bool warm = T >= T0;
    float tc = T - T0, sat0, dsat_fac;
    if (warm) {
        float tw = tc > 100.f ? 100.f : tc;
        if (tw > 0.f) {
            sat0 = expf(34.494f - 4924.99f / (tw + 237.1f)) / powf(tw + 105.0f, 1.57f);
        } else {
            const float t2 = tw * tw;
            sat0 = 100.f * (6.107799961f + 4.436518521e-1f * tw + 1.428945805e-2f * t2 + 2.650648471e-4f * t2 * tw
                            + 3.031240396e-6f * t2 * t2 + 2.034080948e-8f * t2 * t2 * tw
                            + 6.136820929e-11f * t2 * t2 * t2);
        }
        float td = tc > 100.f ? 100.f : (tc < 0.f ? 0.f : tc);
        const float q0 = td + 237.1f;
        dsat_fac = 4924.99f / (q0 * q0) - 1.57f / (td + 105.0f);
    } else {
        float ti = tc < -80.f ? -80.f : (tc > 0.f ? 0.f : tc);
        const float a = ti + 868.0f;
        sat0 = expf(43.494f - 6545.8f / (ti + 278.0f)) / (a * a);
        const float q0 = ti + 278.0f;
        dsat_fac = 6545.8f / (q0 * q0) - 2.0f / (ti + 868.0f);
    }
    const float wvp = rv * float(R_V) * T;
    const float air = (rg - rv) * float(R_D) * T + wvp;
    const float ef = warm ? 1.00071f * expf(0.000000045f * air) : 0.99882f * expf(0.00000008f * air);
    const float sat = ef * sat0;
    const float h_evap = enthalpy_evaporation_f(T), h_subl = enthalpy_sublimation_f(T), h_melt = h_subl - h_evap;
    float cv = 0.f;
    for (int k = 0; k < cond; ++k) cv += r[k] * ((k % 2 == 0) ? cpi : cpw);
    cv += rg * float(C_D_V) + rv * float(C_V_V);
    const float pth = warm ? h_evap : h_subl;
    const float a = -float(R_V) * pth / cv;
    const float b = float(R_V) * T - float(R_V) * rv * pth / cv + ef * (sat0 * dsat_fac) * pth / cv;
    const float pp = b / a, q = (wvp - sat) / a;
    const float sq = sqrtf(0.25f * (pp * pp) - q);
    const float diff = pp < 0.f ? q / (-0.5f * pp + sq) : -0.5f * pp - sq;
    float r0, r1, r2, r3, r4, heat;
    if (sat >= wvp) {
        if (warm) {
            r2 = -r[2] / dt;
            const float ptd = fminf(r[3], diff);
            r4 = ptd / dt;
            r3 = r[2] / dt - ptd / dt;
            heat = r2 * h_melt - ptd * h_evap / dt;
        } else {
            r3 = -r[3] / dt;
            const float ptd = fminf(r[2], diff);
            r4 = ptd / dt;
            r2 = r[3] / dt - ptd / dt;
            heat = -r3 * h_melt - ptd * h_subl / dt;
        }
    } else {
        if (warm) {
            r2 = -r[2] / dt;
            r4 = diff / dt;
            r3 = r[2] / dt - diff / dt;
            heat = r2 * h_melt - diff * h_evap / dt;
        } else {
            r3 = -r[3] / dt;
            r4 = diff / dt;
            r2 = r[3] / dt - diff / dt;
            heat = -r3 * h_melt - diff * h_subl / dt;
        }
    }
    r0 = 0.f;
    r1 = 0.f;
    const float max_cloud_water = 0.2e-3f;
    if (!warm) {
        r0 = fmaxf(r[2] - max_cloud_water * r[4], 0.f) / 1000.f;
        r2 -= r0;
    } else {
        r1 = fmaxf(r[3] - max_cloud_water * r[4], 0.f) / 1000.f;
        r3 -= r1;
    }
    if (warm && r[0] > 0.f) {
        r0 = -r[0] / dt;
        r1 -= r0;
        heat += r0 * h_melt;
    }
    if (!warm && r[1] > 0.f) {
        r1 = -r[1] / dt;
        r0 -= r1;
        heat += -r1 * h_melt;
    }
    /* widened by integer operations (to_double): the FP64 pipe was this
     * kernel's bound */
    pt_rates[i] = to_double(r0);
    pt_rates[ns + i] = to_double(r1);
    pt_rates[2 * ns + i] = to_double(r2);
    pt_rates[3 * ns + i] = to_double(r3);
    pt_rates[4 * ns + i] = to_double(r4);
    pt_heat[i] = to_double(heat);
}

/* FP32 shadow of the state at the start of a mixed step.  Each thread
 * converts the pairs 2i, 2i + 1 of every field with one 16-byte load and one
 * 8-byte store (every field length is even: 10 * 4^RES_ID + 2 cells, 30 *
 * 4^RES_ID edges, so every field of the mirror and of the shadow starts on
 * an even element), rounding with to_float (the conversion instruction's
 * bits, on the integer pipe instead of the FP64 pipe). */
__device__ __forceinline__ void shadow_pair(const double *src, float *dst, long long j)
{
    const double2 v = reinterpret_cast<const double2 *>(src)[j];
    reinterpret_cast<float2 *>(dst)[j] = make_float2(to_float(v.x), to_float(v.y));
}
__global__ void k_make_shadow(long long n_rho, long long ns, long long nw, long long nu, DState s, Shadow sh)
{
    const long long j = gtid();
    if (2 * j < n_rho) shadow_pair(s.rho, sh.rho, j);
    if (2 * j < ns) {
        shadow_pair(s.rhotheta_v, sh.rhotheta_v, j);
        shadow_pair(s.theta_v_pert, sh.theta_v_pert, j);
        shadow_pair(s.exner_pert, sh.exner_pert, j);
    }
    if (2 * j < nw) shadow_pair(s.w, sh.w, j);
    if (2 * j < nu) shadow_pair(s.u, sh.u, j);
}

/* ------------------------------------------------------- k_tri_vort
 * vertical relative vorticity on triangles (vorticities.c:167-222) */
template <typename R>
__global__ void __launch_bounds__(256, sizeof(R) == sizeof(float) ? 8 : 1) k_tri_vort(HGrid<R> g, const R *u, R *tri_vort)
{
    const long long n = (long long)g.nl * g.nt;
    const long long i = gtid();
    if (i >= n) return;
    const int l = (int)(i / g.nt), t = (int)(i - (long long)l * g.nt);
    R acc = R(0);
    for (int j = 0; j < 3; ++j) {
        const int e = g.vort_i[j * g.nt + t];
        const long long le = (long long)l * g.ne + e;
        R vel = u[le];
        R rescale = R(1);
        if (l >= g.nl - g.n_oro) {
            const R zt = g.dual_z_t[i];
            rescale = (g.radius + zt) / (g.radius + g.z_h[le]);
            R dz = zt - g.z_h[le];
            int lo;
            if (dz > R(0)) lo = l - 1;
            else if (l == g.nl - 1) lo = l - 1;
            else lo = l + 1;
            const long long lo_e = (long long)lo * g.ne + e;
            R vgrad = (u[le] - u[lo_e]) / (g.z_h[le] - g.z_h[lo_e]);
            vel += dz * vgrad;
        }
        acc += rescale * g.nd_h[le] * R(g.vort_s[j * g.nt + t]) * vel;
    }
    tri_vort[i] = acc / g.dual_area_t[i];
}

/* tangential relative vorticity at level k, edge e (vorticities.c:104-165) */
template <typename R>
__device__ __forceinline__ R rel_vort_tangential(const HGrid<R> &g, const R *u, const R *w, int k, int e)
{
    const int nl = g.nl;
    if (k == 0) k = 1; /* no vertical shear of the tangential vorticity at the TOA */
    const R inv_area = R(1) / g.dual_area_h[(long long)k * g.ne + e];
    if (k == nl) {
        R c2 = hor_covariant(g, u, w, k - 1, e);
        return inv_area * g.nd_h[(long long)(k - 1) * g.ne + e] * c2;
    }
    const int fr = g.from[e], to = g.to[e];
    R c0 = hor_covariant(g, u, w, k, e);
    R c2 = hor_covariant(g, u, w, k - 1, e);
    return inv_area * (-g.nd_h[(long long)k * g.ne + e] * c0
                       + g.nd_v[(long long)k * g.nc + fr] * w[(long long)k * g.nc + fr]
                       + g.nd_h[(long long)(k - 1) * g.ne + e] * c2
                       - g.nd_v[(long long)k * g.nc + to] * w[(long long)k * g.nc + to]);
}

/* --------------------------------------------------------- k_edge_vort
 * potential vorticity (vorticities.c:18-85) and the horizontal mass flux
 * density (multiplications.c:45-66), one thread per (edge, level 0..L) */
template <typename R>
__global__ void __launch_bounds__(256, sizeof(R) == sizeof(float) ? 8 : 1) k_edge_vort(HGrid<R> g, const R *u, const R *w, const R *rho_gas, const R *tri_vort, R *zh, R *zv,
                            R *flux_h)
{
    const long long n = (long long)(g.nl + 1) * g.ne;
    const long long i = gtid();
    if (i >= n) return;
    const int k = (int)(i / g.ne), e = (int)(i - (long long)k * g.ne);
    const int nl = g.nl, nc = g.nc, ne = g.ne;
    const int fr = g.from[e], to = g.to[e];
    /* tangential component at level k */
    {
        R rel = rel_vort_tangential(g, u, w, k, e);
        R pv = rel + g.f_vec[e];
        R dens;
        if (k == 0) {
            R top = R(0.5) * (rho_gas[fr] + rho_gas[to]);
            R below = R(0.5) * (rho_gas[nc + fr] + rho_gas[nc + to]);
            dens = top + (top - below) / g.pvz[ne + e] * g.pvz[e];
        } else if (k == nl) {
            long long a = (long long)(nl - 1) * nc, b = (long long)(nl - 2) * nc;
            R low = R(0.5) * (rho_gas[a + fr] + rho_gas[a + to]);
            R above = R(0.5) * (rho_gas[b + fr] + rho_gas[b + to]);
            dens = low + (above - low) / g.pvz[3 * (long long)ne + e] * g.pvz[2 * (long long)ne + e];
        } else {
            long long uf = (long long)(k - 1) * nc + fr, ut = (long long)(k - 1) * nc + to;
            dens = R(0.25) * (rho_gas[uf] + rho_gas[ut] + rho_gas[uf + nc] + rho_gas[ut + nc]);
        }
        zh[i] = pv / dens;
    }
    if (k < nl) {
        const long long le = (long long)k * ne + e;
        /* rhombus: area-weighted mean of the two triangles */
        const int tf = g.dual_from[e], tt = g.dual_to[e];
        const long long kt = (long long)k * g.nt;
        R af = g.dual_area_t[kt + tf], at = g.dual_area_t[kt + tt];
        R rel = (af * tri_vort[kt + tf] + at * tri_vort[kt + tt]) / (af + at);
        R pv = rel + g.f_vec[ne + e];
        R dens = R(0);
        for (int j = 0; j < 4; ++j)
            dens += g.rhombi_w[j * (long long)ne + e] * rho_gas[(long long)k * nc + g.rhombi_i[j * (long long)ne + e]];
        zv[le] = pv / dens;
        /* mass flux density */
        R sv = R(0.5) * (rho_gas[(long long)k * nc + to] + rho_gas[(long long)k * nc + fr]);
        flux_h[le] = sv * u[le];
    }
}

/* ------------------------------------------------------ k_cell_kinetic
 * kinetic energy v^2 (inner_product.c:13-43) at (cell, layer) and the vertical
 * mass flux density (multiplications.c:98-117) at the inner interfaces */
template <typename R>
__global__ void k_cell_kinetic(HGrid<R> g, const R *u, const R *w, const R *rho_gas, R *v2, R *flux_v)
{
    const long long ns = (long long)g.nl * g.nc;
    const long long i = gtid();
    if (i >= ns) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const int n_edges = c < N_PENT ? 5 : 6;
    R acc = R(0);
    for (int j = 0; j < n_edges; ++j) {
        R ue = u[(long long)l * g.ne + g.adj[j * g.nc + c]];
        acc += ipw_at(g, j, l, c) * ue * ue;
    }
    R wu = w[i], wl = w[i + g.nc];
    acc += ipw_at(g, 6, l, c) * wu * wu;
    acc += ipw_at(g, 7, l, c) * wl * wl;
    v2[i] = acc;
    if (l >= 1) {
        R sv = R(0.5) * (rho_gas[i - g.nc] + rho_gas[i]);
        flux_v[i] = sv * wu;
    }
}

/* modified TRSK vorticity flux at edge e of layer l (vorticity_flux.c:35-137) */
template <typename R>
__device__ __forceinline__ R vorticity_flux_h(const HGrid<R> &g, const R *flux_h, const R *flux_v, const R *zh,
                                              const R *zv, int l, int e)
{
    const long long ne = g.ne;
    const R *mf = flux_h + (long long)l * ne;
    const R *pv = zv + (long long)l * ne;
    const int fr = g.from[e], to = g.to[e];
    R out = R(0);
    if (fr < N_PENT) {
        for (int j = 0; j < 4; ++j)
            out += g.trsk_w[j * ne + e] * mf[g.trsk_i[j * ne + e]] * pv[g.trsk_m[j * ne + e]];
    } else {
        for (int j = 0; j < 5; ++j) {
            if (j == 2)
                out += g.trsk_w[j * ne + e] * mf[g.trsk_i[j * ne + e]] * R(0.5) * (pv[g.trsk_m[j * ne + e]] + pv[e]);
            else
                out += g.trsk_w[j * ne + e] * mf[g.trsk_i[j * ne + e]] * pv[g.trsk_m[j * ne + e]];
        }
    }
    if (to < N_PENT) {
        for (int j = 5; j < 9; ++j)
            out += g.trsk_w[j * ne + e] * mf[g.trsk_i[j * ne + e]] * pv[g.trsk_m[j * ne + e]];
    } else {
        for (int j = 5; j < 10; ++j) {
            if (j == 7)
                out += g.trsk_w[j * ne + e] * mf[g.trsk_i[j * ne + e]] * R(0.5) * (pv[g.trsk_m[j * ne + e]] + pv[e]);
            else
                out += g.trsk_w[j * ne + e] * mf[g.trsk_i[j * ne + e]] * pv[g.trsk_m[j * ne + e]];
        }
    }
    const R zt = zh[(long long)l * ne + e], zb = zh[(long long)(l + 1) * ne + e];
    const long long nc = g.nc;
    out -= R(0.5) * ipw_at(g, 6, l, fr) * flux_v[l * nc + fr] * zt;
    out -= R(0.5) * ipw_at(g, 6, l, to) * flux_v[l * nc + to] * zt;
    out -= R(0.5) * ipw_at(g, 7, l, fr) * flux_v[(l + 1) * nc + fr] * zb;
    out -= R(0.5) * ipw_at(g, 7, l, to) * flux_v[(l + 1) * nc + to] * zb;
    return out;
}

/* sum of all constituent densities in R (derived_quantities.c:83-95) */
template <typename R>
__device__ __forceinline__ R density_total_r(const R *rho, int n_const, long long ns, long long i)
{
    R r = R(0);
    for (int k = 0; k < n_const; ++k) r += rho[k * ns + i];
    return r;
}

/* decelerated pressure-gradient sum nl + l at edge e, layer l
 * (manage_pressure_gradient.c:17-72) */
template <typename R>
__device__ __forceinline__ void pgrad_h_parts(const HGrid<R> &g, const StepParams &p, const SView<R> &s, int l, int e,
                                              R &nl, R &l_term)
{
    const long long ns = (long long)g.nl * g.nc;
    const int fr = g.from[e], to = g.to[e];
    const long long cf = (long long)l * g.nc + fr, ct = (long long)l * g.nc + to;
    const R cdp = R(C_D_P);
    nl = grad_h(g, s.exner_pert, l, e);
    R s_to = cdp * (g.theta_v_bg[ct] + s.theta_v_pert[ct]), s_fr = cdp * (g.theta_v_bg[cf] + s.theta_v_pert[cf]);
    nl = (R(0.5) * (s_to + s_fr)) * nl;
    l_term = (R(0.5) * (cdp * s.theta_v_pert[ct] + cdp * s.theta_v_pert[cf])) * g.exner_bg_grad_h[(long long)l * g.ne + e];
    R d_to = s.rho[p.n_cond * ns + ct] / density_total_r(s.rho, p.n_const, ns, ct);
    R d_fr = s.rho[p.n_cond * ns + cf] / density_total_r(s.rho, p.n_const, ns, cf);
    R dec = R(0.5) * (d_to + d_fr);
    nl = dec * nl;
    l_term = dec * l_term;
}

/* the sum nl + l, the only form the step reads */
template <typename R>
__device__ __forceinline__ R pgrad_h(const HGrid<R> &g, const StepParams &p, const SView<R> &s, int l, int e)
{
    R nl, l_term;
    pgrad_h_parts(g, p, s, l, e, nl, l_term);
    return nl + l_term;
}

/* the same at the inner interface k of cell c */
template <typename R>
__device__ __forceinline__ void pgrad_v_parts(const HGrid<R> &g, const StepParams &p, const SView<R> &s, int k, int c,
                                              R &nl, R &l_term)
{
    const long long ns = (long long)g.nl * g.nc;
    const long long up = (long long)(k - 1) * g.nc + c, lo = (long long)k * g.nc + c;
    const R cdp = R(C_D_P);
    nl = grad_v(g, s.exner_pert, k, c);
    R s_up = cdp * (g.theta_v_bg[up] + s.theta_v_pert[up]), s_lo = cdp * (g.theta_v_bg[lo] + s.theta_v_pert[lo]);
    nl = (R(0.5) * (s_up + s_lo)) * nl;
    l_term = (R(0.5) * (cdp * s.theta_v_pert[up] + cdp * s.theta_v_pert[lo])) * g.exner_bg_grad_v[(long long)k * g.nc + c];
    R d_up = s.rho[p.n_cond * ns + up] / density_total_r(s.rho, p.n_const, ns, up);
    R d_lo = s.rho[p.n_cond * ns + lo] / density_total_r(s.rho, p.n_const, ns, lo);
    R dec = R(0.5) * (d_up + d_lo);
    nl = dec * nl;
    l_term = dec * l_term;
}

template <typename R>
__device__ __forceinline__ R pgrad_v(const HGrid<R> &g, const StepParams &p, const SView<R> &s, int k, int c)
{
    R nl, l_term;
    pgrad_v_parts(g, p, s, k, c, nl, l_term);
    return nl + l_term;
}

/* Mixed path: the cell factors of the pressure gradient at the step start,
 * one float4 per (layer, cell): x = Pi', y = c_p (theta_v_bg + theta_v'),
 * z = c_p theta_v', w = rho_gas / (sum of all densities) -- the float
 * expressions of pgrad_h_parts / pgrad_v_parts, so that the first
 * substage's gradients gather two float4 per edge (or interface) instead of
 * some twenty scalars.  Read from the FP32 shadow of state_new, which the
 * first substage's pressure gradient reads. */
__global__ void k_pg_cells(HGrid<float> g, StepParams p, SView<float> s, float4 *pc)
{
    const long long ns = (long long)g.nl * g.nc;
    const long long i = gtid();
    if (i >= ns) return;
    const float cdp = float(C_D_P);
    const float tp = s.theta_v_pert[i];
    pc[i] = make_float4(s.exner_pert[i], cdp * (g.theta_v_bg[i] + tp), cdp * tp,
                        s.rho[p.n_cond * ns + i] / density_total_r(s.rho, p.n_const, ns, i));
}

/* pgrad_h from the cell factors (mixed path, first substage) */
__device__ __forceinline__ float pgrad_h_packed(const HGrid<float> &g, const float4 *pc, const SView<float> &s, int l,
                                                int e)
{
    const int fr = g.from[e], to = g.to[e];
    const long long le = (long long)l * g.ne + e;
    const float4 a = pc[(long long)l * g.nc + fr], b = pc[(long long)l * g.nc + to];
    float nl = (b.x - a.x) / g.nd_h[le];
    const float slope = l >= g.nl - g.n_oro ? g.slope_h[le] : 0.0f;
    if (slope != 0.0f) { /* a zero slope adds -0 */
        float c = ipw_at(g, 6, l, fr) * grad_v(g, s.exner_pert, l, fr);
        c += ipw_at(g, 6, l, to) * grad_v(g, s.exner_pert, l, to);
        if (l < g.nl - 1) {
            c += ipw_at(g, 7, l, fr) * grad_v(g, s.exner_pert, l + 1, fr);
            c += ipw_at(g, 7, l, to) * grad_v(g, s.exner_pert, l + 1, to);
        }
        c = 0.5f * c;
        nl += -slope * c;
    }
    nl = (0.5f * (b.y + a.y)) * nl;
    float l_term = (0.5f * (b.z + a.z)) * g.exner_bg_grad_h[le];
    const float dec = 0.5f * (b.w + a.w);
    nl = dec * nl;
    l_term = dec * l_term;
    return nl + l_term;
}

/* pgrad_v from the cell factors of the interface's two cells */
__device__ __forceinline__ float pgrad_v_packed(const HGrid<float> &g, float4 u, float4 d, int k, int c)
{
    float nl = (u.x - d.x) / g.nd_v[(long long)k * g.nc + c];
    nl = (0.5f * (u.y + d.y)) * nl;
    float l_term = (0.5f * (u.z + d.z)) * g.exner_bg_grad_v[(long long)k * g.nc + c];
    const float dec = 0.5f * (u.w + d.w);
    nl = dec * nl;
    l_term = dec * l_term;
    return nl + l_term;
}

/* ------------------------------------------------------- k_momentum_h
 * horizontal momentum: explicit tendency (vector_tendencies_expl.c:74-131) and
 * the wind update (manage_rkhevi.c:67-75).  ADV: the advection terms are
 * recomputed in this substage; PG: the pressure gradient is recomputed (on
 * the mixed path from the cell factors pc of k_pg_cells).  The wind update
 * is FP64; u_shadow (mixed path) receives its FP32 copy. */
template <typename R, bool ADV, bool PG>
__global__ void __launch_bounds__(256, sizeof(R) == sizeof(float) ? 8 : 1) k_momentum_h(HGrid<R> g, StepParams p, SView<R> sv, double *u_new, float *u_shadow, const double *u_old,
                             double *tend_u, R *P_h, R *pg_old_h, R *pvt_h, R *v2g_h, const R *flux_h,
                             const R *flux_v, const R *zh, const R *zv, const R *v2, double new_w, double old_w,
                             const double *fric_u, const float4 *pc)
{
    const long long n = (long long)g.nl * g.ne;
    const long long i = gtid();
    if (i >= n) return;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    R P, pgo;
    if (PG) {
        if constexpr (sizeof(R) == sizeof(float))
            P = pgrad_h_packed(g, pc, sv, l, e);
        else
            P = pgrad_h(g, p, sv, l, e);
        pgo = p.first_step ? -P : -P_h[i];
        P_h[i] = P;
        pg_old_h[i] = pgo;
    } else {
        P = P_h[i];
        pgo = pg_old_h[i];
    }
    R pvt, v2g;
    if (ADV) {
        pvt = vorticity_flux_h(g, flux_h, flux_v, zh, zv, l, e);
        v2g = grad_h(g, v2, l, e);
        pvt_h[i] = pvt;
        v2g_h[i] = v2g;
    } else {
        pvt = pvt_h[i];
        v2g = v2g_h[i];
    }
    constexpr bool F = sizeof(R) == sizeof(float);
    const R cur_hor = F ? R(p.cur_hor_f) : R(p.cur_hor), old_hor = F ? R(p.old_hor_f) : R(p.old_hor);
    R y = old_hor * pgo - cur_hor * P + pvt - R(0.5) * v2g;
    /* friction acceleration of the diffusion branch, when it is active */
    if (fric_u) y = y + R(fric_u[i]);
    /* the pressure gradient is recomputed in substage 0 only, where the new
     * weight is 1 */
    double t = PG ? wide(y) : old_w * tend_u[i] + new_w * wide(y);
    tend_u[i] = t;
    const double un = u_old[i] + p.dt * t;
    u_new[i] = un;
    if (u_shadow) u_shadow[i] = to_float(un);
}

/* ------------------------------------------------------- k_momentum_v
 * vertical momentum at interface k of cell c: tendency including the
 * condensate term (manage_pressure_gradient.c:74-87) */
template <typename R, bool ADV, bool PG>
__global__ void __launch_bounds__(256, sizeof(R) == sizeof(float) ? 8 : 1) k_momentum_v(HGrid<R> g, StepParams p, SView<R> sv, double *tend_w, R *P_v, R *pvt_v, R *v2g_v,
                             const R *flux_h, const R *zh, const R *v2, double new_w, double old_w,
                             const double *fric_w, const float4 *pc)
{
    const long long n = (long long)(g.nl + 1) * g.nc;
    const long long i = gtid();
    if (i >= n) return;
    const int k = (int)(i / g.nc), c = (int)(i - (long long)k * g.nc);
    const int nl = g.nl;
    R pvt = R(0);
    if (ADV) {
        /* vertical part of the vorticity flux (vorticity_flux.c:143-183), all levels */
        const int n_edges = c < N_PENT ? 5 : 6;
        const R vw = (k == 0 || k == nl) ? R(1) : R(0.5);
        const R *z = zh + (long long)k * g.ne;
        if (k >= 1)
            for (int j = 0; j < n_edges; ++j) {
                const int a = g.adj[j * g.nc + c];
                pvt += vw * ipw_at(g, j, k - 1, c) * flux_h[(long long)(k - 1) * g.ne + a] * z[a];
            }
        if (k <= nl - 1)
            for (int j = 0; j < n_edges; ++j) {
                const int a = g.adj[j * g.nc + c];
                pvt += vw * ipw_at(g, j, k, c) * flux_h[(long long)k * g.ne + a] * z[a];
            }
        pvt_v[i] = pvt;
    }
    if (k == 0 || k == nl) {
        tend_w[i] = 0.0;
        return;
    }
    /* the mixed path's first substage takes the pressure gradient and the
     * condensate factors from the cell factors pc of k_pg_cells */
    constexpr bool PACKED = PG && sizeof(R) == sizeof(float);
    R P, v2g, d_up, d_lo;
    if (PG) {
        if constexpr (PACKED) {
            const float4 fu = pc[(long long)(k - 1) * g.nc + c], fd = pc[(long long)k * g.nc + c];
            P = pgrad_v_packed(g, fu, fd, k, c);
            d_up = fu.w - 1.0f;
            d_lo = fd.w - 1.0f;
        } else {
            P = pgrad_v(g, p, sv, k, c);
        }
        P_v[i] = P;
    } else {
        P = P_v[i];
    }
    if (ADV) {
        v2g = grad_v(g, v2, k, c);
        v2g_v[i] = v2g;
    } else {
        pvt = pvt_v[i];
        v2g = v2g_v[i];
    }
    if constexpr (!PACKED) {
        const long long ns = (long long)nl * g.nc;
        const long long up = (long long)(k - 1) * g.nc + c, lo = (long long)k * g.nc + c;
        d_up = sv.rho[p.n_cond * ns + up] / density_total_r(sv.rho, p.n_const, ns, up) - R(1);
        d_lo = sv.rho[p.n_cond * ns + lo] / density_total_r(sv.rho, p.n_const, ns, lo) - R(1);
    }
    R pgc = (R(0.5) * (d_up + d_lo)) * g.gravity_m_v[i];
    const R cur_ver = sizeof(R) == sizeof(float) ? R(p.cur_ver_f) : R(p.cur_ver);
    R y = -cur_ver * P + pvt - R(0.5) * v2g;
    if (fric_w) y = y + R(fric_w[i]);
    y = y + pgc;
    double t = PG ? wide(y) : old_w * tend_w[i] + new_w * wide(y);
    tend_w[i] = t;
}

/* ------------------------------------------------------ k_scalar_tend2
 * explicit mass and rho*theta_v tendencies (scalar_tendencies_expl.c:90-178)
 * at (cell, layer) */

/* vertical_contravariant_corr (averaging.c:41-95) of an edge field given
 * by the functor flux(l, j) at level k of cell c */
template <typename R, typename FX>
__device__ __forceinline__ R contra_corr(const HGrid<R> &g, int k, int c, int n_edges, FX flux)
{
    R r = R(0);
    if (k >= g.nl - g.n_oro) {
        if (k > g.nl - g.n_oro)
            for (int j = 0; j < n_edges; ++j) {
                const int a = g.adj[j * g.nc + c];
                r += R(-0.5) * ipw_at(g, j, k - 1, c) * g.slope_h[(long long)(k - 1) * g.ne + a] * flux(k - 1, j);
            }
        for (int j = 0; j < n_edges; ++j) {
            const int a = g.adj[j * g.nc + c];
            r += R(-0.5) * ipw_at(g, j, k, c) * g.slope_h[(long long)k * g.ne + a] * flux(k, j);
        }
    }
    return r;
}

template <typename R>
__global__ void k_theta(int nl, int nc, int n_cond, SView<R> sv, R *theta)
{
    const long long ns = (long long)nl * nc;
    const long long i = gtid();
    if (i >= ns) return;
    theta[i] = sv.rhotheta_v[i] / sv.rho[n_cond * ns + i];
}

/* Sum of edge fluxes of one cell.  R = double: plain double accumulation
 * (the reference's).  R = float: Knuth's TwoSum keeps the exact rounding
 * error of every FP32 addition in a second FP32 word, so the pair (hi, lo)
 * carries the sum to ~2^-48 relative before being rounded once to double --
 * FP64-class accumulation of the mass fluxes at FP32 instruction cost. */
template <typename R>
struct FluxSum {
    double s = 0.0;
    __device__ __forceinline__ void add(R x) { s += double(x); }
    __device__ __forceinline__ double value() const { return s; }
};
template <>
struct FluxSum<float> {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float x)
    {
        const float t = hi + x;
        const float bp = t - hi;
        const float err = (hi - (t - bp)) + (x - bp);
        hi = t;
        lo += err;
    }
    __device__ __forceinline__ double value() const { return to_double(hi) + to_double(lo); }
};

/* Explicit mass and rho*theta_v tendencies (scalar_tendencies_expl.c:90-178)
 * at (cell, layer).  The cell's edges are streamed one layer at a time
 * (layer l-1, l, l+1) so that only one layer's fluxes are live; every
 * accumulator still receives its terms in the reference's order (layer
 * l-1 before l, edges j = 0..5), so with R = double every sum and product is
 * the reference's, bit for bit.  The main mass flux is reused for the
 * rho*theta_v flux; the terrain correction of the wind is computed once for
 * all tracers.  Edge fluxes are products in R, divergences accumulate in
 * double (FluxSum) and tendencies are formed in double. */
/* irreversible terms of the tendencies (scalar_tendencies_expl.c:125-176):
 * dissipative and diffusive heating, radiation, mass diffusion [C][L][Nc] */
struct IrrTerms {
    const double *heating_diss, *temp_diff_heating, *radiation, *mass_diff;
};

template <typename R, bool IRR>
__global__ void __launch_bounds__(128) k_scalar_tend2(HGrid<R> g, StepParams p, SView<R> sv, DState st,
                                                      const R *theta, const R *cp_ice, const R *cp_water,
                                                      const double *pt_rates, const double *pt_heat,
                                                      const double *sed_heat, const double *inv_vol_tab, int rk,
                                                      IrrTerms irr)
{
    const long long ns = (long long)g.nl * g.nc;
    const long long i = gtid();
    if (i >= ns) return;
    const int nl = g.nl, n_oro = g.n_oro;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const long long nc = g.nc, ne = g.ne;
    const int n_edges = c < N_PENT ? 5 : 6;
    const int cond = p.n_cond;
    /* terrain-following corrections: in the orography layers (on the mixed
     * path only where the cell's edges slope; elsewhere they are zero) */
    const bool oro = l >= nl - n_oro - 1 && (sizeof(R) == sizeof(double) || g.tilt[c]);
    const bool up_corr = oro && l >= nl - n_oro;            /* contra_corr at level l needed   */
    const bool lo_corr = oro && l < nl - 1;                 /* contra_corr at level l+1 needed */
    const bool up_has_prev = up_corr && l > nl - n_oro;     /* level l sums layer l-1, then l  */
    const bool lo_has_curr = lo_corr && l + 1 > nl - n_oro; /* level l+1 sums layer l, then l+1 */
    const double inv_vol = sizeof(R) == sizeof(double) ? 1.0 / double(g.volume[i]) : inv_vol_tab[i];
    const R area_up = g.area_v[(long long)l * nc + c], area_lo = g.area_v[(long long)(l + 1) * nc + c];
    auto edge = [&](int j) { return g.adj[j * nc + c]; };
    auto wcorr = [&](int ll, int j) {
        return R(-0.5) * ipw_at(g, j, ll, c) * g.slope_h[(long long)ll * ne + edge(j)];
    };
    auto uval = [&](int ll, int j) { return sv.u[(long long)ll * ne + edge(j)]; };
    auto comp_v = [&](R up, R lo) -> double {
        if (!oro) return 0.0;
        if (l == nl - n_oro - 1) return wide(-lo * area_lo);
        if (l == nl - 1) return wide(up * area_up);
        return wide(up * area_up - lo * area_lo);
    };
    /* terrain correction of the wind at levels l and l+1 (shared by the tracers) */
    R w_up = R(0), w_lo = R(0);
    if (oro) {
        if (up_has_prev)
            for (int j = 0; j < n_edges; ++j) w_up += wcorr(l - 1, j) * uval(l - 1, j);
        for (int j = 0; j < n_edges; ++j) {
            const R t = wcorr(l, j) * uval(l, j);
            if (up_corr) w_up += t;
            if (lo_has_curr) w_lo += t;
        }
        if (lo_corr)
            for (int j = 0; j < n_edges; ++j) w_lo += wcorr(l + 1, j) * uval(l + 1, j);
    }
    /* the main gas: centred mass flux and, from it, the rho*theta_v flux
     * (new weight 1 in both substages) */
    {
        const R *f = sv.rho + cond * ns;
        FluxSum<R> hm, ht;
        R um = R(0), ut = R(0), lm = R(0), lt = R(0);
        auto layer_pass = [&](int ll, bool to_h, bool to_up, bool to_lo) {
            const long long o = (long long)ll * nc;
            const R fs = f[o + c], ts = theta[o + c];
            for (int j = 0; j < n_edges; ++j) {
                const int nb = g.adj_nbr[j * nc + c];
                const R fm = (R(0.5) * (fs + f[o + nb])) * uval(ll, j);
                const R ft = (R(0.5) * (ts + theta[o + nb])) * fm;
                if (to_h) {
                    const R ar = g.area_h[(long long)ll * ne + edge(j)];
                    const bool self_from = g.adj_sign[j * nc + c] > 0;
                    const R am = fm * ar, at = ft * ar;
                    hm.add(self_from ? am : -am);
                    ht.add(self_from ? at : -at);
                }
                if (to_up || to_lo) {
                    const R wc = wcorr(ll, j);
                    if (to_up) {
                        um += wc * fm;
                        ut += wc * ft;
                    }
                    if (to_lo) {
                        lm += wc * fm;
                        lt += wc * ft;
                    }
                }
            }
        };
        if (up_has_prev) layer_pass(l - 1, false, true, false);
        layer_pass(l, true, up_corr, lo_has_curr);
        if (lo_corr) layer_pass(l + 1, false, false, true);
        const double div = inv_vol * (hm.value() + comp_v(um, lm));
        double y = -div;
        if (IRR) y = y + irr.mass_diff[cond * ns + i];
        if (p.moist) y = y + pt_rates[cond * ns + i];
        st.rho[cond * ns + i] = rk == 0 ? y : 0.0 * st.rho[cond * ns + i] + 1.0 * y;
        const double div_t = inv_vol * (ht.value() + comp_v(ut, lt));
        double yt = -div_t;
        if (p.moist || IRR) {
            /* diabatic heating: c_v-weighted, divided by c_p * Pi */
            R cv = R(0);
            for (int kk = 0; kk < cond; ++kk) cv += sv.rho[kk * ns + i] * ((kk % 2 == 0) ? cp_ice[i] : cp_water[i]);
            cv += sv.rho[cond * ns + i] * R(C_D_V);
            if (p.moist) cv += sv.rho[(cond + 1) * ns + i] * R(C_V_V);
            double heat = pt_heat[i] + sed_heat[i], rate = pt_rates[cond * ns + i];
            if (IRR) {
                heat = irr.heating_diss[i] + irr.temp_diff_heating[i] + irr.radiation[i] + pt_heat[i] + sed_heat[i];
                rate = pt_rates[cond * ns + i] + irr.mass_diff[cond * ns + i];
            }
            if (sizeof(R) == sizeof(double)) {
                yt = yt + C_D_V * double(sv.rho[cond * ns + i]) / double(cv) * heat
                              / (C_D_P * (double(g.exner_bg[i]) + double(sv.exner_pert[i])))
                     + rate * double(theta[i]);
            } else {
                const R fac = R(C_D_V) * sv.rho[cond * ns + i] / cv / (R(C_D_P) * (g.exner_bg[i] + sv.exner_pert[i]));
                yt = yt + wide(fac) * heat + rate * wide(theta[i]);
            }
        }
        st.rhotheta_v[i] = rk == 0 ? yt : 0.0 * st.rhotheta_v[i] + 1.0 * yt;
    }
    if (p.n_const == 1) return;
    /* the other constituents: upstream flux.  The cell's edges, neighbours,
     * orientation and layer-l wind and face areas are loaded once for all
     * of them. */
    int ej[6], nbj[6];
    bool sfj[6];
    R uj[6], arj[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        const bool on = j < n_edges;
        ej[j] = on ? g.adj[j * nc + c] : 0;
        nbj[j] = on ? g.adj_nbr[j * nc + c] : c;
        sfj[j] = on && g.adj_sign[j * nc + c] > 0;
        uj[j] = on ? sv.u[(long long)l * ne + ej[j]] : R(0);
        arj[j] = on ? g.area_h[(long long)l * ne + ej[j]] : R(0);
    }
    const long long o = (long long)l * nc;
    for (int k = 0; k < p.n_const; ++k) {
        if (k == cond) continue;
        const double new_w = rk == 1 ? 0.5 : 1.0, old_w = 1.0 - new_w;
        const R *f = sv.rho + k * ns;
        FluxSum<R> h;
        const R fs = f[o + c];
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            if (j >= n_edges) continue;
            const R ue = uj[j];
            const R fv = ((ue >= R(0)) == sfj[j] ? fs : f[o + nbj[j]]) * ue;
            const R a = fv * arj[j];
            h.add(sfj[j] ? a : -a);
        }
        double cv = 0.0;
        if (oro) {
            const R d_here = f[i];
            if (l == nl - n_oro - 1) {
                const R d_lo = w_lo <= R(0) ? d_here : f[i + nc];
                cv = wide(-d_lo * w_lo * area_lo);
            } else if (l == nl - 1) {
                const R d_up = w_up <= R(0) ? f[i - nc] : d_here;
                cv = wide(d_up * w_up * area_up);
            } else {
                const R d_up = w_up <= R(0) ? f[i - nc] : d_here;
                const R d_lo = w_lo <= R(0) ? d_here : f[i + nc];
                cv = wide(d_up * w_up * area_up - d_lo * w_lo * area_lo);
            }
        }
        const double div = inv_vol * (h.value() + cv);
        double y = -div;
        if (IRR) y = y + irr.mass_diff[k * ns + i];
        if (p.moist) {
            long long pt = k * ns;
            if (k == cond + 1) pt -= ns;
            y = y + pt_rates[pt + i];
        }
        st.rho[k * ns + i] = rk == 0 ? y : old_w * st.rho[k * ns + i] + new_w * y;
    }
}

/* per-thread column sweeps of the adjoint hold at most this many layers */
constexpr int MAX_L = 64;

}  // namespace
}  // namespace game

