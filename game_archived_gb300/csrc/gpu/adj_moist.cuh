/*
 * The moist build's terms of the differentiable step (adj_fwd.cuh) and their
 * adjoints: temperature and phase transitions once per step
 * (src/constituents/derived_quantities.c:15-40, phase_trans.c:16-311),
 * the moist scalar tendencies (src/time_stepping/scalar_tendencies_expl.c:
 * 90-178: phase-transition rates, the c_v-weighted diabatic heating, the
 * upstream flux divergences of the non-main constituents), the tracer
 * column solve with its sedimentation heat (column_solvers.c:385-639) and
 * the moist surface pressure of the objective (write_output.c:105-121).
 *
 * Forward kernels are templated on the value type as in adj_fwd.cuh (double:
 * the fused FP64 step's operations in its order; Dual: the tangent-linear
 * model).  The adjoints of the pointwise maps (a cell's phase transitions,
 * its diabatic heating term, a column's surface pressure) are J^T ybar with
 * the local Jacobian J formed column by column in forward mode (one Dual
 * evaluation per input seed): the derivatives of exactly the implemented
 * arithmetic, branch by branch, with no hand derivation to get wrong.  The
 * stencil part (the tracers' upstream fluxes) has its own reverse kernel;
 * the tracer column solve reuses the operator adjoint of
 * three_band_solver_gen_densities (adj_ops_f64.cu).
 */
#pragma once

#include "adj_bwd.cuh"
#include "adj_fwd.cuh"
#include "solvers.cuh"

namespace game {
namespace {

/* ---------------------------------------------------- Dual elementary math
 * (the double versions stay visible beside the Dual overloads) */
using ::exp;
using ::fmax;
using ::fmin;
using ::pow;
using ::sqrt;
__device__ __forceinline__ double dval(double x) { return x; }
__device__ __forceinline__ double dval(Dual x) { return x.v; }
__device__ __forceinline__ Dual exp(Dual a)
{
    const double e = ::exp(a.v);
    return {e, a.d * e};
}
__device__ __forceinline__ Dual sqrt(Dual a)
{
    const double s = ::sqrt(a.v);
    return {s, a.d * 0.5 / s};
}
__device__ __forceinline__ Dual pow(Dual a, double b)
{
    return {::pow(a.v, b), a.d * b * ::pow(a.v, b - 1.0)};
}
__device__ __forceinline__ Dual pow(Dual a, Dual b)
{
    const double pv = ::pow(a.v, b.v);
    return {pv, pv * (b.d * ::log(a.v) + b.v * a.d / a.v)};
}
__device__ __forceinline__ Dual fmin(Dual a, Dual b) { return a.v <= b.v ? a : b; }
__device__ __forceinline__ Dual fmax(Dual a, double b) { return a.v >= b ? a : Dual{b, 0.0}; }
__device__ __forceinline__ Dual &operator+=(Dual &a, double b) { return a = a + b; }
__device__ __forceinline__ Dual &operator-=(Dual &a, double b) { return a = a - b; }

/* ------------------------------------------- thermodynamics (dictionary.c)
 * the expressions of kernels.cuh, templated */
template <class T>
__device__ __forceinline__ T t_c_p_ice(T t)
{
    if (dval(t) > T_0) t = tconst<T>(T_0);
    if (dval(t) < 20.0) t = tconst<T>(20.0);
    T q = t / 125.1;
    T r = -2.0572 + 0.14644 * t + 0.06163 * t * exp(-(q * q));
    return r / M_V;
}

template <class T>
__device__ __forceinline__ T t_c_p_water(T t)
{
    T tc = t - T_0, r;
    if (dval(tc) >= 0.0) {
        if (dval(tc) > 35.0) tc = tconst<T>(35.0);
        T a = tc - 35.0;
        r = 0.9979 + 3.1e-6 * (a * a) + 3.8e-9 * pow(a, 4.0);
    } else {
        if (dval(tc) < -37.0) tc = tconst<T>(-37.0);
        r = 1.000938 - 2.7052e-3 * tc - 2.3235e-5 * (tc * tc) + 4.3778e-6 * pow(tc, 3.0) + 2.7136e-7 * pow(tc, 4.0);
    }
    return 4186.8 * r;
}

template <class T>
__device__ __forceinline__ T t_enthalpy_evaporation(T t)
{
    T r;
    if (dval(t) < T_0) {
        if (dval(t) < 30.0) t = tconst<T>(30.0);
        r = 56579.0 - 42.212 * t + exp(0.1149 * (281.6 - t));
        r = r / M_V;
    } else {
        if (dval(t) > T_0 + 100.0) t = tconst<T>(T_0 + 100.0);
        r = 3151378.0 - 2386.0 * t;
    }
    return r;
}

template <class T>
__device__ __forceinline__ T t_enthalpy_sublimation(T t)
{
    if (dval(t) < 30.0) t = tconst<T>(30.0);
    if (dval(t) > T_0) t = tconst<T>(T_0);
    T q = t / 123.75;
    T r = 46782.5 + 35.8925 * t - 0.07414 * (t * t) + 541.5 * exp(-(q * q));
    return r / M_V;
}

template <class T>
__device__ __forceinline__ T t_sat_pressure_water(T t)
{
    T tc = t - T_0, r;
    if (dval(tc) > 100.0) tc = tconst<T>(100.0);
    if (dval(tc) > 0.0) {
        r = exp(34.494 - 4924.99 / (tc + 237.1)) / pow(tc + 105.0, 1.57);
    } else {
        if (dval(tc) < -50.0) tc = tconst<T>(-50.0);
        r = 6.107799961 + 4.436518521e-1 * tc + 1.428945805e-2 * (tc * tc) + 2.650648471e-4 * pow(tc, 3.0)
            + 3.031240396e-6 * pow(tc, 4.0) + 2.034080948e-8 * pow(tc, 5.0) + 6.136820929e-11 * pow(tc, 6.0);
        r = 100.0 * r;
    }
    return r;
}

template <class T>
__device__ __forceinline__ T t_sat_pressure_ice(T t)
{
    T tc = t - T_0;
    if (dval(tc) < -80.0) tc = tconst<T>(-80.0);
    if (dval(tc) > 0.0) tc = tconst<T>(0.0);
    T a = tc + 868.0;
    return exp(43.494 - 6545.8 / (tc + 278.0)) / (a * a);
}

/* number of inputs and outputs of a cell's moist prelude: inputs the six
 * constituent densities, theta_v' and Pi'; outputs the temperature, the
 * five phase-transition rates, the heating and c_p of ice and of water */
constexpr int PRE_IN = 8, PRE_OUT = 9;

/* temperature, phase-transition rates and heating of one cell (k_cell_prepare
 * of kernels.cuh, EXACT path): x[0..5] densities, x[6] theta_v', x[7] Pi';
 * y[0] T, y[1..5] rates, y[6] heating, y[7] c_p of ice, y[8] c_p of water */
template <class T>
__device__ __forceinline__ void moist_prelude(const VGrid &vg, double dt, long long i, const T *x, T *y)
{
    const T *rho = x; /* rho[k] for k < 6 */
    const T Tc = (vg.theta_v_bg[i] + x[6]) * (vg.exner_bg[i] + x[7]) / (1.0 + rho[5] / rho[4] * (M_D / M_V - 1.0));
    const T cpi = t_c_p_ice(Tc), cpw = t_c_p_water(Tc);
    const double max_cloud_water = 0.2e-3;
    const bool warm = dval(Tc) >= T_0;
    const T sat0 = warm ? t_sat_pressure_water(Tc) : t_sat_pressure_ice(Tc);
    const T wvp = rho[5] * R_V * Tc;
    const T dry = (rho[4] - rho[5]) * R_D * Tc;
    const T air = dry + wvp;
    const T ef = warm ? 1.00071 * exp(0.000000045 * air) : 0.99882 * exp(0.00000008 * air);
    const T sat = ef * sat0;
    T dsat;
    if (warm) {
        T tc = Tc - T_0;
        if (dval(tc) > 100.0) tc = tconst<T>(100.0);
        if (dval(tc) < 0.0) tc = tconst<T>(0.0);
        const T q0 = tc + 237.1;
        dsat = sat0 * (4924.99 / (q0 * q0) - 1.57 / (tc + 105.0));
    } else {
        T tc = Tc - T_0;
        if (dval(tc) < -80.0) tc = tconst<T>(-80.0);
        if (dval(tc) > 0.0) tc = tconst<T>(0.0);
        const T q0 = tc + 278.0;
        dsat = sat0 * (6545.8 / (q0 * q0) - 2.0 / (tc + 868.0));
    }
    const T h_evap = t_enthalpy_evaporation(Tc), h_subl = t_enthalpy_sublimation(Tc);
    const T h_melt = h_subl - h_evap;
    T cv = tzero<T>();
    for (int k = 0; k < 4; ++k) cv += rho[k] * ((k % 2 == 0) ? cpi : cpw);
    cv += rho[4] * C_D_V;
    cv += rho[5] * C_V_V;
    const T pth = warm ? h_evap : h_subl;
    const T a = -R_V * pth / cv;
    const T b = R_V * Tc - R_V * rho[5] * pth / cv + ef * dsat * pth / cv;
    const T cc = wvp - sat;
    const T pp = b / a;
    const T q = cc / a;
    const T diff = -0.5 * pp - sqrt(0.25 * (pp * pp) - q);
    T r0, r1, r2, r3, r4, heat;
    if (dval(sat) >= dval(wvp)) {
        if (warm) {
            r2 = -rho[2] / dt;
            const T ptd = fmin(rho[3], diff);
            r4 = ptd / dt;
            r3 = rho[2] / dt - ptd / dt;
            heat = r2 * h_melt - ptd * h_evap / dt;
        } else {
            r3 = -rho[3] / dt;
            const T ptd = fmin(rho[2], diff);
            r4 = ptd / dt;
            r2 = rho[3] / dt - ptd / dt;
            heat = -r3 * h_melt - ptd * h_subl / dt;
        }
    } else {
        if (warm) {
            r2 = -rho[2] / dt;
            r4 = diff / dt;
            r3 = rho[2] / dt - diff / dt;
            heat = r2 * h_melt - diff * h_evap / dt;
        } else {
            r3 = -rho[3] / dt;
            r4 = diff / dt;
            r2 = rho[3] / dt - diff / dt;
            heat = -r3 * h_melt - diff * h_subl / dt;
        }
    }
    r0 = tzero<T>();
    r1 = tzero<T>();
    if (!warm) {
        r0 = fmax(rho[2] - max_cloud_water * rho[4], 0.0) / 1000.0;
        r2 -= r0;
    } else {
        r1 = fmax(rho[3] - max_cloud_water * rho[4], 0.0) / 1000.0;
        r3 -= r1;
    }
    if (warm && dval(rho[0]) > 0.0) {
        r0 = -rho[0] / dt;
        r1 -= r0;
        heat += r0 * h_melt;
    }
    if (!warm && dval(rho[1]) > 0.0) {
        r1 = -rho[1] / dt;
        r0 -= r1;
        heat += -r1 * h_melt;
    }
    y[0] = Tc;
    y[1] = r0;
    y[2] = r1;
    y[3] = r2;
    y[4] = r3;
    y[5] = r4;
    y[6] = heat;
    y[7] = cpi;
    y[8] = cpw;
}

/* the prelude over all cells; pre = [PRE_OUT][L][Nc] */
template <class T>
__global__ void fa_prelude(VGrid vg, AParams ap, AState<T> s, T *pre)
{
    const long long ns = (long long)vg.nl * vg.nc, i = gtid();
    if (i >= ns) return;
    T x[PRE_IN], y[PRE_OUT];
    for (int k = 0; k < 6; ++k) x[k] = s.rho_all[k * ns + i];
    x[6] = s.tp[i];
    x[7] = s.ep[i];
    moist_prelude<T>(vg, ap.dt, i, x, y);
    for (int k = 0; k < PRE_OUT; ++k) pre[k * ns + i] = y[k];
}

/* its adjoint: xbar += J^T ybar, J by forward mode, one seed per input */
__global__ void ba_prelude(VGrid vg, AParams ap, AState<double> s, const double *pre_b, AState<double> sb)
{
    const long long ns = (long long)vg.nl * vg.nc, i = gtid();
    if (i >= ns) return;
    double yb[PRE_OUT];
    bool any = false;
    for (int k = 0; k < PRE_OUT; ++k) {
        yb[k] = pre_b[k * ns + i];
        any = any || yb[k] != 0.0;
    }
    if (!any) return;
    double xv[PRE_IN];
    for (int k = 0; k < 6; ++k) xv[k] = s.rho_all[k * ns + i];
    xv[6] = s.tp[i];
    xv[7] = s.ep[i];
    for (int m = 0; m < PRE_IN; ++m) {
        Dual x[PRE_IN], y[PRE_OUT];
        for (int k = 0; k < PRE_IN; ++k) x[k] = {xv[k], k == m ? 1.0 : 0.0};
        moist_prelude<Dual>(vg, ap.dt, i, x, y);
        double g = 0.0;
        for (int k = 0; k < PRE_OUT; ++k) g += y[k].d * yb[k];
        if (m < 6) sb.rho_all[m * ns + i] += g;
        else if (m == 6) sb.tp[i] += g;
        else sb.ep[i] += g;
    }
}

/* ------------------------------------------------- moist scalar tendencies
 * k_scalar_tend2 (kernels.cuh) with R = double: the main gas's mass flux and
 * rho theta_v flux as fa_scalar, plus the phase-transition rates, the
 * c_v-weighted diabatic heating, and the non-main constituents' upstream
 * fluxes with their rk 1 blend 0.5 old + 0.5 new.  str = [C][L][Nc]. */

/* the diabatic part of the rho theta_v tendency at one cell (inputs: six
 * densities, c_p of ice and water, the heating, the rate of the main gas,
 * theta_v, Pi'; Pi_bg a constant) */
constexpr int HEAT_IN = 12;
/* a = C_D_V rho_gas / c_v * heating / (c_p Pi), b = rate * theta_v: the step
 * adds them to the flux divergence one after the other */
template <class T>
__device__ __forceinline__ void heat_terms(double exner_bg, const T *x, T &a, T &b)
{
    T cv = tzero<T>();
    for (int kk = 0; kk < 4; ++kk) cv += x[kk] * ((kk % 2 == 0) ? x[6] : x[7]);
    cv += x[4] * C_D_V;
    cv += x[5] * C_V_V;
    a = C_D_V * x[4] / cv * x[8] / (C_D_P * (exner_bg + x[11]));
    b = x[9] * x[10];
}

template <class T>
__global__ void fa_scalar_moist(HGrid<double> g, AParams ap, int rk, const T *rho_all, const T *theta, const T *u,
                                const T *ep, const T *pre, const T *sed, const T *str_prev, T *str, T *strt)
{
    const long long ns = (long long)g.nl * g.nc;
    const long long i = gtid();
    if (i >= ns) return;
    const int nl = g.nl, n_oro = g.n_oro, cond = ap.n_cond, n_const = ap.n_const;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const long long nc = g.nc, ne = g.ne;
    const int n_edges = c < N_PENT ? 5 : 6;
    const bool oro = l >= nl - n_oro - 1;
    const bool up_corr = oro && l >= nl - n_oro;
    const bool lo_corr = oro && l < nl - 1;
    const bool up_has_prev = up_corr && l > nl - n_oro;
    const bool lo_has_curr = lo_corr && l + 1 > nl - n_oro;
    const double inv_vol = 1.0 / g.volume[i];
    const double area_up = g.area_v[(long long)l * nc + c], area_lo = g.area_v[(long long)(l + 1) * nc + c];
    const T *rho = rho_all + (long long)cond * ns;
    auto wcorr = [&](int ll, int j) {
        return -0.5 * ipw_d(g, j, ll, c) * g.slope_h[(long long)ll * ne + g.adj[j * nc + c]];
    };
    auto uval = [&](int ll, int j) { return u[(long long)ll * ne + g.adj[j * nc + c]]; };
    /* terrain correction of the wind at levels l and l + 1 */
    T w_up = tzero<T>(), w_lo = tzero<T>();
    if (oro) {
        if (up_has_prev)
            for (int j = 0; j < n_edges; ++j) w_up += wcorr(l - 1, j) * uval(l - 1, j);
        for (int j = 0; j < n_edges; ++j) {
            const T t = wcorr(l, j) * uval(l, j);
            if (up_corr) w_up += t;
            if (lo_has_curr) w_lo += t;
        }
        if (lo_corr)
            for (int j = 0; j < n_edges; ++j) w_lo += wcorr(l + 1, j) * uval(l + 1, j);
    }
    /* the main gas */
    T hm = tzero<T>(), ht = tzero<T>(), um = tzero<T>(), ut = tzero<T>(), lm = tzero<T>(), lt = tzero<T>();
    auto layer_pass = [&](int ll, bool to_h, bool to_up, bool to_lo) {
        const long long o = (long long)ll * nc;
        const T fs = rho[o + c], ts = theta[o + c];
        for (int j = 0; j < n_edges; ++j) {
            const int nb = g.adj_nbr[j * nc + c], ed = g.adj[j * nc + c];
            const T fm = (0.5 * (fs + rho[o + nb])) * u[(long long)ll * ne + ed];
            const T ft = (0.5 * (ts + theta[o + nb])) * fm;
            if (to_h) {
                const double ar = g.area_h[(long long)ll * ne + ed];
                const bool self_from = g.adj_sign[j * nc + c] > 0;
                const T am = fm * ar, at = ft * ar;
                hm += self_from ? am : -am;
                ht += self_from ? at : -at;
            }
            if (to_up || to_lo) {
                const double wc = wcorr(ll, j);
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
    auto comp_v = [&](T up, T lo) -> T {
        if (!oro) return tzero<T>();
        if (l == nl - n_oro - 1) return -lo * area_lo;
        if (l == nl - 1) return up * area_up;
        return up * area_up - lo * area_lo;
    };
    str[cond * ns + i] = -(inv_vol * (hm + comp_v(um, lm))) + pre[(1 + cond) * ns + i];
    {
        T x[HEAT_IN];
        for (int k = 0; k < 6; ++k) x[k] = rho_all[k * ns + i];
        x[6] = pre[7 * ns + i];
        x[7] = pre[8 * ns + i];
        x[8] = pre[6 * ns + i] + sed[i];
        x[9] = pre[(1 + cond) * ns + i];
        x[10] = theta[i];
        x[11] = ep[i];
        T a, b;
        heat_terms<T>(g.exner_bg[i], x, a, b);
        strt[i] = -(inv_vol * (ht + comp_v(ut, lt))) + a + b;
    }
    /* the other constituents: upstream flux */
    const long long o = (long long)l * nc;
    for (int k = 0; k < n_const; ++k) {
        if (k == cond) continue;
        const T *f = rho_all + (long long)k * ns;
        T h = tzero<T>();
        const T fs = f[o + c];
        for (int j = 0; j < n_edges; ++j) {
            const int ed = g.adj[j * nc + c], nb = g.adj_nbr[j * nc + c];
            const bool sf = g.adj_sign[j * nc + c] > 0;
            const T ue = u[(long long)l * ne + ed];
            const T fv = ((dval(ue) >= 0.0) == sf ? fs : f[o + nb]) * ue;
            const T a = fv * g.area_h[(long long)l * ne + ed];
            h += sf ? a : -a;
        }
        T cvr = tzero<T>();
        if (oro) {
            const T d_here = f[i];
            if (l == nl - n_oro - 1) {
                const T d_lo = dval(w_lo) <= 0.0 ? d_here : f[i + nc];
                cvr = -d_lo * w_lo * area_lo;
            } else if (l == nl - 1) {
                const T d_up = dval(w_up) <= 0.0 ? f[i - nc] : d_here;
                cvr = d_up * w_up * area_up;
            } else {
                const T d_up = dval(w_up) <= 0.0 ? f[i - nc] : d_here;
                const T d_lo = dval(w_lo) <= 0.0 ? d_here : f[i + nc];
                cvr = d_up * w_up * area_up - d_lo * w_lo * area_lo;
            }
        }
        const int pt = k == cond + 1 ? k - 1 : k;
        const T y = -(inv_vol * (h + cvr)) + pre[(1 + pt) * ns + i];
        str[k * ns + i] = rk == 0 ? y : 0.5 * str_prev[k * ns + i] + 0.5 * y;
    }
}

/* adjoint of fa_scalar_moist: the main gas's fluxes (as ba_scalar), the
 * heating term (J^T by forward mode), the rates, the upstream fluxes (the
 * upstream choice held) and the rk 1 blend */
__global__ void ba_scalar_moist(HGrid<double> g, AParams ap, int rk, const double *rho_all, const double *theta,
                                const double *u, const double *ep, const double *pre, const double *sed,
                                const double *str_b, const double *strt_b, double *rho_all_b, double *theta_b,
                                double *u_b, double *ep_b, double *pre_b, double *sed_b, double *str_prev_b)
{
    const long long ns = (long long)g.nl * g.nc;
    const long long i = gtid();
    if (i >= ns) return;
    const int nl = g.nl, n_oro = g.n_oro, cond = ap.n_cond, n_const = ap.n_const;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const long long nc = g.nc, ne = g.ne;
    const int n_edges = c < N_PENT ? 5 : 6;
    const bool oro = l >= nl - n_oro - 1;
    const bool up_corr = oro && l >= nl - n_oro;
    const bool lo_corr = oro && l < nl - 1;
    const bool up_has_prev = up_corr && l > nl - n_oro;
    const bool lo_has_curr = lo_corr && l + 1 > nl - n_oro;
    const double inv_vol = 1.0 / g.volume[i];
    const double area_up = g.area_v[(long long)l * nc + c], area_lo = g.area_v[(long long)(l + 1) * nc + c];
    const double *rho = rho_all + (long long)cond * ns;
    double *rho_b = rho_all_b + (long long)cond * ns;
    auto wcorr = [&](int ll, int j) {
        return -0.5 * ipw_d(g, j, ll, c) * g.slope_h[(long long)ll * ne + g.adj[j * nc + c]];
    };
    /* ---- the main gas and rho theta_v (as ba_scalar) */
    const double yb = str_b[cond * ns + i], ytb = strt_b[i];
    if (yb != 0.0) acc(&pre_b[(1 + cond) * ns + i], yb);
    if (ytb != 0.0) {
        /* heating term */
        double xv[HEAT_IN];
        for (int k = 0; k < 6; ++k) xv[k] = rho_all[k * ns + i];
        xv[6] = pre[7 * ns + i];
        xv[7] = pre[8 * ns + i];
        xv[8] = pre[6 * ns + i] + sed[i];
        xv[9] = pre[(1 + cond) * ns + i];
        xv[10] = theta[i];
        xv[11] = ep[i];
        double gb[HEAT_IN];
        for (int m = 0; m < HEAT_IN; ++m) {
            Dual x[HEAT_IN];
            for (int k = 0; k < HEAT_IN; ++k) x[k] = {xv[k], k == m ? 1.0 : 0.0};
            Dual a, b;
            heat_terms<Dual>(g.exner_bg[i], x, a, b);
            gb[m] = (a.d + b.d) * ytb;
        }
        for (int k = 0; k < 6; ++k) acc(&rho_all_b[k * ns + i], gb[k]);
        acc(&pre_b[7 * ns + i], gb[6]);
        acc(&pre_b[8 * ns + i], gb[7]);
        acc(&pre_b[6 * ns + i], gb[8]);
        acc(&sed_b[i], gb[8]);
        acc(&pre_b[(1 + cond) * ns + i], gb[9]);
        acc(&theta_b[i], gb[10]);
        acc(&ep_b[i], gb[11]);
    }
    if (yb != 0.0 || ytb != 0.0) {
        const double hb = -inv_vol * yb, htb = -inv_vol * ytb;
        double umb = 0.0, lmb = 0.0, utb = 0.0, ltb = 0.0;
        if (oro) {
            if (l == nl - n_oro - 1) {
                lmb = -area_lo * hb;
                ltb = -area_lo * htb;
            } else if (l == nl - 1) {
                umb = area_up * hb;
                utb = area_up * htb;
            } else {
                umb = area_up * hb;
                utb = area_up * htb;
                lmb = -area_lo * hb;
                ltb = -area_lo * htb;
            }
        }
        auto layer_pass = [&](int ll, bool to_h, bool to_up, bool to_lo) {
            const long long o = (long long)ll * nc;
            const double fs = rho[o + c], ts = theta[o + c];
            for (int j = 0; j < n_edges; ++j) {
                const int nb = g.adj_nbr[j * nc + c], ed = g.adj[j * nc + c];
                const long long le = (long long)ll * ne + ed;
                double fmb = 0.0, ftb = 0.0;
                if (to_h) {
                    const double ar = g.area_h[le];
                    const double sg = g.adj_sign[j * nc + c] > 0 ? 1.0 : -1.0;
                    fmb += sg * ar * hb;
                    ftb += sg * ar * htb;
                }
                if (to_up || to_lo) {
                    const double wc = wcorr(ll, j);
                    if (to_up) {
                        fmb += wc * umb;
                        ftb += wc * utb;
                    }
                    if (to_lo) {
                        fmb += wc * lmb;
                        ftb += wc * ltb;
                    }
                }
                const double uv = u[le];
                const double fm = (0.5 * (fs + rho[o + nb])) * uv;
                fmb += 0.5 * (ts + theta[o + nb]) * ftb;
                const double qt = 0.5 * fm * ftb;
                acc(&theta_b[o + c], qt);
                acc(&theta_b[o + nb], qt);
                const double qr = 0.5 * uv * fmb;
                acc(&rho_b[o + c], qr);
                acc(&rho_b[o + nb], qr);
                acc(&u_b[le], 0.5 * (fs + rho[o + nb]) * fmb);
            }
        };
        if (up_has_prev) layer_pass(l - 1, false, true, false);
        layer_pass(l, true, up_corr, lo_has_curr);
        if (lo_corr) layer_pass(l + 1, false, false, true);
    }
    /* ---- the other constituents */
    double w_up = 0.0, w_lo = 0.0;
    if (oro) {
        auto uval = [&](int ll, int j) { return u[(long long)ll * ne + g.adj[j * nc + c]]; };
        if (up_has_prev)
            for (int j = 0; j < n_edges; ++j) w_up += wcorr(l - 1, j) * uval(l - 1, j);
        for (int j = 0; j < n_edges; ++j) {
            const double t = wcorr(l, j) * uval(l, j);
            if (up_corr) w_up += t;
            if (lo_has_curr) w_lo += t;
        }
        if (lo_corr)
            for (int j = 0; j < n_edges; ++j) w_lo += wcorr(l + 1, j) * uval(l + 1, j);
    }
    double w_up_b = 0.0, w_lo_b = 0.0;
    const long long o = (long long)l * nc;
    for (int k = 0; k < n_const; ++k) {
        if (k == cond) continue;
        double y_b = str_b[k * ns + i];
        if (y_b == 0.0) continue;
        if (rk != 0) {
            acc(&str_prev_b[k * ns + i], 0.5 * y_b);
            y_b = 0.5 * y_b;
        }
        const int pt = k == cond + 1 ? k - 1 : k;
        acc(&pre_b[(1 + pt) * ns + i], y_b);
        const double s_b = -inv_vol * y_b; /* bar of h + cvr */
        const double *f = rho_all + (long long)k * ns;
        double *f_b = rho_all_b + (long long)k * ns;
        const double fs = f[o + c];
        for (int j = 0; j < n_edges; ++j) {
            const int ed = g.adj[j * nc + c], nb = g.adj_nbr[j * nc + c];
            const bool sf = g.adj_sign[j * nc + c] > 0;
            const long long le = (long long)l * ne + ed;
            const double ue = u[le];
            const bool self = (ue >= 0.0) == sf;
            const double fup = self ? fs : f[o + nb];
            const double a_b = (sf ? 1.0 : -1.0) * s_b * g.area_h[le]; /* bar of fv */
            acc(&f_b[self ? o + c : o + nb], ue * a_b);
            acc(&u_b[le], fup * a_b);
        }
        if (oro) {
            const double d_here = f[i];
            if (l == nl - n_oro - 1) {
                const bool here = w_lo <= 0.0;
                const double d_lo = here ? d_here : f[i + nc];
                acc(&f_b[here ? i : i + nc], -w_lo * area_lo * s_b);
                w_lo_b += -d_lo * area_lo * s_b;
            } else if (l == nl - 1) {
                const bool above = w_up <= 0.0;
                const double d_up = above ? f[i - nc] : d_here;
                acc(&f_b[above ? i - nc : i], w_up * area_up * s_b);
                w_up_b += d_up * area_up * s_b;
            } else {
                const bool above = w_up <= 0.0, here = w_lo <= 0.0;
                const double d_up = above ? f[i - nc] : d_here;
                const double d_lo = here ? d_here : f[i + nc];
                acc(&f_b[above ? i - nc : i], w_up * area_up * s_b);
                w_up_b += d_up * area_up * s_b;
                acc(&f_b[here ? i : i + nc], -w_lo * area_lo * s_b);
                w_lo_b += -d_lo * area_lo * s_b;
            }
        }
    }
    if (oro && (w_up_b != 0.0 || w_lo_b != 0.0)) {
        auto ub = [&](int ll, int j, double v) { acc(&u_b[(long long)ll * ne + g.adj[j * nc + c]], v); };
        if (up_has_prev)
            for (int j = 0; j < n_edges; ++j) ub(l - 1, j, wcorr(l - 1, j) * w_up_b);
        for (int j = 0; j < n_edges; ++j) {
            double v = 0.0;
            if (up_corr) v += w_up_b;
            if (lo_has_curr) v += w_lo_b;
            ub(l, j, wcorr(l, j) * v);
        }
        if (lo_corr)
            for (int j = 0; j < n_edges; ++j) ub(l + 1, j, wcorr(l + 1, j) * w_lo_b);
    }
}

/* -------------------------------------------------------- tracer solve
 * k_tracers_solve (solvers.cuh, EXACT path) and k_tracers_sedheat, templated:
 * the non-main constituents' implicit vertical advection and sedimentation
 * from the old densities so.rho_all, the old and new vertical wind and the
 * tendency str, into out.rho_all; at rk 0 the sedimentation heat from the old
 * condensates, the new wind, the temperature and c_p (pre) */
template <class T>
__global__ void fa_tracer_solve(VGrid vg, StepParams p, AState<T> so, const T *w_new, const T *str, AState<T> out)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long ns = (long long)nl * nc;
    const long long q = gtid();
    const int n_tr = p.n_const - 1;
    if (q >= (long long)n_tr * nc) return;
    const int slot = (int)(q / nc), i = (int)(q - (long long)slot * nc);
    const int k = slot < p.n_cond ? slot : slot + 1;
    bool has_sink;
    const double vsink = sink_velocity(p, k, has_sink);
    const double dt = p.dt, iw = 0.5, ew = 1.0 - iw;
    const T *ro = so.rho_all + k * ns;
    const T *tr = str + k * ns;
    const long long bot = i + ns - nc;
    const double a_sfc = vg.area_v[(long long)nl * nc + i];
    T ep[MAX_L], rp[MAX_L];
    T fi_prev = tzero<T>(), fr_prev = tzero<T>(), c_prev = tzero<T>();
    for (int j = 0; j < nl; ++j) {
        const long long b = i + (long long)j * nc;
        const double vol = vg.volume[b];
        T fi = tzero<T>(), fr = tzero<T>(), cj = tzero<T>(), ej = tzero<T>();
        if (j < nl - 1) {
            const long long wi = b + nc;
            T a_ = so.w[wi], b_ = w_new[wi];
            if (has_sink) {
                a_ = a_ - vsink;
                b_ = b_ - vsink;
            }
            const double ar = vg.area_v[wi];
            a_ = ar * a_;
            b_ = ar * b_;
            const T dio = dval(b_) >= 0.0 ? ro[b + nc] : ro[b];
            fi = a_;
            fr = dio * b_;
            if (dval(fi) >= 0.0) ej = -iw * dt / vol * fi;
            else cj = iw * dt / vg.volume[b + nc] * fi;
        }
        T dj, rj = ro[b] + dt * tr[b];
        if (j == 0) {
            dj = dval(fi) >= 0.0 ? tconst<T>(1.0) : 1.0 - iw * dt / vol * fi;
            rj += ew * dt * fr / vol;
        } else if (j == nl - 1) {
            dj = dval(fi_prev) >= 0.0 ? 1.0 + iw * dt / vol * fi_prev : tconst<T>(1.0);
            if (has_sink) dj += iw * vsink * dt * a_sfc / vol;
            rj += -ew * dt * fr_prev / vol;
            if (has_sink) rj += -ew * vsink * dt * ro[bot] * a_sfc / vol;
        } else {
            dj = tconst<T>(1.0);
            if (dval(fi_prev) >= 0.0) dj += iw * dt / vol * fi_prev;
            if (dval(fi) < 0.0) dj -= iw * dt / vol * fi;
            rj += ew * dt * (-fr_prev + fr) / vol;
        }
        if (j == 0) {
            ep[0] = ej / dj;
            rp[0] = rj / dj;
        } else {
            const T den = dj - ep[j - 1] * c_prev;
            if (j < nl - 1) ep[j] = ej / den;
            rp[j] = (rj - rp[j - 1] * c_prev) / den;
        }
        fi_prev = fi;
        fr_prev = fr;
        c_prev = cj;
    }
    T *rn = out.rho_all + k * ns;
    T x = rp[nl - 1];
    rn[(long long)(nl - 1) * nc + i] = dval(x) < 0.0 ? tzero<T>() : x;
    for (int j = nl - 2; j >= 0; --j) {
        x = rp[j] - ep[j] * x;
        rn[(long long)j * nc + i] = dval(x) < 0.0 ? tzero<T>() : x;
    }
}

template <class T>
__global__ void fa_sedheat(VGrid vg, StepParams p, AState<T> so, const T *w_new, const T *pre, T *sed)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long ns = (long long)nl * nc;
    const long long ii = gtid();
    if (ii >= nc) return;
    const int i = (int)ii, n_cond = p.n_cond;
    const long long bot = i + ns - nc;
    const double a_sfc = vg.area_v[(long long)nl * nc + i];
    const T *temperature = pre, *cp_ice = pre + 7 * ns, *cp_water = pre + 8 * ns;
    auto fe = [&](int k, int jj, double vsink, bool has) {
        const long long bb = i + (long long)jj * nc, wi = bb + nc;
        T b_ = w_new[wi];
        if (has) b_ = b_ - vsink;
        b_ = vg.area_v[wi] * b_;
        const long long up = dval(b_) >= 0.0 ? bb + nc : bb;
        const T fr = so.rho_all[k * ns + up] * b_;
        const T cp = (k % 2 == 0) ? cp_ice[up] : cp_water[up];
        return cp * temperature[up] * fr;
    };
    T h_up[SEDHEAT_MAX_COND];
    for (int j = 0; j < nl; ++j) {
        const long long b = i + (long long)j * nc;
        const double vol = vg.volume[b];
        T sh = tzero<T>();
        for (int k = 0; k < SEDHEAT_MAX_COND; ++k) {
            if (k >= n_cond) break;
            bool has;
            const double vs = sink_velocity(p, k, has);
            if (j == 0) {
                h_up[k] = fe(k, j, vs, has);
                sh += h_up[k] / vol;
            } else if (j == nl - 1) {
                sh += -h_up[k] / vol;
                const T cp = (k % 2 == 0) ? cp_ice[bot] : cp_water[bot];
                sh += -vs * temperature[bot] * cp * so.rho_all[k * ns + bot] * a_sfc / vol;
            } else {
                const T h = fe(k, j, vs, has);
                sh += (-h_up[k] + h) / vol;
                h_up[k] = h;
            }
        }
        sed[b] = sh;
    }
}

/* ------------------------------------------------------ moist objective
 * surface pressure of a column (write_output.c:105-121) from the lowest
 * layer: x = rho_gas, rho_vapour, theta_v', Pi' there */
constexpr int SFC_IN = 4;
template <class T>
__device__ __forceinline__ T sfc_pressure_moist(const VGrid &vg, const double *gm_v, int i, const T *x)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long si = (long long)(nl - 1) * nc + i;
    const double lapse = 0.0065;
    const T t_low = (vg.theta_v_bg[si] + x[2]) * (vg.exner_bg[si] + x[3])
                    / (1.0 + x[1] / x[0] * (M_D / M_V - 1.0));
    const T rgas = ((x[0] - x[1]) * R_D + x[1] * R_V) / x[0];
    const T pr = x[0] * rgas * t_low;
    const double gm = gm_v[(long long)(nl - 1) * nc + i];
    const double z = vg.z_scalar[si];
    const T t_sfc = t_low + lapse * (z - vg.z_v[(long long)nl * nc + i]);
    return pr / pow(1.0 - (t_sfc - t_low) / t_sfc, gm / (rgas * lapse));
}

}  // namespace
}  // namespace game
