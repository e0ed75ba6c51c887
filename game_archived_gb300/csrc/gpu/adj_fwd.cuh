/*
 * Differentiable restatement of the dry RKHEVI step for the adjoint and
 * tangent-linear models (adj_f64.cu).
 *
 * Every kernel here computes one operator of the step at one point from
 * explicit input arrays into explicit output arrays (no in-place update), so
 * that a step run keeps all its intermediate fields (the tape of the
 * adjoint).  The kernels are templated on the value type T: with T = double
 * they perform the same floating-point operations in the same order as the
 * fused FP64 step (the translation unit is compiled without FMA
 * contraction), with T = Dual they carry a directional derivative alongside
 * every value -- the tangent-linear model of exactly this arithmetic.  Grid
 * tables are double in both cases.
 *
 * Both builds: in the dry one (one constituent) the condensate deceleration
 * factor of the pressure gradient is rho/rho = 1 and the condensate term of
 * the vertical momentum equation is 0, and both are left out; the moist
 * build's own terms (phase transitions, the moist scalar tendencies, the
 * tracer solve) are in adj_moist.cuh.
 */
#pragma once

#include "kernels.cuh"

namespace game {
namespace {

/* ------------------------------------------------------------ dual numbers */
struct Dual {
    double v, d;
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b)
{
    const double q = a.v / b.v;
    return {q, (a.d - q * b.d) / b.v};
}
__device__ __forceinline__ Dual operator+(Dual a, double b) { return {a.v + b, a.d}; }
__device__ __forceinline__ Dual operator+(double a, Dual b) { return {a + b.v, b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, double b) { return {a.v - b, a.d}; }
__device__ __forceinline__ Dual operator-(double a, Dual b) { return {a - b.v, -b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return {a.v * b, a.d * b}; }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, double b) { return {a.v / b, a.d / b}; }
__device__ __forceinline__ Dual operator/(double a, Dual b)
{
    const double q = a / b.v;
    return {q, -q * b.d / b.v};
}
__device__ __forceinline__ Dual &operator+=(Dual &a, Dual b) { return a = a + b; }
__device__ __forceinline__ Dual &operator-=(Dual &a, Dual b) { return a = a - b; }

template <class T>
__device__ __forceinline__ T tzero();
template <>
__device__ __forceinline__ double tzero<double>() { return 0.0; }
template <>
__device__ __forceinline__ Dual tzero<Dual>() { return {0.0, 0.0}; }
/* a constant (derivative 0) */
template <class T>
__device__ __forceinline__ T tconst(double v);
template <>
__device__ __forceinline__ double tconst<double>(double v) { return v; }
template <>
__device__ __forceinline__ Dual tconst<Dual>(double v) { return {v, 0.0}; }

/* one state in device layout, value type T: rho is the main gas's density
 * (the only constituent of the dry build), rho_all all constituents
 * [C][L][Nc] (rho_all == rho when C = 1) */
template <class T>
struct AState {
    T *rho, *rt, *tp, *ep, *w, *u; /* [L][Nc] x4, [L+1][Nc], [L][Ne] */
    T *rho_all;
};

/* run constants of the differentiable step */
struct AParams {
    double dt, impl_thermo_weight;
    int n_const, n_cond; /* constituents; condensates (the main gas's index) */
};

template <class T>
__device__ __forceinline__ T a_density_total(const T *rho_all, int n_const, long long ns, long long i)
{
    T r = tzero<T>();
    for (int k = 0; k < n_const; ++k) r += rho_all[k * ns + i];
    return r;
}

__device__ __forceinline__ double ipw_d(const HGrid<double> &g, int j, int l, int c)
{
    return g.ipw[((long long)j * g.nl + l) * g.nc + c];
}

/* ----------------------------------------------------- operator restatements
 * (same order of operations as kernels.cuh / solvers.cuh, EXACT branches) */
template <class T>
__device__ __forceinline__ T a_gv(const HGrid<double> &g, const T *f, int k, int c)
{
    return (f[(long long)(k - 1) * g.nc + c] - f[(long long)k * g.nc + c]) / g.nd_v[(long long)k * g.nc + c];
}

template <class T>
__device__ __forceinline__ T a_grad_h(const HGrid<double> &g, const T *f, int l, int e)
{
    const int fr = g.from[e], to = g.to[e];
    const long long le = (long long)l * g.ne + e;
    T out = (f[(long long)l * g.nc + to] - f[(long long)l * g.nc + fr]) / g.nd_h[le];
    if (l >= g.nl - g.n_oro) {
        T c = ipw_d(g, 6, l, fr) * a_gv(g, f, l, fr);
        c += ipw_d(g, 6, l, to) * a_gv(g, f, l, to);
        if (l < g.nl - 1) {
            c += ipw_d(g, 7, l, fr) * a_gv(g, f, l + 1, fr);
            c += ipw_d(g, 7, l, to) * a_gv(g, f, l + 1, to);
        }
        c = 0.5 * c;
        out += -g.slope_h[le] * c;
    }
    return out;
}

template <class T>
__device__ __forceinline__ T a_hor_cov(const HGrid<double> &g, const T *u, const T *w, int l, int e)
{
    const long long le = (long long)l * g.ne + e;
    T r = u[le];
    if (l >= g.nl - g.n_oro) {
        const int fr = g.from[e], to = g.to[e];
        T c = ipw_d(g, 6, l, fr) * w[(long long)l * g.nc + fr];
        c += ipw_d(g, 6, l, to) * w[(long long)l * g.nc + to];
        if (l < g.nl - 1) {
            c += ipw_d(g, 7, l, fr) * w[(long long)(l + 1) * g.nc + fr];
            c += ipw_d(g, 7, l, to) * w[(long long)(l + 1) * g.nc + to];
        }
        c = 0.5 * c;
        r += g.slope_h[le] * c;
    }
    return r;
}

/* pressure gradient nl + l (manage_pressure_gradient.c:32-60) at every edge
 * and inner interface; device vector layout [w (L+1) Nc][u L Ne] */
template <class T>
__global__ void fa_pgrad(HGrid<double> g, AParams ap, AState<T> s, T *P)
{
    const long long nw = (long long)(g.nl + 1) * g.nc, n = nw + (long long)g.nl * g.ne;
    const long long ns = (long long)g.nl * g.nc;
    const long long i = gtid();
    if (i >= n) return;
    const double cdp = C_D_P;
    /* deceleration by the condensates (manage_pressure_gradient.c:63-69):
     * the gas share of the total density, averaged to the edge or interface
     * (1 exactly in the dry build, where it is left out) */
    auto decel = [&](long long a, long long b) {
        const T d_a = s.rho[a] / a_density_total(s.rho_all, ap.n_const, ns, a);
        const T d_b = s.rho[b] / a_density_total(s.rho_all, ap.n_const, ns, b);
        return 0.5 * (d_a + d_b);
    };
    if (i < nw) {
        const int k = (int)(i / g.nc), c = (int)(i - (long long)k * g.nc);
        if (k == 0 || k == g.nl) return;
        const long long up = (long long)(k - 1) * g.nc + c, lo = (long long)k * g.nc + c;
        T nl = a_gv(g, s.ep, k, c);
        T s_up = cdp * (g.theta_v_bg[up] + s.tp[up]), s_lo = cdp * (g.theta_v_bg[lo] + s.tp[lo]);
        nl = (0.5 * (s_up + s_lo)) * nl;
        T lt = (0.5 * (cdp * s.tp[up] + cdp * s.tp[lo])) * g.exner_bg_grad_v[(long long)k * g.nc + c];
        if (ap.n_const > 1) {
            const T dec = decel(up, lo);
            nl = dec * nl;
            lt = dec * lt;
        }
        P[i] = nl + lt;
    } else {
        const long long j = i - nw;
        const int l = (int)(j / g.ne), e = (int)(j - (long long)l * g.ne);
        const int fr = g.from[e], to = g.to[e];
        const long long cf = (long long)l * g.nc + fr, ct = (long long)l * g.nc + to;
        T nl = a_grad_h(g, s.ep, l, e);
        T s_to = cdp * (g.theta_v_bg[ct] + s.tp[ct]), s_fr = cdp * (g.theta_v_bg[cf] + s.tp[cf]);
        nl = (0.5 * (s_to + s_fr)) * nl;
        T lt = (0.5 * (cdp * s.tp[ct] + cdp * s.tp[cf])) * g.exner_bg_grad_h[(long long)l * g.ne + e];
        if (ap.n_const > 1) {
            const T dec = decel(ct, cf);
            nl = dec * nl;
            lt = dec * lt;
        }
        P[i] = nl + lt;
    }
}

/* relative vorticity on triangles (vorticities.c:167-222) */
template <class T>
__global__ void fa_tri(HGrid<double> g, const T *u, T *tri)
{
    const long long n = (long long)g.nl * g.nt;
    const long long i = gtid();
    if (i >= n) return;
    const int l = (int)(i / g.nt), t = (int)(i - (long long)l * g.nt);
    T acc = tzero<T>();
    for (int j = 0; j < 3; ++j) {
        const int e = g.vort_i[j * g.nt + t];
        const long long le = (long long)l * g.ne + e;
        T vel = u[le];
        double rescale = 1.0;
        if (l >= g.nl - g.n_oro) {
            const double zt = g.dual_z_t[i];
            rescale = (g.radius + zt) / (g.radius + g.z_h[le]);
            const double dz = zt - g.z_h[le];
            int lo;
            if (dz > 0.0) lo = l - 1;
            else if (l == g.nl - 1) lo = l - 1;
            else lo = l + 1;
            const long long lo_e = (long long)lo * g.ne + e;
            T vgrad = (u[le] - u[lo_e]) / (g.z_h[le] - g.z_h[lo_e]);
            vel += dz * vgrad;
        }
        acc += rescale * g.nd_h[le] * double(g.vort_s[j * g.nt + t]) * vel;
    }
    tri[i] = acc / g.dual_area_t[i];
}

/* tangential relative vorticity at level k (vorticities.c:104-165) */
template <class T>
__device__ __forceinline__ T a_rel_tan(const HGrid<double> &g, const T *u, const T *w, int k, int e)
{
    const int nl = g.nl;
    if (k == 0) k = 1;
    const double inv_area = 1.0 / g.dual_area_h[(long long)k * g.ne + e];
    if (k == nl) {
        T c2 = a_hor_cov(g, u, w, k - 1, e);
        return inv_area * g.nd_h[(long long)(k - 1) * g.ne + e] * c2;
    }
    const int fr = g.from[e], to = g.to[e];
    T c0 = a_hor_cov(g, u, w, k, e);
    T c2 = a_hor_cov(g, u, w, k - 1, e);
    return inv_area * (-g.nd_h[(long long)k * g.ne + e] * c0 + g.nd_v[(long long)k * g.nc + fr] * w[(long long)k * g.nc + fr]
                       + g.nd_h[(long long)(k - 1) * g.ne + e] * c2
                       - g.nd_v[(long long)k * g.nc + to] * w[(long long)k * g.nc + to]);
}

/* density of the tangential potential vorticity at level k (vorticities.c:40-70) */
template <class T>
__device__ __forceinline__ T a_dens_tan(const HGrid<double> &g, const T *rho, int k, int e)
{
    const int nl = g.nl, nc = g.nc, ne = g.ne, fr = g.from[e], to = g.to[e];
    if (k == 0) {
        T top = 0.5 * (rho[fr] + rho[to]);
        T below = 0.5 * (rho[nc + fr] + rho[nc + to]);
        return top + (top - below) / g.pvz[ne + e] * g.pvz[e];
    }
    if (k == nl) {
        const long long a = (long long)(nl - 1) * nc, b = (long long)(nl - 2) * nc;
        T low = 0.5 * (rho[a + fr] + rho[a + to]);
        T above = 0.5 * (rho[b + fr] + rho[b + to]);
        return low + (above - low) / g.pvz[3 * (long long)ne + e] * g.pvz[2 * (long long)ne + e];
    }
    const long long uf = (long long)(k - 1) * nc + fr, ut = (long long)(k - 1) * nc + to;
    return 0.25 * (rho[uf] + rho[ut] + rho[uf + nc] + rho[ut + nc]);
}

/* potential vorticity (tangential at levels, rhombus at layers) and the
 * horizontal mass flux (k_edge_vort) */
template <class T>
__global__ void fa_edge(HGrid<double> g, const T *u, const T *w, const T *rho, const T *tri, T *zh, T *zv, T *flux_h)
{
    const long long n = (long long)(g.nl + 1) * g.ne;
    const long long i = gtid();
    if (i >= n) return;
    const int k = (int)(i / g.ne), e = (int)(i - (long long)k * g.ne);
    const int nl = g.nl, nc = g.nc, ne = g.ne;
    zh[i] = (a_rel_tan(g, u, w, k, e) + g.f_vec[e]) / a_dens_tan(g, rho, k, e);
    if (k < nl) {
        const long long le = (long long)k * ne + e;
        const int tf = g.dual_from[e], tt = g.dual_to[e];
        const long long kt = (long long)k * g.nt;
        const double af = g.dual_area_t[kt + tf], at = g.dual_area_t[kt + tt];
        T rel = (af * tri[kt + tf] + at * tri[kt + tt]) / (af + at);
        T pv = rel + g.f_vec[ne + e];
        T dens = tzero<T>();
        for (int j = 0; j < 4; ++j)
            dens += g.rhombi_w[j * (long long)ne + e] * rho[(long long)k * nc + g.rhombi_i[j * (long long)ne + e]];
        zv[le] = pv / dens;
        T sv = 0.5 * (rho[(long long)k * nc + g.to[e]] + rho[(long long)k * nc + g.from[e]]);
        flux_h[le] = sv * u[le];
    }
}

/* kinetic energy and vertical mass flux (k_cell_kinetic); flux_v levels 0
 * and L are not written */
template <class T>
__global__ void fa_kin(HGrid<double> g, const T *u, const T *w, const T *rho, T *v2, T *flux_v)
{
    const long long ns = (long long)g.nl * g.nc;
    const long long i = gtid();
    if (i >= ns) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const int n_edges = c < N_PENT ? 5 : 6;
    T acc = tzero<T>();
    for (int j = 0; j < n_edges; ++j) {
        T ue = u[(long long)l * g.ne + g.adj[j * g.nc + c]];
        acc += ipw_d(g, j, l, c) * ue * ue;
    }
    T wu = w[i], wl = w[i + g.nc];
    acc += ipw_d(g, 6, l, c) * wu * wu;
    acc += ipw_d(g, 7, l, c) * wl * wl;
    v2[i] = acc;
    if (l >= 1) flux_v[i] = (0.5 * (rho[i - g.nc] + rho[i])) * wu;
}

/* modified TRSK vorticity flux at (layer l, edge e) (vorticity_flux.c:35-137) */
template <class T>
__device__ __forceinline__ T a_vflux_h(const HGrid<double> &g, const T *flux_h, const T *flux_v, const T *zh,
                                       const T *zv, int l, int e)
{
    const long long ne = g.ne;
    const T *mf = flux_h + (long long)l * ne;
    const T *pv = zv + (long long)l * ne;
    const int fr = g.from[e], to = g.to[e];
    T out = tzero<T>();
    if (fr < N_PENT) {
        for (int j = 0; j < 4; ++j) out += g.trsk_w[j * ne + e] * mf[g.trsk_i[j * ne + e]] * pv[g.trsk_m[j * ne + e]];
    } else {
        for (int j = 0; j < 5; ++j) {
            if (j == 2)
                out += g.trsk_w[j * ne + e] * mf[g.trsk_i[j * ne + e]] * 0.5 * (pv[g.trsk_m[j * ne + e]] + pv[e]);
            else
                out += g.trsk_w[j * ne + e] * mf[g.trsk_i[j * ne + e]] * pv[g.trsk_m[j * ne + e]];
        }
    }
    if (to < N_PENT) {
        for (int j = 5; j < 9; ++j) out += g.trsk_w[j * ne + e] * mf[g.trsk_i[j * ne + e]] * pv[g.trsk_m[j * ne + e]];
    } else {
        for (int j = 5; j < 10; ++j) {
            if (j == 7)
                out += g.trsk_w[j * ne + e] * mf[g.trsk_i[j * ne + e]] * 0.5 * (pv[g.trsk_m[j * ne + e]] + pv[e]);
            else
                out += g.trsk_w[j * ne + e] * mf[g.trsk_i[j * ne + e]] * pv[g.trsk_m[j * ne + e]];
        }
    }
    const T zt = zh[(long long)l * ne + e], zb = zh[(long long)(l + 1) * ne + e];
    const long long nc = g.nc;
    out -= 0.5 * ipw_d(g, 6, l, fr) * flux_v[l * nc + fr] * zt;
    out -= 0.5 * ipw_d(g, 6, l, to) * flux_v[l * nc + to] * zt;
    out -= 0.5 * ipw_d(g, 7, l, fr) * flux_v[(l + 1) * nc + fr] * zb;
    out -= 0.5 * ipw_d(g, 7, l, to) * flux_v[(l + 1) * nc + to] * zb;
    return out;
}

/* horizontal momentum: advection terms (adv), tendency with weights
 * (vector_tendencies_expl.c:79-131) and the wind update (manage_rkhevi.c:67-75).
 * Vector fields in device layout; tend_out may alias nothing. */
template <class T>
__global__ void fa_mom_h(HGrid<double> g, AParams ap, int adv, double new_w, double old_w, const T *P, const T *pg_old,
                         const T *flux_h, const T *flux_v, const T *zh, const T *zv, const T *v2, T *pvt, T *v2g,
                         const T *tend_in, T *tend_out, const T *u_old, T *u_new)
{
    const long long n = (long long)g.nl * g.ne;
    const long long i = gtid();
    if (i >= n) return;
    const long long nw = (long long)(g.nl + 1) * g.nc, vi = nw + i;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    if (adv) {
        pvt[vi] = a_vflux_h(g, flux_h, flux_v, zh, zv, l, e);
        v2g[vi] = a_grad_h(g, v2, l, e);
    }
    const double cur_hor = 0.5 + ap.impl_thermo_weight, old_hor = 1.0 - (0.5 + ap.impl_thermo_weight);
    T y = old_hor * pg_old[vi] - cur_hor * P[vi] + pvt[vi] - 0.5 * v2g[vi];
    T t = (new_w == 1.0) ? y : old_w * tend_in[vi] + new_w * y;
    tend_out[vi] = t;
    u_new[i] = u_old[i] + ap.dt * t;
}

/* vertical momentum: vertical vorticity flux (all levels), kinetic-energy
 * gradient, tendency; w itself is advanced by the sound-wave solver */
template <class T>
__global__ void fa_mom_v(HGrid<double> g, AParams ap, int adv, double new_w, double old_w, const T *P,
                         const T *flux_h, const T *zh, const T *v2, T *pvt, T *v2g, const T *tend_in, T *tend_out,
                         const T *rho_all = nullptr)
{
    const long long n = (long long)(g.nl + 1) * g.nc;
    const long long i = gtid();
    if (i >= n) return;
    const int k = (int)(i / g.nc), c = (int)(i - (long long)k * g.nc);
    const int nl = g.nl;
    if (adv) {
        T acc = tzero<T>();
        const int n_edges = c < N_PENT ? 5 : 6;
        const double vw = (k == 0 || k == nl) ? 1.0 : 0.5;
        const T *z = zh + (long long)k * g.ne;
        if (k >= 1)
            for (int j = 0; j < n_edges; ++j) {
                const int a = g.adj[j * g.nc + c];
                acc += vw * ipw_d(g, j, k - 1, c) * flux_h[(long long)(k - 1) * g.ne + a] * z[a];
            }
        if (k <= nl - 1)
            for (int j = 0; j < n_edges; ++j) {
                const int a = g.adj[j * g.nc + c];
                acc += vw * ipw_d(g, j, k, c) * flux_h[(long long)k * g.ne + a] * z[a];
            }
        pvt[i] = acc;
    }
    if (k == 0 || k == nl) {
        tend_out[i] = tzero<T>();
        return;
    }
    if (adv) v2g[i] = a_gv(g, v2, k, c);
    const double cur_ver = 1.0 - ap.impl_thermo_weight;
    T y = -cur_ver * P[i] + pvt[i] - 0.5 * v2g[i];
    if (rho_all) {
        /* condensate term (manage_pressure_gradient.c:74-87): the gas
         * deficit of the total density times gravity, averaged to the
         * interface, from the substage's state */
        const long long ns = (long long)nl * g.nc;
        const long long up = (long long)(k - 1) * g.nc + c, lo = (long long)k * g.nc + c;
        const long long gp = (long long)ap.n_cond * ns;
        const T d_up = rho_all[gp + up] / a_density_total(rho_all, ap.n_const, ns, up) - 1.0;
        const T d_lo = rho_all[gp + lo] / a_density_total(rho_all, ap.n_const, ns, lo) - 1.0;
        y = y + (0.5 * (d_up + d_lo)) * g.gravity_m_v[i];
    }
    T t = (new_w == 1.0) ? y : old_w * tend_in[i] + new_w * y;
    tend_out[i] = t;
}

/* theta_v = rho theta_v / rho and its perturbation */
template <class T>
__global__ void fa_theta(long long ns, const T *rho, const T *rt, T *theta)
{
    const long long i = gtid();
    if (i < ns) theta[i] = rt[i] / rho[i];
}

template <class T>
__global__ void fa_rediag(VGrid vg, AState<T> s)
{
    const long long ns = (long long)vg.nl * vg.nc, i = gtid();
    if (i < ns) s.tp[i] = s.rt[i] / s.rho[i] - vg.theta_v_bg[i];
}

/* mass and rho theta_v tendencies of the dry build (k_scalar_tend2, main
 * gas), new weight 1 in both substages */
template <class T>
__global__ void fa_scalar(HGrid<double> g, const T *rho, const T *theta, const T *u, T *st_rho, T *st_rt)
{
    const long long ns = (long long)g.nl * g.nc;
    const long long i = gtid();
    if (i >= ns) return;
    const int nl = g.nl, n_oro = g.n_oro;
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
                const double wc = -0.5 * ipw_d(g, j, ll, c) * g.slope_h[(long long)ll * ne + ed];
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
    st_rho[i] = -(inv_vol * (hm + comp_v(um, lm)));
    st_rt[i] = -(inv_vol * (ht + comp_v(ut, lt)));
}

/* ---------------------------------------------- vertical sound-wave solver
 * (column_solvers.c:19-383, EXACT order).  Per-layer work wl = 8 x [L][Nc]:
 * alpha, beta, gam, rho_expl, rt_expl, tp_expl, ep_expl, thl; per-interface
 * work wr = 8 x [L-1][Nc]: c, d, e, r, x (undamped solution), sol (damped),
 * th_int, rho_io */
enum { WL_A, WL_B, WL_G, WL_REXP, WL_RTEXP, WL_TPEXP, WL_EPEXP, WL_THL, WL_N };
enum { WR_C, WR_D, WR_E, WR_R, WR_X, WR_SOL, WR_TH, WR_RIO, WR_N };

template <class T>
__global__ void fa_waves_layer(VGrid vg, AParams ap, int rk, AState<T> so, AState<T> sn, const T *st_rho,
                               const T *st_rt, T *wl)
{
    const long long ns = (long long)vg.nl * vg.nc, b = gtid();
    if (b >= ns) return;
    const double dt = ap.dt, pdw = 0.5;
    const double vol = vg.volume[b];
    const T ro = so.rho[b], rto = so.rt[b];
    T alpha, beta, gam;
    if (rk == 0) {
        alpha = -rto / (ro * ro) / vol;
        beta = 1.0 / ro / vol;
        gam = R_D / (C_D_V * rto) * (vg.exner_bg[b] + so.ep[b]) / vol;
    } else {
        const T rn = sn.rho[b];
        const T ao = -rto / (ro * ro), bo = 1.0 / ro;
        const T go = R_D / (C_D_V * rto) * (vg.exner_bg[b] + so.ep[b]);
        const T an = -sn.rt[b] / (rn * rn), bn = 1.0 / rn;
        const T gn = R_D / (C_D_V * sn.rt[b]) * (vg.exner_bg[b] + sn.ep[b]);
        alpha = ((1.0 - pdw) * ao + pdw * an) / vol;
        beta = ((1.0 - pdw) * bo + pdw * bn) / vol;
        gam = ((1.0 - pdw) * go + pdw * gn) / vol;
    }
    wl[WL_A * ns + b] = alpha;
    wl[WL_B * ns + b] = beta;
    wl[WL_G * ns + b] = gam;
    wl[WL_REXP * ns + b] = ro + dt * st_rho[b];
    wl[WL_RTEXP * ns + b] = rto + dt * st_rt[b];
    wl[WL_TPEXP * ns + b] = so.tp[b] + dt * vol * (alpha * st_rho[b] + beta * st_rt[b]);
    wl[WL_EPEXP * ns + b] = so.ep[b] + dt * vol * gam * st_rt[b];
    wl[WL_THL * ns + b] = sn.rt[b] / sn.rho[b];
}

template <class T>
__global__ void fa_waves_rows(VGrid vg, AParams ap, AState<T> so, const T *st_w, const T *wl, T *wr)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long n = (long long)(nl - 1) * nc, q = gtid();
    if (q >= n) return;
    const int j = (int)(q / nc);
    const long long ns = (long long)nl * nc;
    const long long b = q, lo = q + nc, wi = q + nc;
    const double dt = ap.dt, iw = ap.impl_thermo_weight, dt2 = dt * dt;
    const T *al = wl + WL_A * ns, *be = wl + WL_B * ns, *ga = wl + WL_G * ns, *rexp = wl + WL_REXP * ns;
    const T *tpx = wl + WL_TPEXP * ns, *epx = wl + WL_EPEXP * ns, *thl = wl + WL_THL * ns;
    const T rho_io = 0.5 * (so.rho[b] + so.rho[lo]);
    const T rho_ie = 0.5 * (rexp[b] + rexp[lo]);
    const T th = 0.5 * (thl[b] + thl[lo]);
    const double dz = vg.z_scalar[b] - vg.z_scalar[lo], dpi = vg.exner_bg[b] - vg.exner_bg[lo];
    const T wo = so.w[wi];
    const T a0 = al[b], a1 = al[lo], b0 = be[b], b1 = be[lo], g0 = ga[b], g1 = ga[lo];
    wr[WR_D * n + q] = -(th * th) * (g0 + g1) + 0.5 * dpi * (a1 - a0 + th * (b1 - b0))
                       - dz / (iw * dt2 * C_D_P * rho_io)
                             * (2.0 / vg.area_v[wi] + dt * wo * 0.5 * (-1.0 / vg.volume[b] + 1.0 / vg.volume[lo]));
    wr[WR_R * n + q] = -(wo + dt * st_w[wi]) * dz / (iw * dt2 * C_D_P) + th * (epx[b] - epx[lo]) / dt
                       + 0.5 / dt * (tpx[b] + tpx[lo]) * dpi - dz / (iw * dt2 * C_D_P) * wo * rho_ie / rho_io;
    wr[WR_TH * n + q] = th;
    wr[WR_RIO * n + q] = rho_io;
    if (j < nl - 2) {
        const long long lo2 = lo + nc;
        const T th1 = 0.5 * (thl[lo] + thl[lo2]);
        const T rho_io1 = 0.5 * (so.rho[lo] + so.rho[lo2]);
        wr[WR_C * n + q] = th1 * g1 * th + 0.5 * (vg.exner_bg[lo] - vg.exner_bg[lo2]) * (a1 + b1 * th)
                           - (vg.z_scalar[lo] - vg.z_scalar[lo2]) / (iw * dt * C_D_P) * 0.5 * so.w[wi + nc]
                                 / (vg.volume[lo] * rho_io1);
        wr[WR_E * n + q] = th * g1 * th1 - 0.5 * dpi * (a1 + b1 * th1)
                           + dz / (iw * dt * C_D_P) * 0.5 * wo / (vg.volume[lo] * rho_io);
    }
}

/* Thomas elimination per column (column_solvers.c:641-669), then the Klemp
 * damping division; n = L - 1 <= 64 */
template <class T>
__global__ void fa_waves_thomas(int nc, int nl, const double *dden, T *wr)
{
    const int i = (int)gtid();
    if (i >= nc) return;
    const int n = nl - 1;
    const long long m = (long long)n * nc;
    T ep[MAX_L], rp[MAX_L];
    for (int j = 0; j < n; ++j) {
        const long long q = (long long)j * nc + i;
        const T dj = wr[WR_D * m + q], rj = wr[WR_R * m + q];
        if (j == 0) {
            ep[0] = wr[WR_E * m + q] / dj;
            rp[0] = rj / dj;
        } else {
            const T cm = wr[WR_C * m + q - nc];
            const T den = dj - ep[j - 1] * cm;
            if (j < n - 1) ep[j] = wr[WR_E * m + q] / den;
            rp[j] = (rj - rp[j - 1] * cm) / den;
        }
    }
    T x = rp[n - 1];
    wr[WR_X * m + (long long)(n - 1) * nc + i] = x;
    wr[WR_SOL * m + (long long)(n - 1) * nc + i] = x / dden[(long long)(n - 1) * nc + i];
    for (int j = n - 2; j >= 0; --j) {
        x = rp[j] - ep[j] * x;
        wr[WR_X * m + (long long)j * nc + i] = x;
        wr[WR_SOL * m + (long long)j * nc + i] = x / dden[(long long)j * nc + i];
    }
}

/* back-substitution into the new state (column_solvers.c:305-370); w at the
 * TOA and the surface is copied from the input state */
template <class T>
__global__ void fa_waves_apply(VGrid vg, AParams ap, AState<T> so, const T *wl, const T *wr, AState<T> out)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long ns = (long long)nl * nc, b = gtid();
    if (b >= ns) return;
    const int j = (int)(b / nc);
    const long long m = (long long)(nl - 1) * nc;
    const double dt = ap.dt;
    const T *sol = wr + WR_SOL * m, *th_int = wr + WR_TH * m, *rio = wr + WR_RIO * m;
    auto rho_new = [&](int jj, long long bb) {
        T num;
        if (jj == 0) num = sol[bb];
        else if (jj == nl - 1) num = -sol[bb - nc];
        else num = -sol[bb - nc] + sol[bb];
        return wl[WL_REXP * ns + bb] + dt * (num) / vg.volume[bb];
    };
    const T r_new = rho_new(j, b);
    T num;
    if (j == 0) num = th_int[b] * sol[b];
    else if (j == nl - 1) num = -th_int[b - nc] * sol[b - nc];
    else num = -th_int[b - nc] * sol[b - nc] + th_int[b] * sol[b];
    const T rt_new = wl[WL_RTEXP * ns + b] + dt * num / vg.volume[b];
    out.rho[b] = r_new;
    out.rt[b] = rt_new;
    out.tp[b] = rt_new / r_new - vg.theta_v_bg[b];
    out.ep[b] = so.ep[b] + vg.volume[b] * wl[WL_G * ns + b] * (rt_new - so.rt[b]);
    if (j < nl - 1) {
        const long long wi = b + nc;
        const T dint = 0.5 * (r_new + rho_new(j + 1, b + nc));
        out.w[wi] = (2.0 * sol[b] / vg.area_v[wi] - dint * so.w[wi]) / rio[b];
    }
    if (j == 0) out.w[b] = so.w[b];                     /* TOA: interface 0 */
    if (j == nl - 1) out.w[b + nc] = so.w[b + nc];      /* surface: interface L */
}

}  // namespace
}  // namespace game
