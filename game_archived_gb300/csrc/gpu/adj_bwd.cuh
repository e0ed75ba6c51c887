/*
 * Hand-written adjoint kernels of the dry RKHEVI step (the reverse mode of
 * adj_fwd.cuh).  Each kernel takes the bar (adjoint) of one forward
 * kernel's outputs, recomputes the forward point values it needs from the
 * tape, and accumulates the bars of that kernel's inputs: x_bar += (dy/dx)^T
 * y_bar.  Gathers of the forward become scatters here; they use FP64
 * atomicAdd, so the summation order of a bar varies between runs by rounding
 * (about 1e-16 relative), which the dot-product test tolerates by orders of
 * magnitude.  Pointwise inputs are accumulated without atomics.
 */
#pragma once

#include "adj_fwd.cuh"

namespace game {
namespace {

__device__ __forceinline__ void acc(double *p, double v) { atomicAdd(p, v); }

/* ---------------------------------------------------- operator adjoints */
__device__ __forceinline__ void b_gv(const HGrid<double> &g, double *fb, int k, int c, double gb)
{
    const double q = gb / g.nd_v[(long long)k * g.nc + c];
    acc(&fb[(long long)(k - 1) * g.nc + c], q);
    acc(&fb[(long long)k * g.nc + c], -q);
}

__device__ __forceinline__ void b_grad_h(const HGrid<double> &g, double *fb, int l, int e, double ob)
{
    const int fr = g.from[e], to = g.to[e];
    const long long le = (long long)l * g.ne + e;
    const double q = ob / g.nd_h[le];
    acc(&fb[(long long)l * g.nc + to], q);
    acc(&fb[(long long)l * g.nc + fr], -q);
    if (l >= g.nl - g.n_oro) {
        const double cb = 0.5 * (-g.slope_h[le] * ob);
        b_gv(g, fb, l, fr, ipw_d(g, 6, l, fr) * cb);
        b_gv(g, fb, l, to, ipw_d(g, 6, l, to) * cb);
        if (l < g.nl - 1) {
            b_gv(g, fb, l + 1, fr, ipw_d(g, 7, l, fr) * cb);
            b_gv(g, fb, l + 1, to, ipw_d(g, 7, l, to) * cb);
        }
    }
}

__device__ __forceinline__ void b_hor_cov(const HGrid<double> &g, double *ub, double *wb, int l, int e, double rb)
{
    const long long le = (long long)l * g.ne + e;
    acc(&ub[le], rb);
    if (l >= g.nl - g.n_oro) {
        const int fr = g.from[e], to = g.to[e];
        const double cb = 0.5 * (g.slope_h[le] * rb);
        acc(&wb[(long long)l * g.nc + fr], ipw_d(g, 6, l, fr) * cb);
        acc(&wb[(long long)l * g.nc + to], ipw_d(g, 6, l, to) * cb);
        if (l < g.nl - 1) {
            acc(&wb[(long long)(l + 1) * g.nc + fr], ipw_d(g, 7, l, fr) * cb);
            acc(&wb[(long long)(l + 1) * g.nc + to], ipw_d(g, 7, l, to) * cb);
        }
    }
}

__device__ __forceinline__ void b_rel_tan(const HGrid<double> &g, double *ub, double *wb, int k, int e, double rb)
{
    const int nl = g.nl;
    if (k == 0) k = 1;
    const double ia = 1.0 / g.dual_area_h[(long long)k * g.ne + e];
    if (k == nl) {
        b_hor_cov(g, ub, wb, k - 1, e, ia * g.nd_h[(long long)(k - 1) * g.ne + e] * rb);
        return;
    }
    const int fr = g.from[e], to = g.to[e];
    const double s = ia * rb;
    b_hor_cov(g, ub, wb, k, e, -g.nd_h[(long long)k * g.ne + e] * s);
    acc(&wb[(long long)k * g.nc + fr], g.nd_v[(long long)k * g.nc + fr] * s);
    b_hor_cov(g, ub, wb, k - 1, e, g.nd_h[(long long)(k - 1) * g.ne + e] * s);
    acc(&wb[(long long)k * g.nc + to], -g.nd_v[(long long)k * g.nc + to] * s);
}

__device__ __forceinline__ void b_dens_tan(const HGrid<double> &g, double *rb, int k, int e, double db)
{
    const int nl = g.nl, nc = g.nc, ne = g.ne, fr = g.from[e], to = g.to[e];
    if (k == 0) {
        const double f = g.pvz[e] / g.pvz[ne + e];
        const double tb = 0.5 * (db * (1.0 + f)), bb = 0.5 * (-db * f);
        acc(&rb[fr], tb);
        acc(&rb[to], tb);
        acc(&rb[nc + fr], bb);
        acc(&rb[nc + to], bb);
        return;
    }
    if (k == nl) {
        const long long a = (long long)(nl - 1) * nc, b = (long long)(nl - 2) * nc;
        const double f = g.pvz[2 * (long long)ne + e] / g.pvz[3 * (long long)ne + e];
        const double lb = 0.5 * (db * (1.0 - f)), ab = 0.5 * (db * f);
        acc(&rb[a + fr], lb);
        acc(&rb[a + to], lb);
        acc(&rb[b + fr], ab);
        acc(&rb[b + to], ab);
        return;
    }
    const long long uf = (long long)(k - 1) * nc + fr, ut = (long long)(k - 1) * nc + to;
    const double q = 0.25 * db;
    acc(&rb[uf], q);
    acc(&rb[ut], q);
    acc(&rb[uf + nc], q);
    acc(&rb[ut + nc], q);
}

/* theta_v' = rho theta_v / rho - theta_bg: the bar of theta_v' moves to
 * rho theta_v and rho and is consumed */
__global__ void ba_rediag(long long ns, const double *rho, const double *rt, double *tp_b, double *rho_b, double *rt_b)
{
    const long long i = gtid();
    if (i >= ns) return;
    const double tb = tp_b[i], r = rho[i];
    rt_b[i] += tb / r;
    rho_b[i] -= tb * (rt[i] / r) / r;
    tp_b[i] = 0.0;
}

/* theta = rho theta_v / rho */
__global__ void ba_theta(long long ns, const double *rho, const double *rt, const double *theta_b, double *rho_b,
                         double *rt_b)
{
    const long long i = gtid();
    if (i >= ns) return;
    const double tb = theta_b[i], r = rho[i];
    rt_b[i] += tb / r;
    rho_b[i] -= tb * (rt[i] / r) / r;
}

__global__ void ba_pgrad(HGrid<double> g, AParams ap, AState<double> s, const double *P_b, double *tp_b,
                         double *ep_b, double *rho_all_b = nullptr)
{
    const long long nw = (long long)(g.nl + 1) * g.nc, n = nw + (long long)g.nl * g.ne;
    const long long ns = (long long)g.nl * g.nc;
    const long long i = gtid();
    if (i >= n) return;
    const double cdp = C_D_P;
    double pb = P_b[i];
    if (pb == 0.0) return;
    const bool moist = ap.n_const > 1 && rho_all_b;
    /* moist: P = dec (nl + l), dec = 0.5 (d_a + d_b), d = rho_gas / rho_total */
    auto decel = [&](long long a, long long b, double nl_plus_l) {
        double d = 0.0;
        for (const long long cell : {a, b}) {
            double tot = 0.0;
            for (int q = 0; q < ap.n_const; ++q) tot += s.rho_all[q * ns + cell];
            const double rg = s.rho[cell];
            d += 0.5 * (rg / tot);
            const double hb = 0.5 * nl_plus_l * pb;
            for (int q = 0; q < ap.n_const; ++q) {
                const double dq = ((q == ap.n_cond ? tot : 0.0) - rg) / (tot * tot);
                acc(&rho_all_b[q * ns + cell], dq * hb);
            }
        }
        return d;
    };
    if (i < nw) {
        const int k = (int)(i / g.nc), c = (int)(i - (long long)k * g.nc);
        if (k == 0 || k == g.nl) return;
        const long long up = (long long)(k - 1) * g.nc + c, lo = (long long)k * g.nc + c;
        const double G = a_gv(g, s.ep, k, c);
        const double S = 0.5 * (cdp * (g.theta_v_bg[up] + s.tp[up]) + cdp * (g.theta_v_bg[lo] + s.tp[lo]));
        if (moist) {
            const double lt = (0.5 * (cdp * s.tp[up] + cdp * s.tp[lo])) * g.exner_bg_grad_v[(long long)k * g.nc + c];
            pb = pb * decel(up, lo, S * G + lt);
        }
        const double tb = 0.5 * cdp * (G * pb) + 0.5 * cdp * g.exner_bg_grad_v[(long long)k * g.nc + c] * pb;
        acc(&tp_b[up], tb);
        acc(&tp_b[lo], tb);
        b_gv(g, ep_b, k, c, S * pb);
    } else {
        const long long j = i - nw;
        const int l = (int)(j / g.ne), e = (int)(j - (long long)l * g.ne);
        const int fr = g.from[e], to = g.to[e];
        const long long cf = (long long)l * g.nc + fr, ct = (long long)l * g.nc + to;
        const double G = a_grad_h(g, s.ep, l, e);
        const double S = 0.5 * (cdp * (g.theta_v_bg[ct] + s.tp[ct]) + cdp * (g.theta_v_bg[cf] + s.tp[cf]));
        if (moist) {
            const double lt = (0.5 * (cdp * s.tp[ct] + cdp * s.tp[cf])) * g.exner_bg_grad_h[(long long)l * g.ne + e];
            pb = pb * decel(ct, cf, S * G + lt);
        }
        const double tb = 0.5 * cdp * (G * pb) + 0.5 * cdp * g.exner_bg_grad_h[(long long)l * g.ne + e] * pb;
        acc(&tp_b[ct], tb);
        acc(&tp_b[cf], tb);
        b_grad_h(g, ep_b, l, e, S * pb);
    }
}

__global__ void ba_tri(HGrid<double> g, const double *tri_b, double *u_b)
{
    const long long n = (long long)g.nl * g.nt;
    const long long i = gtid();
    if (i >= n) return;
    const double tb = tri_b[i] / g.dual_area_t[i];
    if (tb == 0.0) return;
    const int l = (int)(i / g.nt), t = (int)(i - (long long)l * g.nt);
    for (int j = 0; j < 3; ++j) {
        const int e = g.vort_i[j * g.nt + t];
        const long long le = (long long)l * g.ne + e;
        double rescale = 1.0, dz = 0.0;
        long long lo_e = le;
        if (l >= g.nl - g.n_oro) {
            const double zt = g.dual_z_t[i];
            rescale = (g.radius + zt) / (g.radius + g.z_h[le]);
            dz = zt - g.z_h[le];
            int lo;
            if (dz > 0.0) lo = l - 1;
            else if (l == g.nl - 1) lo = l - 1;
            else lo = l + 1;
            lo_e = (long long)lo * g.ne + e;
        }
        const double vb = rescale * g.nd_h[le] * double(g.vort_s[j * g.nt + t]) * tb;
        acc(&u_b[le], vb);
        if (l >= g.nl - g.n_oro) {
            const double q = dz * vb / (g.z_h[le] - g.z_h[lo_e]);
            acc(&u_b[le], q);
            acc(&u_b[lo_e], -q);
        }
    }
}

__global__ void ba_edge(HGrid<double> g, const double *u, const double *rho, const double *zh, const double *zv,
                        const double *zh_b, const double *zv_b, const double *fh_b, double *u_b, double *w_b,
                        double *rho_b, double *tri_b)
{
    const long long n = (long long)(g.nl + 1) * g.ne;
    const long long i = gtid();
    if (i >= n) return;
    const int k = (int)(i / g.ne), e = (int)(i - (long long)k * g.ne);
    const int nl = g.nl, nc = g.nc, ne = g.ne;
    {
        const double zb = zh_b[i];
        if (zb != 0.0) {
            const double dens = a_dens_tan(g, rho, k, e);
            b_rel_tan(g, u_b, w_b, k, e, zb / dens);
            b_dens_tan(g, rho_b, k, e, -zb * zh[i] / dens);
        }
    }
    if (k < nl) {
        const long long le = (long long)k * ne + e;
        const double vb = zv_b[le];
        if (vb != 0.0) {
            double dens = 0.0;
            for (int j = 0; j < 4; ++j)
                dens += g.rhombi_w[j * (long long)ne + e] * rho[(long long)k * nc + g.rhombi_i[j * (long long)ne + e]];
            const double pb = vb / dens, db = -vb * zv[le] / dens;
            for (int j = 0; j < 4; ++j)
                acc(&rho_b[(long long)k * nc + g.rhombi_i[j * (long long)ne + e]], g.rhombi_w[j * (long long)ne + e] * db);
            const int tf = g.dual_from[e], tt = g.dual_to[e];
            const long long kt = (long long)k * g.nt;
            const double af = g.dual_area_t[kt + tf], at = g.dual_area_t[kt + tt];
            acc(&tri_b[kt + tf], af / (af + at) * pb);
            acc(&tri_b[kt + tt], at / (af + at) * pb);
        }
        const double fb = fh_b[le];
        if (fb != 0.0) {
            const long long ct = (long long)k * nc + g.to[e], cf = (long long)k * nc + g.from[e];
            acc(&u_b[le], 0.5 * (rho[ct] + rho[cf]) * fb);
            const double q = 0.5 * u[le] * fb;
            acc(&rho_b[ct], q);
            acc(&rho_b[cf], q);
        }
    }
}

__global__ void ba_kin(HGrid<double> g, const double *u, const double *w, const double *rho, const double *v2_b,
                       const double *fv_b, double *u_b, double *w_b, double *rho_b)
{
    const long long ns = (long long)g.nl * g.nc;
    const long long i = gtid();
    if (i >= ns) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const int n_edges = c < N_PENT ? 5 : 6;
    const double vb = v2_b[i];
    if (vb != 0.0) {
        for (int j = 0; j < n_edges; ++j) {
            const long long le = (long long)l * g.ne + g.adj[j * g.nc + c];
            acc(&u_b[le], 2.0 * ipw_d(g, j, l, c) * u[le] * vb);
        }
        acc(&w_b[i], 2.0 * ipw_d(g, 6, l, c) * w[i] * vb);
        acc(&w_b[i + g.nc], 2.0 * ipw_d(g, 7, l, c) * w[i + g.nc] * vb);
    }
    if (l >= 1) {
        const double fb = fv_b[i];
        if (fb != 0.0) {
            acc(&w_b[i], 0.5 * (rho[i - g.nc] + rho[i]) * fb);
            const double q = 0.5 * w[i] * fb;
            acc(&rho_b[i - g.nc], q);
            acc(&rho_b[i], q);
        }
    }
}

__device__ __forceinline__ void b_vflux_h(const HGrid<double> &g, const double *flux_h, const double *flux_v,
                                          const double *zh, const double *zv, double *fh_b, double *fv_b,
                                          double *zh_b, double *zv_b, int l, int e, double ob)
{
    const long long ne = g.ne, nc = g.nc;
    const double *mf = flux_h + (long long)l * ne, *pv = zv + (long long)l * ne;
    double *mfb = fh_b + (long long)l * ne, *pvb = zv_b + (long long)l * ne;
    const int fr = g.from[e], to = g.to[e];
    auto term = [&](int j, bool half) {
        const double w = g.trsk_w[j * ne + e];
        const int ti = g.trsk_i[j * ne + e], tm = g.trsk_m[j * ne + e];
        if (half) {
            acc(&mfb[ti], w * 0.5 * (pv[tm] + pv[e]) * ob);
            const double q = w * mf[ti] * 0.5 * ob;
            acc(&pvb[tm], q);
            acc(&pvb[e], q);
        } else {
            acc(&mfb[ti], w * pv[tm] * ob);
            acc(&pvb[tm], w * mf[ti] * ob);
        }
    };
    if (fr < N_PENT)
        for (int j = 0; j < 4; ++j) term(j, false);
    else
        for (int j = 0; j < 5; ++j) term(j, j == 2);
    if (to < N_PENT)
        for (int j = 5; j < 9; ++j) term(j, false);
    else
        for (int j = 5; j < 10; ++j) term(j, j == 7);
    const double zt = zh[(long long)l * ne + e], zb = zh[(long long)(l + 1) * ne + e];
    const double i6f = 0.5 * ipw_d(g, 6, l, fr), i6t = 0.5 * ipw_d(g, 6, l, to);
    const double i7f = 0.5 * ipw_d(g, 7, l, fr), i7t = 0.5 * ipw_d(g, 7, l, to);
    acc(&fv_b[l * nc + fr], -i6f * zt * ob);
    acc(&fv_b[l * nc + to], -i6t * zt * ob);
    acc(&fv_b[(l + 1) * nc + fr], -i7f * zb * ob);
    acc(&fv_b[(l + 1) * nc + to], -i7t * zb * ob);
    acc(&zh_b[(long long)l * ne + e], -(i6f * flux_v[l * nc + fr] + i6t * flux_v[l * nc + to]) * ob);
    acc(&zh_b[(long long)(l + 1) * ne + e],
        -(i7f * flux_v[(l + 1) * nc + fr] + i7t * flux_v[(l + 1) * nc + to]) * ob);
}

/* horizontal momentum: t_b holds the bar of this substage's tendency from its
 * later uses, u_new_b the bar of the new wind; pvt_b / v2g_b may already hold
 * bars from the next step (they are lagged into it) */
__global__ void ba_mom_h(HGrid<double> g, AParams ap, int adv, double new_w, double old_w, const double *flux_h,
                         const double *flux_v, const double *zh, const double *zv, const double *t_b,
                         const double *u_new_b, double *u_old_b, double *tend_in_b, double *P_b, double *pgo_b,
                         double *pvt_b, double *v2g_b, double *fh_b, double *fv_b, double *zh_b, double *zv_b,
                         double *v2_b)
{
    const long long n = (long long)g.nl * g.ne;
    const long long i = gtid();
    if (i >= n) return;
    const long long nw = (long long)(g.nl + 1) * g.nc, vi = nw + i;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    const double ub = u_new_b[i];
    u_old_b[i] += ub;
    const double tb = t_b[vi] + ap.dt * ub;
    double yb;
    if (new_w == 1.0) {
        yb = tb;
    } else {
        tend_in_b[vi] += old_w * tb;
        yb = new_w * tb;
    }
    const double cur_hor = 0.5 + ap.impl_thermo_weight, old_hor = 1.0 - (0.5 + ap.impl_thermo_weight);
    pgo_b[vi] += old_hor * yb;
    P_b[vi] += -cur_hor * yb;
    const double pb = pvt_b[vi] + yb, gb = v2g_b[vi] - 0.5 * yb;
    pvt_b[vi] = pb;
    v2g_b[vi] = gb;
    if (adv) {
        if (pb != 0.0) b_vflux_h(g, flux_h, flux_v, zh, zv, fh_b, fv_b, zh_b, zv_b, l, e, pb);
        if (gb != 0.0) b_grad_h(g, v2_b, l, e, gb);
    }
}

__global__ void ba_mom_v(HGrid<double> g, AParams ap, int adv, double new_w, double old_w, const double *flux_h,
                         const double *zh, const double *t_b, double *tend_in_b, double *P_b, double *pvt_b,
                         double *v2g_b, double *fh_b, double *zh_b, double *v2_b, const double *rho_all = nullptr,
                         double *rho_all_b = nullptr)
{
    const long long n = (long long)(g.nl + 1) * g.nc;
    const long long i = gtid();
    if (i >= n) return;
    const int k = (int)(i / g.nc), c = (int)(i - (long long)k * g.nc);
    const int nl = g.nl;
    double pb = pvt_b[i];
    if (k != 0 && k != nl) {
        const double tb = t_b[i];
        double yb;
        if (new_w == 1.0) {
            yb = tb;
        } else {
            tend_in_b[i] += old_w * tb;
            yb = new_w * tb;
        }
        const double cur_ver = 1.0 - ap.impl_thermo_weight;
        P_b[i] += -cur_ver * yb;
        pb += yb;
        if (rho_all && yb != 0.0) {
            /* condensate term 0.5 (d_up + d_lo) g_m, d = rho_gas / rho_total - 1 */
            const long long ns = (long long)nl * g.nc, gp = (long long)ap.n_cond * ns;
            const double hb = 0.5 * g.gravity_m_v[i] * yb;
            for (const long long cell : {(long long)(k - 1) * g.nc + c, (long long)k * g.nc + c}) {
                double tot = 0.0;
                for (int q = 0; q < ap.n_const; ++q) tot += rho_all[q * ns + cell];
                const double rg = rho_all[gp + cell];
                /* d(rg / tot) / d rho_q = (delta_q,gas tot - rg) / tot^2 */
                for (int q = 0; q < ap.n_const; ++q) {
                    const double dq = ((q == ap.n_cond ? tot : 0.0) - rg) / (tot * tot);
                    acc(&rho_all_b[q * ns + cell], dq * hb);
                }
            }
        }
        const double gb = v2g_b[i] - 0.5 * yb;
        v2g_b[i] = gb;
        if (adv && gb != 0.0) b_gv(g, v2_b, k, c, gb);
    }
    pvt_b[i] = pb;
    if (adv && pb != 0.0) {
        const int n_edges = c < N_PENT ? 5 : 6;
        const double vw = (k == 0 || k == nl) ? 1.0 : 0.5;
        const double *z = zh + (long long)k * g.ne;
        double *zb = zh_b + (long long)k * g.ne;
        if (k >= 1)
            for (int j = 0; j < n_edges; ++j) {
                const int a = g.adj[j * g.nc + c];
                const double wv = vw * ipw_d(g, j, k - 1, c);
                acc(&fh_b[(long long)(k - 1) * g.ne + a], wv * z[a] * pb);
                acc(&zb[a], wv * flux_h[(long long)(k - 1) * g.ne + a] * pb);
            }
        if (k <= nl - 1)
            for (int j = 0; j < n_edges; ++j) {
                const int a = g.adj[j * g.nc + c];
                const double wv = vw * ipw_d(g, j, k, c);
                acc(&fh_b[(long long)k * g.ne + a], wv * z[a] * pb);
                acc(&zb[a], wv * flux_h[(long long)k * g.ne + a] * pb);
            }
    }
}

/* mass and rho theta_v tendencies (fa_scalar) */
__global__ void ba_scalar(HGrid<double> g, const double *rho, const double *theta, const double *u,
                          const double *st_rho_b, const double *st_rt_b, double *rho_b, double *theta_b, double *u_b)
{
    const long long ns = (long long)g.nl * g.nc;
    const long long i = gtid();
    if (i >= ns) return;
    const double yb = st_rho_b[i], ytb = st_rt_b[i];
    if (yb == 0.0 && ytb == 0.0) return;
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
                const double wc = -0.5 * ipw_d(g, j, ll, c) * g.slope_h[le];
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
            /* ft = 0.5 (theta_c + theta_nb) fm */
            fmb += 0.5 * (ts + theta[o + nb]) * ftb;
            const double qt = 0.5 * fm * ftb;
            acc(&theta_b[o + c], qt);
            acc(&theta_b[o + nb], qt);
            /* fm = 0.5 (rho_c + rho_nb) u */
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

/* ------------------------------------------------- sound-wave solver adjoints */

/* apply, phase 1 (per layer): theta_v', Pi' and the TOA / surface copies of w */
__global__ void ba_apply_layer(VGrid vg, AState<double> so, const double *wl, AState<double> out, AState<double> out_b,
                               double *rn_b, double *rtn_b, AState<double> so_b, double *wl_b)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long ns = (long long)nl * nc, b = gtid();
    if (b >= ns) return;
    const int j = (int)(b / nc);
    const double vol = vg.volume[b], gam = wl[WL_G * ns + b];
    const double rn = out.rho[b], rtn = out.rt[b];
    const double tpb = out_b.tp[b], epb = out_b.ep[b];
    rtn_b[b] = out_b.rt[b] + tpb / rn + epb * vol * gam;
    rn_b[b] = out_b.rho[b] - tpb * (rtn / rn) / rn;
    so_b.ep[b] += epb;
    wl_b[WL_G * ns + b] += epb * vol * (rtn - so.rt[b]);
    so_b.rt[b] -= epb * vol * gam;
    if (j == 0) so_b.w[b] += out_b.w[b];
    if (j == nl - 1) so_b.w[b + nc] += out_b.w[b + nc];
}

/* apply, phase 2 (per inner interface): w */
__global__ void ba_apply_w(VGrid vg, AState<double> so, const double *wr, AState<double> out, AState<double> out_b,
                           double *rn_b, AState<double> so_b, double *wr_b)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long m = (long long)(nl - 1) * nc, q = gtid();
    if (q >= m) return;
    const long long wi = q + nc;
    const double wb = out_b.w[wi];
    if (wb == 0.0) return;
    const double rio = wr[WR_RIO * m + q];
    const double dint = 0.5 * (out.rho[q] + out.rho[q + nc]);
    wr_b[WR_SOL * m + q] += 2.0 * wb / (vg.area_v[wi] * rio);
    const double db = -wb * so.w[wi] / rio;
    so_b.w[wi] += -wb * dint / rio;
    wr_b[WR_RIO * m + q] += -wb * out.w[wi] / rio;
    acc(&rn_b[q], 0.5 * db);
    acc(&rn_b[q + nc], 0.5 * db);
}

/* apply, phase 3 (per layer): rho and rho theta_v from the solution */
__global__ void ba_apply_rho(VGrid vg, AParams ap, const double *wr, const double *rn_b, const double *rtn_b,
                             double *wl_b, double *wr_b)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long ns = (long long)nl * nc, b = gtid();
    if (b >= ns) return;
    const int j = (int)(b / nc);
    const long long m = (long long)(nl - 1) * nc;
    const double dt = ap.dt, vol = vg.volume[b];
    const double rb = rn_b[b], rtb = rtn_b[b];
    wl_b[WL_REXP * ns + b] += rb;
    wl_b[WL_RTEXP * ns + b] += rtb;
    const double nb = rb * dt / vol, ntb = rtb * dt / vol;
    const double *sol = wr + WR_SOL * m, *th = wr + WR_TH * m;
    double *sol_b = wr_b + WR_SOL * m, *th_b = wr_b + WR_TH * m;
    if (j < nl - 1) {
        acc(&sol_b[b], nb + th[b] * ntb);
        acc(&th_b[b], sol[b] * ntb);
    }
    if (j > 0) {
        acc(&sol_b[b - nc], -nb - th[b - nc] * ntb);
        acc(&th_b[b - nc], -sol[b - nc] * ntb);
    }
}

/* transposed tridiagonal solve per column: lambda = A^-T xbar with xbar the
 * bar of the undamped solution; then rbar = lambda and the coefficient bars
 * -lambda x^T on the three diagonals */
__global__ void ba_thomas(int nc, int nl, const double *dden, const double *wr, double *wr_b)
{
    const int i = (int)gtid();
    if (i >= nc) return;
    const int n = nl - 1;
    const long long m = (long long)n * nc;
    const double *cc = wr + WR_C * m, *dd = wr + WR_D * m, *ee = wr + WR_E * m, *x = wr + WR_X * m;
    double ep[MAX_L], rp[MAX_L];
    for (int j = 0; j < n; ++j) {
        const long long q = (long long)j * nc + i;
        const double xb = wr_b[WR_SOL * m + q] / dden[q];
        const double dj = dd[q];
        if (j == 0) {
            if (n > 1) ep[0] = cc[q] / dj;
            rp[0] = xb / dj;
        } else {
            const double sub = ee[q - nc]; /* (A^T)_{j,j-1} = e_{j-1} */
            const double den = dj - ep[j - 1] * sub;
            if (j < n - 1) ep[j] = cc[q] / den; /* (A^T)_{j,j+1} = c_j */
            rp[j] = (xb - rp[j - 1] * sub) / den;
        }
    }
    double lam_next = 0.0;
    for (int j = n - 1; j >= 0; --j) {
        const long long q = (long long)j * nc + i;
        const double lam = (j == n - 1) ? rp[j] : rp[j] - ep[j] * lam_next;
        wr_b[WR_R * m + q] += lam;
        wr_b[WR_D * m + q] += -lam * x[q];
        if (j < n - 1) {
            wr_b[WR_E * m + q] += -lam * x[q + nc];
            wr_b[WR_C * m + q] += -lam_next * x[q];
        }
        lam_next = lam;
    }
}

/* the rows (fa_waves_rows) per inner interface: bars of c, d, e, r, th_int
 * and rho_io scattered to the per-layer work bars, rho and w of the old
 * state and the vertical-wind tendency */
__global__ void ba_waves_rows(VGrid vg, AParams ap, AState<double> so, const double *wl, const double *wr,
                              const double *wr_b, double *wl_b, AState<double> so_b, double *st_w_b)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long n = (long long)(nl - 1) * nc, q = gtid();
    if (q >= n) return;
    const int j = (int)(q / nc);
    const long long ns = (long long)nl * nc;
    const long long b = q, lo = q + nc, wi = q + nc;
    const double dt = ap.dt, iw = ap.impl_thermo_weight, dt2 = dt * dt;
    const double K1 = iw * dt2 * C_D_P, K2 = iw * dt * C_D_P;
    const double *al = wl + WL_A * ns, *be = wl + WL_B * ns, *ga = wl + WL_G * ns, *rexp = wl + WL_REXP * ns;
    const double *epx = wl + WL_EPEXP * ns, *thl = wl + WL_THL * ns;
    const double rho_io = wr[WR_RIO * n + q];
    const double rho_ie = 0.5 * (rexp[b] + rexp[lo]);
    const double th = wr[WR_TH * n + q];
    const double dz = vg.z_scalar[b] - vg.z_scalar[lo], dpi = vg.exner_bg[b] - vg.exner_bg[lo];
    const double wo = so.w[wi];
    const double a1 = al[lo], b0 = be[b], b1 = be[lo], g0 = ga[b], g1 = ga[lo];
    const double db = wr_b[WR_D * n + q], rb = wr_b[WR_R * n + q];
    double thb = wr_b[WR_TH * n + q], riob = wr_b[WR_RIO * n + q];
    double a0b = 0.0, a1b = 0.0, b0b = 0.0, b1b = 0.0, g0b = 0.0, g1b = 0.0, wob = 0.0, rieb = 0.0;
    /* d */
    const double geo = 2.0 / vg.area_v[wi] + dt * wo * 0.5 * (-1.0 / vg.volume[b] + 1.0 / vg.volume[lo]);
    thb += db * (-2.0 * th * (g0 + g1) + 0.5 * dpi * (b1 - b0));
    g0b += db * -(th * th);
    g1b += db * -(th * th);
    a1b += db * 0.5 * dpi;
    a0b -= db * 0.5 * dpi;
    b1b += db * 0.5 * dpi * th;
    b0b -= db * 0.5 * dpi * th;
    riob += db * dz / (K1 * rho_io * rho_io) * geo;
    wob += db * -dz / (K1 * rho_io) * dt * 0.5 * (-1.0 / vg.volume[b] + 1.0 / vg.volume[lo]);
    /* r */
    wob += rb * (-dz / K1 - dz / K1 * rho_ie / rho_io);
    acc(&st_w_b[wi], rb * (-dt * dz / K1));
    thb += rb * (epx[b] - epx[lo]) / dt;
    acc(&wl_b[WL_EPEXP * ns + b], rb * th / dt);
    acc(&wl_b[WL_EPEXP * ns + lo], -rb * th / dt);
    acc(&wl_b[WL_TPEXP * ns + b], rb * 0.5 / dt * dpi);
    acc(&wl_b[WL_TPEXP * ns + lo], rb * 0.5 / dt * dpi);
    rieb += rb * (-dz / K1 * wo / rho_io);
    riob += rb * dz / K1 * wo * rho_ie / (rho_io * rho_io);
    if (j < nl - 2) {
        const long long lo2 = lo + nc;
        const double th1 = 0.5 * (thl[lo] + thl[lo2]);
        const double rho_io1 = 0.5 * (so.rho[lo] + so.rho[lo2]);
        const double w1 = so.w[wi + nc];
        const double cb = wr_b[WR_C * n + q], eb = wr_b[WR_E * n + q];
        const double H1 = 0.5 * (vg.exner_bg[lo] - vg.exner_bg[lo2]), dz1 = vg.z_scalar[lo] - vg.z_scalar[lo2];
        double th1b = 0.0, rio1b = 0.0;
        /* c = th1 g1 th + H1 (a1 + b1 th) - dz1 / K2 0.5 w1 / (V_lo rho_io1) */
        th1b += cb * g1 * th;
        g1b += cb * th1 * th;
        thb += cb * (th1 * g1 + H1 * b1);
        a1b += cb * H1;
        b1b += cb * H1 * th;
        acc(&so_b.w[wi + nc], cb * -(dz1 / K2 * 0.5 / (vg.volume[lo] * rho_io1)));
        rio1b += cb * dz1 / K2 * 0.5 * w1 / (vg.volume[lo] * rho_io1 * rho_io1);
        /* e = th g1 th1 - 0.5 dpi (a1 + b1 th1) + dz / K2 0.5 wo / (V_lo rho_io) */
        thb += eb * g1 * th1;
        g1b += eb * th * th1;
        th1b += eb * (th * g1 - 0.5 * dpi * b1);
        a1b += eb * -0.5 * dpi;
        b1b += eb * -0.5 * dpi * th1;
        wob += eb * dz / K2 * 0.5 / (vg.volume[lo] * rho_io);
        riob += eb * -(dz / K2 * 0.5 * wo / (vg.volume[lo] * rho_io * rho_io));
        acc(&wl_b[WL_THL * ns + lo], 0.5 * th1b);
        acc(&wl_b[WL_THL * ns + lo2], 0.5 * th1b);
        acc(&so_b.rho[lo], 0.5 * rio1b);
        acc(&so_b.rho[lo2], 0.5 * rio1b);
    }
    acc(&wl_b[WL_THL * ns + b], 0.5 * thb);
    acc(&wl_b[WL_THL * ns + lo], 0.5 * thb);
    acc(&so_b.rho[b], 0.5 * riob);
    acc(&so_b.rho[lo], 0.5 * riob);
    acc(&wl_b[WL_REXP * ns + b], 0.5 * rieb);
    acc(&wl_b[WL_REXP * ns + lo], 0.5 * rieb);
    acc(&wl_b[WL_A * ns + b], a0b);
    acc(&wl_b[WL_A * ns + lo], a1b);
    acc(&wl_b[WL_B * ns + b], b0b);
    acc(&wl_b[WL_B * ns + lo], b1b);
    acc(&wl_b[WL_G * ns + b], g0b);
    acc(&wl_b[WL_G * ns + lo], g1b);
    acc(&so_b.w[wi], wob);
}

/* the per-layer predictors (fa_waves_layer); at rk 0 sn is so and sn_b is so_b */
__global__ void ba_waves_layer(VGrid vg, AParams ap, int rk, AState<double> so, AState<double> sn, const double *st_rho,
                               const double *st_rt, const double *wl, const double *wl_b, AState<double> so_b,
                               AState<double> sn_b, double *st_rho_b, double *st_rt_b)
{
    const long long ns = (long long)vg.nl * vg.nc, b = gtid();
    if (b >= ns) return;
    const double dt = ap.dt, vol = vg.volume[b];
    const double alpha = wl[WL_A * ns + b], beta = wl[WL_B * ns + b], gam = wl[WL_G * ns + b];
    double ab = wl_b[WL_A * ns + b], bb = wl_b[WL_B * ns + b], gb = wl_b[WL_G * ns + b];
    const double rexpb = wl_b[WL_REXP * ns + b], rtxb = wl_b[WL_RTEXP * ns + b];
    const double tpxb = wl_b[WL_TPEXP * ns + b], epxb = wl_b[WL_EPEXP * ns + b], thlb = wl_b[WL_THL * ns + b];
    const double sr = st_rho[b], srt = st_rt[b];
    double ro_b = 0.0, rto_b = 0.0, epo_b = 0.0, rn_b = 0.0, rtn_b = 0.0, epn_b = 0.0, sr_b = 0.0, srt_b = 0.0;
    /* tp_expl, ep_expl, rho_expl, rt_expl */
    so_b.tp[b] += tpxb;
    ab += tpxb * dt * vol * sr;
    bb += tpxb * dt * vol * srt;
    sr_b += tpxb * dt * vol * alpha;
    srt_b += tpxb * dt * vol * beta;
    epo_b += epxb;
    gb += epxb * dt * vol * srt;
    srt_b += epxb * dt * vol * gam;
    ro_b += rexpb;
    sr_b += dt * rexpb;
    rto_b += rtxb;
    srt_b += dt * rtxb;
    /* thl = rt_n / rho_n */
    const double rn = sn.rho[b], rtn = sn.rt[b];
    rtn_b += thlb / rn;
    rn_b -= thlb * (rtn / rn) / rn;
    /* alpha, beta, gamma */
    const double ro = so.rho[b], rto = so.rt[b], pe = vg.exner_bg[b] + so.ep[b];
    const double kg = R_D / C_D_V;
    if (rk == 0) {
        ro_b += ab * 2.0 * rto / (ro * ro * ro) / vol;
        rto_b += -ab / (ro * ro) / vol;
        ro_b += -bb / (ro * ro) / vol;
        rto_b += -gb * kg * pe / (rto * rto) / vol;
        epo_b += gb * kg / rto / vol;
    } else {
        const double hab = 0.5 * ab / vol, hbb = 0.5 * bb / vol, hgb = 0.5 * gb / vol;
        const double pn = vg.exner_bg[b] + sn.ep[b];
        ro_b += hab * 2.0 * rto / (ro * ro * ro);
        rto_b += -hab / (ro * ro);
        rn_b += hab * 2.0 * rtn / (rn * rn * rn);
        rtn_b += -hab / (rn * rn);
        ro_b += -hbb / (ro * ro);
        rn_b += -hbb / (rn * rn);
        rto_b += -hgb * kg * pe / (rto * rto);
        epo_b += hgb * kg / rto;
        rtn_b += -hgb * kg * pn / (rtn * rtn);
        epn_b += hgb * kg / rtn;
    }
    so_b.rho[b] += ro_b;
    so_b.rt[b] += rto_b;
    so_b.ep[b] += epo_b;
    sn_b.rho[b] += rn_b;
    sn_b.rt[b] += rtn_b;
    sn_b.ep[b] += epn_b;
    st_rho_b[b] += sr_b;
    st_rt_b[b] += srt_b;
}

}  // namespace
}  // namespace game
