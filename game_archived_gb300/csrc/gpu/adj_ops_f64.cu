/*
 * Adjoints of the single operators (the reverse mode of grad, divv_h,
 * scalar_times_vector, inner_product, calc_pot_vort and vorticity_flux on
 * device-layout fields), compiled with --fmad=false.  They use the scatter
 * helpers of the step adjoint (adj_bwd.cuh): bars of a forward's inputs are
 * accumulated, x_bar += (dy/dx)^T y_bar.
 */
#include "adj_bwd.cuh"
#include "adj_ops.h"

namespace game {
namespace {

inline unsigned nb(long long n, int bs = 256) { return (unsigned)((n + bs - 1) / bs); }

/* grad (gradient_operators.c:66-74): vector bar [w | u] -> scalar bar; the
 * TOA and surface entries of the output are not written by grad and carry
 * no dependence on the input */
__global__ void kop_grad_adj(HGrid<double> g, const double *out_b, double *in_b)
{
    const long long nw = (long long)(g.nl + 1) * g.nc, n = nw + (long long)g.nl * g.ne;
    const long long i = gtid();
    if (i >= n) return;
    const double ob = out_b[i];
    if (ob == 0.0) return;
    if (i < nw) {
        const int k = (int)(i / g.nc), c = (int)(i - (long long)k * g.nc);
        if (k == 0 || k == g.nl) return;
        b_gv(g, in_b, k, c, ob);
    } else {
        const long long j = i - nw;
        const int l = (int)(j / g.ne), e = (int)(j - (long long)l * g.ne);
        b_grad_h(g, in_b, l, e, ob);
    }
}

/* divv_h (divergences.c:14-64): scalar bar -> bar of the horizontal part of
 * the vector field, through the edge sum and the terrain correction */
__global__ void kop_divv_adj(HGrid<double> g, const double *out_b, double *in_b_u)
{
    const long long ns = (long long)g.nl * g.nc;
    const long long i = gtid();
    if (i >= ns) return;
    const double yb = out_b[i];
    if (yb == 0.0) return;
    const int nl = g.nl, n_oro = g.n_oro;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const long long nc = g.nc, ne = g.ne;
    const int n_edges = c < N_PENT ? 5 : 6;
    const bool oro = l >= nl - n_oro - 1;
    const bool up_corr = oro && l >= nl - n_oro;
    const bool lo_corr = oro && l < nl - 1;
    const bool up_has_prev = up_corr && l > nl - n_oro;
    const bool lo_has_curr = lo_corr && l + 1 > nl - n_oro;
    const double hb = yb / g.volume[i];
    const double area_up = g.area_v[(long long)l * nc + c], area_lo = g.area_v[(long long)(l + 1) * nc + c];
    double upb = 0.0, lob = 0.0;
    if (oro) {
        if (l == nl - n_oro - 1) lob = -area_lo * hb;
        else if (l == nl - 1) upb = area_up * hb;
        else {
            upb = area_up * hb;
            lob = -area_lo * hb;
        }
    }
    auto pass = [&](int ll, bool to_h, bool to_up, bool to_lo) {
        for (int j = 0; j < n_edges; ++j) {
            const int ed = g.adj[j * nc + c];
            const long long le = (long long)ll * ne + ed;
            double fb = 0.0;
            if (to_h) fb += double(g.adj_sign[j * nc + c]) * g.area_h[le] * hb;
            if (to_up || to_lo) {
                const double wc = -0.5 * ipw_d(g, j, ll, c) * g.slope_h[le];
                if (to_up) fb += wc * upb;
                if (to_lo) fb += wc * lob;
            }
            if (fb != 0.0) acc(&in_b_u[le], fb);
        }
    };
    if (up_has_prev) pass(l - 1, false, true, false);
    pass(l, true, up_corr, lo_has_curr);
    if (lo_corr) pass(l + 1, false, false, true);
}

/* scalar_times_vector (multiplications.c:35-117): edge average (all edges)
 * and interface average (inner interfaces) times the vector */
__global__ void kop_stv_adj(HGrid<double> g, const double *s, const double *v, const double *out_b, double *s_b,
                            double *v_b)
{
    const long long nw = (long long)(g.nl + 1) * g.nc, n = nw + (long long)g.nl * g.ne;
    const long long i = gtid();
    if (i >= n) return;
    const double ob = out_b[i];
    if (ob == 0.0) return;
    if (i < nw) {
        const int k = (int)(i / g.nc), c = (int)(i - (long long)k * g.nc);
        if (k == 0 || k == g.nl) return;
        const long long up = (long long)(k - 1) * g.nc + c, lo = (long long)k * g.nc + c;
        acc(&v_b[i], 0.5 * (s[up] + s[lo]) * ob);
        const double q = 0.5 * v[i] * ob;
        acc(&s_b[up], q);
        acc(&s_b[lo], q);
    } else {
        const long long j = i - nw;
        const int l = (int)(j / g.ne), e = (int)(j - (long long)l * g.ne);
        const long long ct = (long long)l * g.nc + g.to[e], cf = (long long)l * g.nc + g.from[e];
        acc(&v_b[i], 0.5 * (s[ct] + s[cf]) * ob);
        const double q = 0.5 * v[i] * ob;
        acc(&s_b[ct], q);
        acc(&s_b[cf], q);
    }
}

/* inner_product (inner_product.c:13-43) of vectors a, b (device layout) */
__global__ void kop_inner_adj(HGrid<double> g, const double *a, const double *b, const double *out_b, double *a_b,
                              double *b_b)
{
    const long long ns = (long long)g.nl * g.nc;
    const long long i = gtid();
    if (i >= ns) return;
    const double ob = out_b[i];
    if (ob == 0.0) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const int n_edges = c < N_PENT ? 5 : 6;
    const long long nw = (long long)(g.nl + 1) * g.nc;
    for (int j = 0; j < n_edges; ++j) {
        const long long vi = nw + (long long)l * g.ne + g.adj[j * g.nc + c];
        const double wgt = ipw_d(g, j, l, c);
        acc(&a_b[vi], wgt * b[vi] * ob);
        acc(&b_b[vi], wgt * a[vi] * ob);
    }
    const long long top = i, bot = i + g.nc;
    acc(&a_b[top], ipw_d(g, 6, l, c) * b[top] * ob);
    acc(&b_b[top], ipw_d(g, 6, l, c) * a[top] * ob);
    acc(&a_b[bot], ipw_d(g, 7, l, c) * b[bot] * ob);
    acc(&b_b[bot], ipw_d(g, 7, l, c) * a[bot] * ob);
}

/* vorticity_flux (vorticity_flux.c:16-187): horizontal part per edge */
__global__ void kop_vflux_h_adj(HGrid<double> g, const double *flux_v, const double *flux_h, const double *zh,
                                const double *zv, const double *out_b_u, double *fv_b, double *fh_b, double *zh_b,
                                double *zv_b)
{
    const long long n = (long long)g.nl * g.ne;
    const long long i = gtid();
    if (i >= n) return;
    const double ob = out_b_u[i];
    if (ob == 0.0) return;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    b_vflux_h(g, flux_h, flux_v, zh, zv, fh_b, fv_b, zh_b, zv_b, l, e, ob);
}

/* vertical part per interface (all levels) */
__global__ void kop_vflux_v_adj(HGrid<double> g, const double *flux_h, const double *zh, const double *out_b_w,
                                double *fh_b, double *zh_b)
{
    const long long n = (long long)(g.nl + 1) * g.nc;
    const long long i = gtid();
    if (i >= n) return;
    const double pb = out_b_w[i];
    if (pb == 0.0) return;
    const int k = (int)(i / g.nc), c = (int)(i - (long long)k * g.nc);
    const int nl = g.nl, n_edges = c < N_PENT ? 5 : 6;
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

}  // namespace

void op_grad_adj(Context *c, const double *out_b, double *in_b)
{
    kop_grad_adj<<<nb(c->nv), 256, 0, c->stream>>>(c->hg64, out_b, in_b);
    c->kernel_launches++;
}

void op_divv_adj(Context *c, const double *out_b, double *in_b)
{
    kop_divv_adj<<<nb(c->ns), 256, 0, c->stream>>>(c->hg64, out_b, in_b + (long long)(c->nl + 1) * c->nc);
    c->kernel_launches++;
}

void op_stv_adj(Context *c, const double *s, const double *v, const double *out_b, double *s_b, double *v_b)
{
    kop_stv_adj<<<nb(c->nv), 256, 0, c->stream>>>(c->hg64, s, v, out_b, s_b, v_b);
    c->kernel_launches++;
}

void op_inner_adj(Context *c, const double *a, const double *b, const double *out_b, double *a_b, double *b_b)
{
    kop_inner_adj<<<nb(c->ns), 256, 0, c->stream>>>(c->hg64, a, b, out_b, a_b, b_b);
    c->kernel_launches++;
}

void op_vflux_adj(Context *c, const double *flux, const double *pv, const double *out_b, double *flux_b, double *pv_b)
{
    const long long nw = (long long)(c->nl + 1) * c->nc, nzh = (long long)(c->nl + 1) * c->ne;
    kop_vflux_h_adj<<<nb((long long)c->nl * c->ne), 256, 0, c->stream>>>(c->hg64, flux, flux + nw, pv, pv + nzh,
                                                                          out_b + nw, flux_b, flux_b + nw, pv_b,
                                                                          pv_b + nzh);
    kop_vflux_v_adj<<<nb(nw), 256, 0, c->stream>>>(c->hg64, flux + nw, pv, out_b, flux_b + nw, pv_b);
    c->kernel_launches += 2;
}

void op_pot_vort_adj(Context *c, const double *wind, const double *rho, const double *pv, const double *pv_b,
                     const double *zero_u, double *wind_b, double *rho_b, double *tri_b)
{
    const long long nw = (long long)(c->nl + 1) * c->nc, nzh = (long long)(c->nl + 1) * c->ne;
    ba_edge<<<nb(nzh), 256, 0, c->stream>>>(c->hg64, wind + nw, rho, pv, pv + nzh, pv_b, pv_b + nzh, zero_u,
                                            wind_b + nw, wind_b, rho_b, tri_b);
    ba_tri<<<nb((long long)c->nl * c->nt), 256, 0, c->stream>>>(c->hg64, tri_b, wind_b + nw);
    c->kernel_launches += 2;
}

}  // namespace game
