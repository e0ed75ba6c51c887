/*
 * Single-operator kernels behind the per-operator C entry points (grad,
 * divv_h, calc_pot_vort, vorticity_flux, inner_product, ...).  FP64, compiled
 * with --fmad=false, on device-layout fields:
 *   scalar field  [L][Nc]
 *   vector field  [w: (L+1)][Nc] followed by [u: L][Ne]
 *   curl field    [tangential: (L+1)][Ne] followed by [rhombus: L][Ne]
 */
#include "kernels.cuh"
#include "ops.h"

namespace game {
namespace {

using G = HGrid<double>;

__global__ void k_op_grad_h(G g, const double *f, double *u, int with_correction)
{
    const long long n = (long long)g.nl * g.ne, i = gtid();
    if (i >= n) return;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    if (with_correction) {
        u[i] = grad_h(g, f, l, e);
    } else {
        const int fr = g.from[e], to = g.to[e];
        u[i] = (f[(long long)l * g.nc + to] - f[(long long)l * g.nc + fr]) / g.nd_h[i];
    }
}

__global__ void k_op_grad_v(G g, const double *f, double *w)
{
    const long long n = (long long)(g.nl - 1) * g.nc, i = gtid();
    if (i >= n) return;
    const int k = (int)(i / g.nc) + 1, c = (int)(i - (long long)(k - 1) * g.nc);
    w[(long long)k * g.nc + c] = grad_v(g, f, k, c);
}

/* vector_field_hor_cov_to_con (averaging.c:113-133) on a vector field */
__global__ void k_op_cov_to_con(G g, const double *w, double *u)
{
    const long long n = (long long)g.n_oro * g.ne, i = gtid();
    if (i >= n) return;
    const int l = (int)(i / g.ne) + (g.nl - g.n_oro), e = (int)(i % g.ne);
    const int fr = g.from[e], to = g.to[e];
    double c = ipw_at(g, 6, l, fr) * w[(long long)l * g.nc + fr];
    c += ipw_at(g, 6, l, to) * w[(long long)l * g.nc + to];
    if (l < g.nl - 1) {
        c += ipw_at(g, 7, l, fr) * w[(long long)(l + 1) * g.nc + fr];
        c += ipw_at(g, 7, l, to) * w[(long long)(l + 1) * g.nc + to];
    }
    c = 0.5 * c;
    const long long le = (long long)l * g.ne + e;
    u[le] += -g.slope_h[le] * c;
}

/* scalar_times_vector_h / _h_upstream (multiplications.c:45-96) */
__global__ void k_op_stv_h(G g, const double *s, const double *v, double *out, int upstream)
{
    const long long n = (long long)g.nl * g.ne, i = gtid();
    if (i >= n) return;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    const long long o = (long long)l * g.nc;
    double sv;
    if (upstream) sv = v[i] >= 0.0 ? s[o + g.from[e]] : s[o + g.to[e]];
    else sv = 0.5 * (s[o + g.to[e]] + s[o + g.from[e]]);
    out[i] = sv * v[i];
}

/* scalar_times_vector_v (multiplications.c:98-117), inner interfaces */
__global__ void k_op_stv_v(G g, const double *s, const double *v, double *out)
{
    const long long n = (long long)(g.nl - 1) * g.nc, i0 = gtid();
    if (i0 >= n) return;
    const long long i = i0 + g.nc;
    const double sv = 0.5 * (s[i - g.nc] + s[i]);
    out[i] = sv * v[i];
}

/* divv_h / divv_h_tracer (divergences.c:14-148) of an edge field in_u */
__global__ void k_op_divv(G g, const double *in_u, const double *density, const double *wind_u, double *out,
                          int tracer)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const int n_edges = c < N_PENT ? 5 : 6, nl = g.nl, n_oro = g.n_oro;
    const long long nc = g.nc;
    double comp_h = 0.0;
    for (int j = 0; j < n_edges; ++j) {
        const long long vi = (long long)l * g.ne + g.adj[j * nc + c];
        comp_h += in_u[vi] * double(g.adj_sign[j * nc + c]) * g.area_h[vi];
    }
    auto fin = [&](int ll, int j) { return in_u[(long long)ll * g.ne + g.adj[j * nc + c]]; };
    auto fw = [&](int ll, int j) { return wind_u[(long long)ll * g.ne + g.adj[j * nc + c]]; };
    double comp_v = 0.0;
    if (!tracer) {
        if (l == nl - n_oro - 1) {
            double lo = contra_corr(g, l + 1, c, n_edges, fin);
            comp_v = -lo * g.area_v[(long long)(l + 1) * nc + c];
        } else if (l == nl - 1) {
            double up = contra_corr(g, l, c, n_edges, fin);
            comp_v = up * g.area_v[(long long)l * nc + c];
        } else if (l > nl - n_oro - 1) {
            double up = contra_corr(g, l, c, n_edges, fin);
            double lo = contra_corr(g, l + 1, c, n_edges, fin);
            comp_v = up * g.area_v[(long long)l * nc + c] - lo * g.area_v[(long long)(l + 1) * nc + c];
        }
    } else {
        if (l == nl - n_oro - 1) {
            double lo = contra_corr(g, l + 1, c, n_edges, fw);
            double d_lo = lo <= 0.0 ? density[i] : density[i + nc];
            comp_v = -d_lo * lo * g.area_v[(long long)(l + 1) * nc + c];
        } else if (l == nl - 1) {
            double up = contra_corr(g, l, c, n_edges, fw);
            double d_up = up <= 0.0 ? density[i - nc] : density[i];
            comp_v = d_up * up * g.area_v[(long long)l * nc + c];
        } else if (l > nl - n_oro - 1) {
            double up = contra_corr(g, l, c, n_edges, fw);
            double d_up = up <= 0.0 ? density[i - nc] : density[i];
            double lo = contra_corr(g, l + 1, c, n_edges, fw);
            double d_lo = lo <= 0.0 ? density[i] : density[i + nc];
            comp_v = d_up * up * g.area_v[(long long)l * nc + c] - d_lo * lo * g.area_v[(long long)(l + 1) * nc + c];
        }
    }
    out[i] = 1.0 / g.volume[i] * (comp_h + comp_v);
}

/* inner_product (inner_product.c:13-43) */
__global__ void k_op_inner(G g, const double *aw, const double *au, const double *bw, const double *bu, double *out)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const int n_edges = c < N_PENT ? 5 : 6;
    double r = 0;
    for (int j = 0; j < n_edges; ++j) {
        const long long vi = (long long)l * g.ne + g.adj[j * g.nc + c];
        r += ipw_at(g, j, l, c) * au[vi] * bu[vi];
    }
    r += ipw_at(g, 6, l, c) * aw[i] * bw[i];
    r += ipw_at(g, 7, l, c) * aw[i + g.nc] * bw[i + g.nc];
    out[i] = r;
}

/* calc_rel_vort (vorticities.c:104-165): tangential [L+1][Ne], rhombus [L][Ne] */
__global__ void k_op_rel_vort(G g, const double *u, const double *w, const double *tri, double *zh, double *zv)
{
    const long long n = (long long)(g.nl + 1) * g.ne, i = gtid();
    if (i >= n) return;
    const int k = (int)(i / g.ne), e = (int)(i - (long long)k * g.ne);
    zh[i] = rel_vort_tangential(g, u, w, k, e);
    if (k < g.nl) {
        const int tf = g.dual_from[e], tt = g.dual_to[e];
        const long long kt = (long long)k * g.nt;
        const double af = g.dual_area_t[kt + tf], at = g.dual_area_t[kt + tt];
        zv[(long long)k * g.ne + e] = (af * tri[kt + tf] + at * tri[kt + tt]) / (af + at);
    }
}

/* add_f_to_rel_vort (vorticities.c:87-102) and, when rho is given, the
 * division by the density of calc_pot_vort (vorticities.c:27-83) */
__global__ void k_op_pot_vort(G g, const double *rzh, const double *rzv, const double *rho, double *pzh, double *pzv)
{
    const long long n = (long long)(g.nl + 1) * g.ne, i = gtid();
    if (i >= n) return;
    const int k = (int)(i / g.ne), e = (int)(i - (long long)k * g.ne);
    const int nl = g.nl, nc = g.nc, ne = g.ne, fr = g.from[e], to = g.to[e];
    double pv = rzh[i] + g.f_vec[e];
    if (rho) {
        double dens;
        if (k == 0) {
            double top = 0.5 * (rho[fr] + rho[to]), below = 0.5 * (rho[nc + fr] + rho[nc + to]);
            dens = top + (top - below) / g.pvz[ne + e] * g.pvz[e];
        } else if (k == nl) {
            long long a = (long long)(nl - 1) * nc, b = (long long)(nl - 2) * nc;
            double low = 0.5 * (rho[a + fr] + rho[a + to]), above = 0.5 * (rho[b + fr] + rho[b + to]);
            dens = low + (above - low) / g.pvz[3 * (long long)ne + e] * g.pvz[2 * (long long)ne + e];
        } else {
            long long uf = (long long)(k - 1) * nc + fr, ut = (long long)(k - 1) * nc + to;
            dens = 0.25 * (rho[uf] + rho[ut] + rho[uf + nc] + rho[ut + nc]);
        }
        pv = pv / dens;
    }
    pzh[i] = pv;
    if (k < nl) {
        const long long le = (long long)k * ne + e;
        double pr = rzv[le] + g.f_vec[ne + e];
        if (rho) {
            double dens = 0;
            for (int j = 0; j < 4; ++j) dens += g.rhombi_w[j * (long long)ne + e] * rho[(long long)k * nc + g.rhombi_i[j * (long long)ne + e]];
            pr = pr / dens;
        }
        pzv[le] = pr;
    }
}

/* vorticity_flux (vorticity_flux.c:16-187) */
__global__ void k_op_vflux_h(G g, const double *fw, const double *fu, const double *zh, const double *zv, double *out_u)
{
    const long long n = (long long)g.nl * g.ne, i = gtid();
    if (i >= n) return;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    out_u[i] = vorticity_flux_h(g, fu, fw, zh, zv, l, e);
}

__global__ void k_op_vflux_v(G g, const double *fu, const double *zh, double *out_w)
{
    const long long n = (long long)(g.nl + 1) * g.nc, i = gtid();
    if (i >= n) return;
    const int k = (int)(i / g.nc), c = (int)(i - (long long)k * g.nc), nl = g.nl;
    const int n_edges = c < N_PENT ? 5 : 6;
    const double vw = (k == 0 || k == nl) ? 1 : 0.5;
    const double *z = zh + (long long)k * g.ne;
    double r = 0;
    if (k >= 1)
        for (int j = 0; j < n_edges; ++j) {
            const int a = g.adj[j * g.nc + c];
            r += vw * ipw_at(g, j, k - 1, c) * fu[(long long)(k - 1) * g.ne + a] * z[a];
        }
    if (k <= nl - 1)
        for (int j = 0; j < n_edges; ++j) {
            const int a = g.adj[j * g.nc + c];
            r += vw * ipw_at(g, j, k, c) * fu[(long long)k * g.ne + a] * z[a];
        }
    out_w[i] = r;
}

/* linear_combine_two_states (linear_combine_two_states.c:14-43) on device
 * state blocks: all fields, then theta_v_pert from the combined fields */
__global__ void k_op_lincomb(long long n, const double *a, const double *b, double *o, double c0, double c1)
{
    const long long i = gtid();
    if (i < n) o[i] = c0 * a[i] + c1 * b[i];
}

__global__ void k_op_lincomb_theta(VGrid vg, int n_cond, DState o)
{
    const long long ns = (long long)vg.nl * vg.nc, i = gtid();
    if (i < ns) o.theta_v_pert[i] = o.rhotheta_v[i] / o.rho[n_cond * ns + i] - vg.theta_v_bg[i];
}

/* scalar_times_scalar, vector_times_vector (multiplications.c:15-33):
 * pointwise products, in any element order */
__global__ void k_op_mul(long long n, const double *a, const double *b, double *out)
{
    const long long i = gtid();
    if (i < n) out[i] = a[i] * b[i];
}

/* add_vertical_divv (divergences.c:150-185): out += 1 / V * the divergence of
 * the vertical part w [L+1][Nc] of a vector field, zero flux at the top and
 * bottom of the column */
__global__ void k_op_add_vertical_divv(G g, const double *w, double *out)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const long long up = (long long)l * g.nc + c, lo = (long long)(l + 1) * g.nc + c;
    const double contra_upper = l == 0 ? 0.0 : w[up];
    const double contra_lower = l == g.nl - 1 ? 0.0 : w[lo];
    const double comp_v = contra_upper * g.area_v[up] - contra_lower * g.area_v[lo];
    out[i] += 1 / g.volume[i] * comp_v;
}

}  // namespace

static unsigned nb(long long n) { return (unsigned)((n + 255) / 256); }

void op_mul(Context *c, long long n, const double *a, const double *b, double *out)
{
    k_op_mul<<<nb(n), 256, 0, c->stream>>>(n, a, b, out);
    c->kernel_launches++;
}

void op_add_vertical_divv(Context *c, const double *vec, double *out)
{
    k_op_add_vertical_divv<<<nb(c->ns), 256, 0, c->stream>>>(c->hg64, vec, out);
    c->kernel_launches++;
}

void op_grad(Context *c, const double *f, double *vec, int parts)
{
    double *w = vec, *u = vec + (long long)(c->nl + 1) * c->nc;
    if (parts & OP_GRAD_V) k_op_grad_v<<<nb((long long)(c->nl - 1) * c->nc), 256, 0, c->stream>>>(c->hg64, f, w);
    if (parts & OP_GRAD_H)
        k_op_grad_h<<<nb((long long)c->nl * c->ne), 256, 0, c->stream>>>(c->hg64, f, u, (parts & OP_GRAD_CON) ? 1 : 0);
    c->kernel_launches += 2;
}

void op_cov_to_con(Context *c, double *vec)
{
    double *w = vec, *u = vec + (long long)(c->nl + 1) * c->nc;
    k_op_cov_to_con<<<nb((long long)c->n_oro * c->ne), 256, 0, c->stream>>>(c->hg64, w, u);
    c->kernel_launches++;
}

void op_scalar_times_vector(Context *c, const double *s, const double *vec, double *out, int parts)
{
    const long long off = (long long)(c->nl + 1) * c->nc;
    if (parts & OP_STV_H)
        k_op_stv_h<<<nb((long long)c->nl * c->ne), 256, 0, c->stream>>>(c->hg64, s, vec + off, out + off,
                                                                       (parts & OP_STV_UPSTREAM) ? 1 : 0);
    if (parts & OP_STV_V) k_op_stv_v<<<nb((long long)(c->nl - 1) * c->nc), 256, 0, c->stream>>>(c->hg64, s, vec, out);
    c->kernel_launches += 2;
}

void op_divv(Context *c, const double *vec, const double *density, const double *wind, double *out, int tracer)
{
    const long long off = (long long)(c->nl + 1) * c->nc;
    k_op_divv<<<nb(c->ns), 256, 0, c->stream>>>(c->hg64, vec + off, density, wind ? wind + off : nullptr, out, tracer);
    c->kernel_launches++;
}

void op_inner_product(Context *c, const double *a, const double *b, double *out)
{
    const long long off = (long long)(c->nl + 1) * c->nc;
    k_op_inner<<<nb(c->ns), 256, 0, c->stream>>>(c->hg64, a, a + off, b, b + off, out);
    c->kernel_launches++;
}

void op_rel_vort(Context *c, const double *wind, double *tri, double *curl)
{
    const long long off = (long long)(c->nl + 1) * c->nc, coff = (long long)(c->nl + 1) * c->ne;
    k_tri_vort<double><<<nb((long long)c->nl * c->nt), 256, 0, c->stream>>>(c->hg64, wind + off, tri);
    k_op_rel_vort<<<nb(coff), 256, 0, c->stream>>>(c->hg64, wind + off, wind, tri, curl, curl + coff);
    c->kernel_launches += 2;
}

void op_pot_vort(Context *c, const double *rel, const double *rho, double *pv)
{
    const long long coff = (long long)(c->nl + 1) * c->ne;
    k_op_pot_vort<<<nb(coff), 256, 0, c->stream>>>(c->hg64, rel, rel + coff, rho, pv, pv + coff);
    c->kernel_launches++;
}

void op_vorticity_flux(Context *c, const double *flux, const double *pv, double *out)
{
    const long long off = (long long)(c->nl + 1) * c->nc, coff = (long long)(c->nl + 1) * c->ne;
    k_op_vflux_h<<<nb((long long)c->nl * c->ne), 256, 0, c->stream>>>(c->hg64, flux, flux + off, pv, pv + coff,
                                                                       out + off);
    k_op_vflux_v<<<nb(off), 256, 0, c->stream>>>(c->hg64, flux + off, pv, out);
    c->kernel_launches += 2;
}

void op_linear_combine(Context *c, StateMirror *a, StateMirror *b, StateMirror *o, double c0, double c1)
{
    k_op_lincomb<<<nb(c->state_len), 256, 0, c->stream>>>(c->state_len, a->dev, b->dev, o->dev, c0, c1);
    k_op_lincomb_theta<<<nb(c->ns), 256, 0, c->stream>>>(c->vg, c->n_cond, o->ds);
    c->kernel_launches += 2;
}

}  // namespace game
