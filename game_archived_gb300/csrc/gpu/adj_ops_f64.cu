/*
 * Adjoints of the single operators (the reverse mode of grad, divv_h,
 * divv_h_tracer, scalar_times_vector, inner_product, calc_pot_vort,
 * vorticity_flux and the tracer column solver on device-layout fields),
 * compiled with --fmad=false.  They use the scatter
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


/* divv_h_tracer (divergences.c:66-148): the horizontal part is linear in the
 * flux field; the terrain vertical term is rho_up * corr(wind) * area_v with
 * rho_up the density upstream of the contravariant correction corr (the
 * pick is held fixed: the derivative of the piecewise form) */
__global__ void kop_divv_tracer_adj(HGrid<double> g, const double *density, const double *wind_u,
                                    const double *out_b, double *in_b_u, double *dens_b, double *wind_b_u)
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
    const double hb = yb / g.volume[i];
    for (int j = 0; j < n_edges; ++j) {
        const long long vi = (long long)l * ne + g.adj[j * nc + c];
        acc(&in_b_u[vi], double(g.adj_sign[j * nc + c]) * g.area_h[vi] * hb);
    }
    auto fw = [&](int ll, int j) { return wind_u[(long long)ll * ne + g.adj[j * nc + c]]; };
    /* bar of contra_corr(g, k, c, ...) into the edge winds it reads */
    auto corr_b = [&](int k, double cb) {
        if (k < nl - n_oro || cb == 0.0) return;
        for (int kk = (k > nl - n_oro ? k - 1 : k); kk <= k; ++kk)
            for (int j = 0; j < n_edges; ++j) {
                const long long le = (long long)kk * ne + g.adj[j * nc + c];
                acc(&wind_b_u[le], -0.5 * ipw_at(g, j, kk, c) * g.slope_h[le] * cb);
            }
    };
    if (l == nl - n_oro - 1 || (l > nl - n_oro - 1 && l < nl - 1)) { /* lower interface term, - rho * corr * A */
        const double lo = contra_corr(g, l + 1, c, n_edges, fw);
        const long long id = lo <= 0.0 ? i : i + nc;
        const double a = g.area_v[(long long)(l + 1) * nc + c];
        acc(&dens_b[id], -lo * a * hb);
        corr_b(l + 1, -density[id] * a * hb);
    }
    if (l > nl - n_oro - 1) { /* upper interface term, + rho * corr * A */
        const double up = contra_corr(g, l, c, n_edges, fw);
        const long long id = up <= 0.0 ? i - nc : i;
        const double a = g.area_v[(long long)l * nc + c];
        acc(&dens_b[id], up * a * hb);
        corr_b(l, density[id] * a * hb);
    }
}

/* d/dT of c_p(T) * T for the condensate kinds of c_p_cond (dictionary.c:111-190),
 * from the same fits: Murphy and Koop (2005) Eq. (4) for ice, Pruppacher and
 * Klett (2010) Eqs. (3-15), (3-16) for water; zero where the fits clip */
__device__ double d_cpT(int id, double t)
{
    double dcp = 0.0;
    if (id % 2 == 0) {
        if (t <= T_0 && t >= 20.0) {
            const double q = t / 125.1;
            dcp = (0.14644 + 0.06163 * exp(-(q * q)) * (1.0 - 2.0 * q * q)) / M_V;
        }
    } else {
        const double tc = t - T_0;
        if (tc >= 0.0) {
            if (tc <= 35.0) {
                const double a = tc - 35.0;
                dcp = 4186.8 * (2.0 * 3.1e-6 * a + 4.0 * 3.8e-9 * a * a * a);
            }
        } else if (tc >= -37.0) {
            dcp = 4186.8 * (-2.7052e-3 - 2.0 * 2.3235e-5 * tc + 3.0 * 4.3778e-6 * tc * tc
                            + 4.0 * 2.7136e-7 * tc * tc * tc);
        }
    }
    return dcp * t + c_p_cond(id, t);
}

/* three_band_solver_gen_densities (column_solvers.c:385-639) in reverse mode;
 * thread = (tracer slot, column).  The column's rows and unclipped solution
 * are rebuilt, the transposed tridiagonal system gives the bar of the
 * right-hand side, and the bars of the rows move to the inputs: the old
 * density and tendency of the tracer (owned by the thread), the old and new
 * vertical wind and, at rk 0, the temperature through the sedimentation heat
 * (shared by the tracer slots: atomic).  Upwind picks and flux-sign branches
 * are held fixed; clipped outputs carry no derivative.  The thread takes the
 * bar of its tracer's new density and leaves it zero (the forward overwrites
 * that field without reading it). */
template <int CAP>
__global__ void ka_gen_densities(VGrid vg, StepParams p, DState so, DState sn, DState st, const double *temperature,
                                 int rk, const double *sed_b, DState so_b, DState sn_b, DState st_b, double *t_b)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long ns = (long long)nl * nc;
    const long long q = gtid();
    if (q >= (long long)(p.n_const - 1) * nc) return;
    const int slot = (int)(q / nc), i = (int)(q - (long long)slot * nc);
    const int k = slot < p.n_cond ? slot : slot + 1;
    const int cond = p.n_cond;
    const bool sink = k < cond, heat = rk == 0 && k < cond;
    const double vs = k < cond / 4 ? p.snow_velocity : k < cond / 2 ? p.rain_velocity : sink ? p.cloud_velocity : 0.0;
    const double dt = p.dt, iw = 0.5, ew = 0.5;
    const double *ro = so.rho + k * ns, *tr = st.rho + k * ns;
    double *ro_b = so_b.rho + k * ns, *tr_b = st_b.rho + k * ns, *rn_b = sn_b.rho + k * ns;
    const long long bot = i + ns - nc;
    const double a_sfc = vg.area_v[(long long)nl * nc + i];
    auto vol = [&](int j) { return vg.volume[i + (long long)j * nc]; };
    auto fi = [&](int j) { const long long wi = i + (long long)(j + 1) * nc; return vg.area_v[wi] * (so.w[wi] - vs); };
    auto bw = [&](int j) { const long long wi = i + (long long)(j + 1) * nc; return vg.area_v[wi] * (sn.w[wi] - vs); };
    auto io = [&](int j) { return bw(j) >= 0.0 ? i + (long long)(j + 1) * nc : i + (long long)j * nc; };
    double cc[CAP], dd[CAP], ee[CAP], xx[CAP], ep[CAP], rp[CAP];
    /* rows */
    for (int j = 0; j < nl; ++j) {
        const double v = vol(j);
        double d = 1.0, r = ro[i + (long long)j * nc] + dt * tr[i + (long long)j * nc];
        if (j < nl - 1) {
            const double f = fi(j), fr = ro[io(j)] * bw(j);
            ee[j] = f >= 0.0 ? -iw * dt / v * f : 0.0;
            cc[j] = f < 0.0 ? iw * dt / vol(j + 1) * f : 0.0;
            if (f < 0.0) d -= iw * dt / v * f;
            r += ew * dt * fr / v;
        }
        if (j > 0) {
            const double f = fi(j - 1), fr = ro[io(j - 1)] * bw(j - 1);
            if (f >= 0.0) d += iw * dt / v * f;
            r -= ew * dt * fr / v;
        }
        if (j == nl - 1 && sink) {
            d += iw * vs * dt * a_sfc / v;
            r -= ew * vs * dt * ro[bot] * a_sfc / v;
        }
        dd[j] = d;
        /* forward elimination */
        if (j == 0) {
            ep[0] = nl > 1 ? ee[0] / d : 0.0;
            rp[0] = r / d;
        } else {
            const double den = d - ep[j - 1] * cc[j - 1];
            if (j < nl - 1) ep[j] = ee[j] / den;
            rp[j] = (r - rp[j - 1] * cc[j - 1]) / den;
        }
    }
    xx[nl - 1] = rp[nl - 1];
    for (int j = nl - 2; j >= 0; --j) xx[j] = rp[j] - ep[j] * xx[j + 1];
    /* transposed system A^T y = xbar (sub-diagonal ee, super-diagonal cc) */
    for (int j = 0; j < nl; ++j) {
        const long long b = i + (long long)j * nc;
        const double g = xx[j] < 0.0 ? 0.0 : rn_b[b];
        rn_b[b] = 0.0;
        if (j == 0) {
            ep[0] = nl > 1 ? cc[0] / dd[0] : 0.0;
            rp[0] = g / dd[0];
        } else {
            const double den = dd[j] - ep[j - 1] * ee[j - 1];
            if (j < nl - 1) ep[j] = cc[j] / den;
            rp[j] = (g - rp[j - 1] * ee[j - 1]) / den;
        }
    }
    for (int j = nl - 2; j >= 0; --j) rp[j] = rp[j] - ep[j] * rp[j + 1];
    const double *y = rp;
    /* bars of the inputs */
    for (int j = 0; j < nl; ++j) {
        const long long b = i + (long long)j * nc;
        ro_b[b] += y[j];
        tr_b[b] += dt * y[j];
    }
    if (sink) {
        const double v = vol(nl - 1);
        double rb = -ew * vs * dt * a_sfc / v * y[nl - 1];
        if (heat) {
            const double hb = sed_b[bot], tb = temperature[bot];
            rb += -vs * c_p_cond(k, tb) * tb * a_sfc / v * hb;
            acc(&t_b[bot], -vs * d_cpT(k, tb) * ro[bot] * a_sfc / v * hb);
        }
        ro_b[bot] += rb;
    }
    for (int j = 0; j < nl - 1; ++j) {
        const double vj = vol(j), vj1 = vol(j + 1);
        const long long wi = i + (long long)(j + 1) * nc, id = io(j);
        const double f = fi(j), b_ = bw(j), dio = ro[id];
        double frb = ew * dt * (y[j] / vj - y[j + 1] / vj1);
        if (heat) {
            const double hb = sed_b[i + (long long)j * nc] / vj - sed_b[i + (long long)(j + 1) * nc] / vj1;
            const double t = temperature[id];
            frb += c_p_cond(k, t) * t * hb;
            acc(&t_b[id], d_cpT(k, t) * dio * b_ * hb);
        }
        ro_b[id] += b_ * frb;
        acc(&sn_b.w[wi], vg.area_v[wi] * dio * frb);
        /* rows j (e, d) and j + 1 (c, d) */
        double fb;
        if (f >= 0.0)
            fb = -iw * dt / vj * (-y[j] * xx[j + 1]) + iw * dt / vj1 * (-y[j + 1] * xx[j + 1]);
        else
            fb = iw * dt / vj1 * (-y[j + 1] * xx[j]) - iw * dt / vj * (-y[j] * xx[j]);
        acc(&so_b.w[wi], vg.area_v[wi] * fb);
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

void op_divv_tracer_adj(Context *c, const double *density, const double *wind, const double *out_b, double *in_b,
                        double *dens_b, double *wind_b)
{
    const long long nw = (long long)(c->nl + 1) * c->nc;
    kop_divv_tracer_adj<<<nb(c->ns), 256, 0, c->stream>>>(c->hg64, density, wind + nw, out_b, in_b + nw, dens_b,
                                                          wind_b + nw);
    c->kernel_launches++;
}

int adj_gen_densities(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st,
                      const double *temperature, int rk, double *sed_b, StateMirror *so_b, StateMirror *sn_b,
                      StateMirror *st_b, double *t_b)
{
    if (c->n_const <= 1) return 0;
    const long long nsys = (long long)(c->n_const - 1) * c->nc;
    if (c->nl <= 64)
        ka_gen_densities<64><<<nb(nsys, 64), 64, 0, c->stream>>>(c->vg, p, so->ds, sn->ds, st->ds, temperature, rk,
                                                                 sed_b, so_b->ds, sn_b->ds, st_b->ds, t_b);
    else if (c->nl <= 256)
        ka_gen_densities<256><<<nb(nsys, 64), 64, 0, c->stream>>>(c->vg, p, so->ds, sn->ds, st->ds, temperature, rk,
                                                                  sed_b, so_b->ds, sn_b->ds, st_b->ds, t_b);
    else
        return -1;
    c->kernel_launches++;
    /* the forward overwrites the sedimentation heat at rk 0 */
    if (rk == 0 && cudaMemsetAsync(sed_b, 0, (size_t)c->ns * sizeof(double), c->stream) != cudaSuccess) return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace game
