/*
 * The sub-steps of manage_rkhevi as separate operations on device buffers
 * (compiled with --fmad=false, reference operation order), for the drop-in
 * entry points manage_pressure_gradient, calc_pressure_grad_condensates_v,
 * vector_tendencies_expl, scalar_tendencies_expl,
 * three_band_solver_ver_waves and three_band_solver_gen_densities
 * (src/time_stepping/time_stepping.h:7-12).
 *
 * The fused step computes the same quantities inside its own kernels; these
 * launchers produce them in the reference's separate output arrays (the
 * nonlinear and linear pressure-gradient parts, the saved old gradient, the
 * deceleration factor, the condensate term) and run the step's scalar
 * tendency and column-solver kernels on caller-provided buffers, so that a
 * sub-step call never touches the fields the device-resident step keeps
 * between calls.
 */
#include "ops.h"
#include "step.cuh"
#include "substeps.h"

namespace game {
namespace {

/* manage_pressure_gradient.c:32-60 at every vector point the reference
 * writes: all edges, the inner interfaces (grad and scalar_times_vector_v
 * leave the TOA and surface entries alone).  Device vector layout
 * [w (L+1) Nc][u L Ne]. */
__global__ void k_sub_pgrad(HGrid<double> g, StepParams p, SView<double> s, double *nl_out, double *l_out)
{
    const long long nw = (long long)(g.nl + 1) * g.nc, n = nw + (long long)g.nl * g.ne;
    const long long i = gtid();
    if (i >= n) return;
    double nl, lt;
    if (i < nw) {
        const int k = (int)(i / g.nc), c = (int)(i - (long long)k * g.nc);
        if (k == 0 || k == g.nl) return;
        pgrad_v_parts(g, p, s, k, c, nl, lt);
    } else {
        const long long j = i - nw;
        const int l = (int)(j / g.ne), e = (int)(j - (long long)l * g.ne);
        pgrad_h_parts(g, p, s, l, e, nl, lt);
    }
    nl_out[i] = nl;
    l_out[i] = lt;
}

/* pgrad_acc_old = -nl - l over the whole vector field (:25-31, :63-70) */
__global__ void k_sub_neg_sum(long long n, const double *a, const double *b, double *out)
{
    const long long i = gtid();
    if (i < n) out[i] = -a[i] - b[i];
}

/* rho_gas / density_total (:56-59), minus 1 for the condensate term (:80-84) */
__global__ void k_sub_decel(long long ns, const double *rho, int n_const, int n_cond, int minus_one, double *out)
{
    const long long i = gtid();
    if (i >= ns) return;
    double r = rho[n_cond * ns + i] / density_total(rho, n_const, ns, i);
    if (minus_one) r = r - 1.0;
    out[i] = r;
}

/* scalar_times_vector_v(decel - 1, gravity_m) at the inner interfaces (:85) */
__global__ void k_sub_condensates_v(HGrid<double> g, const double *f, double *out)
{
    const long long n = (long long)(g.nl - 1) * g.nc, i0 = gtid();
    if (i0 >= n) return;
    const long long i = i0 + g.nc;
    out[i] = 0.5 * (f[i - g.nc] + f[i]) * g.gravity_m_v[i];
}

/* the explicit momentum tendency (vector_tendencies_expl.c:79-131) at every
 * vector point; TOA and surface w get 0 */
__global__ void k_sub_vec_tend(int nl, int nc, int ne, double *tend, const double *pg_old, const double *p_nl,
                               const double *p_l, const double *pvt, const double *v2g, const double *friction,
                               const double *cond_v, double old_w, double new_w, double cur_hor, double old_hor,
                               double cur_ver)
{
    const long long nw = (long long)(nl + 1) * nc, n = nw + (long long)nl * ne;
    const long long i = gtid();
    if (i >= n) return;
    if (i < nw) {
        const int k = (int)(i / nc);
        if (k == 0 || k == nl) {
            tend[i] = 0.0;
            return;
        }
        tend[i] = old_w * tend[i]
                  + new_w * (-cur_ver * (p_nl[i] + p_l[i]) + pvt[i] - 0.5 * v2g[i] + friction[i] + cond_v[i]);
    } else {
        tend[i] = old_w * tend[i]
                  + new_w * (old_hor * pg_old[i] - cur_hor * (p_nl[i] + p_l[i]) + pvt[i] - 0.5 * v2g[i] + friction[i]);
    }
}

/* c_p of ice and liquid water at the given temperature (dictionary.c) */
__global__ void k_sub_cp_tables(long long ns, const double *t, double *cp_ice, double *cp_water)
{
    const long long i = gtid();
    if (i >= ns) return;
    cp_ice[i] = c_p_ice(t[i]);
    cp_water[i] = c_p_water(t[i]);
}

}  // namespace

void sub_pressure_gradient(Context *c, const StepParams &p, StateMirror *s, double *p_nl, double *p_l, double *pg_old,
                           double *decel)
{
    const long long nv = c->nv;
    SView<double> sv{s->ds.rho, s->ds.rhotheta_v, s->ds.theta_v_pert, s->ds.exner_pert, s->ds.w, s->ds.u};
    if (!p.first_step) k_sub_neg_sum<<<nblocks(nv, 256), 256, 0, c->stream>>>(nv, p_nl, p_l, pg_old);
    k_sub_pgrad<<<nblocks(nv, 256), 256, 0, c->stream>>>(c->hg64, p, sv, p_nl, p_l);
    k_sub_decel<<<nblocks(c->ns, 256), 256, 0, c->stream>>>(c->ns, s->ds.rho, c->n_const, c->n_cond, 0, decel);
    if (p.first_step) k_sub_neg_sum<<<nblocks(nv, 256), 256, 0, c->stream>>>(nv, p_nl, p_l, pg_old);
    c->kernel_launches += 3;
}

void sub_condensates_v(Context *c, StateMirror *s, double *decel, double *cond_v)
{
    k_sub_decel<<<nblocks(c->ns, 256), 256, 0, c->stream>>>(c->ns, s->ds.rho, c->n_const, c->n_cond, 1, decel);
    k_sub_condensates_v<<<nblocks((long long)(c->nl - 1) * c->nc, 256), 256, 0, c->stream>>>(c->hg64, decel, cond_v);
    c->kernel_launches += 2;
}

void sub_vector_tendency(Context *c, const StepParams &p, int rk, double *tend_wind, const double *pg_old,
                         const double *p_nl, const double *p_l, const double *pvt, const double *v2g,
                         const double *friction, const double *cond_v)
{
    const double new_w = rk == 1 ? 0.5 : 1.0, old_w = 1.0 - new_w;
    const double cur_hor = 0.5 + p.impl_thermo_weight, old_hor = 1.0 - cur_hor, cur_ver = 1.0 - p.impl_thermo_weight;
    k_sub_vec_tend<<<nblocks(c->nv, 256), 256, 0, c->stream>>>(c->nl, c->nc, c->ne, tend_wind, pg_old, p_nl, p_l, pvt,
                                                               v2g, friction, cond_v, old_w, new_w, cur_hor, old_hor,
                                                               cur_ver);
    c->kernel_launches++;
}

void sub_cp_tables(Context *c, const double *temperature, double *cp_ice, double *cp_water)
{
    k_sub_cp_tables<<<nblocks(c->ns, 256), 256, 0, c->stream>>>(c->ns, temperature, cp_ice, cp_water);
    c->kernel_launches++;
}

void sub_scalar_tendencies(Context *c, const StepParams &p, StateMirror *sn, StateMirror *st, int rk, double *theta,
                           const double *cp_ice, const double *cp_water, const double *pt_rates,
                           const double *pt_heat, const double *sed_heat)
{
    const Views<double> v = views<double>(c, sn);
    k_theta<double><<<nblocks(c->ns, 256), 256, 0, c->stream>>>(c->nl, c->nc, c->n_cond, v.sv, theta);
    k_scalar_tend2<double, false><<<nblocks(c->ns, 128), 128, 0, c->stream>>>(
        c->hg64, p, v.sv, st->ds, theta, cp_ice, cp_water, pt_rates, pt_heat, sed_heat, c->inv_vol, rk, IrrTerms{});
    c->kernel_launches += 2;
}

int sub_ver_waves(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st, int rk)
{
    if (launch_damping_table(c, p)) return -1;
    launch_waves<true>(c, p, so, sn, st, rk, Shadow{});
    return 0;
}

void sub_gen_densities(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st, int rk,
                       const double *temperature, const double *cp_ice, const double *cp_water, double *sed_heat)
{
    launch_tracers<true>(c, p, so, sn, st, rk, Shadow{}, temperature, cp_ice, cp_water, sed_heat);
}

}  // namespace game
