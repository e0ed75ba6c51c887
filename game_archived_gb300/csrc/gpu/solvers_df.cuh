/*
 * The mixed path's vertical eliminations in double-float arithmetic
 * (dfloat.cuh), so that they issue on the FP32 pipe instead of GB300's FP64
 * pipe (1/64 of the FP32 rate), at close to FP64 precision (about 2^-45 per
 * operation against 2^-53).  Same rows, same branch structure and the same
 * elimination order as the mixed-path kernels of solvers.cuh; the prognostic
 * results are joined back to FP64 (one FP64 addition each) and clipped as
 * there.
 *
 * k_tracers_solve_df  vertical advection and sedimentation of the non-main
 *                     constituents (column_solvers.c:385-639), one thread
 *                     per (constituent, column), the Thomas sweep in
 *                     registers (layer count a compile-time constant)
 * k_waves_df          the whole implicit sound-wave solve of one column
 *                     (column_solvers.c:19-383) in one kernel, one thread
 *                     per column: going down, each layer's explicit
 *                     predictors and partial derivatives (:102-139), each
 *                     inner interface's tridiagonal row (:142-189) and its
 *                     forward elimination (:641-669) at once, the
 *                     elimination coefficients in registers; going up, the
 *                     back-substitution, the Klemp damping (:285-298) and
 *                     the new rho, rho theta_v, theta_v', Pi' and w
 *                     (:305-370).  Nothing but the new state is written.
 */
#pragma once

#include "dfloat.cuh"
#include "solvers.cuh"

namespace game {
namespace {


template <int NL>
__global__ void __launch_bounds__(64) k_tracers_solve_df(VGrid vg, StepParams p, DState so, DState sn, DState st,
                                                         DfGrid dg, float *sh_rho)
{
    const int nc = vg.nc;
    constexpr int nl = NL;
    const long long ns = (long long)nl * nc;
    const long long q = gtid();
    const int n_tr = p.n_const - 1;
    if (q >= (long long)n_tr * nc) return;
    const int slot = (int)(q / nc), i = (int)(q - (long long)slot * nc);
    const int k = slot < p.n_cond ? slot : slot + 1; /* skip the main gas */
    bool has_sink;
    const double vsink = sink_velocity(p, k, has_sink);
    const df vs = df_from_double(vsink);
    const df dtd = df_from_double(p.dt);
    const df half_dt = {0.5f * dtd.hi, 0.5f * dtd.lo}; /* exact */
    const double *ro = so.rho + k * ns;
    const double *tr = st.rho + k * ns;
    const df a_sfc = ld_df(dg.area_v, (long long)nl * nc + i);
    df ep[NL], rp[NL];
    df fi_prev = df_zero(), fr_prev = df_zero();
    df ro_j = df_from_double(ro[i]);
#pragma unroll
    for (int j = 0; j < nl; ++j) {
        const long long b = i + (long long)j * nc;
        /* implicit and explicit weights are both 1/2: every flux term of row
         * j carries the factor g = dt / (2 V_j) */
        const df g = df_mul(half_dt, ld_df(dg.inv_vol, b));
        /* flux at interface j (below layer j) */
        df fi = df_zero(), fr = df_zero(), ej = df_zero(), ro_next = df_zero();
        if (j < nl - 1) {
            const long long wi = b + nc;
            df a_ = df_from_double(so.w[wi]), b_ = df_from_double(sn.w[wi]);
            if (has_sink) {
                a_ = df_sub(a_, vs);
                b_ = df_sub(b_, vs);
            }
            const df ar = ld_df(dg.area_v, wi);
            a_ = df_mul(ar, a_);
            b_ = df_mul(ar, b_);
            ro_next = df_from_double(ro[b + nc]);
            const df dio = df_nonneg(b_) ? ro_next : ro_j;
            fi = a_;
            fr = df_mul(dio, b_);
            if (df_nonneg(fi)) ej = df_neg(df_mul(g, fi));
        }
        /* sub-diagonal of row j (coupling to layer j - 1), formed with row
         * j's factor */
        const df c_j = df_nonneg(fi_prev) ? df_zero() : df_mul(g, fi_prev);
        df dj, rj = df_add(ro_j, df_mul(dtd, df_from_double(tr[b])));
        if (j == 0) {
            dj = df_nonneg(fi) ? df_one() : df_sub(df_one(), df_mul(g, fi));
            rj = df_add(rj, df_mul(g, fr));
        } else if (j == nl - 1) {
            dj = df_nonneg(fi_prev) ? df_add(df_one(), df_mul(g, fi_prev)) : df_one();
            rj = df_sub(rj, df_mul(g, fr_prev));
            if (has_sink) {
                const df gs = df_mul(df_mul(g, vs), a_sfc);
                dj = df_add(dj, gs);
                rj = df_sub(rj, df_mul(gs, ro_j));
            }
        } else {
            dj = df_one();
            if (df_nonneg(fi_prev)) dj = df_add(dj, df_mul(g, fi_prev));
            if (!df_nonneg(fi)) dj = df_sub(dj, df_mul(g, fi));
            rj = df_add(rj, df_mul(g, df_sub(fr, fr_prev)));
        }
        /* forward elimination */
        if (j == 0) {
            const df inv = df_rcp(dj);
            ep[0] = df_mul(ej, inv);
            rp[0] = df_mul(rj, inv);
        } else {
            const df inv = df_rcp(df_sub_mul(dj, ep[j - 1], c_j));
            if (j < nl - 1) ep[j] = df_mul(ej, inv);
            rp[j] = df_mul(df_sub_mul(rj, rp[j - 1], c_j), inv);
        }
        fi_prev = fi;
        fr_prev = fr;
        ro_j = ro_next;
    }
    double *rn = sn.rho + k * ns;
    float *rs = sh_rho + k * ns;
    df x = rp[nl - 1];
    {
        const df v = df_nonneg(x) ? x : df_zero();
        rn[(long long)(nl - 1) * nc + i] = df_to_double(v);
        rs[(long long)(nl - 1) * nc + i] = v.hi;
    }
#pragma unroll
    for (int j = nl - 2; j >= 0; --j) {
        x = df_sub_mul(rp[j], ep[j], x);
        const df v = df_nonneg(x) ? x : df_zero();
        rn[(long long)j * nc + i] = df_to_double(v);
        rs[(long long)j * nc + i] = v.hi;
    }
}

/* per-layer quantities of the sound-wave solve (the mixed-path forms of
 * k_waves_layer, solvers.cuh), at layer j of column i */
struct WaveLayer {
    df alpha, beta, gam, rho_expl, tp_expl, ep_expl, thl, ro;
};

template <int NL>
__global__ void __launch_bounds__(64) k_waves_df(VGrid vg, StepParams p, DState so, DState sn, DState st, DfGrid dg,
                                                 Shadow sh, int rk)
{
    constexpr int n = NL - 1; /* inner interfaces = rows */
    const int nc = vg.nc;
    const int i = (int)gtid();
    if (i >= nc) return;
    const long long ns = (long long)NL * nc, gp = (long long)p.n_cond * ns, ni = (long long)n * nc;
    const df dt = df_from_double(p.dt), inv_dt = df_from_double(p.inv_dt);
    const df k_rows = df_from_double(p.k_rows), k_rows2 = df_from_double(p.k_rows2);
    const df rcv = df_from_double(R_D / C_D_V);
    const bool rk1 = rk != 0;

    /* theta_v of state_new at layer j (read before the layer is overwritten) */
    auto thl_at = [&](int j) {
        const long long b = (long long)j * nc + i;
        return df_mul(df_from_double(sn.rhotheta_v[b]), df_rcp(df_from_double(sn.rho[gp + b])));
    };
    /* gamma = d Pi / d (rho theta_v) per volume, averaged over old and new
     * state at rk 1 */
    auto gam_at = [&](long long b, df rto, df iv) {
        const df go = df_mul(df_mul(rcv, df_add(ld_df(dg.exner_bg, b), df_from_double(so.exner_pert[b]))),
                             df_rcp(rto));
        if (!rk1) return df_mul(go, iv);
        const df gn = df_mul(df_mul(rcv, df_add(ld_df(dg.exner_bg, b), df_from_double(sn.exner_pert[b]))),
                             df_rcp(df_from_double(sn.rhotheta_v[b])));
        return df_mul(df_half(df_add(go, gn)), iv);
    };
    auto layer = [&](int j) {
        const long long b = (long long)j * nc + i;
        WaveLayer L;
        const df iv = ld_df(dg.inv_vol, b), vol = ld_df(dg.volume, b);
        const df ro = df_from_double(so.rho[gp + b]), rto = df_from_double(so.rhotheta_v[b]);
        const df iro = df_rcp(ro);
        const df rn = df_from_double(sn.rho[gp + b]), rtn = df_from_double(sn.rhotheta_v[b]);
        const df irn = df_rcp(rn);
        L.gam = gam_at(b, rto, iv);
        if (!rk1) {
            L.alpha = df_neg(df_mul(df_mul(df_mul(rto, iro), iro), iv));
            L.beta = df_mul(iro, iv);
        } else {
            L.alpha = df_mul(df_half(df_neg(df_add(df_mul(df_mul(rto, iro), iro), df_mul(df_mul(rtn, irn), irn)))),
                             iv);
            L.beta = df_mul(df_half(df_add(iro, irn)), iv);
        }
        const df str = df_from_double(st.rho[gp + b]), strt = df_from_double(st.rhotheta_v[b]);
        L.rho_expl = df_add(ro, df_mul(dt, str));
        L.tp_expl = df_add(df_from_double(so.theta_v_pert[b]),
                           df_mul(df_mul(dt, vol), df_add(df_mul(L.alpha, str), df_mul(L.beta, strt))));
        L.ep_expl = df_add(df_from_double(so.exner_pert[b]), df_mul(df_mul(df_mul(dt, vol), L.gam), strt));
        L.thl = df_mul(rtn, irn);
        L.ro = ro;
        return L;
    };

    /* ---- down: rows and forward elimination */
    df ep[n], rp[n];
    WaveLayer L0 = layer(0);
    df thl_prev = df_zero();
    df c_prev_row = df_zero();
    (void)c_prev_row;
#pragma unroll
    for (int j = 0; j < n; ++j) {
        const WaveLayer L1 = layer(j + 1);
        const long long q = (long long)j * nc + i, wi = q + nc;
        const df dz = ld_df(dg.geo, q), H = ld_df(dg.geo, ni + q), G1 = ld_df(dg.geo, 2 * ni + q),
                 G2 = ld_df(dg.geo, 3 * ni + q);
        const df irio = df_rcp(df_half(df_add(L0.ro, L1.ro)));
        const df rho_ie = df_half(df_add(L0.rho_expl, L1.rho_expl));
        const df th = df_half(df_add(L0.thl, L1.thl));
        const df wo = df_from_double(so.w[wi]);
        const df k1 = df_mul(dz, k_rows);
        /* d_j, r_j */
        const df d = df_sub(
            df_add(df_neg(df_mul(df_mul(th, th), df_add(L0.gam, L1.gam))),
                   df_mul(H, df_add(df_sub(L1.alpha, L0.alpha), df_mul(th, df_sub(L1.beta, L0.beta))))),
            df_mul(df_mul(k1, irio), df_add(G1, df_mul(df_mul(dt, wo), G2))));
        const df r = df_sub(
            df_add(df_add(df_neg(df_mul(df_add(wo, df_mul(dt, df_from_double(st.w[wi]))), k1)),
                          df_mul(df_mul(th, df_sub(L0.ep_expl, L1.ep_expl)), inv_dt)),
                   df_mul(df_mul(inv_dt, df_add(L0.tp_expl, L1.tp_expl)), H)),
            df_mul(df_mul(df_mul(k1, wo), rho_ie), irio));
        const df sw = df_mul(df_mul(k_rows2, wo), irio);
        /* e_j: super-diagonal of row j */
        df e = df_zero();
        if (j < n - 1) {
            const df th_next = df_half(df_add(L1.thl, thl_at(j + 2)));
            e = df_add(df_sub(df_mul(df_mul(th, L1.gam), th_next),
                              df_mul(H, df_add(L1.alpha, df_mul(L1.beta, th_next)))),
                       df_mul(ld_df(dg.geo, 5 * ni + q), sw));
        }
        /* c_{j-1}: sub-diagonal of row j (its coupling to interface j - 1) */
        if (j == 0) {
            const df inv = df_rcp(d);
            ep[0] = df_mul(e, inv);
            rp[0] = df_mul(r, inv);
        } else {
            const df th_prev = df_half(df_add(thl_prev, L0.thl));
            const df cm = df_sub(df_add(df_mul(df_mul(th, L0.gam), th_prev),
                                        df_mul(H, df_add(L0.alpha, df_mul(L0.beta, th_prev)))),
                                 df_mul(ld_df(dg.geo, 4 * ni + q), sw));
            const df inv = df_rcp(df_sub_mul(d, ep[j - 1], cm));
            if (j < n - 1) ep[j] = df_mul(e, inv);
            rp[j] = df_mul(df_sub_mul(r, rp[j - 1], cm), inv);
        }
        thl_prev = L0.thl;
        L0 = L1;
    }

    /* ---- up: back-substitution, damping and the new state, layer by layer
     * from the surface; the interface below layer jj is jj, the one above
     * jj - 1 */
    df x_below = df_zero(), sol_below = df_zero(), thl_below = df_zero(), rnew_below = df_zero(),
       ro_below = df_zero();
    df thl_here = thl_at(NL - 1);
#pragma unroll
    for (int jj = NL - 1; jj >= 0; --jj) {
        const long long b = (long long)jj * nc + i;
        df x_above = df_zero(), sol_above = df_zero(), thl_above = df_zero();
        if (jj > 0) {
            x_above = jj - 1 == n - 1 ? rp[n - 1] : df_sub_mul(rp[jj - 1], ep[jj - 1], x_below);
            sol_above = df_mul(x_above, ld_df(dg.damp_inv, b - nc));
            thl_above = thl_at(jj - 1);
        }
        const df iv = ld_df(dg.inv_vol, b);
        const df ro = df_from_double(so.rho[gp + b]), rto = df_from_double(so.rhotheta_v[b]);
        const df gam = gam_at(b, rto, iv);
        const df rho_expl = df_add(ro, df_mul(dt, df_from_double(st.rho[gp + b])));
        const df rt_expl = df_add(rto, df_mul(dt, df_from_double(st.rhotheta_v[b])));
        const df th_above = df_half(df_add(thl_above, thl_here)), th_below = df_half(df_add(thl_here, thl_below));
        df num, num2;
        if (jj == 0) {
            num = sol_below;
            num2 = df_mul(th_below, sol_below);
        } else if (jj == NL - 1) {
            num = df_neg(sol_above);
            num2 = df_neg(df_mul(th_above, sol_above));
        } else {
            num = df_sub(sol_below, sol_above);
            num2 = df_sub(df_mul(th_below, sol_below), df_mul(th_above, sol_above));
        }
        const df r_new = df_add(rho_expl, df_mul(df_mul(dt, num), iv));
        const df rt_new = df_add(rt_expl, df_mul(df_mul(dt, num2), iv));
        const df tp_new = df_sub(df_mul(rt_new, df_rcp(r_new)), ld_df(dg.theta_v_bg, b));
        const df ep_new = df_add(df_from_double(so.exner_pert[b]),
                                 df_mul(df_mul(ld_df(dg.volume, b), gam), df_sub(rt_new, rto)));
        sn.rho[gp + b] = df_to_double(r_new);
        sn.rhotheta_v[b] = df_to_double(rt_new);
        sn.theta_v_pert[b] = df_to_double(tp_new);
        sn.exner_pert[b] = df_to_double(ep_new);
        if (sh.rho) {
            sh.rho[gp + b] = r_new.hi;
            sh.rhotheta_v[b] = rt_new.hi;
            sh.theta_v_pert[b] = tp_new.hi;
            sh.exner_pert[b] = ep_new.hi;
        }
        if (jj < NL - 1) { /* w at the interface below */
            const long long wi = b + nc;
            const df irio = df_rcp(df_half(df_add(ro, ro_below)));
            const df dint = df_half(df_add(r_new, rnew_below));
            const df wn = df_mul(df_sub(df_mul(df_mul({2.0f, 0.0f}, sol_below), ld_df(dg.inv_area_v, wi)),
                                        df_mul(dint, df_from_double(so.w[wi]))),
                                 irio);
            sn.w[wi] = df_to_double(wn);
            if (sh.w) sh.w[wi] = wn.hi;
        }
        x_below = x_above;
        sol_below = sol_above;
        thl_below = thl_here;
        thl_here = thl_above;
        rnew_below = r_new;
        ro_below = ro;
    }
}

}  // namespace
}  // namespace game
