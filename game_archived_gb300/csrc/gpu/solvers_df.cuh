/*
 * The mixed path's vertical eliminations in double-float arithmetic
 * (dfloat.cuh), so that they issue on the FP32 pipe instead of GB300's FP64
 * pipe (1/64 of the FP32 rate), at close to FP64 precision (about 2^-45 per
 * operation against 2^-53).  Same rows, same branch structure and the same
 * elimination order as the mixed-path kernels of solvers.cuh.  A double
 * carried in double-float keeps 48 of its 53 significand bits, so the
 * kernels compute only increments in double-float and add them to the FP64
 * state with one FP64 addition each: the densities, rho theta_v and Pi' keep
 * their full precision, and the mass-flux form of the density update stays
 * conservative to FP64 rounding.
 *
 * k_tracers_solve_df  vertical advection and sedimentation of the non-main
 *                     constituents (column_solvers.c:385-639), one thread
 *                     per (constituent, column), the elimination
 *                     coefficients in shared memory, solved for the
 *                     increment of the density
 * k_waves_*_df        the implicit sound-wave solve (column_solvers.c:19-383):
 *                     per (layer, column) the explicit predictors and
 *                     partial derivatives (:102-139), per (interface,
 *                     column) the tridiagonal rows (:142-189), per column
 *                     the elimination (:641-669) with the Klemp damping
 *                     (:285-298), per (layer, column) the new rho,
 *                     rho theta_v, theta_v', Pi' and w (:305-370)
 */
#pragma once

#include "dfloat.cuh"
#include "solvers.cuh"

namespace game {
namespace {


/* threads per block of the double-float tracer solve; its elimination
 * coefficients live in shared memory, NL x TRACER_BLOCK (hi, lo) pairs each */
constexpr int TRACER_BLOCK = 64;

/* The column system A x = r of the tracer (rows as k_tracers_solve's mixed
 * path) is solved for the increment delta = x - rho_old: A delta = r - A
 * rho_old, whose right-hand side holds only the tendency and flux terms
 * (dt tr + g (fr_j - fr_{j-1}) - (A - I) rho_old), so that the new density
 * is the FP64 old value plus a double-float increment: the state keeps its
 * 53 bits (a double carried in double-float keeps 48). */
template <int NL>
__global__ void __launch_bounds__(TRACER_BLOCK) k_tracers_solve_df(VGrid vg, StepParams p, DState so, DState sn,
                                                                   DState st, DfGrid dg, float *sh_rho)
{
    /* the loops are not unrolled (the unrolled double-float sweep overflowed
     * the instruction cache), so the coefficients cannot be registers */
    __shared__ float2 s_ep[NL][TRACER_BLOCK], s_rp[NL][TRACER_BLOCK];
    const int nc = vg.nc;
    constexpr int nl = NL;
    const long long ns = (long long)nl * nc;
    const long long q = gtid();
    const int n_tr = p.n_const - 1;
    if (q >= (long long)n_tr * nc) return;
    const int t = threadIdx.x;
    const int slot = (int)(q / nc), i = (int)(q - (long long)slot * nc);
    const int k = slot < p.n_cond ? slot : slot + 1; /* skip the main gas */
    bool has_sink;
    const double vsink = sink_velocity(p, k, has_sink);
    const df vs = df_from_double(vsink);
    const df dtd = df_from_double(p.dt);
    const df half_dt = df_half(dtd);
    const double *ro = so.rho + k * ns;
    const double *tr = st.rho + k * ns;
    {
        /* a constituent absent from the column, old density and tendency 0 in
         * every layer (a cloud-free column's condensates): the system's
         * right-hand side is 0 and so is the new density, exactly */
        bool empty = true;
#pragma unroll 1
        for (int j = 0; j < nl && empty; ++j) {
            const long long b = (long long)j * nc + i;
            empty = is_zero(ro[b]) && is_zero(tr[b]);
        }
        if (empty) {
            double *rn = sn.rho + k * ns;
            float *rs = sh_rho + k * ns;
#pragma unroll 1
            for (int j = 0; j < nl; ++j) {
                rn[(long long)j * nc + i] = 0.0;
                rs[(long long)j * nc + i] = 0.0f;
            }
            return;
        }
    }
    const df a_sfc = ld_df(dg.area_v, (long long)nl * nc + i);
    df fi_prev = df_zero(), fr_prev = df_zero(), ep_prev = df_zero(), rp_prev = df_zero();
    df ro_j = df_from_double(ro[i]), ro_prev = df_zero();
    /* inputs of row j, loaded one row ahead (indices clamped to the column) */
    auto wi_of = [&](int j) { return (long long)(j < nl - 1 ? j + 1 : nl - 1) * nc + i; };
    float2 iv_c = dg.inv_vol[i];
    double tr_c = tr[i], wo_c = so.w[wi_of(0)], wn_c = sn.w[wi_of(0)], ron_c = ro[wi_of(0)];
    float2 ar_c = dg.area_v[wi_of(0)];
#pragma unroll 1
    for (int j = 0; j < nl; ++j) {
        const int jn = j + 1 < nl ? j + 1 : j;
        const long long bn = (long long)jn * nc + i, wn_i = wi_of(jn);
        const float2 iv_n = dg.inv_vol[bn];
        const double tr_n = tr[bn], wo_n = so.w[wn_i], wn_n = sn.w[wn_i], ron_n = ro[wn_i];
        const float2 ar_n = dg.area_v[wn_i];
        /* implicit and explicit weights are both 1/2: every flux term of row
         * j carries the factor g = dt / (2 V_j) */
        const df g = df_mul(half_dt, df{iv_c.x, iv_c.y});
        /* flux at interface j (below layer j) */
        df fi = df_zero(), fr = df_zero(), ej = df_zero(), ro_next = df_zero();
        if (j < nl - 1) {
            df a_ = df_from_double(wo_c), b_ = df_from_double(wn_c);
            if (has_sink) {
                a_ = df_sub(a_, vs);
                b_ = df_sub(b_, vs);
            }
            const df ar = {ar_c.x, ar_c.y};
            a_ = df_mul(ar, a_);
            b_ = df_mul(ar, b_);
            ro_next = df_from_double(ron_c);
            const df dio = df_nonneg(b_) ? ro_next : ro_j;
            fi = a_;
            fr = df_mul(dio, b_);
            if (df_nonneg(fi)) ej = df_neg(df_mul(g, fi));
        }
        /* sub-diagonal of row j (coupling to layer j - 1), formed with row
         * j's factor */
        const df c_j = df_nonneg(fi_prev) ? df_zero() : df_mul(g, fi_prev);
        /* dm1 = d_j - 1 and the explicit right-hand side minus rho_old */
        df dm1, rx = df_mul(dtd, df_from_double(tr_c));
        if (j == 0) {
            dm1 = df_nonneg(fi) ? df_zero() : df_neg(df_mul(g, fi));
            rx = df_add(rx, df_mul(g, fr));
        } else if (j == nl - 1) {
            dm1 = df_nonneg(fi_prev) ? df_mul(g, fi_prev) : df_zero();
            rx = df_sub(rx, df_mul(g, fr_prev));
            if (has_sink) {
                const df gs = df_mul(df_mul(g, vs), a_sfc);
                dm1 = df_add(dm1, gs);
                rx = df_sub(rx, df_mul(gs, ro_j));
            }
        } else {
            dm1 = df_zero();
            if (df_nonneg(fi_prev)) dm1 = df_add(dm1, df_mul(g, fi_prev));
            if (!df_nonneg(fi)) dm1 = df_sub(dm1, df_mul(g, fi));
            rx = df_add(rx, df_mul(g, df_sub(fr, fr_prev)));
        }
        /* the increment's right-hand side r - A rho_old */
        df r_inc = df_sub(rx, df_mul(dm1, ro_j));
        if (j > 0) r_inc = df_sub_mul(r_inc, c_j, ro_prev);
        if (j < nl - 1) r_inc = df_sub_mul(r_inc, ej, ro_next);
        /* forward elimination (row 0: ep_prev = rp_prev = c_0 = 0) */
        const df inv = df_rcp(df_sub_mul(df_add(df_one(), dm1), ep_prev, c_j));
        ep_prev = df_mul(ej, inv);
        rp_prev = df_mul(df_sub_mul(r_inc, rp_prev, c_j), inv);
        s_ep[j][t] = make_float2(ep_prev.hi, ep_prev.lo);
        s_rp[j][t] = make_float2(rp_prev.hi, rp_prev.lo);
        fi_prev = fi;
        fr_prev = fr;
        ro_prev = ro_j;
        ro_j = ro_next;
        iv_c = iv_n;
        tr_c = tr_n;
        wo_c = wo_n;
        wn_c = wn_n;
        ron_c = ron_n;
        ar_c = ar_n;
    }
    double *rn = sn.rho + k * ns;
    float *rs = sh_rho + k * ns;
    df x = df_zero();
#pragma unroll 1
    for (int j = nl - 1; j >= 0; --j) {
        const float2 e2 = s_ep[j][t], r2 = s_rp[j][t];
        x = df_sub_mul(df{r2.x, r2.y}, df{e2.x, e2.y}, x); /* e_{nl-1} = 0 */
        const long long b = (long long)j * nc + i;
        const double xn = ro[b] + df_to_double(x);
        const double v = nonneg<false>(xn) ? xn : 0.0;
        rn[b] = v;
        rs[b] = to_float(v);
    }
}

/* sedimentation heating (rk 0, column_solvers.c:455-462, 551-623): the
 * divergence of the condensates' enthalpy fluxes c_p T rho w_sink A at the
 * interfaces, summed over the condensates in the reference's order.  One
 * thread per (layer, column), each forming the fluxes of its two
 * interfaces (the per-column FP64 kernel of solvers.cuh forms each once but
 * has 26 times fewer threads). */
__global__ void k_tracers_sedheat_df(VGrid vg, StepParams p, DState so, DState sn, const double *temperature,
                                     TracerWork tw, DfGrid dg, double *sed_heat)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long ns = (long long)nl * nc, b = gtid();
    if (b >= ns) return;
    const int j = (int)(b / nc), i = (int)(b - (long long)j * nc);
    const int n_cond = p.n_cond < SEDHEAT_MAX_COND ? p.n_cond : SEDHEAT_MAX_COND;
    /* enthalpy flux of constituent k at interface jj (below layer jj) */
    /* a condensate's flux is c_p T rho w A with rho its upstream density:
     * exactly zero where that density is (no cloud), so the double-float
     * products are skipped there, and the upwind choice too where both
     * candidate densities are zero */
    auto fe = [&](int k, int jj, df vs, bool has) {
        const long long bb = i + (long long)jj * nc, wi = bb + nc;
        /* no density on either side: zero whichever way the wind blows */
        if (is_zero(so.rho[k * ns + bb]) && is_zero(so.rho[k * ns + bb + nc])) return df_zero();
        df b_ = df_from_double(sn.w[wi]);
        if (has) b_ = df_sub(b_, vs);
        b_ = df_mul(ld_df(dg.area_v, wi), b_);
        const long long up = df_nonneg(b_) ? bb + nc : bb;
        const double r_up = so.rho[k * ns + up];
        if (is_zero(r_up)) return df_zero();
        const df fr = df_mul(df_from_double(r_up), b_);
        const df cp = df_from_double((k % 2 == 0) ? tw.cp_ice[up] : tw.cp_water[up]);
        return df_mul(df_mul(cp, df_from_double(temperature[up])), fr);
    };
    const df ivol = ld_df(dg.inv_vol, b);
    df sh = df_zero();
#pragma unroll 1
    for (int k = 0; k < n_cond; ++k) {
        bool has;
        const double vsd = sink_velocity(p, k, has);
        const df vs = df_from_double(vsd);
        if (j == 0) {
            sh = df_add(sh, df_mul(fe(k, 0, vs, has), ivol));
        } else if (j == nl - 1) {
            sh = df_add(sh, df_mul(df_neg(fe(k, j - 1, vs, has)), ivol));
            const long long bot = b;
            const double r_bot = so.rho[k * ns + bot];
            if (!is_zero(r_bot)) {
                const df cp = df_from_double((k % 2 == 0) ? tw.cp_ice[bot] : tw.cp_water[bot]);
                const df e = df_mul(df_mul(df_mul(df_mul(df_neg(vs), df_from_double(temperature[bot])), cp),
                                           df_from_double(r_bot)),
                                    ld_df(dg.area_v, (long long)nl * nc + i));
                sh = df_add(sh, df_mul(e, ivol));
            }
        } else {
            sh = df_add(sh, df_mul(df_add(df_neg(fe(k, j - 1, vs, has)), fe(k, j, vs, has)), ivol));
        }
    }
    sed_heat[b] = df_to_double(sh);
}

/* ---------------------------------------------------------- sound waves
 * The four kernels of solvers.cuh's mixed path (k_waves_layer,
 * k_waves_rows_mixed, k_waves_thomas, k_waves_apply) with their FP64
 * arithmetic in double-float; the WavesWork arrays hold (hi, lo) pairs in
 * place of doubles (same size).  A single fused kernel with one thread per
 * column (rows, elimination and back-substitution in one pass) was slower
 * than this chain on GB300: 41k columns give too few threads to hide its
 * latency, and its unrolled body overflowed the instruction cache. */
__device__ __forceinline__ float2 f2(df x) { return make_float2(x.hi, x.lo); }
__device__ __forceinline__ df ldw(const double *a, long long i) { return ld_df((const float2 *)a, i); }
__device__ __forceinline__ void stw(double *a, long long i, df x) { ((float2 *)a)[i] = f2(x); }

__global__ void k_waves_layer_df(VGrid vg, StepParams p, DState so, DState sn, DState st, WavesWork ww, DfGrid dg,
                                 int rk)
{
    const long long ns = (long long)vg.nl * vg.nc, b = gtid();
    if (b >= ns) return;
    const long long gp = p.n_cond * ns;
    const df dt = df_from_double(p.dt), rcv = df_from_double(R_D / C_D_V);
    const df iv = ld_df(dg.inv_vol, b), vol = ld_df(dg.volume, b), ebg = ld_df(dg.exner_bg, b);
    const df ro = df_from_double(so.rho[gp + b]), rto = df_from_double(so.rhotheta_v[b]);
    const df rn = df_from_double(sn.rho[gp + b]), rtn = df_from_double(sn.rhotheta_v[b]);
    const df iro = df_rcp(ro), irn = df_rcp(rn);
    const df go = df_mul(df_mul(rcv, df_add(ebg, df_from_double(so.exner_pert[b]))), df_rcp(rto));
    df alpha, beta, gam;
    if (rk == 0) {
        alpha = df_neg(df_mul(df_mul(df_mul(rto, iro), iro), iv));
        beta = df_mul(iro, iv);
        gam = df_mul(go, iv);
    } else {
        const df gn = df_mul(df_mul(rcv, df_add(ebg, df_from_double(sn.exner_pert[b]))), df_rcp(rtn));
        alpha = df_mul(df_half(df_neg(df_add(df_mul(df_mul(rto, iro), iro), df_mul(df_mul(rtn, irn), irn)))), iv);
        beta = df_mul(df_half(df_add(iro, irn)), iv);
        gam = df_mul(df_half(df_add(go, gn)), iv);
    }
    const df str = df_from_double(st.rho[gp + b]), strt = df_from_double(st.rhotheta_v[b]);
    const df dtv = df_mul(dt, vol);
    stw(ww.alpha, b, alpha);
    stw(ww.beta, b, beta);
    stw(ww.gam, b, gam);
    /* the explicit increments dt * tendency (not the predictors themselves):
     * the new densities are formed as the FP64 old value plus an increment,
     * so the double-float arithmetic never rounds the state itself */
    stw(ww.rho_expl, b, df_mul(dt, str));
    stw(ww.rt_expl, b, df_mul(dt, strt));
    stw(ww.tp_expl, b, df_add(df_from_double(so.theta_v_pert[b]),
                              df_mul(dtv, df_add(df_mul(alpha, str), df_mul(beta, strt)))));
    stw(ww.ep_expl, b, df_add(df_from_double(so.exner_pert[b]), df_mul(df_mul(dtv, gam), strt)));
    stw(ww.thl, b, df_mul(rtn, irn));
}

/* the rows of k_waves_rows_mixed: d_j, r_j, e_j of row j and c_{j-1} of row
 * j (its coupling to interface j - 1), one reciprocal of rho per interface */
__global__ void k_waves_rows_df(VGrid vg, StepParams p, DState so, DState st, WavesWork ww, DfGrid dg)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long n = (long long)(nl - 1) * nc, q = gtid();
    if (q >= n) return;
    const int j = (int)(q / nc);
    const long long ns = (long long)nl * nc, gp = p.n_cond * ns;
    const long long b = q, lo = q + nc, wi = q + nc;
    const df dt = df_from_double(p.dt), inv_dt = df_from_double(p.inv_dt);
    const df dz = ld_df(dg.geo, q), H = ld_df(dg.geo, n + q), G1 = ld_df(dg.geo, 2 * n + q),
             G2 = ld_df(dg.geo, 3 * n + q);
    const df ro_b = df_from_double(so.rho[gp + b]), ro_lo = df_from_double(so.rho[gp + lo]);
    const df irio = df_rcp(df_half(df_add(ro_b, ro_lo)));
    const df rho_ie = df_half(df_add(df_add(ro_b, ldw(ww.rho_expl, b)), df_add(ro_lo, ldw(ww.rho_expl, lo))));
    const df tl_b = ldw(ww.thl, b), tl_lo = ldw(ww.thl, lo);
    const df th = df_half(df_add(tl_b, tl_lo));
    const df wo = df_from_double(so.w[wi]);
    const df a0 = ldw(ww.alpha, b), a1 = ldw(ww.alpha, lo), b0 = ldw(ww.beta, b), b1 = ldw(ww.beta, lo);
    const df g0 = ldw(ww.gam, b), g1 = ldw(ww.gam, lo);
    const df k1 = df_mul(dz, df_from_double(p.k_rows));
    stw(ww.d, q, df_sub(df_add(df_neg(df_mul(df_mul(th, th), df_add(g0, g1))),
                               df_mul(H, df_add(df_sub(a1, a0), df_mul(th, df_sub(b1, b0))))),
                        df_mul(df_mul(k1, irio), df_add(G1, df_mul(df_mul(dt, wo), G2)))));
    stw(ww.r, q, df_sub(df_add(df_add(df_neg(df_mul(df_add(wo, df_mul(dt, df_from_double(st.w[wi]))), k1)),
                                      df_mul(df_mul(th, df_sub(ldw(ww.ep_expl, b), ldw(ww.ep_expl, lo))), inv_dt)),
                               df_mul(df_mul(inv_dt, df_add(ldw(ww.tp_expl, b), ldw(ww.tp_expl, lo))), H)),
                        df_mul(df_mul(df_mul(k1, wo), rho_ie), irio)));
    stw(ww.th_int, q, th);
    stw(ww.rho_io, q, irio);
    const df sw = df_mul(df_mul(df_from_double(p.k_rows2), wo), irio);
    if (j < nl - 2) {
        const df th_next = df_half(df_add(tl_lo, ldw(ww.thl, lo + nc)));
        stw(ww.e, q, df_add(df_sub(df_mul(df_mul(th, g1), th_next), df_mul(H, df_add(a1, df_mul(b1, th_next)))),
                            df_mul(ld_df(dg.geo, 5 * n + q), sw)));
    }
    if (j > 0) {
        const df th_prev = df_half(df_add(ldw(ww.thl, b - nc), tl_b));
        stw(ww.c, q - nc, df_sub(df_add(df_mul(df_mul(th, g0), th_prev), df_mul(H, df_add(a0, df_mul(b0, th_prev)))),
                                 df_mul(ld_df(dg.geo, 4 * n + q), sw)));
    }
}

/* threads per block of the double-float sound-wave sweep: two per column
 * (its coefficients in shared memory, (NL - 1) x (WAVES_BLOCK / 2) pairs
 * each) */
constexpr int WAVES_BLOCK = 64;

/* the tridiagonal elimination of one column (column_solvers.c:641-669),
 * solution times the damping factor written over r.  Twisted elimination,
 * two lanes per column: the even lane eliminates the inner interfaces
 * 0 .. m-1 downwards (x_j = r'_j - e'_j x_{j+1}), the odd lane n-1 .. m+1
 * upwards (x_j = r''_j - c''_j x_{j-1}); both solve row m from the shuffled
 * last coefficients and each back-substitutes its half.  The dependent
 * chain is half the Thomas sweep's and twice the warps hide its latency
 * (24.7 against 32.9 us at RES_ID=6; the same scheme for the tracer
 * columns, with their rows built inside the sweep, was slower: 141 against
 * 129 us). */
template <int NL>
__global__ void __launch_bounds__(WAVES_BLOCK) k_waves_thomas_df(int nc, WavesWork ww, DfGrid dg)
{
    constexpr int n = NL - 1, SYS = WAVES_BLOCK / 2, M = n / 2;
    __shared__ float2 s_a[n][SYS], s_r[n][SYS];
    const long long tq = gtid();
    const bool live = (tq >> 1) < nc;
    const unsigned mask = __ballot_sync(0xffffffffu, live);
    if (!live) return;
    const int i = (int)(tq >> 1);
    const bool up = tq & 1; /* the odd lane eliminates upwards */
    const int t = threadIdx.x >> 1;
    auto at = [&](int j) { return (long long)j * nc + i; };
    /* couplings of row j to rows j - 1 and j + 1 */
    auto sub = [&](int j) { return j > 0 ? ldw(ww.c, at(j - 1)) : df_zero(); };
    auto sup = [&](int j) { return j < n - 1 ? ldw(ww.e, at(j)) : df_zero(); };
    df ca = df_zero(), cr = df_zero(); /* e'_{j-1}, r'_{j-1} or c''_{j+1}, r''_{j+1} */
    const int j0 = up ? n - 1 : 0, dj = up ? -1 : 1;
#pragma unroll 1
    for (int j = j0; j != M; j += dj) {
        const df cn = up ? sup(j) : sub(j); /* coupling to the swept side */
        const df cf = up ? sub(j) : sup(j); /* coupling to the far side */
        const df inv = df_rcp(df_sub_mul(ldw(ww.d, at(j)), ca, cn));
        ca = df_mul(cf, inv);
        cr = df_mul(df_sub_mul(ldw(ww.r, at(j)), cr, cn), inv);
        s_a[j][t] = f2(ca);
        s_r[j][t] = f2(cr);
    }
    /* row M, read by both lanes before the even lane overwrites its r with
     * the solution: __syncwarp orders the pair's reads before that store */
    const df a_m = sub(M), e_m = sup(M), d_m = ldw(ww.d, at(M)), r_m = ldw(ww.r, at(M));
    __syncwarp(mask);
    auto shfl_df = [&](df v) {
        return df{__shfl_xor_sync(mask, v.hi, 1), __shfl_xor_sync(mask, v.lo, 1)};
    };
    const df oa = shfl_df(ca), orr = shfl_df(cr);
    const df ea = up ? oa : ca, er = up ? orr : cr;  /* e'_{M-1}, r'_{M-1} */
    const df cb = up ? ca : oa, cbr = up ? cr : orr; /* c''_{M+1}, r''_{M+1} */
    const df den = df_sub_mul(df_sub_mul(d_m, a_m, ea), e_m, cb);
    df x = df_mul(df_sub_mul(df_sub_mul(r_m, a_m, er), e_m, cbr), df_rcp(den));
    if (!up) stw(ww.r, at(M), df_mul(x, ld_df(dg.damp_inv, at(M))));
#pragma unroll 1
    for (int j = M - dj; j != j0 - dj; j -= dj) {
        const float2 a2 = s_a[j][t], r2 = s_r[j][t];
        x = df_sub_mul(df{r2.x, r2.y}, df{a2.x, a2.y}, x);
        stw(ww.r, at(j), df_mul(x, ld_df(dg.damp_inv, at(j))));
    }
}

__global__ void k_waves_apply_df(VGrid vg, StepParams p, DState so, DState sn, WavesWork ww, DfGrid dg, Shadow sh)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long ns = (long long)nl * nc, b = gtid();
    if (b >= ns) return;
    const int j = (int)(b / nc);
    const long long gp = p.n_cond * ns;
    const df dt = df_from_double(p.dt);
    /* the new density as the FP64 old value plus the increment
     * dt (tendency + flux divergence / V), joined in FP64 */
    auto rho_new = [&](int jj, long long bb) {
        df num;
        if (jj == 0) num = ldw(ww.r, bb);
        else if (jj == nl - 1) num = df_neg(ldw(ww.r, bb - nc));
        else num = df_sub(ldw(ww.r, bb), ldw(ww.r, bb - nc));
        const df inc = df_add(ldw(ww.rho_expl, bb), df_mul(df_mul(dt, num), ld_df(dg.inv_vol, bb)));
        return so.rho[gp + bb] + df_to_double(inc);
    };
    const double r_new = rho_new(j, b);
    df num;
    if (j == 0) num = df_mul(ldw(ww.th_int, b), ldw(ww.r, b));
    else if (j == nl - 1) num = df_neg(df_mul(ldw(ww.th_int, b - nc), ldw(ww.r, b - nc)));
    else num = df_sub(df_mul(ldw(ww.th_int, b), ldw(ww.r, b)), df_mul(ldw(ww.th_int, b - nc), ldw(ww.r, b - nc)));
    const df rt_inc = df_add(ldw(ww.rt_expl, b), df_mul(df_mul(dt, num), ld_df(dg.inv_vol, b)));
    const double rt_new = so.rhotheta_v[b] + df_to_double(rt_inc);
    const df rn = df_from_double(r_new), rtn = df_from_double(rt_new);
    const df tp_new = df_sub(df_mul(rtn, df_rcp(rn)), ld_df(dg.theta_v_bg, b));
    /* Pi' = Pi'_old + V gamma (rho theta_v new - old): the increment */
    const double ep_new = so.exner_pert[b] + df_to_double(df_mul(df_mul(ld_df(dg.volume, b), ldw(ww.gam, b)), rt_inc));
    sn.rho[gp + b] = r_new;
    sn.rhotheta_v[b] = rt_new;
    sn.theta_v_pert[b] = df_to_double(tp_new);
    sn.exner_pert[b] = ep_new;
    if (sh.rho) {
        sh.rho[gp + b] = to_float(r_new);
        sh.rhotheta_v[b] = to_float(rt_new);
        sh.theta_v_pert[b] = tp_new.hi;
        sh.exner_pert[b] = to_float(ep_new);
    }
    if (j < nl - 1) {
        const long long wi = b + nc;
        const df dint = df_half(df_add(rn, df_from_double(rho_new(j + 1, b + nc))));
        /* rho_io holds 1 / rho at the interface */
        const df wn = df_mul(df_sub(df_mul(df_mul({2.0f, 0.0f}, ldw(ww.r, b)), ld_df(dg.inv_area_v, wi)),
                                    df_mul(dint, df_from_double(so.w[wi]))),
                             ldw(ww.rho_io, b));
        sn.w[wi] = df_to_double(wn);
        if (sh.w) sh.w[wi] = wn.hi;
    }
}

}  // namespace
}  // namespace game
