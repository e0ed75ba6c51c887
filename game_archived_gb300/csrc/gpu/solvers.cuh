/*
 * Vertical implicit solvers of the RKHEVI step (src/time_stepping/column_solvers.c),
 * FP64, restructured for the GPU:
 *
 * sound waves (column_solvers.c:19-383) in four kernels
 *   k_waves_layer   per (layer, column): explicit predictors and the
 *                   partial derivatives alpha, beta, gamma (:102-139)
 *   k_waves_rows    per (interface, column): the tridiagonal rows c, d, e, r
 *                   (:142-189) and the Klemp damping denominator (:285-298);
 *                   k_waves_rows_mixed is its mixed-path rearrangement
 *   k_waves_thomas  per column: the elimination, with the sweep held in
 *                   registers (layer count a compile-time constant)
 *   k_waves_apply   per (layer, column): back-substitution into rho, rho*theta_v,
 *                   w, theta_v', Pi' (:305-370)
 * tracers (column_solvers.c:385-639)
 *   k_tracers_solve per (constituent, column): rows built on the fly, Thomas
 *                   sweep in registers, clipping
 *   k_tracers_sedheat per column: sedimentation enthalpy flux
 *                   divergence, accumulated over the condensates in the
 *                   reference's order
 *
 * EXACT = true keeps the reference's operation order bit for bit (FP64
 * parity path); EXACT = false (mixed path) multiplies by precomputed
 * reciprocals of the grid metrics and of repeated denominators, which moves
 * results by a few ulps but removes most FP64 divisions.
 */
#pragma once

#include "kernels.cuh"

namespace game {
namespace {

struct WavesWork {
    /* per layer [L][Nc] */
    double *rho_expl, *rt_expl, *alpha, *beta, *gam, *tp_expl, *ep_expl, *thl;
    /* per inner interface [L-1][Nc] */
    double *c, *d, *e, *r, *th_int, *rho_io, *dden;
    /* mixed path: reciprocal grid metrics */
    const double *inv_vol;    /* [L][Nc] */
    const double *inv_area_v; /* [L+1][Nc] */
    /* Klemp damping coefficient of the inner interfaces [L-1][Nc]; mixed
     * path: 1 / (1 + dt * coefficient) for the current dt */
    const double *damp_dc, *damp_inv;
    /* mixed path: grid terms of the rows of inner interface j [6][L-1][Nc]:
     * dz = z(j) - z(j+1), H = (Pi_bg(j) - Pi_bg(j+1)) / 2, G1 = 2 / A_v,
     * G2 = (1/V(j+1) - 1/V(j)) / 2, Cz = dz / V(j), Ez = dz / V(j+1)
     * (layers j, j+1 above and below the interface) */
    const double *geo;
};

/* Klemp (2008) damping coefficient at inner interface j + 1 of every column
 * (column_solvers.c:285-298).  It depends on the grid and the two damping
 * parameters only, so it is tabulated once per parameter pair instead of
 * once per substage. */
__global__ void k_damping_table(VGrid vg, double start_height, double coeff_max, double dt, double *dc,
                                double *inv_den, float2 *inv_den_df)
{
    const long long n = (long long)(vg.nl - 1) * vg.nc, q = gtid();
    if (q >= n) return;
    const long long wi = q + vg.nc;
    const double zad = vg.z_v[wi] - start_height;
    double r = 0.0;
    if (zad >= 0.0) {
        const double s = sin(0.5 * M_PI * zad / (vg.z_v[0] - start_height));
        r = coeff_max * (s * s);
    }
    dc[q] = r;
    const double inv = 1.0 / (1.0 + dt * r);
    inv_den[q] = inv;
    const float hi = (float)inv;
    inv_den_df[q] = make_float2(hi, (float)(inv - (double)hi));
}

template <bool EXACT>
__global__ void k_waves_layer(VGrid vg, StepParams p, DState so, DState sn, DState st, WavesWork ww, int rk)
{
    const long long ns = (long long)vg.nl * vg.nc, b = gtid();
    if (b >= ns) return;
    const long long gp = p.n_cond * ns;
    const double dt = p.dt, pdw = 0.5;
    const double vol = vg.volume[b];
    const double ro = so.rho[gp + b], rto = so.rhotheta_v[b];
    double alpha, beta, gam;
    if (EXACT) {
        if (rk == 0) {
            alpha = -rto / (ro * ro) / vol;
            beta = 1.0 / ro / vol;
            gam = R_D / (C_D_V * rto) * (vg.exner_bg[b] + so.exner_pert[b]) / vol;
        } else {
            const double rn = sn.rho[gp + b];
            const double ao = -rto / (ro * ro), bo = 1.0 / ro;
            const double go = R_D / (C_D_V * rto) * (vg.exner_bg[b] + so.exner_pert[b]);
            const double an = -sn.rhotheta_v[b] / (rn * rn), bn = 1.0 / rn;
            const double gn = R_D / (C_D_V * sn.rhotheta_v[b]) * (vg.exner_bg[b] + sn.exner_pert[b]);
            alpha = ((1.0 - pdw) * ao + pdw * an) / vol;
            beta = ((1.0 - pdw) * bo + pdw * bn) / vol;
            gam = ((1.0 - pdw) * go + pdw * gn) / vol;
        }
    } else {
        const double iv = ww.inv_vol[b], iro = rcp_nr<1>(ro);
        const double rn = sn.rho[gp + b], rtn = sn.rhotheta_v[b], irn = rk == 0 ? 0.0 : rcp_nr<1>(rn);
        const double go = (R_D / C_D_V) * (vg.exner_bg[b] + so.exner_pert[b]) * rcp_nr<1>(rto);
        if (rk == 0) {
            alpha = -rto * iro * iro * iv;
            beta = iro * iv;
            gam = go * iv;
        } else {
            const double gn = (R_D / C_D_V) * (vg.exner_bg[b] + sn.exner_pert[b]) * rcp_nr<1>(rtn);
            alpha = 0.5 * (-rto * iro * iro - rtn * irn * irn) * iv;
            beta = 0.5 * (iro + irn) * iv;
            gam = 0.5 * (go + gn) * iv;
        }
        const double str = st.rho[gp + b], strt = st.rhotheta_v[b];
        ww.alpha[b] = alpha;
        ww.beta[b] = beta;
        ww.gam[b] = gam;
        ww.rho_expl[b] = ro + dt * str;
        ww.rt_expl[b] = rto + dt * strt;
        ww.tp_expl[b] = so.theta_v_pert[b] + dt * vol * (alpha * str + beta * strt);
        ww.ep_expl[b] = so.exner_pert[b] + dt * vol * gam * strt;
        ww.thl[b] = rtn * (rk == 0 ? rcp_nr<1>(rn) : irn);
        return;
    }
    ww.alpha[b] = alpha;
    ww.beta[b] = beta;
    ww.gam[b] = gam;
    ww.rho_expl[b] = ro + dt * st.rho[gp + b];
    ww.rt_expl[b] = rto + dt * st.rhotheta_v[b];
    ww.tp_expl[b] = so.theta_v_pert[b] + dt * vol * (alpha * st.rho[gp + b] + beta * st.rhotheta_v[b]);
    ww.ep_expl[b] = so.exner_pert[b] + dt * vol * gam * st.rhotheta_v[b];
    ww.thl[b] = sn.rhotheta_v[b] / sn.rho[gp + b];
}

/* FP64 path: the rows in the reference's operation order */
__global__ void k_waves_rows(VGrid vg, StepParams p, DState so, DState st, WavesWork ww)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long n = (long long)(nl - 1) * nc, q = gtid();
    if (q >= n) return;
    const int j = (int)(q / nc);
    const long long ns = (long long)nl * nc, gp = p.n_cond * ns;
    const long long b = q, lo = q + nc, wi = q + nc;
    const double dt = p.dt, iw = p.impl_thermo_weight, dt2 = dt * dt;
    const double rho_io = 0.5 * (so.rho[gp + b] + so.rho[gp + lo]);
    const double rho_ie = 0.5 * (ww.rho_expl[b] + ww.rho_expl[lo]);
    const double th = 0.5 * (ww.thl[b] + ww.thl[lo]);
    const double dz = vg.z_scalar[b] - vg.z_scalar[lo], dpi = vg.exner_bg[b] - vg.exner_bg[lo];
    const double wo = so.w[wi];
    const double a0 = ww.alpha[b], a1 = ww.alpha[lo], b0 = ww.beta[b], b1 = ww.beta[lo];
    const double g0 = ww.gam[b], g1 = ww.gam[lo];
    ww.d[q] = -(th * th) * (g0 + g1) + 0.5 * dpi * (a1 - a0 + th * (b1 - b0))
              - dz / (iw * dt2 * C_D_P * rho_io) * (2.0 / vg.area_v[wi] + dt * wo * 0.5 * (-1.0 / vg.volume[b] + 1.0 / vg.volume[lo]));
    ww.r[q] = -(wo + dt * st.w[wi]) * dz / (iw * dt2 * C_D_P) + th * (ww.ep_expl[b] - ww.ep_expl[lo]) / dt
              + 0.5 / dt * (ww.tp_expl[b] + ww.tp_expl[lo]) * dpi - dz / (iw * dt2 * C_D_P) * wo * rho_ie / rho_io;
    ww.th_int[q] = th;
    ww.rho_io[q] = rho_io;
    if (j < nl - 2) {
        const long long lo2 = lo + nc;
        const double th1 = 0.5 * (ww.thl[lo] + ww.thl[lo2]);
        const double rho_io1 = 0.5 * (so.rho[gp + lo] + so.rho[gp + lo2]);
        ww.c[q] = th1 * g1 * th + 0.5 * (vg.exner_bg[lo] - vg.exner_bg[lo2]) * (a1 + b1 * th)
                  - (vg.z_scalar[lo] - vg.z_scalar[lo2]) / (iw * dt * C_D_P) * 0.5 * so.w[wi + nc] / (vg.volume[lo] * rho_io1);
        ww.e[q] = th * g1 * th1 - 0.5 * dpi * (a1 + b1 * th1)
                  + dz / (iw * dt * C_D_P) * 0.5 * wo / (vg.volume[lo] * rho_io);
    }
    /* Klemp (2008) damping denominator of the solution at interface j + 1 */
    ww.dden[q] = 1.0 + dt * ww.damp_dc[q];
}

/* Mixed path: the rows of column_solvers.c:142-189 rearranged so that every
 * inner interface needs one reciprocal.  Thread (interface j, column) forms
 * d_j, r_j, the super-diagonal e_j of row j and the sub-diagonal c_{j-1} of
 * row j-1: c_{j-1} depends on the quantities of interface j (theta_v, rho,
 * w, heights) and on layer j, so the thread of interface j owns it.  Grid
 * terms come from the geo tables; 1/rho at the interface is kept in rho_io
 * for k_waves_apply. */
__global__ void k_waves_rows_mixed(VGrid vg, StepParams p, DState so, DState st, WavesWork ww)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long n = (long long)(nl - 1) * nc, q = gtid();
    if (q >= n) return;
    const int j = (int)(q / nc);
    const long long ns = (long long)nl * nc, gp = p.n_cond * ns;
    const long long b = q, lo = q + nc, wi = q + nc;
    const double dt = p.dt;
    const double *geo = ww.geo;
    const double dz = geo[q], H = geo[n + q], G1 = geo[2 * n + q], G2 = geo[3 * n + q];
    const double rho_io = 0.5 * (so.rho[gp + b] + so.rho[gp + lo]);
    const double irio = rcp_nr<1>(rho_io);
    const double rho_ie = 0.5 * (ww.rho_expl[b] + ww.rho_expl[lo]);
    const double tl_b = ww.thl[b], tl_lo = ww.thl[lo];
    const double th = 0.5 * (tl_b + tl_lo);
    const double wo = so.w[wi];
    const double a0 = ww.alpha[b], a1 = ww.alpha[lo], b0 = ww.beta[b], b1 = ww.beta[lo];
    const double g0 = ww.gam[b], g1 = ww.gam[lo];
    const double k1 = dz * p.k_rows;
    ww.d[q] = -(th * th) * (g0 + g1) + H * (a1 - a0 + th * (b1 - b0)) - k1 * irio * (G1 + dt * wo * G2);
    ww.r[q] = -(wo + dt * st.w[wi]) * k1 + th * (ww.ep_expl[b] - ww.ep_expl[lo]) * p.inv_dt
              + p.inv_dt * (ww.tp_expl[b] + ww.tp_expl[lo]) * H - k1 * wo * rho_ie * irio;
    ww.th_int[q] = th;
    ww.rho_io[q] = irio;
    const double sw = p.k_rows2 * wo * irio;
    if (j < nl - 2) {
        const double th_next = 0.5 * (tl_lo + ww.thl[lo + nc]);
        ww.e[q] = th * g1 * th_next - H * (a1 + b1 * th_next) + geo[5 * n + q] * sw;
    }
    if (j > 0) {
        const double th_prev = 0.5 * (ww.thl[b - nc] + tl_b);
        ww.c[q - nc] = th * g0 * th_prev + H * (a0 + b0 * th_prev) - geo[4 * n + q] * sw;
    }
}

/* tridiagonal elimination of one column (column_solvers.c:641-669), forward
 * sweep kept in registers; solution divided by the damping denominator and
 * written over r */
template <int NL, bool EXACT>
__global__ void k_waves_thomas(int nc, WavesWork ww)
{
    const int i = (int)gtid();
    if (i >= nc) return;
    constexpr int n = NL - 1;
    double ep[n], rp[n];
#pragma unroll
    for (int j = 0; j < n; ++j) {
        const long long q = (long long)j * nc + i;
        const double dj = ww.d[q], rj = ww.r[q];
        if (j == 0) {
            if (EXACT) {
                ep[0] = ww.e[q] / dj;
                rp[0] = rj / dj;
            } else {
                const double inv = rcp_nr<2>(dj);
                ep[0] = ww.e[q] * inv;
                rp[0] = rj * inv;
            }
        } else {
            const double cm = ww.c[q - nc];
            const double den = dj - ep[j - 1] * cm;
            if (EXACT) {
                if (j < n - 1) ep[j] = ww.e[q] / den;
                rp[j] = (rj - rp[j - 1] * cm) / den;
            } else {
                const double inv = rcp_nr<2>(den);
                if (j < n - 1) ep[j] = ww.e[q] * inv;
                rp[j] = (rj - rp[j - 1] * cm) * inv;
            }
        }
    }
    /* damping: divide by 1 + dt * coefficient (mixed path: multiply by the
     * tabulated reciprocal) */
    auto damp = [&](double x, long long q) { return EXACT ? x / ww.dden[q] : x * ww.damp_inv[q]; };
    double x = rp[n - 1];
    ww.r[(long long)(n - 1) * nc + i] = damp(x, (long long)(n - 1) * nc + i);
#pragma unroll
    for (int j = n - 2; j >= 0; --j) {
        x = rp[j] - ep[j] * x;
        ww.r[(long long)j * nc + i] = damp(x, (long long)j * nc + i);
    }
}

/* generic layer count (nl - 1 <= CAP): the sweep in local memory, FP64
 * divisions on both paths */
template <int CAP, bool EXACT>
__global__ void k_waves_thomas_any(int nc, int nl, WavesWork ww)
{
    const int i = (int)gtid();
    if (i >= nc) return;
    const int n = nl - 1;
    double ep[CAP], rp[CAP];
    for (int j = 0; j < n; ++j) {
        const long long q = (long long)j * nc + i;
        const double dj = ww.d[q], rj = ww.r[q];
        if (j == 0) {
            ep[0] = ww.e[q] / dj;
            rp[0] = rj / dj;
        } else {
            const double cm = ww.c[q - nc];
            const double den = dj - ep[j - 1] * cm;
            if (j < n - 1) ep[j] = ww.e[q] / den;
            rp[j] = (rj - rp[j - 1] * cm) / den;
        }
    }
    auto damp = [&](double x, long long q) { return EXACT ? x / ww.dden[q] : x * ww.damp_inv[q]; };
    double x = rp[n - 1];
    ww.r[(long long)(n - 1) * nc + i] = damp(x, (long long)(n - 1) * nc + i);
    for (int j = n - 2; j >= 0; --j) {
        x = rp[j] - ep[j] * x;
        ww.r[(long long)j * nc + i] = damp(x, (long long)j * nc + i);
    }
}

template <bool EXACT>
__global__ void k_waves_apply(VGrid vg, StepParams p, DState so, DState sn, WavesWork ww, Shadow sh)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long ns = (long long)nl * nc, b = gtid();
    if (b >= ns) return;
    const int j = (int)(b / nc);
    const long long gp = p.n_cond * ns;
    const double dt = p.dt;
    const double *sol = ww.r;
    auto rho_new = [&](int jj, long long bb) {
        const double ve = EXACT ? vg.volume[bb] : 0.0;
        const double iv = EXACT ? 0.0 : ww.inv_vol[bb];
        double num;
        if (jj == 0) num = sol[bb];
        else if (jj == nl - 1) num = -sol[bb - nc];
        else num = -sol[bb - nc] + sol[bb];
        return EXACT ? ww.rho_expl[bb] + dt * (num) / ve : ww.rho_expl[bb] + dt * num * iv;
    };
    const double r_new = rho_new(j, b);
    double num;
    if (j == 0) num = ww.th_int[b] * sol[b];
    else if (j == nl - 1) num = -ww.th_int[b - nc] * sol[b - nc];
    else num = -ww.th_int[b - nc] * sol[b - nc] + ww.th_int[b] * sol[b];
    const double rt_new = EXACT ? ww.rt_expl[b] + dt * num / vg.volume[b] : ww.rt_expl[b] + dt * num * ww.inv_vol[b];
    const double tp_new = (EXACT ? rt_new / r_new : rt_new * rcp_nr<1>(r_new)) - vg.theta_v_bg[b];
    const double ep_new = so.exner_pert[b] + vg.volume[b] * ww.gam[b] * (rt_new - so.rhotheta_v[b]);
    sn.rho[gp + b] = r_new;
    sn.rhotheta_v[b] = rt_new;
    sn.theta_v_pert[b] = tp_new;
    sn.exner_pert[b] = ep_new;
    if (sh.rho) {
        sh.rho[gp + b] = to_float(r_new);
        sh.rhotheta_v[b] = to_float(rt_new);
        sh.theta_v_pert[b] = to_float(tp_new);
        sh.exner_pert[b] = to_float(ep_new);
    }
    if (j < nl - 1) {
        const long long wi = b + nc;
        const double r_below = rho_new(j + 1, b + nc);
        const double dint = 0.5 * (r_new + r_below);
        double wn;
        if (EXACT)
            wn = (2.0 * sol[b] / vg.area_v[wi] - dint * so.w[wi]) / ww.rho_io[b];
        else /* rho_io holds 1 / rho at the interface on the mixed path */
            wn = (2.0 * sol[b] * ww.inv_area_v[wi] - dint * so.w[wi]) * ww.rho_io[b];
        sn.w[wi] = wn;
        if (sh.w) sh.w[wi] = to_float(wn);
    }
}

/* ------------------------------------------------------------- tracers */
struct TracerWork {
    const double *cp_ice, *cp_water; /* c_p of ice / liquid water at the cell temperature [L][Nc] */
    const double *inv_vol;           /* mixed path */
};

__device__ __forceinline__ double sink_velocity(const StepParams &p, int k, bool &has)
{
    const int cond = p.n_cond;
    has = true;
    if (k < cond / 4) return p.snow_velocity;
    if (k < cond / 2) return p.rain_velocity;
    if (k < cond) return p.cloud_velocity;
    has = false;
    return 0.0;
}

/* vertical advection + sedimentation of constituent k in one column
 * (column_solvers.c:398-635); thread = (k-slot, column).  NL > 0: the layer
 * count is a compile-time constant and the sweep stays in registers; NL = 0:
 * the layer count is vg.nl (at most CAP) and the sweep lives in local memory */
template <int NL, int CAP, bool EXACT>
__global__ void k_tracers_solve(VGrid vg, StepParams p, DState so, DState sn, DState st, TracerWork tw, float *sh_rho)
{
    const int nc = vg.nc;
    const int nl = NL > 0 ? NL : vg.nl;
    const long long ns = (long long)nl * nc;
    const long long q = gtid();
    const int n_tr = p.n_const - 1;
    if (q >= (long long)n_tr * nc) return;
    const int slot = (int)(q / nc), i = (int)(q - (long long)slot * nc);
    const int k = slot < p.n_cond ? slot : slot + 1; /* skip the main gas */
    bool has_sink;
    const double vsink = sink_velocity(p, k, has_sink);
    const double dt = p.dt, iw = 0.5, ew = 1.0 - iw, half_dt = 0.5 * dt;
    const double *ro = so.rho + k * ns;
    const double *tr = st.rho + k * ns;
    const long long bot = i + ns - nc;
    const double a_sfc = vg.area_v[(long long)nl * nc + i];
    double ep[NL > 0 ? NL : CAP], rp[NL > 0 ? NL : CAP];
    double fi_prev = 0.0, fr_prev = 0.0, c_prev = 0.0;
#pragma unroll
    for (int j = 0; j < nl; ++j) {
        const long long b = i + (long long)j * nc;
        const double vol = EXACT ? vg.volume[b] : 0.0;
        /* mixed path: implicit and explicit weights are both 1/2, so every
         * flux term of row j carries the factor g = dt / (2 V_j) */
        const double g = EXACT ? 0.0 : half_dt * tw.inv_vol[b];
        /* flux at interface j (below layer j) */
        double fi = 0.0, fr = 0.0, cj = 0.0, ej = 0.0;
        if (j < nl - 1) {
            const long long wi = b + nc;
            double a_ = so.w[wi], b_ = sn.w[wi];
            if (has_sink) {
                a_ -= vsink;
                b_ -= vsink;
            }
            const double ar = vg.area_v[wi];
            a_ = ar * a_;
            b_ = ar * b_;
            const double dio = nonneg<EXACT>(b_) ? ro[b + nc] : ro[b];
            fi = a_;
            fr = dio * b_;
            if (EXACT) {
                if (fi >= 0.0) ej = -iw * dt / vol * fi;
                else cj = iw * dt / vg.volume[b + nc] * fi;
            } else if (nonneg<EXACT>(fi)) {
                ej = -g * fi;
            }
        }
        if (!EXACT) /* sub-diagonal of row j - 1, formed with row j's factor */
            c_prev = nonneg<EXACT>(fi_prev) ? 0.0 : g * fi_prev;
        double dj, rj = ro[b] + dt * tr[b];
        if (EXACT) {
            if (j == 0) {
                dj = fi >= 0.0 ? 1.0 : 1.0 - iw * dt / vol * fi;
                rj += ew * dt * fr / vol;
            } else if (j == nl - 1) {
                dj = fi_prev >= 0.0 ? 1.0 + iw * dt / vol * fi_prev : 1.0;
                if (has_sink) dj += iw * vsink * dt * a_sfc / vol;
                rj += -ew * dt * fr_prev / vol;
                if (has_sink) rj += -ew * vsink * dt * ro[bot] * a_sfc / vol;
            } else {
                dj = 1.0;
                if (fi_prev >= 0.0) dj += iw * dt / vol * fi_prev;
                if (fi < 0.0) dj -= iw * dt / vol * fi;
                rj += ew * dt * (-fr_prev + fr) / vol;
            }
        } else {
            if (j == 0) {
                dj = nonneg<EXACT>(fi) ? 1.0 : 1.0 - g * fi;
                rj += g * fr;
            } else if (j == nl - 1) {
                dj = nonneg<EXACT>(fi_prev) ? 1.0 + g * fi_prev : 1.0;
                rj -= g * fr_prev;
                if (has_sink) {
                    const double gs = g * vsink * a_sfc;
                    dj += gs;
                    rj -= gs * ro[bot];
                }
            } else {
                dj = 1.0 + (nonneg<EXACT>(fi_prev) ? g * fi_prev : 0.0) - (nonneg<EXACT>(fi) ? 0.0 : g * fi);
                rj += g * (fr - fr_prev);
            }
        }
        /* forward elimination */
        if (j == 0) {
            if (EXACT) {
                ep[0] = ej / dj;
                rp[0] = rj / dj;
            } else {
                const double inv = rcp_nr<2>(dj);
                ep[0] = ej * inv;
                rp[0] = rj * inv;
            }
        } else {
            const double den = dj - ep[j - 1] * c_prev;
            if (EXACT) {
                if (j < nl - 1) ep[j] = ej / den;
                rp[j] = (rj - rp[j - 1] * c_prev) / den;
            } else {
                const double inv = rcp_nr<2>(den);
                if (j < nl - 1) ep[j] = ej * inv;
                rp[j] = (rj - rp[j - 1] * c_prev) * inv;
            }
        }
        fi_prev = fi;
        fr_prev = fr;
        if (EXACT) c_prev = cj;
    }
    double *rn = sn.rho + k * ns;
    float *rs = sh_rho ? sh_rho + k * ns : nullptr;
    double x = rp[nl - 1];
    {
        const double v = EXACT ? (x < 0.0 ? 0.0 : x) : (nonneg<false>(x) ? x : 0.0);
        rn[(long long)(nl - 1) * nc + i] = v;
        if (rs) rs[(long long)(nl - 1) * nc + i] = to_float(v);
    }
#pragma unroll
    for (int j = nl - 2; j >= 0; --j) {
        x = rp[j] - ep[j] * x;
        const double v = EXACT ? (x < 0.0 ? 0.0 : x) : (nonneg<false>(x) ? x : 0.0);
        rn[(long long)j * nc + i] = v;
        if (rs) rs[(long long)j * nc + i] = to_float(v);
    }
}

/* sedimentation heating (rk 0 only): thread = column, walking down the
 * layers so that each interface's enthalpy fluxes are formed once and reused
 * by the layer below; the condensates' contributions are added in the
 * reference's constituent order, with the same operations as the per-layer
 * form (column_solvers.c:455-462, 551-623) */
constexpr int SEDHEAT_MAX_COND = 4;
template <bool EXACT>
__global__ void k_tracers_sedheat(VGrid vg, StepParams p, DState so, DState sn, const double *temperature,
                                  TracerWork tw, double *sed_heat)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long ns = (long long)nl * nc;
    const long long ii = gtid();
    if (ii >= nc) return;
    const int i = (int)ii, n_cond = p.n_cond;
    const long long bot = i + ns - nc;
    const double a_sfc = vg.area_v[(long long)nl * nc + i];
    /* enthalpy flux of constituent k at interface jj (below layer jj) */
    auto fe = [&](int k, int jj, double vsink, bool has) {
        const long long bb = i + (long long)jj * nc, wi = bb + nc;
        double b_ = sn.w[wi];
        if (has) b_ -= vsink;
        b_ = vg.area_v[wi] * b_;
        const long long up = nonneg<EXACT>(b_) ? bb + nc : bb;
        const double dio = so.rho[k * ns + up], tio = temperature[up];
        const double fr = dio * b_;
        const double cp = (k % 2 == 0) ? tw.cp_ice[up] : tw.cp_water[up];
        return cp * tio * fr;
    };
    double h_up[SEDHEAT_MAX_COND];
    for (int j = 0; j < nl; ++j) {
        const long long b = i + (long long)j * nc;
        const double vol = vg.volume[b];
        const double ivol = EXACT ? 0.0 : tw.inv_vol[b];
        auto per_vol = [&](double x) { return EXACT ? x / vol : x * ivol; };
        double sh = 0.0;
#pragma unroll
        for (int k = 0; k < SEDHEAT_MAX_COND; ++k) {
            if (k >= n_cond) break;
            bool has;
            const double vs = sink_velocity(p, k, has);
            if (j == 0) {
                h_up[k] = fe(k, j, vs, has);
                sh += per_vol(h_up[k]);
            } else if (j == nl - 1) {
                sh += per_vol(-h_up[k]);
                const double tb = temperature[bot];
                const double cp = (k % 2 == 0) ? tw.cp_ice[bot] : tw.cp_water[bot];
                sh += per_vol(-vs * tb * cp * so.rho[k * ns + bot] * a_sfc);
            } else {
                const double h = fe(k, j, vs, has);
                sh += per_vol(-h_up[k] + h);
                h_up[k] = h;
            }
        }
        sed_heat[b] = sh;
    }
}


/* ------------------------------------------------ deep columns: warp PCR
 * One warp solves one tridiagonal system a_j x_{j-1} + b_j x_j + c_j x_{j+1}
 * = d_j (j < n, a_0 = c_{n-1} = 0) by parallel cyclic reduction (Hockney and
 * Jesshope): in step s = 1, 2, 4, ... every row eliminates its couplings at
 * distance s with the rows j - s and j + s, so after ceil(log2 n) steps row j
 * reads x_j = d_j.  Rows are kept normalised to b_j = 1, one reciprocal per
 * row and step (an FP64 division on the FP64 path, a Newton-refined
 * reciprocal on the mixed path).
 * A block holds PCR_WARPS systems of neighbouring columns.  Its threads load
 * and store the rows cooperatively, PCR_WARPS consecutive columns of one row
 * per group of threads, so that the [layer][cell] accesses fill whole
 * sectors; warp w then reduces system w in shared memory, double-buffered
 * (one __syncwarp per step), lane l handling rows l, l + 32, ....
 * Shared memory: 6 n doubles per system, 48 KB per block at n = 256. */
constexpr int PCR_MAX_ROWS = 256;
constexpr int PCR_WARPS = 4; /* systems (warps) per block */
static_assert(PCR_WARPS * 6 * PCR_MAX_ROWS * sizeof(double) <= 48 * 1024, "PCR block exceeds 48 KB");

template <bool EXACT>
__device__ __forceinline__ double pcr_inv(double b)
{
    return EXACT ? 1.0 / b : rcp_nr<2>(b);
}

/* reduction steps for n rows: ceil(log2 n) */
__device__ __forceinline__ int pcr_steps(int n)
{
    int s = 0;
    for (int st = 1; st < n; st <<= 1) ++s;
    return s;
}

/* s: [a | c | d] of n normalised rows followed by the second buffer; the
 * solution ends in d of buffer pcr_steps(n) & 1 */
template <bool EXACT>
__device__ __forceinline__ void pcr_warp(double *s, int n)
{
    const int lane = threadIdx.x & 31;
    double *cur = s, *nxt = s + 3 * n;
    for (int st = 1; st < n; st <<= 1) {
        const double *a = cur, *c = cur + n, *d = cur + 2 * n;
        for (int j = lane; j < n; j += 32) {
            double an = 0.0, cn = 0.0, bn = 1.0, dn = d[j];
            if (j - st >= 0) {
                const double k = a[j];
                an = -k * a[j - st];
                bn -= k * c[j - st];
                dn -= k * d[j - st];
            }
            if (j + st < n) {
                const double k = c[j];
                cn = -k * c[j + st];
                bn -= k * a[j + st];
                dn -= k * d[j + st];
            }
            const double r = pcr_inv<EXACT>(bn);
            nxt[j] = an * r;
            nxt[n + j] = cn * r;
            nxt[2 * n + j] = dn * r;
        }
        __syncwarp();
        double *tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
}

__device__ __forceinline__ const double *pcr_solution(const double *s, int n)
{
    return s + (pcr_steps(n) & 1) * 3 * n + 2 * n;
}

/* sound waves: the rows of k_waves_rows(_mixed) of PCR_WARPS neighbouring
 * columns, solution divided by the damping denominator into r */
template <bool EXACT>
__global__ void __launch_bounds__(32 * PCR_WARPS) k_waves_pcr(int nc, int nl, WavesWork ww)
{
    extern __shared__ double smem[];
    const int n = nl - 1;
    const int t = threadIdx.x, warp = t >> 5, sys = t % PCR_WARPS, row0 = t / PCR_WARPS;
    const int i0 = blockIdx.x * PCR_WARPS, i = i0 + sys;
    double *s = smem + (size_t)sys * 6 * n;
    if (i < nc)
        for (int j = row0; j < n; j += 32) {
            const long long q = (long long)j * nc + i;
            const double r = pcr_inv<EXACT>(ww.d[q]);
            s[j] = j > 0 ? ww.c[q - nc] * r : 0.0;
            s[n + j] = j < n - 1 ? ww.e[q] * r : 0.0;
            s[2 * n + j] = ww.r[q] * r;
        }
    __syncthreads();
    if (i0 + warp < nc) pcr_warp<EXACT>(smem + (size_t)warp * 6 * n, n);
    __syncthreads();
    if (i < nc) {
        const double *x = pcr_solution(s, n);
        for (int j = row0; j < n; j += 32) {
            const long long q = (long long)j * nc + i;
            ww.r[q] = EXACT ? x[j] / ww.dden[q] : x[j] * ww.damp_inv[q];
        }
    }
}

/* tracers: vertical advection and sedimentation of constituent k (the rows of
 * k_tracers_solve, column_solvers.c:398-635) for PCR_WARPS consecutive
 * (k-slot, column) systems, clipped at 0; the sedimentation heat comes from
 * k_tracers_sedheat.  The interface fluxes are staged in the second buffer,
 * which the reduction overwrites only after the rows are built. */
template <bool EXACT>
__global__ void __launch_bounds__(32 * PCR_WARPS)
    k_tracers_pcr(VGrid vg, StepParams p, DState so, DState sn, DState st, TracerWork tw, float *sh_rho)
{
    extern __shared__ double smem[];
    const int nc = vg.nc, nl = vg.nl, n = nl;
    const int t = threadIdx.x, warp = t >> 5, sys = t % PCR_WARPS, row0 = t / PCR_WARPS;
    const int n_tr = p.n_const - 1;
    const long long nsys = (long long)n_tr * nc, q0 = (long long)blockIdx.x * PCR_WARPS, q = q0 + sys;
    const bool valid = q < nsys;
    const int slot = valid ? (int)(q / nc) : 0, i = valid ? (int)(q - (long long)slot * nc) : 0;
    const int k = slot < p.n_cond ? slot : slot + 1;
    const long long ns = (long long)nl * nc;
    bool has_sink;
    const double vsink = sink_velocity(p, k, has_sink);
    const double dt = p.dt, iw = 0.5, ew = 1.0 - iw, half_dt = 0.5 * dt;
    const double *ro = so.rho + k * ns, *tr = st.rho + k * ns;
    double *s = smem + (size_t)sys * 6 * n;
    double *fi = s + 3 * n, *fr = s + 4 * n;
    /* interface fluxes (below layer j) */
    if (valid)
        for (int j = row0; j < n; j += 32) {
            double a_ = 0.0, f_ = 0.0;
            if (j < nl - 1) {
                const long long b = i + (long long)j * nc, wi = b + nc;
                double wo = so.w[wi], wn = sn.w[wi];
                if (has_sink) {
                    wo -= vsink;
                    wn -= vsink;
                }
                const double ar = vg.area_v[wi];
                a_ = ar * wo;
                const double b_ = ar * wn;
                f_ = (nonneg<EXACT>(b_) ? ro[b + nc] : ro[b]) * b_;
            }
            fi[j] = a_;
            fr[j] = f_;
        }
    __syncthreads();
    if (valid) {
        const long long bot = i + ns - nc;
        const double a_sfc = vg.area_v[(long long)nl * nc + i];
        for (int j = row0; j < n; j += 32) {
            const long long b = i + (long long)j * nc;
            const double fij = j < nl - 1 ? fi[j] : 0.0, fip = j > 0 ? fi[j - 1] : 0.0;
            const double frj = j < nl - 1 ? fr[j] : 0.0, frp = j > 0 ? fr[j - 1] : 0.0;
            double aj = 0.0, cj = 0.0, dj, rj = ro[b] + dt * tr[b];
            if (EXACT) {
                const double vol = vg.volume[b];
                if (j > 0 && fip < 0.0) aj = iw * dt / vol * fip;
                if (j < nl - 1 && fij >= 0.0) cj = -iw * dt / vol * fij;
                if (j == 0) {
                    dj = fij >= 0.0 ? 1.0 : 1.0 - iw * dt / vol * fij;
                    rj += ew * dt * frj / vol;
                } else if (j == nl - 1) {
                    dj = fip >= 0.0 ? 1.0 + iw * dt / vol * fip : 1.0;
                    if (has_sink) dj += iw * vsink * dt * a_sfc / vol;
                    rj += -ew * dt * frp / vol;
                    if (has_sink) rj += -ew * vsink * dt * ro[bot] * a_sfc / vol;
                } else {
                    dj = 1.0;
                    if (fip >= 0.0) dj += iw * dt / vol * fip;
                    if (fij < 0.0) dj -= iw * dt / vol * fij;
                    rj += ew * dt * (-frp + frj) / vol;
                }
            } else {
                const double g = half_dt * tw.inv_vol[b];
                if (j > 0 && !nonneg<false>(fip)) aj = g * fip;
                if (j < nl - 1 && nonneg<false>(fij)) cj = -g * fij;
                if (j == 0) {
                    dj = nonneg<false>(fij) ? 1.0 : 1.0 - g * fij;
                    rj += g * frj;
                } else if (j == nl - 1) {
                    dj = nonneg<false>(fip) ? 1.0 + g * fip : 1.0;
                    rj -= g * frp;
                    if (has_sink) {
                        const double gs = g * vsink * a_sfc;
                        dj += gs;
                        rj -= gs * ro[bot];
                    }
                } else {
                    dj = 1.0 + (nonneg<false>(fip) ? g * fip : 0.0) - (nonneg<false>(fij) ? 0.0 : g * fij);
                    rj += g * (frj - frp);
                }
            }
            const double r = pcr_inv<EXACT>(dj);
            s[j] = aj * r;
            s[n + j] = cj * r;
            s[2 * n + j] = rj * r;
        }
    }
    __syncthreads();
    if (q0 + warp < nsys) pcr_warp<EXACT>(smem + (size_t)warp * 6 * n, n);
    __syncthreads();
    if (valid) {
        const double *x = pcr_solution(s, n);
        double *rn = sn.rho + k * ns;
        float *rs = sh_rho ? sh_rho + k * ns : nullptr;
        for (int j = row0; j < n; j += 32) {
            const double v = EXACT ? (x[j] < 0.0 ? 0.0 : x[j]) : (nonneg<false>(x[j]) ? x[j] : 0.0);
            rn[i + (long long)j * nc] = v;
            if (rs) rs[i + (long long)j * nc] = to_float(v);
        }
    }
}

}  // namespace
}  // namespace game
