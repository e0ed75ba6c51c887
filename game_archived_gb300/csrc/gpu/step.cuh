/*
 * One RKHEVI step on device mirrors (src/time_stepping/manage_rkhevi.c:20-100),
 * templated on the horizontal precision R.  Included by step_f64.cu (R =
 * double, compiled without FMA contraction, every operation in the
 * reference's order) and step_mixed.cu (R = float).
 */
#pragma once

#include "context.h"
#include "diff.h"
#include "kernels.cuh"
#include "solvers.cuh"
#include "solvers_df.cuh"

namespace game {

inline unsigned nblocks(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

template <typename R>
HGrid<R> &hgrid(Context *c);
template <>
inline HGrid<double> &hgrid<double>(Context *c) { return c->hg64; }
template <>
inline HGrid<float> &hgrid<float>(Context *c) { return c->hg32; }
template <typename R>
Work<R> &work(Context *c);
template <>
inline Work<double> &work<double>(Context *c) { return c->w64; }
template <>
inline Work<float> &work<float>(Context *c) { return c->w32; }

/* the layer count the register-resident column sweeps are compiled for
 * (NO_OF_LAYERS of every GAME configuration) */
constexpr int NL_FIXED = 26;
/* capacities of the local-memory sweeps for other layer counts */
constexpr int SWEEP_SMALL = 64, SWEEP_LARGE = 256;
/* the mixed path solves a batch of fewer systems than this with the warp
 * cyclic reduction: one thread per system leaves most of the 152 SMs idle
 * there, while above it the per-thread sweeps, with log2(n) times less FP64
 * work, are faster (measured on GB300 from 642 to 40962 columns and 64 to 256
 * layers).  The FP64 path keeps the reference's elimination order at any
 * depth. */
constexpr long long PCR_SYSTEMS_BELOW = 6144;

enum { COLUMN_REGISTERS, COLUMN_LOCAL, COLUMN_PCR };
/* the solver for a batch of n_systems columns (game_gpu_set_column_solver:
 * 0 chosen by layer count, batch size and precision, 1 per-thread Thomas
 * sweeps, 2 warp cyclic reduction) */
inline int column_mode(const Context *c, bool exact, long long n_systems)
{
    if (c->column_solver == 2) return COLUMN_PCR;
    if (c->nl == NL_FIXED) return COLUMN_REGISTERS;
    if (c->column_solver == 0 && !exact && n_systems < PCR_SYSTEMS_BELOW) return COLUMN_PCR;
    return COLUMN_LOCAL;
}

inline WavesWork waves_work(Context *c)
{
    WavesWork w;
    const long long ns = c->ns, ni = (long long)(c->nl - 1) * c->nc;
    double *a = c->wv_layer, *b = c->wv_rows;
    w.rho_expl = a; w.rt_expl = a + ns; w.alpha = a + 2 * ns; w.beta = a + 3 * ns; w.gam = a + 4 * ns;
    w.tp_expl = a + 5 * ns; w.ep_expl = a + 6 * ns; w.thl = a + 7 * ns;
    w.c = b; w.d = b + ni; w.e = b + 2 * ni; w.r = b + 3 * ni; w.th_int = b + 4 * ni; w.rho_io = b + 5 * ni;
    w.dden = b + 6 * ni;
    w.inv_vol = c->inv_vol;
    w.inv_area_v = c->inv_area_v;
    w.damp_dc = c->damp_dc;
    w.damp_inv = c->damp_inv;
    w.geo = c->wv_geo;
    return w;
}

/* read view of state_new in precision R and the FP32 shadow (mixed path) */
template <typename R>
struct Views {
    SView<R> sv;
    Shadow sh;
};
template <typename R>
Views<R> views(Context *c, StateMirror *sn);
template <>
inline Views<double> views<double>(Context *c, StateMirror *sn)
{
    Views<double> v{};
    v.sv = {sn->ds.rho, sn->ds.rhotheta_v, sn->ds.theta_v_pert, sn->ds.exner_pert, sn->ds.w, sn->ds.u};
    v.sh = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    return v;
}
template <>
inline Views<float> views<float>(Context *c, StateMirror *sn)
{
    Views<float> v{};
    const long long ns = c->ns;
    float *b = c->shadow;
    v.sh.rho = b;
    v.sh.rhotheta_v = b + (long long)c->n_const * ns;
    v.sh.theta_v_pert = v.sh.rhotheta_v + ns;
    v.sh.exner_pert = v.sh.theta_v_pert + ns;
    v.sh.w = v.sh.exner_pert + ns;
    v.sh.u = v.sh.w + (long long)(c->nl + 1) * c->nc;
    v.sv = {v.sh.rho, v.sh.rhotheta_v, v.sh.theta_v_pert, v.sh.exner_pert, v.sh.w, v.sh.u};
    return v;
}

template <typename R, bool ADV, bool PG>
static void launch_momentum_v(Context *c, const StepParams &p, const Views<R> &v, StateMirror *st, double new_w,
                              double old_w)
{
    HGrid<R> &g = hgrid<R>(c);
    Work<R> &w = work<R>(c);
    ProfScope ps(c, "k_momentum_v");
    const double *fric_w = p.irr ? c->dbuf->fric : nullptr;
    const float4 *pc = sizeof(R) == sizeof(float) && PG ? c->pg_cell : nullptr;
    k_momentum_v<R, ADV, PG><<<nblocks((long long)(c->nl + 1) * c->nc, 256), 256, 0, c->stream>>>(
        g, p, v.sv, st->ds.w, w.P_v, w.pvt_v, w.v2g_v, w.flux_h, w.zh, w.v2, new_w, old_w, fric_w, pc);
    c->kernel_launches++;
}

template <typename R, bool ADV, bool PG>
static void launch_momentum_h(Context *c, const StepParams &p, const Views<R> &v, StateMirror *so, StateMirror *sn,
                              StateMirror *st, double new_w, double old_w)
{
    HGrid<R> &g = hgrid<R>(c);
    Work<R> &w = work<R>(c);
    ProfScope ps(c, "k_momentum_h");
    const double *fric_u = p.irr ? c->dbuf->fric + (long long)(c->nl + 1) * c->nc : nullptr;
    const float4 *pc = sizeof(R) == sizeof(float) && PG ? c->pg_cell : nullptr;
    k_momentum_h<R, ADV, PG><<<nblocks((long long)c->nl * c->ne, 256), 256, 0, c->stream>>>(
        g, p, v.sv, sn->ds.u, v.sh.u, so->ds.u, st->ds.u, w.P_h, w.pg_old_h, w.pvt_h, w.v2g_h, w.flux_h, w.flux_v,
        w.zh, w.zv, w.v2, new_w, old_w, fric_u, pc);
    c->kernel_launches++;
}

template <typename R, bool ADV, bool PG>
static void launch_momentum(Context *c, const StepParams &p, const Views<R> &v, StateMirror *so, StateMirror *sn,
                            StateMirror *st, double new_w, double old_w)
{
    launch_momentum_v<R, ADV, PG>(c, p, v, st, new_w, old_w);
    launch_momentum_h<R, ADV, PG>(c, p, v, so, sn, st, new_w, old_w);
}

/* implicit vertical sound waves (column_solvers.c:19-383) */
template <bool EXACT>
void launch_waves(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st, int rk,
                  const Shadow &sh)
{
    const long long ns = c->ns;
    WavesWork ww = waves_work(c);
    if constexpr (!EXACT) {
        if (p.dfloat && column_mode(c, EXACT, c->nc) == COLUMN_REGISTERS) {
            {
                ProfScope ps(c, "k_waves_layer");
                k_waves_layer_df<<<nblocks(ns, 256), 256, 0, c->stream>>>(c->vg, p, so->ds, sn->ds, st->ds, ww,
                                                                          c->dfg, rk);
            }
            {
                ProfScope ps(c, "k_waves_rows");
                k_waves_rows_df<<<nblocks((long long)(c->nl - 1) * c->nc, 256), 256, 0, c->stream>>>(
                    c->vg, p, so->ds, st->ds, ww, c->dfg);
            }
            {
                ProfScope ps(c, "k_waves_thomas");
                /* two lanes per column (twisted elimination) */
                k_waves_thomas_df<NL_FIXED><<<nblocks(2 * (long long)c->nc, WAVES_BLOCK), WAVES_BLOCK, 0,
                                              c->stream>>>(c->nc, ww, c->dfg);
            }
            {
                ProfScope ps(c, "k_waves_apply");
                k_waves_apply_df<<<nblocks(ns, 256), 256, 0, c->stream>>>(c->vg, p, so->ds, sn->ds, ww, c->dfg, sh);
            }
            c->kernel_launches += 4;
            return;
        }
    }
    {
        ProfScope ps(c, "k_waves_layer");
        k_waves_layer<EXACT><<<nblocks(ns, 256), 256, 0, c->stream>>>(c->vg, p, so->ds, sn->ds, st->ds, ww, rk);
    }
    {
        ProfScope ps(c, "k_waves_rows");
        const unsigned nb = nblocks((long long)(c->nl - 1) * c->nc, 256);
        if (EXACT)
            k_waves_rows<<<nb, 256, 0, c->stream>>>(c->vg, p, so->ds, st->ds, ww);
        else
            k_waves_rows_mixed<<<nb, 256, 0, c->stream>>>(c->vg, p, so->ds, st->ds, ww);
    }
    {
        ProfScope ps(c, "k_waves_thomas");
        const int mode = column_mode(c, EXACT, c->nc);
        if (mode == COLUMN_REGISTERS)
            k_waves_thomas<NL_FIXED, EXACT><<<nblocks(c->nc, 64), 64, 0, c->stream>>>(c->nc, ww);
        else if (mode == COLUMN_LOCAL && c->nl - 1 <= SWEEP_SMALL)
            k_waves_thomas_any<SWEEP_SMALL, EXACT><<<nblocks(c->nc, 64), 64, 0, c->stream>>>(c->nc, c->nl, ww);
        else if (mode == COLUMN_LOCAL)
            k_waves_thomas_any<SWEEP_LARGE, EXACT><<<nblocks(c->nc, 64), 64, 0, c->stream>>>(c->nc, c->nl, ww);
        else
            k_waves_pcr<EXACT><<<nblocks(c->nc, PCR_WARPS), 32 * PCR_WARPS,
                                 (size_t)PCR_WARPS * 6 * (c->nl - 1) * sizeof(double), c->stream>>>(c->nc, c->nl, ww);
    }
    {
        ProfScope ps(c, "k_waves_apply");
        k_waves_apply<EXACT><<<nblocks(ns, 256), 256, 0, c->stream>>>(c->vg, p, so->ds, sn->ds, ww, sh);
    }
    c->kernel_launches += 4;
}

/* implicit vertical advection and sedimentation of the non-main constituents
 * (column_solvers.c:385-639); temperature and its c_p tables as of the start
 * of the step, sedimentation heat written at rk 0 */
template <bool EXACT>
void launch_tracers(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st, int rk,
                    const Shadow &sh, const double *temperature, const double *cp_ice, const double *cp_water,
                    double *sed_heat, cudaStream_t strm = nullptr)
{
    if (c->n_const <= 1) return;
    if (!strm) strm = c->stream;
    const long long ns = c->ns;
    TracerWork tw{cp_ice, cp_water, c->inv_vol};
    const long long nsys = (long long)(c->n_const - 1) * c->nc;
    const int mode = column_mode(c, EXACT, nsys);
    if (rk == 0) {
        ProfScope ps(c, "k_tracers_sedheat");
        if (!EXACT && p.dfloat)
            k_tracers_sedheat_df<<<nblocks(ns, 128), 128, 0, strm>>>(c->vg, p, so->ds, sn->ds, temperature, tw,
                                                                     c->dfg, sed_heat);
        else
            k_tracers_sedheat<EXACT><<<nblocks(c->nc, 128), 128, 0, strm>>>(c->vg, p, so->ds, sn->ds, temperature,
                                                                                tw, sed_heat);
        c->kernel_launches++;
    }
    ProfScope ps(c, "k_tracers_solve");
    if constexpr (!EXACT) {
        if (p.dfloat && mode == COLUMN_REGISTERS) {
            k_tracers_solve_df<NL_FIXED><<<nblocks(nsys, TRACER_BLOCK), TRACER_BLOCK, 0, strm>>>(
                c->vg, p, so->ds, sn->ds, st->ds, c->dfg, sh.rho);
            c->kernel_launches++;
            return;
        }
    }
    if (mode == COLUMN_REGISTERS)
        k_tracers_solve<NL_FIXED, NL_FIXED, EXACT><<<nblocks(nsys, 64), 64, 0, strm>>>(c->vg, p, so->ds, sn->ds,
                                                                                        st->ds, tw, sh.rho);
    else if (mode == COLUMN_LOCAL && c->nl <= SWEEP_SMALL)
        k_tracers_solve<0, SWEEP_SMALL, EXACT><<<nblocks(nsys, 64), 64, 0, strm>>>(c->vg, p, so->ds, sn->ds, st->ds,
                                                                                    tw, sh.rho);
    else if (mode == COLUMN_LOCAL)
        k_tracers_solve<0, SWEEP_LARGE, EXACT><<<nblocks(nsys, 64), 64, 0, strm>>>(c->vg, p, so->ds, sn->ds, st->ds,
                                                                                    tw, sh.rho);
    else
        k_tracers_pcr<EXACT><<<nblocks(nsys, PCR_WARPS), 32 * PCR_WARPS,
                               (size_t)PCR_WARPS * 6 * c->nl * sizeof(double), strm>>>(c->vg, p, so->ds, sn->ds,
                                                                                       st->ds, tw, sh.rho);
    c->kernel_launches++;
}

/* the kernel sequence of one step on c->stream (and c->stream2 for the tracer branch) */
template <typename R>
void launch_step(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st)
{
    constexpr bool EXACT = sizeof(R) == sizeof(double);
    HGrid<R> &g = hgrid<R>(c);
    Work<R> &w = work<R>(c);
    const int bs = 256;
    const long long ns = c->ns;
    const Views<R> v = views<R>(c, sn);
    R *theta = EXACT ? (R *)c->theta : (R *)c->theta32;
    const R *cpi = EXACT ? (const R *)c->cp_ice : (const R *)c->cp32_ice;
    const R *cpw = EXACT ? (const R *)c->cp_water : (const R *)c->cp32_water;
    if (!EXACT) {
        ProfScope ps(c, "k_make_shadow");
        const long long n_rho = (long long)c->n_const * ns, nw = (long long)(c->nl + 1) * c->nc,
                        nu = (long long)c->nl * c->ne;
        const long long pairs = (std::max(std::max(n_rho, nw), nu) + 1) / 2;
        k_make_shadow<<<nblocks(pairs, bs), bs, 0, c->stream>>>(n_rho, ns, nw, nu, sn->ds, v.sh);
        c->kernel_launches++;
    }
    if constexpr (!EXACT) {
        /* the first substage's pressure-gradient factors per cell (the
         * diffusion branch, which runs before it, changes none of its inputs) */
        ProfScope ps(c, "k_pg_cells");
        k_pg_cells<<<nblocks(ns, bs), bs, 0, c->stream>>>(c->hg32, p, v.sv, c->pg_cell);
        c->kernel_launches++;
    }
    {
        ProfScope ps(c, "k_cell_prepare");
        if (EXACT)
            k_cell_prepare<<<nblocks(ns, bs), bs, 0, c->stream>>>(c->vg, p, so->ds, c->temperature, c->pt_rates,
                                                                  c->pt_heat, c->cp_ice, c->cp_water);
        else
            k_cell_prepare_f32<<<nblocks(ns, bs), bs, 0, c->stream>>>(c->vg, p, so->ds, c->temperature, c->pt_rates,
                                                                      c->pt_heat, c->cp_ice, c->cp_water, c->cp32_ice,
                                                                      c->cp32_water);
    }
    c->kernel_launches++;
    const R *rho_gas = v.sv.rho + (long long)c->n_cond * ns;
    /* Substage 0's tracer solve (FP64-bound) and substage 1's advection and
     * horizontal momentum (FP32, memory-bound) read and write disjoint
     * fields: the tracer solve runs on a second stream (a parallel branch of
     * the captured graph) and joins before substage 1's vertical momentum,
     * whose condensate term reads the tracer densities.  Serial while
     * profiling. */
    const bool fork = c->n_const > 1 && !c->profiling;
    bool join_pending = false;
    for (int rk = 0; rk < 2; ++rk) {
        const bool adv = rk == 1 || p.first_step;
        const double new_w = rk == 1 ? 0.5 : 1.0, old_w = 1.0 - new_w;
        if (adv) {
            {
                ProfScope ps(c, "k_tri_vort");
                k_tri_vort<R><<<nblocks((long long)c->nl * c->nt, bs), bs, 0, c->stream>>>(g, v.sv.u, w.tri_vort);
            }
            {
                ProfScope ps(c, "k_edge_vort");
                k_edge_vort<R><<<nblocks((long long)(c->nl + 1) * c->ne, bs), bs, 0, c->stream>>>(
                    g, v.sv.u, v.sv.w, rho_gas, w.tri_vort, w.zh, w.zv, w.flux_h);
            }
            {
                ProfScope ps(c, "k_cell_kinetic");
                k_cell_kinetic<R><<<nblocks(ns, bs), bs, 0, c->stream>>>(g, v.sv.u, v.sv.w, rho_gas, w.v2, w.flux_v);
            }
            c->kernel_launches += 3;
        }
        /* diffusion branch: momentum part on state_new before the wind update */
        if (rk == 0 && p.diff) launch_diffusion_momentum(c, p, v.sv);
        if (rk == 0 && adv) {
            launch_momentum<R, true, true>(c, p, v, so, sn, st, new_w, old_w);
        } else if (rk == 0) {
            launch_momentum<R, false, true>(c, p, v, so, sn, st, new_w, old_w);
        } else {
            launch_momentum_h<R, true, false>(c, p, v, so, sn, st, new_w, old_w);
            if (join_pending) {
                cudaEventRecord(c->ev_join, c->stream2);
                cudaStreamWaitEvent(c->stream, c->ev_join, 0);
                join_pending = false;
            }
            launch_momentum_v<R, true, false>(c, p, v, st, new_w, old_w);
        }
        /* diffusion branch: temperature and mass diffusion */
        if (rk == 0 && (p.diff & DIFF_RAD_HS)) launch_held_suarez_radiation(c, so->ds);
        if (rk == 0 && p.diff) launch_diffusion_scalar(c, p, v.sv);
        {
            ProfScope ps(c, "k_theta");
            k_theta<R><<<nblocks(ns, bs), bs, 0, c->stream>>>(c->nl, c->nc, c->n_cond, v.sv, theta);
        }
        {
            ProfScope ps(c, "k_scalar_tend");
            if (p.irr) {
                const DiffBufs &b = *c->dbuf;
                k_scalar_tend2<R, true><<<nblocks(ns, 128), 128, 0, c->stream>>>(
                    g, p, v.sv, st->ds, theta, cpi, cpw, c->pt_rates, c->pt_heat, c->sed_heat, c->inv_vol, rk,
                    IrrTerms{b.hdiss, b.tdh, b.rad, b.mdt});
            } else {
                k_scalar_tend2<R, false><<<nblocks(ns, 128), 128, 0, c->stream>>>(
                    g, p, v.sv, st->ds, theta, cpi, cpw, c->pt_rates, c->pt_heat, c->sed_heat, c->inv_vol, rk,
                    IrrTerms{});
            }
        }
        c->kernel_launches += 2;
        /* the tendency is final from here on: a host-in/host-out call copies
         * it out while the solvers run */
        if (rk == 1) {
            /* inside a graph capture: an external event node, which streams
             * outside the graph can wait on */
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            cudaStreamIsCapturing(c->stream, &cs);
            if (cs == cudaStreamCaptureStatusActive)
                cudaEventRecordWithFlags(c->ev_tend, c->stream, cudaEventRecordExternal);
            else
                cudaEventRecord(c->ev_tend, c->stream);
        }
        launch_waves<EXACT>(c, p, so, sn, st, rk, v.sh);
        if (rk == 0 && fork) {
            cudaEventRecord(c->ev_fork, c->stream);
            cudaStreamWaitEvent(c->stream2, c->ev_fork, 0);
            launch_tracers<EXACT>(c, p, so, sn, st, rk, v.sh, c->temperature, c->cp_ice, c->cp_water, c->sed_heat,
                                  c->stream2);
            join_pending = true;
        } else {
            launch_tracers<EXACT>(c, p, so, sn, st, rk, v.sh, c->temperature, c->cp_ice, c->cp_water, c->sed_heat);
        }
    }
}

}  // namespace game
