/*
 * Adjoint and tangent-linear models of the RKHEVI step, dry and moist builds,
 * over multi-step windows (compiled with --fmad=false, like the FP64 step).
 *
 * Window forward: the initial State and, unless the window starts with the
 * model's first step, the lagged fields of the previous step (pressure
 * gradient nl + l, vorticity flux, kinetic-energy gradient) are
 * checkpointed; every step is run with the differentiable kernels of
 * adj_fwd.cuh and adj_moist.cuh (the same operations as the fused FP64 step)
 * and its end state and lagged fields are checkpointed.  The moist build
 * adds the per-step prelude (temperature, phase transitions), the moist
 * scalar tendencies, the tracer solve and, as a fourth lagged field, the
 * sedimentation heat (the first substage's scalar tendencies read the
 * previous step's).
 * Window backward (reverse mode): from the last step to the first, the step
 * is recomputed from its checkpoint with every intermediate field kept (both
 * RK stage states, the momentum, scalar and solver work of both substages),
 * then the hand-written adjoint kernels of adj_bwd.cuh run in reverse order.
 * The bars of the lagged fields carry over to the earlier step.
 * Window tangent-linear: the same forward kernels instantiated with dual
 * numbers, each step linearised about its checkpoint (values from the
 * checkpoint, derivatives carried from the previous step), so that it is the
 * transpose of the backward sweep whatever computed the checkpoints.
 *
 * Mixed precision: when the library's precision is the mixed one, the
 * forward of record is the fused mixed step itself (FP32 horizontal
 * operators, double-float eliminations, FP64 state), run on private state
 * blocks; its step-start states and lagged fields (widened to FP64) are the
 * checkpoints, so the window's end state is the mixed run's.  The
 * tangent-linear and adjoint models are the FP64 ones, linearised about
 * that trajectory: the backward sweep recomputes each step in FP64 from its
 * mixed checkpoint.  The library's own lagged step fields (those a
 * device-resident run carries from one manage_rkhevi call to the next) are
 * saved before the mixed window and restored after it.
 *
 * The control is the State at the window start: rho, rho theta_v, Pi', w and
 * u.  theta_v' is rediagnosed from rho theta_v / rho at every step start
 * (linear_combine_two_states, src/coordinator.c:305), so its input bar is 0.
 */
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "adj.h"
#include "adj_moist.cuh"
#include "adj_ops.h"
#include "diag.h"
#include "ops.h"

namespace game {
namespace {

/* --------------------------------------------------------------- utilities */
template <class T>
__global__ void ku_copy(long long n, const T *src, T *dst)
{
    const long long i = gtid();
    if (i < n) dst[i] = src[i];
}
template <class T>
__global__ void ku_neg(long long n, const T *src, T *dst)
{
    const long long i = gtid();
    if (i < n) dst[i] = -src[i];
}
__global__ void ku_axpy(long long n, double a, const double *x, double *y)
{
    const long long i = gtid();
    if (i < n) y[i] += a * x[i];
}
__global__ void ku_to_dual(long long n, const double *v, const double *d, Dual *out)
{
    const long long i = gtid();
    if (i < n) out[i] = Dual{v[i], d ? d[i] : 0.0};
}
/* out = (v, derivative of dsrc): a tangent-linear value re-seeded from a
 * checkpoint */
__global__ void ku_reseed(long long n, const double *v, const Dual *dsrc, Dual *out)
{
    const long long i = gtid();
    if (i < n) out[i] = Dual{v[i], dsrc[i].d};
}
__global__ void ku_dual_part(long long n, const Dual *in, double *d)
{
    const long long i = gtid();
    if (i < n) d[i] = in[i].d;
}
__global__ void ku_dden(long long n, double dt, const double *dc, double *dden)
{
    const long long i = gtid();
    if (i < n) dden[i] = 1.0 + dt * dc[i];
}
/* flux_v levels 0 and L (never written by the step) */
template <class T>
__global__ void ku_fv_bounds(int nc, int nl, const double *src, T *fv)
{
    const int i = (int)gtid();
    if (i >= nc) return;
    fv[i] = tconst<T>(src[i]);
    fv[(long long)nl * nc + i] = tconst<T>(src[(long long)nl * nc + i]);
}

inline unsigned nbk(long long n, int bs = 256) { return (unsigned)((n + bs - 1) / bs); }

/* ------------------------------------------------------------- step buffers */
template <class T>
struct StepBufs {
    T *so = nullptr, *sn1 = nullptr, *sn2 = nullptr;
    T *pre = nullptr; /* moist: temperature, rates, heating, c_p of ice and water [PRE_OUT][L][Nc] */
    T *sed = nullptr; /* moist: this step's sedimentation heat [L][Nc] */
    T *P = nullptr, *pgo = nullptr;
    T *tri[2] = {}, *zh[2] = {}, *zv[2] = {}, *fh[2] = {}, *fv[2] = {}, *v2[2] = {};
    T *pvt[2] = {}, *v2g[2] = {}, *tend[2] = {};
    T *theta[2] = {}, *str[2] = {}, *strt[2] = {};
    T *wl[2] = {}, *wr[2] = {};
};

}  // namespace

struct AdjState {
    std::vector<void *> owned;
    long long ns = 0, nw = 0, nu = 0, nv = 0, nblk = 0, ntri = 0, nzh = 0, nwi = 0, nrho = 0;
    int n_const = 1, n_cond = 0; /* constituents; the main gas's index */
    StepBufs<double> B;          /* forward tape of one step */
    StepBufs<double> Z;          /* bars of one step */
    StepBufs<Dual> D;            /* tangent-linear run */
    double *rn_b = nullptr, *rtn_b = nullptr;
    double *dden = nullptr, *fv_bounds = nullptr; /* (L+1) Nc */
    /* checkpoints of every ck_every-th step start and of the window's end,
     * (state block + 3 Vt [+ S]) each, and one scratch slot for the start
     * of a step recomputed from the nearest checkpoint before it */
    double *ck = nullptr, *ck_tmp = nullptr;
    long long ck_cap = -1;       /* slots allocated */
    int ck_every = 1;
    double *obj_w = nullptr, *obj_p = nullptr, *obj_out = nullptr; /* objective work */
    /* lagged fields between tangent-linear steps: P, pvt, v2g and (moist) the
     * sedimentation heat */
    Dual *tl_aux[4] = {};
    double *bar_state = nullptr; /* bar of the current step-end state */
    double *bar_aux[4] = {}, *bar_aux_prev[4] = {}; /* bars of the lagged fields */
    /* mixed forward of record: the fused step's three state blocks, and the
     * library's lagged step fields saved around the window (FP32: P, the
     * old pressure gradient, vorticity flux, KE gradient, mass flux;
     * FP64: temperature, phase-transition rates and heating, sedimentation
     * heat) */
    StateMirror mso{}, msn{}, mst{};
    float *save32 = nullptr;
    double *save64 = nullptr;
    /* the window of the last forward run */
    int n_steps = 0, first = 0, have = 0;
    AParams ap{};
    StepParams p{};
};

namespace {

template <class T>
T *aalloc(AdjState *a, long long n)
{
    void *p = nullptr;
    if (cudaMalloc(&p, (size_t)(n > 0 ? n : 1) * sizeof(T)) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, (size_t)(n > 0 ? n : 1) * sizeof(T));
    a->owned.push_back(p);
    return (T *)p;
}

template <class T>
bool alloc_step(AdjState *a, StepBufs<T> &S)
{
    bool ok = true;
    auto A = [&](T *&p, long long n) {
        p = aalloc<T>(a, n);
        ok = ok && p;
    };
    A(S.so, a->nblk);
    A(S.sn1, a->nblk);
    A(S.sn2, a->nblk);
    if (a->n_const > 1) {
        A(S.pre, PRE_OUT * a->ns);
        A(S.sed, a->ns);
    }
    A(S.P, a->nv);
    A(S.pgo, a->nv);
    for (int r = 0; r < 2; ++r) {
        A(S.tri[r], a->ntri);
        A(S.zh[r], a->nzh);
        A(S.zv[r], a->nu);
        A(S.fh[r], a->nu);
        A(S.fv[r], a->nw);
        A(S.v2[r], a->ns);
        A(S.pvt[r], a->nv);
        A(S.v2g[r], a->nv);
        A(S.tend[r], a->nv);
        A(S.theta[r], a->ns);
        A(S.str[r], a->nrho);
        A(S.strt[r], a->ns);
        A(S.wl[r], WL_N * a->ns);
        A(S.wr[r], WR_N * a->nwi);
    }
    return ok;
}

void adj_release_fn(Context *c)
{
    if (!c->adj) return;
    for (void *p : c->adj->owned) cudaFree(p);
    delete c->adj;
    c->adj = nullptr;
}

int ensure_adj(Context *c)
{
    if (c->adj) return 0;
    if (c->n_const != 1 && c->n_const != 6)
        return fail("adjoint: the adjoint and tangent-linear models cover the dry build and the moist build of six "
                    "constituents");
    if (c->nl > MAX_L) return fail("adjoint: more layers than the column solvers support");
    AdjState *a = new AdjState();
    c->adj = a;
    c->adj_release = adj_release_fn;
    a->ns = c->ns;
    a->n_const = c->n_const;
    a->n_cond = c->n_cond;
    a->nrho = (long long)c->n_const * c->ns;
    a->nw = (long long)(c->nl + 1) * c->nc;
    a->nu = (long long)c->nl * c->ne;
    a->nv = a->nw + a->nu;
    a->nblk = a->nrho + 3 * a->ns + a->nv;
    a->ntri = (long long)c->nl * c->nt;
    a->nzh = (long long)(c->nl + 1) * c->ne;
    a->nwi = (long long)(c->nl - 1) * c->nc;
    bool ok = alloc_step(a, a->B) && alloc_step(a, a->Z) && alloc_step(a, a->D);
    ok = ok && (a->rn_b = aalloc<double>(a, a->ns)) && (a->rtn_b = aalloc<double>(a, a->ns));
    ok = ok && (a->dden = aalloc<double>(a, a->nwi)) && (a->fv_bounds = aalloc<double>(a, a->nw));
    ok = ok && (a->obj_w = aalloc<double>(a, c->nc)) && (a->obj_p = aalloc<double>(a, c->nc))
         && (a->obj_out = aalloc<double>(a, 1)) && (a->bar_state = aalloc<double>(a, a->nblk));
    for (int k = 0; k < 4; ++k)
        ok = ok && (a->tl_aux[k] = aalloc<Dual>(a, a->nv)) && (a->bar_aux[k] = aalloc<double>(a, a->nv))
             && (a->bar_aux_prev[k] = aalloc<double>(a, a->nv));
    if (!ok) {
        adj_release_fn(c);
        return fail("adjoint: device allocation failed");
    }
    return 0;
}

template <class T>
AState<T> view(const AdjState *a, T *blk)
{
    AState<T> s;
    s.rho_all = blk;
    s.rho = blk + (long long)a->n_cond * a->ns;
    s.rt = blk + a->nrho;
    s.tp = s.rt + a->ns;
    s.ep = s.tp + a->ns;
    s.w = s.ep + a->ns;
    s.u = s.w + a->nw;
    return s;
}

/* the same block as the DState of the operator adjoints */
DState dview(const AdjState *a, double *blk)
{
    const AState<double> v = view(a, blk);
    return DState{v.rho_all, v.rt, v.tp, v.ep, v.w, v.u};
}

bool moist_of(const AdjState *a) { return a->n_const > 1; }

/* checkpoint: the state block and the lagged fields P, pvt, v2g (Vt each)
 * and, moist, the sedimentation heat (S) */
long long ck_stride(const AdjState *a) { return a->nblk + 3 * a->nv + (moist_of(a) ? a->ns : 0); }

/* ----------------------------------------------------------- step forward */
/* the substage rk of a step: sn its input state (so at rk 0), out its
 * output (sn1, sn2); sed_prev the previous step's sedimentation heat */
template <class T>
void substage_fwd(Context *c, AdjState *a, StepBufs<T> &B, int rk, bool first, const T *sed_prev)
{
    const HGrid<double> &g = c->hg64;
    const VGrid &vg = c->vg;
    const AParams ap = a->ap;
    cudaStream_t st = c->stream;
    const long long ns = a->ns, nv = a->nv;
    const bool moist = moist_of(a);
    AState<T> so = view(a, B.so), sn = view(a, rk ? B.sn1 : B.so), out = view(a, rk ? B.sn2 : B.sn1);
    const bool adv = rk == 1 || first;
    const double new_w = rk ? 0.5 : 1.0, old_w = 1.0 - new_w;
    if (adv) {
        fa_tri<T><<<nbk(a->ntri), 256, 0, st>>>(g, sn.u, B.tri[rk]);
        fa_edge<T><<<nbk(a->nzh), 256, 0, st>>>(g, sn.u, sn.w, sn.rho, B.tri[rk], B.zh[rk], B.zv[rk], B.fh[rk]);
        fa_kin<T><<<nbk(ns), 256, 0, st>>>(g, sn.u, sn.w, sn.rho, B.v2[rk], B.fv[rk]);
    }
    fa_mom_v<T><<<nbk(a->nw), 256, 0, st>>>(g, ap, adv, new_w, old_w, B.P, B.fh[rk], B.zh[rk], B.v2[rk], B.pvt[rk],
                                            B.v2g[rk], B.tend[0], B.tend[rk], moist ? sn.rho_all : nullptr);
    fa_mom_h<T><<<nbk(a->nu), 256, 0, st>>>(g, ap, adv, new_w, old_w, B.P, B.pgo, B.fh[rk], B.fv[rk], B.zh[rk],
                                            B.zv[rk], B.v2[rk], B.pvt[rk], B.v2g[rk], B.tend[0], B.tend[rk], so.u,
                                            out.u);
    fa_theta<T><<<nbk(ns), 256, 0, st>>>(ns, sn.rho, sn.rt, B.theta[rk]);
    if (moist)
        fa_scalar_moist<T><<<nbk(ns, 128), 128, 0, st>>>(g, ap, rk, sn.rho_all, B.theta[rk], out.u, sn.ep, B.pre,
                                                          rk == 0 ? sed_prev : B.sed, B.str[0], B.str[rk],
                                                          B.strt[rk]);
    else
        fa_scalar<T><<<nbk(ns, 128), 128, 0, st>>>(g, sn.rho, B.theta[rk], out.u, B.str[rk], B.strt[rk]);
    const T *str_gas = B.str[rk] + (long long)a->n_cond * ns;
    fa_waves_layer<T><<<nbk(ns), 256, 0, st>>>(vg, ap, rk, so, sn, str_gas, B.strt[rk], B.wl[rk]);
    fa_waves_rows<T><<<nbk(a->nwi), 256, 0, st>>>(vg, ap, so, B.tend[rk], B.wl[rk], B.wr[rk]);
    fa_waves_thomas<T><<<nbk(c->nc, 64), 64, 0, st>>>(c->nc, c->nl, a->dden, B.wr[rk]);
    fa_waves_apply<T><<<nbk(ns), 256, 0, st>>>(vg, ap, so, B.wl[rk], B.wr[rk], out);
    c->kernel_launches += adv ? 11 : 8;
    if (moist) {
        if (rk == 0) {
            fa_sedheat<T><<<nbk(c->nc, 128), 128, 0, st>>>(vg, a->p, so, out.w, B.pre, B.sed);
            c->kernel_launches++;
        }
        fa_tracer_solve<T><<<nbk((long long)(a->n_const - 1) * c->nc, 64), 64, 0, st>>>(vg, a->p, so, out.w,
                                                                                        B.str[rk], out);
        c->kernel_launches++;
    }
    (void)nv;
}

template <class T>
void step_fwd(Context *c, AdjState *a, StepBufs<T> &B, const T *P_prev, const T *pvt_prev, const T *v2g_prev,
              const T *sed_prev, bool first)
{
    const HGrid<double> &g = c->hg64;
    const AParams ap = a->ap;
    cudaStream_t st = c->stream;
    const long long nv = a->nv;
    AState<T> so = view(a, B.so);
    if (moist_of(a)) {
        fa_prelude<T><<<nbk(a->ns), 256, 0, st>>>(c->vg, ap, so, B.pre);
        c->kernel_launches++;
    }
    fa_pgrad<T><<<nbk(nv), 256, 0, st>>>(g, ap, so, B.P);
    ku_neg<T><<<nbk(nv), 256, 0, st>>>(nv, first ? B.P : P_prev, B.pgo);
    if (!first) {
        ku_copy<T><<<nbk(nv), 256, 0, st>>>(nv, pvt_prev, B.pvt[0]);
        ku_copy<T><<<nbk(nv), 256, 0, st>>>(nv, v2g_prev, B.v2g[0]);
    }
    c->kernel_launches += first ? 2 : 4;
    substage_fwd<T>(c, a, B, 0, first, sed_prev);
    substage_fwd<T>(c, a, B, 1, first, sed_prev);
}

/* ---------------------------------------------------------- step backward
 * s2b: bar of the step's end state (modified); P_next_b, pvt_next_b,
 * v2g_next_b, sed_next_b: bars of this step's lagged outputs from the next
 * step (may be null); writes sob (bar of the step-start state, theta_v' bar
 * consumed) and, for a step that is not the model's first, the bars of the
 * lagged inputs; sed_prev_b (moist) receives the bar of the previous step's
 * sedimentation heat in every case. */
void step_bwd(Context *c, AdjState *a, bool first, double *s2b, const double *P_next_b, const double *pvt_next_b,
              const double *v2g_next_b, const double *sed_next_b, const double *sed_prev, double *sob,
              double *P_prev_b, double *pvt_prev_b, double *v2g_prev_b, double *sed_prev_b)
{
    const HGrid<double> &g = c->hg64;
    const VGrid &vg = c->vg;
    const AParams ap = a->ap;
    cudaStream_t st = c->stream;
    const long long ns = a->ns, nv = a->nv, nw = a->nw;
    const bool moist = moist_of(a);
    StepBufs<double> &B = a->B, &Z = a->Z;
    /* zero all bars of the step */
    auto zero = [&](double *p, long long n) { cudaMemsetAsync(p, 0, (size_t)n * sizeof(double), st); };
    zero(sob, a->nblk);
    zero(Z.sn1, a->nblk);
    zero(Z.P, nv);
    zero(Z.pgo, nv);
    if (moist) {
        zero(Z.pre, PRE_OUT * ns);
        zero(Z.sed, ns);
        zero(sed_prev_b, ns);
    }
    for (int r = 0; r < 2; ++r) {
        zero(Z.tri[r], a->ntri);
        zero(Z.zh[r], a->nzh);
        zero(Z.zv[r], a->nu);
        zero(Z.fh[r], a->nu);
        zero(Z.fv[r], a->nw);
        zero(Z.v2[r], ns);
        zero(Z.pvt[r], nv);
        zero(Z.v2g[r], nv);
        zero(Z.tend[r], nv);
        zero(Z.theta[r], ns);
        zero(Z.str[r], a->nrho);
        zero(Z.strt[r], ns);
        zero(Z.wl[r], WL_N * ns);
        zero(Z.wr[r], WR_N * a->nwi);
    }
    if (pvt_next_b) ku_copy<double><<<nbk(nv), 256, 0, st>>>(nv, pvt_next_b, Z.pvt[1]);
    if (v2g_next_b) ku_copy<double><<<nbk(nv), 256, 0, st>>>(nv, v2g_next_b, Z.v2g[1]);
    if (moist && sed_next_b) ku_copy<double><<<nbk(ns), 256, 0, st>>>(ns, sed_next_b, Z.sed);
    AState<double> so = view(a, B.so), s1 = view(a, B.sn1), s2 = view(a, B.sn2);
    AState<double> sob_v = view(a, sob), s1b = view(a, Z.sn1), s2b_v = view(a, s2b);
    for (int rk = 1; rk >= 0; --rk) {
        AState<double> out = rk ? s2 : s1, out_b = rk ? s2b_v : s1b;
        AState<double> sn = rk ? s1 : so, sn_b = rk ? s1b : sob_v;
        double *out_blk = rk ? B.sn2 : B.sn1, *out_b_blk = rk ? s2b : Z.sn1;
        /* tracer solve (and at rk 0 the sedimentation heat): the operator
         * adjoint of three_band_solver_gen_densities; the temperature's bar
         * goes to the prelude's output bar */
        if (moist) {
            StateMirror mso, msn, mst, mso_b, msn_b, mst_b;
            mso.dev = B.so;
            mso.ds = dview(a, B.so);
            msn.dev = out_blk;
            msn.ds = dview(a, out_blk);
            mst.ds = DState{B.str[rk], nullptr, nullptr, nullptr, nullptr, nullptr};
            mso_b.ds = dview(a, sob);
            msn_b.ds = dview(a, out_b_blk);
            mst_b.ds = DState{Z.str[rk], nullptr, nullptr, nullptr, nullptr, nullptr};
            if (adj_gen_densities(c, a->p, &mso, &msn, &mst, B.pre, rk, Z.sed, &mso_b, &msn_b, &mst_b, Z.pre))
                return;
        }
        ba_apply_layer<<<nbk(ns), 256, 0, st>>>(vg, so, B.wl[rk], out, out_b, a->rn_b, a->rtn_b, sob_v, Z.wl[rk]);
        ba_apply_w<<<nbk(a->nwi), 256, 0, st>>>(vg, so, B.wr[rk], out, out_b, a->rn_b, sob_v, Z.wr[rk]);
        ba_apply_rho<<<nbk(ns), 256, 0, st>>>(vg, ap, B.wr[rk], a->rn_b, a->rtn_b, Z.wl[rk], Z.wr[rk]);
        ba_thomas<<<nbk(c->nc, 64), 64, 0, st>>>(c->nc, c->nl, a->dden, B.wr[rk], Z.wr[rk]);
        ba_waves_rows<<<nbk(a->nwi), 256, 0, st>>>(vg, ap, so, B.wl[rk], B.wr[rk], Z.wr[rk], Z.wl[rk], sob_v,
                                                   Z.tend[rk]);
        const long long gas = (long long)a->n_cond * ns;
        ba_waves_layer<<<nbk(ns), 256, 0, st>>>(vg, ap, rk, so, sn, B.str[rk] + gas, B.strt[rk], B.wl[rk], Z.wl[rk],
                                                sob_v, sn_b, Z.str[rk] + gas, Z.strt[rk]);
        /* scalar tendencies: densities and theta_v of sn, the wind of out */
        if (moist)
            ba_scalar_moist<<<nbk(ns, 128), 128, 0, st>>>(g, ap, rk, sn.rho_all, B.theta[rk], out.u, sn.ep, B.pre,
                                                          rk == 0 ? sed_prev : B.sed, Z.str[rk], Z.strt[rk],
                                                          sn_b.rho_all, Z.theta[rk], out_b.u, sn_b.ep, Z.pre,
                                                          rk == 0 ? sed_prev_b : Z.sed, Z.str[0]);
        else
            ba_scalar<<<nbk(ns, 128), 128, 0, st>>>(g, sn.rho, B.theta[rk], out.u, Z.str[rk], Z.strt[rk], sn_b.rho,
                                                    Z.theta[rk], out_b.u);
        ba_theta<<<nbk(ns), 256, 0, st>>>(ns, sn.rho, sn.rt, Z.theta[rk], sn_b.rho, sn_b.rt);
        /* momentum */
        const int adv = rk == 1 || first;
        const double new_w = rk ? 0.5 : 1.0, old_w = 1.0 - new_w;
        double *tend_in_b = rk ? Z.tend[0] : nullptr;
        ba_mom_v<<<nbk(nw), 256, 0, st>>>(g, ap, adv, new_w, old_w, B.fh[rk], B.zh[rk], Z.tend[rk], tend_in_b, Z.P,
                                          Z.pvt[rk], Z.v2g[rk], Z.fh[rk], Z.zh[rk], Z.v2[rk],
                                          moist ? sn.rho_all : nullptr, moist ? sn_b.rho_all : nullptr);
        ba_mom_h<<<nbk(a->nu), 256, 0, st>>>(g, ap, adv, new_w, old_w, B.fh[rk], B.fv[rk], B.zh[rk], B.zv[rk],
                                             Z.tend[rk], out_b.u, sob_v.u, tend_in_b, Z.P, Z.pgo, Z.pvt[rk], Z.v2g[rk],
                                             Z.fh[rk], Z.fv[rk], Z.zh[rk], Z.zv[rk], Z.v2[rk]);
        if (adv) {
            ba_kin<<<nbk(ns), 256, 0, st>>>(g, sn.u, sn.w, sn.rho, Z.v2[rk], Z.fv[rk], sn_b.u, sn_b.w, sn_b.rho);
            ba_edge<<<nbk(a->nzh), 256, 0, st>>>(g, sn.u, sn.rho, B.zh[rk], B.zv[rk], Z.zh[rk], Z.zv[rk], Z.fh[rk],
                                                 sn_b.u, sn_b.w, sn_b.rho, Z.tri[rk]);
            ba_tri<<<nbk(a->ntri), 256, 0, st>>>(g, Z.tri[rk], sn_b.u);
        }
    }
    if (!first) {
        ku_copy<double><<<nbk(nv), 256, 0, st>>>(nv, Z.pvt[0], pvt_prev_b);
        ku_copy<double><<<nbk(nv), 256, 0, st>>>(nv, Z.v2g[0], v2g_prev_b);
    }
    /* pressure gradient: its use in the next step, then pg_old = -P or -P_prev */
    if (P_next_b) ku_axpy<<<nbk(nv), 256, 0, st>>>(nv, 1.0, P_next_b, Z.P);
    if (first)
        ku_axpy<<<nbk(nv), 256, 0, st>>>(nv, -1.0, Z.pgo, Z.P);
    else
        ku_neg<double><<<nbk(nv), 256, 0, st>>>(nv, Z.pgo, P_prev_b);
    ba_pgrad<<<nbk(nv), 256, 0, st>>>(g, ap, so, Z.P, sob_v.tp, sob_v.ep, moist ? sob_v.rho_all : nullptr);
    if (moist) ba_prelude<<<nbk(ns), 256, 0, st>>>(vg, ap, so, Z.pre, sob_v);
    ba_rediag<<<nbk(ns), 256, 0, st>>>(ns, so.rho, so.rt, sob_v.tp, sob_v.rho, sob_v.rt);
    c->kernel_launches += moist ? 46 : 40;
}

/* checkpoint slot of step start n: every ck_every-th step and the window's
 * end are stored; any other start lives in the scratch slot, valid after the
 * previous step was run (forward) or recomputed (backward) into it */
bool ck_stored(const AdjState *a, int n) { return n % a->ck_every == 0 || n == a->n_steps; }
double *ck_ptr(const AdjState *a, int n)
{
    const int K = a->ck_every;
    if (n % K == 0) return a->ck + (long long)(n / K) * ck_stride(a);
    if (n == a->n_steps) return a->ck + (long long)(a->n_steps / K + 1) * ck_stride(a);
    return a->ck_tmp;
}

/* the step-start state of step n from its checkpoint: theta_v' rediagnosed */
template <class T>
void load_start(Context *c, AdjState *a, int n, T *so_blk)
{
    const double *ck = ck_ptr(a, n);
    if constexpr (sizeof(T) == sizeof(double))
        ku_copy<double><<<nbk(a->nblk), 256, 0, c->stream>>>(a->nblk, ck, (double *)so_blk);
    fa_rediag<T><<<nbk(a->ns), 256, 0, c->stream>>>(c->vg, view(a, so_blk));
}

const double *ck_aux(const AdjState *a, int n, int which) /* 0 P, 1 pvt, 2 v2g, 3 sedimentation heat */
{
    return ck_ptr(a, n) + a->nblk + (long long)which * a->nv;
}

/* the FP64 step n of the window from its start's checkpoint, its end state
 * and lagged fields written to the checkpoint of start n + 1 */
void step_to_checkpoint(Context *c, AdjState *a, int n)
{
    cudaStream_t st = c->stream;
    const bool moist = moist_of(a);
    load_start<double>(c, a, n, a->B.so);
    step_fwd<double>(c, a, a->B, ck_aux(a, n, 0), ck_aux(a, n, 1), ck_aux(a, n, 2), moist ? ck_aux(a, n, 3) : nullptr,
                     a->first && n == 0);
    double *ckn = ck_ptr(a, n + 1);
    ku_copy<double><<<nbk(a->nblk), 256, 0, st>>>(a->nblk, a->B.sn2, ckn);
    ku_copy<double><<<nbk(a->nv), 256, 0, st>>>(a->nv, a->B.P, ckn + a->nblk);
    ku_copy<double><<<nbk(a->nv), 256, 0, st>>>(a->nv, a->B.pvt[1], ckn + a->nblk + a->nv);
    ku_copy<double><<<nbk(a->nv), 256, 0, st>>>(a->nv, a->B.v2g[1], ckn + a->nblk + 2 * a->nv);
    if (moist) ku_copy<double><<<nbk(a->ns), 256, 0, st>>>(a->ns, a->B.sed, ckn + a->nblk + 3 * a->nv);
}

/* --------------------------------------------------------------- objective */
/* surface pressure of a column (write_output.c:105-121, dry) and its partial
 * derivatives by rho, theta_v' and Pi' of the lowest layer */
__device__ __forceinline__ double sfc_p_dry(const VGrid &vg, const double *gm_v, const double *rho, const double *tp,
                                            const double *ep, int i, double *d_rho, double *d_tp, double *d_ep)
{
    const int nc = vg.nc, nl = vg.nl;
    const long long si = (long long)(nl - 1) * nc + i;
    const double lapse = 0.0065, rgas = R_D;
    const double th = vg.theta_v_bg[si] + tp[si], pe = vg.exner_bg[si] + ep[si];
    const double t_low = th * pe;
    const double p = rho[si] * rgas * t_low;
    const double t_sfc = t_low + lapse * (vg.z_scalar[si] - vg.z_v[(long long)nl * nc + i]);
    const double q = 1.0 - (t_sfc - t_low) / t_sfc;
    const double ex = gm_v[(long long)(nl - 1) * nc + i] / (rgas * lapse);
    const double fac = pow(q, ex);
    const double ps = p / fac;
    if (d_rho) {
        const double k = t_sfc - t_low;
        const double dfac_dt = ex * pow(q, ex - 1.0) * (k / (t_sfc * t_sfc));
        const double dps_dt = rho[si] * rgas / fac - ps / fac * dfac_dt;
        *d_rho = rgas * t_low / fac;
        *d_tp = dps_dt * pe;
        *d_ep = dps_dt * th;
    }
    return ps;
}

__global__ void k_obj(VGrid vg, const double *gm_v, AState<double> s, const double *w, double *p2, AState<double> sb,
                      int n_cond, int moist)
{
    const int i = (int)gtid();
    if (i >= vg.nc) return;
    if (moist) {
        /* moist air: the gas constant and temperature of the lowest layer
         * carry the vapour; derivatives by forward mode */
        const long long ns = (long long)vg.nl * vg.nc, si = (long long)(vg.nl - 1) * vg.nc + i;
        const double xv[SFC_IN] = {s.rho_all[n_cond * ns + si], s.rho_all[(n_cond + 1) * ns + si], s.tp[si], s.ep[si]};
        const double ps = sfc_pressure_moist<double>(vg, gm_v, i, xv);
        p2[i] = ps * ps;
        if (sb.rho) {
            const double pb = 2.0 * w[i] * ps;
            double g[SFC_IN];
            for (int m = 0; m < SFC_IN; ++m) {
                Dual x[SFC_IN];
                for (int k = 0; k < SFC_IN; ++k) x[k] = {xv[k], k == m ? 1.0 : 0.0};
                g[m] = sfc_pressure_moist<Dual>(vg, gm_v, i, x).d * pb;
            }
            sb.rho_all[n_cond * ns + si] += g[0];
            sb.rho_all[(n_cond + 1) * ns + si] += g[1];
            sb.tp[si] += g[2];
            sb.ep[si] += g[3];
        }
        return;
    }
    double dr, dt_, de;
    const double ps = sfc_p_dry(vg, gm_v, s.rho, s.tp, s.ep, i, sb.rho ? &dr : nullptr, &dt_, &de);
    p2[i] = ps * ps;
    if (sb.rho) {
        const long long si = (long long)(vg.nl - 1) * vg.nc + i;
        const double pb = 2.0 * w[i] * ps;
        sb.rho[si] += pb * dr;
        sb.tp[si] += pb * dt_;
        sb.ep[si] += pb * de;
    }
}

/* ---------------------------------------------------------- host helpers */
int set_params(Context *c, AdjState *a, const StepParams &p)
{
    a->p = p;
    a->ap.dt = p.dt;
    a->ap.impl_thermo_weight = p.impl_thermo_weight;
    a->ap.n_const = a->n_const;
    a->ap.n_cond = a->n_cond;
    if (launch_damping_table(c, p)) return -1;
    ku_dden<<<nbk(a->nwi), 256, 0, c->stream>>>(a->nwi, p.dt, c->damp_dc, a->dden);
    return 0;
}

/* ------------------------------------------------ mixed forward of record */
int ensure_mixed_fwd(Context *c, AdjState *a)
{
    if (a->mso.dev) return 0;
    for (StateMirror *m : {&a->mso, &a->msn, &a->mst}) {
        m->dev = aalloc<double>(a, c->state_len);
        if (!m->dev) return fail("adjoint window: device allocation of the mixed step's states failed");
        set_mirror_views(c, *m);
    }
    a->save32 = aalloc<float>(a, 5 * a->nu + 4 * a->nw);
    a->save64 = aalloc<double>(a, 8 * a->ns);
    if (!a->save32 || !a->save64) return fail("adjoint window: device allocation failed");
    return 0;
}

/* copies the library's lagged step fields into the save area (save) or back */
int swap_step_fields(Context *c, AdjState *a, bool save)
{
    const Work<float> &w = c->w32;
    const size_t nu = (size_t)a->nu * sizeof(float), nw = (size_t)a->nw * sizeof(float),
                 ns = (size_t)a->ns * sizeof(double);
    const std::pair<void *, size_t> f32[] = {{w.P_h, nu},  {w.pg_old_h, nu}, {w.pvt_h, nu},
                                             {w.v2g_h, nu}, {w.flux_h, nu},   {w.P_v, nw},
                                             {w.pvt_v, nw}, {w.v2g_v, nw},    {w.flux_v, nw}};
    const std::pair<void *, size_t> f64[] = {
        {c->temperature, ns}, {c->pt_rates, 5 * ns}, {c->pt_heat, ns}, {c->sed_heat, ns}};
    char *q = (char *)a->save32;
    for (const auto &f : f32) {
        CK(cudaMemcpyAsync(save ? (void *)q : f.first, save ? f.first : (void *)q, f.second,
                           cudaMemcpyDeviceToDevice, c->stream));
        q += f.second;
    }
    q = (char *)a->save64;
    for (const auto &f : f64) {
        CK(cudaMemcpyAsync(save ? (void *)q : f.first, save ? f.first : (void *)q, f.second,
                           cudaMemcpyDeviceToDevice, c->stream));
        q += f.second;
    }
    return 0;
}

/* the window's steps by the fused mixed step (checkpoint 0 written), started
 * as the reference's time loop starts them (below); each step's end state
 * and its lagged fields become the next checkpoint */
int window_forward_mixed(Context *c, AdjState *a, const StepParams &p, int n_steps, const double *aux_P,
                         const double *aux_pvt, const double *aux_v2g, const double *flux, const double *aux_sed)
{
    if (ensure_mixed_fwd(c, a)) return -1;
    cudaStream_t st = c->stream;
    const bool moist = moist_of(a);
    if (swap_step_fields(c, a, true)) return -1;
    if (a->first)
        aux_load_mixed(c, nullptr, nullptr, nullptr, flux);
    else
        aux_load_mixed(c, aux_P, aux_pvt, aux_v2g, flux);
    if (moist) ku_copy<double><<<nbk(a->ns), 256, 0, st>>>(a->ns, aux_sed, c->sed_heat);
    int rc = 0;
    for (int n = 0; n < n_steps && !rc; ++n) {
        const double *ck_in = ck_ptr(a, n);
        /* the step start as the reference's time loop leaves it:
         * linear_combine_two_states(state_new -> state_old) rediagnoses
         * theta_v' in state_old only, state_new keeps the previous step's
         * solution (the window's state_init for its first step); at the
         * model's first step state_new is state_old, rediagnosed as well
         * (src/coordinator.c:291-305) */
        load_start<double>(c, a, n, a->mso.dev);
        ku_copy<double><<<nbk(a->nblk), 256, 0, st>>>(a->nblk, n == 0 && a->first ? a->mso.dev : ck_in,
                                                      a->msn.dev);
        StepParams pn = p;
        pn.first_step = a->first && n == 0 ? 1 : 0;
        rc = launch_step_mixed(c, pn, &a->mso, &a->msn, &a->mst);
        if (rc) break;
        double *ckn = ck_ptr(a, n + 1);
        ku_copy<double><<<nbk(a->nblk), 256, 0, st>>>(a->nblk, a->msn.dev, ckn);
        aux_store_mixed(c, ckn + a->nblk, ckn + a->nblk + a->nv, ckn + a->nblk + 2 * a->nv);
        if (moist) ku_copy<double><<<nbk(a->ns), 256, 0, st>>>(a->ns, c->sed_heat, ckn + a->nblk + 3 * a->nv);
    }
    if (swap_step_fields(c, a, false)) return -1;
    return rc;
}

}  // namespace

/* ---------------------------------------------------------------- API */
int adj_window_forward(Context *c, StateMirror *init, const StepParams &p, int n_steps, const double *aux_P,
                       const double *aux_pvt, const double *aux_v2g, const double *fv_bounds, const double *aux_sed,
                       StateMirror *final_out)
{
    if (ensure_adj(c)) return -1;
    AdjState *a = c->adj;
    if (n_steps < 1) return fail("adjoint window: n_steps must be at least 1");
    a->ck_every = c->adj_ck_every;
    /* the multiples of ck_every, the end when it is not one, and (stride
     * above 1) the scratch slot after them */
    const int K = a->ck_every;
    const long long stored = n_steps / K + 1 + (n_steps % K != 0 ? 1 : 0);
    const long long slots = stored + (K > 1 ? 1 : 0);
    if (a->ck_cap < slots) {
        double *ck = aalloc<double>(a, slots * ck_stride(a));
        if (!ck) return fail("adjoint window: device allocation of the checkpoints failed");
        a->ck = ck;
        a->ck_cap = slots;
    }
    a->ck_tmp = K > 1 ? a->ck + stored * ck_stride(a) : nullptr;
    if (set_params(c, a, p)) return -1;
    a->n_steps = n_steps;
    a->first = p.first_step ? 1 : 0;
    cudaStream_t st = c->stream;
    ku_copy<double><<<nbk(a->nw), 256, 0, st>>>(a->nw, fv_bounds, a->fv_bounds);
    for (StepBufs<double> *S : {&a->B})
        for (int r = 0; r < 2; ++r) ku_fv_bounds<double><<<nbk(c->nc), 256, 0, st>>>(c->nc, c->nl, a->fv_bounds, S->fv[r]);
    /* checkpoint 0: the initial state and the lagged inputs */
    double *ck0 = a->ck;
    ku_copy<double><<<nbk(a->nblk), 256, 0, st>>>(a->nblk, init->dev, ck0);
    if (!a->first) {
        ku_copy<double><<<nbk(a->nv), 256, 0, st>>>(a->nv, aux_P, ck0 + a->nblk);
        ku_copy<double><<<nbk(a->nv), 256, 0, st>>>(a->nv, aux_pvt, ck0 + a->nblk + a->nv);
        ku_copy<double><<<nbk(a->nv), 256, 0, st>>>(a->nv, aux_v2g, ck0 + a->nblk + 2 * a->nv);
    }
    const bool moist = moist_of(a);
    if (moist) {
        /* the sedimentation heat the first substage of the window's first
         * step reads (the caller's, whatever the first-step flag) */
        if (!aux_sed) return fail("adjoint window: the moist build needs the sedimentation heat");
        ku_copy<double><<<nbk(a->ns), 256, 0, st>>>(a->ns, aux_sed, ck0 + a->nblk + 3 * a->nv);
    }
    a->have = 0;
    if (c->precision == PREC_MIXED) {
        if (window_forward_mixed(c, a, p, n_steps, aux_P, aux_pvt, aux_v2g, fv_bounds, aux_sed)) return -1;
    } else {
        for (int n = 0; n < n_steps; ++n) step_to_checkpoint(c, a, n);
    }
    a->have = 1;
    if (final_out) ku_copy<double><<<nbk(a->nblk), 256, 0, st>>>(a->nblk, ck_ptr(a, n_steps), final_out->dev);
    CK(cudaGetLastError());
    return 0;
}

int adj_window_tl(Context *c, const double *init_dot, double *final_dot)
{
    AdjState *a = c->adj;
    if (!a || !a->have) return fail("adjoint window: run the window forward first");
    cudaStream_t st = c->stream;
    StepBufs<Dual> &D = a->D;
    for (int r = 0; r < 2; ++r) ku_fv_bounds<Dual><<<nbk(c->nc), 256, 0, st>>>(c->nc, c->nl, a->fv_bounds, D.fv[r]);
    /* lagged inputs of the window's first step: values from checkpoint 0,
     * derivative 0 (they are not part of the control) */
    const bool moist = moist_of(a);
    for (int k = 0; k < 3; ++k)
        ku_to_dual<<<nbk(a->nv), 256, 0, st>>>(a->nv, ck_aux(a, 0, k), nullptr, a->tl_aux[k]);
    if (moist) ku_to_dual<<<nbk(a->ns), 256, 0, st>>>(a->ns, ck_aux(a, 0, 3), nullptr, a->tl_aux[3]);
    ku_to_dual<<<nbk(a->nblk), 256, 0, st>>>(a->nblk, a->ck, init_dot, D.so);
    /* every step is linearised about its checkpoint: values from checkpoint
     * n, derivatives carried from step n - 1 */
    for (int n = 0; n < a->n_steps; ++n) {
        /* a step whose start is not stored carries the values of the step
         * before it, as the backward sweep recomputes them */
        if (n > 0 && ck_stored(a, n))
            ku_reseed<<<nbk(a->nblk), 256, 0, st>>>(a->nblk, ck_ptr(a, n), D.sn2, D.so);
        else if (n > 0)
            ku_copy<Dual><<<nbk(a->nblk), 256, 0, st>>>(a->nblk, D.sn2, D.so);
        fa_rediag<Dual><<<nbk(a->ns), 256, 0, st>>>(c->vg, view(a, D.so));
        step_fwd<Dual>(c, a, D, a->tl_aux[0], a->tl_aux[1], a->tl_aux[2], moist ? a->tl_aux[3] : nullptr,
                       a->first && n == 0);
        if (ck_stored(a, n + 1)) {
            ku_reseed<<<nbk(a->nv), 256, 0, st>>>(a->nv, ck_aux(a, n + 1, 0), D.P, a->tl_aux[0]);
            ku_reseed<<<nbk(a->nv), 256, 0, st>>>(a->nv, ck_aux(a, n + 1, 1), D.pvt[1], a->tl_aux[1]);
            ku_reseed<<<nbk(a->nv), 256, 0, st>>>(a->nv, ck_aux(a, n + 1, 2), D.v2g[1], a->tl_aux[2]);
            if (moist) ku_reseed<<<nbk(a->ns), 256, 0, st>>>(a->ns, ck_aux(a, n + 1, 3), D.sed, a->tl_aux[3]);
        } else {
            ku_copy<Dual><<<nbk(a->nv), 256, 0, st>>>(a->nv, D.P, a->tl_aux[0]);
            ku_copy<Dual><<<nbk(a->nv), 256, 0, st>>>(a->nv, D.pvt[1], a->tl_aux[1]);
            ku_copy<Dual><<<nbk(a->nv), 256, 0, st>>>(a->nv, D.v2g[1], a->tl_aux[2]);
            if (moist) ku_copy<Dual><<<nbk(a->ns), 256, 0, st>>>(a->ns, D.sed, a->tl_aux[3]);
        }
    }
    ku_dual_part<<<nbk(a->nblk), 256, 0, st>>>(a->nblk, D.sn2, final_dot);
    CK(cudaGetLastError());
    return 0;
}

int adj_window_backward(Context *c, const double *final_bar, double *init_bar)
{
    AdjState *a = c->adj;
    if (!a || !a->have) return fail("adjoint window: run the window forward first");
    cudaStream_t st = c->stream;
    const long long nv = a->nv;
    ku_copy<double><<<nbk(a->nblk), 256, 0, st>>>(a->nblk, final_bar, a->bar_state);
    const bool moist = moist_of(a);
    bool have_next = false, have_next_sed = false;
    for (int n = a->n_steps - 1; n >= 0; --n) {
        const bool first = a->first && n == 0;
        /* a start that is not stored: recomputed in FP64 from the checkpoint
         * before it into the scratch slot */
        if (!ck_stored(a, n))
            for (int m = (n / a->ck_every) * a->ck_every; m < n; ++m) step_to_checkpoint(c, a, m);
        /* recompute the step from its checkpoint, keeping the tape */
        load_start<double>(c, a, n, a->B.so);
        const double *sed_prev = moist ? ck_aux(a, n, 3) : nullptr;
        step_fwd<double>(c, a, a->B, ck_aux(a, n, 0), ck_aux(a, n, 1), ck_aux(a, n, 2), sed_prev, first);
        step_bwd(c, a, first, a->bar_state, have_next ? a->bar_aux[0] : nullptr,
                 have_next ? a->bar_aux[1] : nullptr, have_next ? a->bar_aux[2] : nullptr,
                 have_next_sed ? a->bar_aux[3] : nullptr, sed_prev, init_bar, a->bar_aux_prev[0],
                 a->bar_aux_prev[1], a->bar_aux_prev[2], a->bar_aux_prev[3]);
        /* the step-start bar is the previous step's end-state bar */
        ku_copy<double><<<nbk(a->nblk), 256, 0, st>>>(a->nblk, init_bar, a->bar_state);
        for (int k = 0; k < 4; ++k) std::swap(a->bar_aux[k], a->bar_aux_prev[k]);
        have_next = !first;
        have_next_sed = moist;
    }
    (void)nv;
    CK(cudaGetLastError());
    return 0;
}

int adj_objective(Context *c, StateMirror *s, const double *w_dev, double *J, double *bar_blk)
{
    if (ensure_adj(c)) return -1;
    AdjState *a = c->adj;
    AState<double> sv = view(a, s->dev);
    AState<double> sb{};
    if (bar_blk) {
        cudaMemsetAsync(bar_blk, 0, (size_t)a->nblk * sizeof(double), c->stream);
        sb = view(a, bar_blk);
    }
    k_obj<<<nbk(c->nc, 128), 128, 0, c->stream>>>(c->vg, c->hg64.gravity_m_v, sv, w_dev, a->obj_p, sb, a->n_cond,
                                                  moist_of(a) ? 1 : 0);
    if (launch_integral(a->obj_p, 0, 1, c->nc, nullptr, w_dev, c->red_partials, c->red_counters, a->obj_out,
                        c->stream))
        return -1;
    c->kernel_launches += 2;
    CK(cudaMemcpyAsync(J, a->obj_out, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

double *adj_obj_weights(Context *c)
{
    if (ensure_adj(c)) return nullptr;
    return c->adj->obj_w;
}

void adj_add_into(Context *c, double *y, const double *x, long long n)
{
    ku_axpy<<<nbk(n), 256, 0, c->stream>>>(n, 1.0, x, y);
    c->kernel_launches++;
}

namespace {
/* pass-through bars of the column solver: wind_h and the TOA / surface w of
 * the output are the input's */
__global__ void ku_waves_passthrough(int nc, int nl, long long nu, double *out_b_w, double *out_b_u, double *in_b_w,
                                     double *in_b_u)
{
    const long long i = gtid();
    if (i < nc) {
        in_b_w[i] += out_b_w[i];
        out_b_w[i] = 0.0;
        in_b_w[(long long)nl * nc + i] += out_b_w[(long long)nl * nc + i];
        out_b_w[(long long)nl * nc + i] = 0.0;
    }
    if (i < nu) {
        in_b_u[i] += out_b_u[i];
        out_b_u[i] = 0.0;
    }
}
}  // namespace

int adj_waves_backward(Context *c, StateMirror *so_m, StateMirror *sn_m, StateMirror *st_m, const StepParams &p, int rk,
                       StateMirror *so_bar, StateMirror *sn_bar, StateMirror *st_bar)
{
    if (ensure_adj(c)) return -1;
    AdjState *a = c->adj;
    if (set_params(c, a, p)) return -1;
    cudaStream_t st = c->stream;
    const HGrid<double> &g = c->hg64;
    (void)g;
    const VGrid &vg = c->vg;
    const AParams ap = a->ap;
    const long long ns = a->ns;
    AState<double> so = view(a, so_m->dev), sn = view(a, sn_m->dev), out = view(a, a->B.sn2);
    double *wl = a->B.wl[0], *wr = a->B.wr[0], *wl_b = a->Z.wl[0], *wr_b = a->Z.wr[0];
    /* forward of the solver, keeping its work */
    fa_waves_layer<double><<<nbk(ns), 256, 0, st>>>(vg, ap, rk, so, sn, st_m->ds.rho, st_m->ds.rhotheta_v, wl);
    fa_waves_rows<double><<<nbk(a->nwi), 256, 0, st>>>(vg, ap, so, st_m->ds.w, wl, wr);
    fa_waves_thomas<double><<<nbk(c->nc, 64), 64, 0, st>>>(c->nc, c->nl, a->dden, wr);
    fa_waves_apply<double><<<nbk(ns), 256, 0, st>>>(vg, ap, so, wl, wr, out);
    /* bars: the output bar moves to a work block, the input bar starts with
     * the pass-through fields */
    double *ob = a->Z.sn2, *ib = sn_bar->dev;
    ku_copy<double><<<nbk(a->nblk), 256, 0, st>>>(a->nblk, ib, ob);
    cudaMemsetAsync(ib, 0, (size_t)a->nblk * sizeof(double), st);
    AState<double> out_b = view(a, ob), in_b = view(a, ib), so_b = view(a, so_bar->dev);
    ku_waves_passthrough<<<nbk(std::max<long long>(a->nu, c->nc)), 256, 0, st>>>(c->nc, c->nl, a->nu, out_b.w,
                                                                                   out_b.u, in_b.w, in_b.u);
    cudaMemsetAsync(wl_b, 0, (size_t)WL_N * ns * sizeof(double), st);
    cudaMemsetAsync(wr_b, 0, (size_t)WR_N * a->nwi * sizeof(double), st);
    ba_apply_layer<<<nbk(ns), 256, 0, st>>>(vg, so, wl, out, out_b, a->rn_b, a->rtn_b, so_b, wl_b);
    ba_apply_w<<<nbk(a->nwi), 256, 0, st>>>(vg, so, wr, out, out_b, a->rn_b, so_b, wr_b);
    ba_apply_rho<<<nbk(ns), 256, 0, st>>>(vg, ap, wr, a->rn_b, a->rtn_b, wl_b, wr_b);
    ba_thomas<<<nbk(c->nc, 64), 64, 0, st>>>(c->nc, c->nl, a->dden, wr, wr_b);
    ba_waves_rows<<<nbk(a->nwi), 256, 0, st>>>(vg, ap, so, wl, wr, wr_b, wl_b, so_b, st_bar->ds.w);
    ba_waves_layer<<<nbk(ns), 256, 0, st>>>(vg, ap, rk, so, sn, st_m->ds.rho, st_m->ds.rhotheta_v, wl, wl_b, so_b,
                                            in_b, st_bar->ds.rho, st_bar->ds.rhotheta_v);
    c->kernel_launches += 12;
    CK(cudaGetLastError());
    return 0;
}

long long adj_block_len(Context *c)
{
    return (long long)(c->n_const + 3) * c->ns + (long long)(c->nl + 1) * c->nc + (long long)c->nl * c->ne;
}

}  // namespace game
