/*
 * extern "C" entry points of include/game_gb300.h.
 */
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cmath>

#include "context.h"
#include "diag.h"
#include "game_gb300.h"
#include "ops.h"
#include "substeps.h"
#include "adj.h"
#include "adj_ops.h"
#include "output.h"
#include "ncwrite.h"

using namespace game;

/* implemented in aux.cu */
namespace game {
void aux_sum_to_work(Context *c, const double *nl, const double *l, const double *pvt, const double *v2g,
                     const double *flux, const double *, const double *);
int aux_export(Context *c, double *P, double *pvt, double *v2g);
}  // namespace game

namespace {

struct Bound {
    const void *grid = nullptr, *dualgrid = nullptr;
    const void *aux_diag = nullptr, *aux_forc = nullptr, *aux_irrev = nullptr;
    /* structs the diffusion fields were checked / imported from */
    const void *diff_diag = nullptr, *diff_forc = nullptr, *diff_irrev = nullptr;
    bool diff_checked = false, diff_imported = false;
} g_bound;

size_t off(int sid, const char *name) { return game_layout_offset(&ctx()->dims, sid, name); }
}  // namespace

namespace game {
/* the lagged fields are imported again from the structs of the next step
 * (after the caller's structs were overwritten, e.g. by a checkpoint) */
void forget_imports()
{
    g_bound.aux_diag = g_bound.aux_forc = g_bound.aux_irrev = nullptr;
    g_bound.diff_diag = g_bound.diff_forc = g_bound.diff_irrev = nullptr;
    g_bound.diff_checked = g_bound.diff_imported = false;
}
}  // namespace game

namespace {
template <typename T>
T *member(const void *base, int sid, const char *name)
{
    return (T *)((char *)base + off(sid, name));
}

int check_ready(const void *grid)
{
    if (!ctx()) return fail("game_gpu_init has not been called");
    if (grid && grid != g_bound.grid) return fail("grid pointer differs from the one given to game_gpu_init");
    return 0;
}

int finish()
{
    Context *c = ctx();
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail(std::string("CUDA error: ") + cudaGetErrorString(e));
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(std::string("CUDA error: ") + cudaGetErrorString(e));
    return 0;
}

/* device-layout offsets inside a scratch vector / curl field */
double *vec_w(double *v) { return v; }

StepParams params_from_config(Context *c, const void *config, double dt)
{
    StepParams p{};
    p.n_const = c->n_const;
    p.n_cond = c->n_cond;
    p.moist = c->moist;
    p.dt = dt;
    p.impl_thermo_weight = *member<double>(config, GAME_CONFIG, "impl_thermo_weight");
    p.damping_start_height = *member<double>(config, GAME_CONFIG, "damping_start_height_over_toa") * c->toa;
    p.damping_coeff_max = *member<double>(config, GAME_CONFIG, "damping_coeff_max");
    p.toa = c->toa;
    p.snow_velocity = *member<double>(config, GAME_CONFIG, "snow_velocity");
    p.rain_velocity = *member<double>(config, GAME_CONFIG, "rain_velocity");
    p.cloud_velocity = *member<double>(config, GAME_CONFIG, "cloud_droplets_velocity");
    p.first_step = *member<int>(config, GAME_CONFIG, "totally_first_step_bool");
    p.dfloat = c->precision == PREC_MIXED && c->double_float == 1 ? 1 : 0;
    p.inv_dt = 1.0 / dt;
    p.k_rows = 1.0 / (p.impl_thermo_weight * dt * dt * C_D_P);
    p.k_rows2 = 0.5 / (p.impl_thermo_weight * dt * C_D_P);
    p.cur_hor = 0.5 + p.impl_thermo_weight;
    p.old_hor = 1.0 - (0.5 + p.impl_thermo_weight);
    p.cur_ver = 1.0 - p.impl_thermo_weight;
    p.cur_hor_f = (float)p.cur_hor;
    p.old_hor_f = (float)p.old_hor;
    p.cur_ver_f = (float)p.cur_ver;
    return p;
}

static const char *const DIFF_SWITCHES[6] = {"momentum_diff_h", "momentum_diff_v", "temperature_diff_h",
                                             "temperature_diff_v", "mass_diff_h", "mass_diff_v"};

/* DIFF_* bits of the config's diffusion switches (same order as DIFF_SWITCHES) */
int diff_flags(const void *config)
{
    int f = 0;
    for (int k = 0; k < 6; ++k)
        if (*member<int>(config, GAME_CONFIG, DIFF_SWITCHES[k]) != 0) f |= 1 << k;
    if (*member<int>(config, GAME_CONFIG, "pbl_scheme") == 2) f |= DIFF_PBL_HS;
    if (*member<int>(config, GAME_CONFIG, "rad_on") == 2 && *member<int>(config, GAME_CONFIG, "rad_update") == 1)
        f |= DIFF_RAD_HS;
    return f;
}

/* RTE+RRTMGP radiation (rad_on = 1), the NWP boundary layer (pbl_scheme = 1),
 * surface fluxes and soil are never part of this library's step.  The
 * diffusion branch and the Held-Suarez forcing (rad_on = 2, pbl_scheme = 2)
 * are, in manage_rkhevi (allow_diffusion); the other entry points refuse
 * every one of these switches */
int check_config(const void *config, bool allow_diffusion = false)
{
    static const char *off_switches[] = {"prog_soil_temp", "sfc_phase_trans", "sfc_sensible_heat_flux"};
    for (const char *s : off_switches)
        if (*member<int>(config, GAME_CONFIG, s) != 0)
            return fail(std::string("config switch ") + s + " is on; surface fluxes and soil are not part of this library's step");
    const int rad_on = *member<int>(config, GAME_CONFIG, "rad_on"), pbl = *member<int>(config, GAME_CONFIG, "pbl_scheme");
    if (rad_on != 0 && !(allow_diffusion && rad_on == 2))
        return fail(allow_diffusion ? "config switch rad_on is 1: RTE+RRTMGP radiation is not part of this library's step (rad_on = 2, Held-Suarez, is)"
                                    : "config switch rad_on is on; this entry point has no radiation (manage_rkhevi has the Held-Suarez forcing)");
    if (pbl != 0 && !(allow_diffusion && pbl == 2))
        return fail(allow_diffusion ? "config switch pbl_scheme is 1: the NWP boundary layer is not part of this library's step (pbl_scheme = 2, Held-Suarez, is)"
                                    : "config switch pbl_scheme is on; this entry point has no boundary layer (manage_rkhevi has the Held-Suarez friction)");
    if (!allow_diffusion)
        for (const char *s : DIFF_SWITCHES)
            if (*member<int>(config, GAME_CONFIG, s) != 0)
                return fail(std::string("config switch ") + s + " is on; this entry point has no diffusion branch (manage_rkhevi has)");
    if (rad_on == 2 && !ctx()->rad_blocks_ok)
        return fail("rad_on = 2: the reference's 18 radiation blocks do not tile this grid (NO_OF_SCALARS / 18 is not a "
                    "multiple of NO_OF_LAYERS; the reference's own block loops write past radiation_tendency here)");
    return 0;
}

static bool any_nonzero(const double *a, long long n)
{
    for (long long i = 0; i < n; ++i)
        if (a[i] != 0.0) return true;
    return false;
}

/* the diffusion branch's fields that persist between steps (the reference
 * carries them in Diagnostics and Irreversible_quantities): imported from the
 * caller's structs on the first call that needs them -- a diffusion switch is
 * on, or one of the irreversible terms the tendencies add is nonzero -- and
 * kept on the device afterwards, like the other lagged fields */
int import_diffusion(Context *c, const void *diag, const void *forc, const void *irrev, int diff)
{
    const bool same = diag == g_bound.diff_diag && forc == g_bound.diff_forc && irrev == g_bound.diff_irrev;
    if (!same) {
        g_bound.diff_diag = diag;
        g_bound.diff_forc = forc;
        g_bound.diff_irrev = irrev;
        g_bound.diff_checked = false;
        g_bound.diff_imported = false;
    }
    if (g_bound.diff_imported) {
        if (diff) c->irr_active = 1;
        return 0;
    }
    const long long ns = c->ns, nv = c->nv;
    bool need = diff != 0 || c->irr_active;
    if (!need && !g_bound.diff_checked) {
        need = any_nonzero(member<double>(irrev, GAME_IRREV, "friction_acc"), nv)
               || any_nonzero(member<double>(irrev, GAME_IRREV, "heating_diss"), ns)
               || any_nonzero(member<double>(irrev, GAME_IRREV, "temperature_diffusion_heating"), ns)
               || any_nonzero(member<double>(irrev, GAME_IRREV, "mass_diff_tendency"), c->n_const * ns)
               || any_nonzero(member<double>(forc, GAME_FORCINGS, "radiation_tendency"), ns);
        g_bound.diff_checked = true;
    }
    if (!need) return 0;
    if (c->nl < 5) return fail("the diffusion branch needs at least 5 layers");
    if (ensure_diff_buffers(c)) return -1;
    DiffBufs &b = *c->dbuf;
    struct {
        const void *base;
        int sid;
        const char *name;
        double *dev;
    } scal[] = {
        {irrev, GAME_IRREV, "tke", b.tke}, {irrev, GAME_IRREV, "viscosity", b.visc},
        {irrev, GAME_IRREV, "heating_diss", b.hdiss}, {irrev, GAME_IRREV, "molecular_diffusion_coeff", b.mol},
        {irrev, GAME_IRREV, "temperature_diffusion_heating", b.tdh}, {diag, GAME_DIAGNOSTICS, "n_squared", b.n2},
        {forc, GAME_FORCINGS, "radiation_tendency", b.rad},
    };
    for (auto &f : scal)
        if (upload_field(member<double>(f.base, f.sid, f.name), f.dev, c->map_s, ns, ns)) return -1;
    const double *mdt = member<double>(irrev, GAME_IRREV, "mass_diff_tendency");
    for (int k = 0; k < c->n_const; ++k)
        if (upload_field(mdt + k * ns, b.mdt + k * ns, c->map_s, ns, ns)) return -1;
    if (upload_field(member<double>(irrev, GAME_IRREV, "friction_acc"), b.fric, c->map_vec, nv, nv)) return -1;
    /* TOA and surface vertical entries of vector_field_placeholder */
    double *t0 = c->dev_tmp[0];
    if (upload_field(member<double>(diag, GAME_DIAGNOSTICS, "vector_field_placeholder"), t0, c->map_vec, nv, nv))
        return -1;
    CK(cudaMemcpyAsync(b.ph_tb, t0, (size_t)c->nc * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(b.ph_tb + c->nc, t0 + (long long)c->nl * c->nc, (size_t)c->nc * sizeof(double),
                       cudaMemcpyDeviceToDevice, c->stream));
    /* TOA row of dv_hdz, in device edge order */
    const double *dv = member<double>(diag, GAME_DIAGNOSTICS, "dv_hdz");
    std::vector<double> top(c->ne);
    for (int e = 0; e < c->ne; ++e) top[e] = dv[c->e_n2o[e]];
    CK(cudaMemcpyAsync(b.dvdz_top, top.data(), (size_t)c->ne * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    g_bound.diff_imported = true;
    c->irr_active = 1;
    return 0;
}

/* first use of a (diagnostics, forcings, irrev) triple: import the lagged
 * step fields the reference carries between calls */
int import_aux(const void *diag, const void *forc, const void *irrev)
{
    Context *c = ctx();
    if (diag == g_bound.aux_diag && forc == g_bound.aux_forc && irrev == g_bound.aux_irrev) return 0;
    const long long nv = c->nv, ns = c->ns;
    const long long woff = (long long)(c->nl + 1) * c->nc;
    double *t0 = c->dev_tmp[0], *t1 = c->dev_tmp[1];
    /* P = nl + l */
    if (upload_field(member<double>(forc, GAME_FORCINGS, "pressure_gradient_acc_neg_nl"), t0, c->map_vec, nv, nv)) return -1;
    if (upload_field(member<double>(forc, GAME_FORCINGS, "pressure_gradient_acc_neg_l"), t1, c->map_vec, nv, nv)) return -1;
    double *t2 = c->dev_tmp[2], *t3 = c->dev_tmp[3];
    if (upload_field(member<double>(forc, GAME_FORCINGS, "pot_vort_tend"), t2, c->map_vec, nv, nv)) return -1;
    if (upload_field(member<double>(forc, GAME_FORCINGS, "v_squared_grad"), t3, c->map_vec, nv, nv)) return -1;
    /* flux_density: the TOA/surface vertical entries are never written by the step */
    CK(cudaStreamSynchronize(c->stream));
    double *fl = nullptr;
    CK(cudaMalloc(&fl, (size_t)nv * sizeof(double)));
    if (upload_field(member<double>(diag, GAME_DIAGNOSTICS, "flux_density"), fl, c->map_vec, nv, nv)) return -1;
    aux_sum_to_work(c, t0, t1, t2, t3, fl, nullptr, nullptr);
    if (upload_field(member<double>(irrev, GAME_IRREV, "condensates_sediment_heat"), c->sed_heat, c->map_s, ns, ns)) return -1;
    CK(cudaStreamSynchronize(c->stream));
    cudaFree(fl);
    (void)woff;
    g_bound.aux_diag = diag;
    g_bound.aux_forc = forc;
    g_bound.aux_irrev = irrev;
    return 0;
}

int run_device_step(Context *c, const StepParams &p, StateMirror *so, StateMirror *sn, StateMirror *st)
{
    /* the damping table is read by the step's kernels: bring it up to date
     * outside any graph, before the first launch */
    if (launch_damping_table(c, p)) return -1;
    auto launch = [&]() {
        return c->precision == PREC_FP64 ? launch_step_f64(c, p, so, sn, st) : launch_step_mixed(c, p, so, sn, st);
    };
    if (!c->use_graphs || c->profiling) {
        if (launch()) return -1;
        c->temperature_from_step = 1;
        return 0;
    }
    Context::GraphKey key{p, c->precision, c->column_solver, so, sn, st};
    auto it = c->graphs.find(key);
    if (it == c->graphs.end()) {
        const int before = c->kernel_launches;
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        int rc = launch();
        cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
        if (rc) return rc;
        if (e != cudaSuccess) return fail(std::string("graph capture: ") + cudaGetErrorString(e));
        cudaGraphExec_t exec;
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(std::string("graph instantiate: ") + cudaGetErrorString(e));
        it = c->graphs.emplace(key, Context::GraphEntry{exec, c->kernel_launches - before}).first;
        c->kernel_launches = before;
    }
    CK(cudaGraphLaunch(it->second.exec, c->stream));
    c->kernel_launches += it->second.launches;
    c->temperature_from_step = 1;
    return 0;
}

}  // namespace

extern "C" {

int game_gpu_init(int res_id, int no_of_layers, int moisture_on, struct grid *grid, struct dualgrid *dualgrid)
{
    g_bound = Bound();
    int rc = init_context(res_id, no_of_layers, moisture_on, grid, dualgrid);
    if (rc) {
        destroy_context();
        return rc;
    }
    g_bound.grid = grid;
    g_bound.dualgrid = dualgrid;
    return 0;
}

int game_gpu_finalize(void)
{
    g_bound = Bound();
    return destroy_context();
}

int game_gpu_set_precision(int precision)
{
    if (check_ready(nullptr)) return -1;
    if (precision != GAME_GPU_FP64 && precision != GAME_GPU_MIXED) return fail("unknown precision");
    ctx()->precision = precision;
    return 0;
}

int game_gpu_set_resident(int resident)
{
    if (check_ready(nullptr)) return -1;
    ctx()->resident = resident ? 1 : 0;
    return 0;
}

int game_gpu_set_column_solver(int mode)
{
    if (check_ready(nullptr)) return -1;
    if (mode < 0 || mode > 2)
        return fail("column solver mode must be 0 (by layer count and precision), 1 (per-thread Thomas sweeps) or 2 "
                    "(warp cyclic reduction)");
    ctx()->column_solver = mode;
    return 0;
}

int game_gpu_set_double_float(int on)
{
    if (check_ready(nullptr)) return -1;
    if (on < 0 || on > 1)
        return fail("game_gpu_set_double_float: 0 (FP64) or 1 (double-float) expected");
    ctx()->double_float = on;
    return 0;
}

int game_gpu_set_graphs(int on)
{
    if (check_ready(nullptr)) return -1;
    ctx()->use_graphs = on ? 1 : 0;
    return 0;
}

int game_gpu_sync_to_device(struct state *state)
{
    if (check_ready(nullptr)) return -1;
    StateMirror *m = mirror(state, 1);
    if (!m) return -1;
    if (upload_state(state, m)) return -1;
    return finish();
}

int game_gpu_sync_to_host(struct state *state)
{
    if (check_ready(nullptr)) return -1;
    StateMirror *m = mirror(state, 0);
    if (!m) return fail("state has no device mirror");
    if (download_state(state, m, 63)) return -1;
    return finish();
}

int game_gpu_sync_aux_to_host(struct diagnostics *diagnostics, struct forcings *forcings,
                              struct irreversible_quantities *irrev)
{
    if (check_ready(nullptr)) return -1;
    Context *c = ctx();
    const long long nv = c->nv, ns = c->ns;
    double *t0 = c->dev_tmp[0], *t1 = c->dev_tmp[1], *t2 = c->dev_tmp[2];
    CK(cudaMemsetAsync(t0, 0, (size_t)nv * sizeof(double), c->stream));
    CK(cudaMemsetAsync(t1, 0, (size_t)nv * sizeof(double), c->stream));
    CK(cudaMemsetAsync(t2, 0, (size_t)nv * sizeof(double), c->stream));
    if (aux_export(c, t0, t1, t2)) return -1;
    if (forcings) {
        double *nl = member<double>(forcings, GAME_FORCINGS, "pressure_gradient_acc_neg_nl");
        double *l = member<double>(forcings, GAME_FORCINGS, "pressure_gradient_acc_neg_l");
        if (download_field(nl, t0, c->map_vec, nv, nv, 0, nv)) return -1;
        CK(cudaStreamSynchronize(c->stream));
        memset(l, 0, (size_t)nv * sizeof(double));
        if (download_field(member<double>(forcings, GAME_FORCINGS, "pot_vort_tend"), t1, c->map_vec, nv, nv, 0, nv)) return -1;
        CK(cudaStreamSynchronize(c->stream));
        if (download_field(member<double>(forcings, GAME_FORCINGS, "v_squared_grad"), t2, c->map_vec, nv, nv, 0, nv)) return -1;
        CK(cudaStreamSynchronize(c->stream));
    }
    if (diagnostics) {
        if (download_field(member<double>(diagnostics, GAME_DIAGNOSTICS, "temperature"), c->temperature, c->map_s, ns, ns,
                           0, ns)) return -1;
        CK(cudaStreamSynchronize(c->stream));
    }
    if (irrev) {
        if (download_field(member<double>(irrev, GAME_IRREV, "condensates_sediment_heat"), c->sed_heat, c->map_s, ns,
                           ns, 0, ns)) return -1;
        CK(cudaStreamSynchronize(c->stream));
        if (c->moist) {
            double *pr = member<double>(irrev, GAME_IRREV, "phase_trans_rates");
            for (int k = 0; k < 5; ++k) {
                if (download_field(pr + k * ns, c->pt_rates + k * ns, c->map_s, ns, ns, 0, ns)) return -1;
                CK(cudaStreamSynchronize(c->stream));
            }
            if (download_field(member<double>(irrev, GAME_IRREV, "phase_trans_heating_rate"), c->pt_heat, c->map_s, ns,
                               ns, 0, ns)) return -1;
        }
    }
    /* fields of the diffusion branch that persist between steps */
    if (c->dbuf && g_bound.diff_imported) {
        DiffBufs &b = *c->dbuf;
        struct {
            const void *base;
            int sid;
            const char *name;
            const double *dev;
        } scal[] = {
            {irrev, GAME_IRREV, "tke", b.tke}, {irrev, GAME_IRREV, "viscosity", b.visc},
            {irrev, GAME_IRREV, "heating_diss", b.hdiss}, {irrev, GAME_IRREV, "molecular_diffusion_coeff", b.mol},
            {irrev, GAME_IRREV, "temperature_diffusion_heating", b.tdh}, {diagnostics, GAME_DIAGNOSTICS, "n_squared", b.n2},
        };
        for (auto &f : scal) {
            if (!f.base) continue;
            if (download_field(member<double>(f.base, f.sid, f.name), f.dev, c->map_s, ns, ns, 0, ns)) return -1;
            CK(cudaStreamSynchronize(c->stream));
        }
        if (forcings) {
            if (download_field(member<double>(forcings, GAME_FORCINGS, "radiation_tendency"), b.rad, c->map_s, ns, ns, 0,
                               ns)) return -1;
            CK(cudaStreamSynchronize(c->stream));
        }
        if (irrev) {
            double *mdt = member<double>(irrev, GAME_IRREV, "mass_diff_tendency");
            for (int k = 0; k < c->n_const; ++k) {
                if (download_field(mdt + k * ns, b.mdt + k * ns, c->map_s, ns, ns, 0, ns)) return -1;
                CK(cudaStreamSynchronize(c->stream));
            }
            if (download_field(member<double>(irrev, GAME_IRREV, "friction_acc"), b.fric, c->map_vec, nv, nv, 0, nv))
                return -1;
        }
    }
    return finish();
}

int game_gpu_synchronize(void)
{
    if (check_ready(nullptr)) return -1;
    return finish();
}

const char *game_gpu_last_error(void) { return last_error(); }

int game_gpu_host_alloc(void **ptr, size_t bytes)
{
    cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocPortable | cudaHostAllocMapped);
    if (e != cudaSuccess) return fail(std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
    memset(*ptr, 0, bytes);
    /* States inside this allocation are copied by kernels that access it
     * directly; without a device address they take the staged copies */
    void *dev = nullptr;
    if (cudaHostGetDevicePointer(&dev, *ptr, 0) == cudaSuccess && dev) pinned_register(*ptr, dev, bytes);
    else cudaGetLastError();
    return 0;
}

int game_gpu_host_free(void *ptr)
{
    pinned_unregister(ptr);
    cudaError_t e = cudaFreeHost(ptr);
    if (e != cudaSuccess) return fail(std::string("cudaFreeHost: ") + cudaGetErrorString(e));
    return 0;
}

long long game_gpu_kernel_launches(int reset)
{
    if (!ctx()) return 0;
    long long n = ctx()->kernel_launches;
    if (reset) ctx()->kernel_launches = 0;
    return n;
}

int game_gpu_set_device(int device)
{
    if (ctx()) return fail("game_gpu_set_device must precede game_gpu_init");
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    return 0;
}

int game_gpu_event_record(int slot)
{
    if (check_ready(nullptr)) return -1;
    Context *c = ctx();
    if (slot < 0 || slot > 1 << 20) return fail("event slot out of range");
    while ((int)c->user_events.size() <= slot) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        c->user_events.push_back(e);
    }
    CK(cudaEventRecord(c->user_events[slot], c->stream));
    return 0;
}

int game_gpu_event_elapsed(int a, int b, float *ms)
{
    if (check_ready(nullptr)) return -1;
    Context *c = ctx();
    if (a < 0 || b < 0 || a >= (int)c->user_events.size() || b >= (int)c->user_events.size())
        return fail("event slot not recorded");
    CK(cudaEventSynchronize(c->user_events[b]));
    CK(cudaEventElapsedTime(ms, c->user_events[a], c->user_events[b]));
    return 0;
}

int game_gpu_profile(int on)
{
    if (check_ready(nullptr)) return -1;
    Context *c = ctx();
    if (!on && profile_flush(c)) return -1;
    if (on) c->prof_totals.clear();
    c->profiling = on ? 1 : 0;
    return 0;
}

int game_gpu_profile_count(void)
{
    if (!ctx()) return 0;
    profile_flush(ctx());
    return (int)ctx()->prof_totals.size();
}

int game_gpu_profile_get(int i, const char **name, double *ms, long long *launches)
{
    if (check_ready(nullptr)) return -1;
    Context *c = ctx();
    if (i < 0 || i >= (int)c->prof_totals.size()) return fail("profile entry out of range");
    auto it = c->prof_totals.begin();
    std::advance(it, i);
    *name = it->first.c_str();
    *ms = it->second.first;
    *launches = it->second.second;
    return 0;
}

int game_gpu_transfer_bytes(long long *h2d, long long *d2h, int reset)
{
    if (check_ready(nullptr)) return -1;
    Context *c = ctx();
    *h2d = c->h2d_bytes;
    *d2h = c->d2h_bytes;
    if (reset) c->h2d_bytes = c->d2h_bytes = 0;
    return 0;
}

/* ---------------------------------------------------------------- the step */
int manage_rkhevi(struct state *state_old, struct state *state_new, struct grid *grid, struct dualgrid *dualgrid,
                  struct state *state_tendency, struct diagnostics *diagnostics, struct forcings *forcings,
                  struct irreversible_quantities *irrev, struct config *config, double delta_t,
                  double time_coordinate)
{
    (void)time_coordinate;
    (void)dualgrid;
    if (check_ready(grid)) return -1;
    if (check_config(config, true)) return -1;
    Context *c = ctx();
    StateMirror *so = mirror(state_old, 1), *sn = mirror(state_new, 1), *st = mirror(state_tendency, 1);
    if (!so || !sn || !st) return -1;
    if (so == sn || so == st || sn == st) return fail("state_old, state_new and state_tendency must be distinct");
    if (import_aux(diagnostics, forcings, irrev)) return -1;
    if (import_diffusion(c, diagnostics, forcings, irrev, diff_flags(config))) return -1;
    if (!c->resident) {
        if (upload_state(state_old, so)) return -1;
        if (upload_state(state_new, sn)) return -1;
    }
    StepParams p = params_from_config(c, config, delta_t);
    p.diff = diff_flags(config);
    p.irr = c->irr_active;
    if (p.diff & DIFF_RAD_HS) {
        /* the Held-Suarez radiation blocks hand back zero surface fluxes
         * (manage_radiation_calls.c:71-72) */
        std::memset(member<double>(forcings, GAME_FORCINGS, "sfc_sw_in"), 0, (size_t)c->rad_covered * sizeof(double));
        std::memset(member<double>(forcings, GAME_FORCINGS, "sfc_lw_out"), 0, (size_t)c->rad_covered * sizeof(double));
    }
    if (run_device_step(c, p, so, sn, st)) return -1;
    if (!c->resident) {
        /* a pinned tendency is copied out on the second stream as soon as the
         * step has finished it, while the vertical solves still run */
        CK(cudaStreamWaitEvent(c->stream2, c->ev_tend, 0));
        const int tend_async = download_state_pinned(state_tendency, st, 1 | 2 | 16, c->stream2);
        if (tend_async) CK(cudaEventRecord(c->ev_tend_copied, c->stream2));
        if (download_state(state_new, sn, 1 | 2 | 4 | 8 | 16)) return -1;
        if (tend_async) CK(cudaStreamWaitEvent(c->stream, c->ev_tend_copied, 0));
        else if (download_state(state_tendency, st, 1 | 2 | 16)) return -1;
    }
    if (finish()) return -1;
    if (c->health_every > 0 && ++c->health_count % c->health_every == 0)
        return check_mirror(c, sn, nullptr, "manage_rkhevi: state_new");
    return 0;
}

int linear_combine_two_states(struct state *state_0, struct state *state_1, struct state *state_out, double coeff_0,
                              double coeff_1, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    StateMirror *a = mirror(state_0, 1), *b = mirror(state_1, 1), *o = mirror(state_out, 1);
    if (!a || !b || !o) return -1;
    if (!c->resident) {
        if (upload_state(state_0, a)) return -1;
        if (b != a && upload_state(state_1, b)) return -1;
    }
    op_linear_combine(c, a, b, o, coeff_0, coeff_1);
    if (!c->resident && download_state(state_out, o, 63)) return -1;
    return finish();
}

/* --------------------------------------------------------- single operators */
/* pointwise product of two host fields of n values (no layout change) */
static int pointwise_product(const double *a, const double *b, double *out, long long n)
{
    Context *c = ctx();
    double *da = c->dev_tmp[0], *db = c->dev_tmp[1], *dout = c->dev_tmp[2];
    CK(cudaMemcpyAsync(da, a, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(db, b, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    c->h2d_bytes += 2 * n * (long long)sizeof(double);
    op_mul(c, n, da, db, dout);
    CK(cudaMemcpyAsync(out, dout, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    c->d2h_bytes += n * (long long)sizeof(double);
    return finish();
}

int scalar_times_scalar(double *in_field_0, double *in_field_1, double *out_field)
{
    if (check_ready(nullptr)) return -1;
    return pointwise_product(in_field_0, in_field_1, out_field, ctx()->ns);
}

int vector_times_vector(double *in_field_0, double *in_field_1, double *out_field)
{
    if (check_ready(nullptr)) return -1;
    return pointwise_product(in_field_0, in_field_1, out_field, ctx()->nv);
}

int add_vertical_divv(double *in_field, double *out_field, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    double *v = c->dev_tmp[1], *o = c->dev_tmp[0];
    if (upload_field(in_field, v, c->map_vec, c->nv, c->nv)) return -1;
    if (upload_field(out_field, o, c->map_s, c->ns, c->ns)) return -1;
    op_add_vertical_divv(c, v, o);
    if (download_field(out_field, o, c->map_s, c->ns, c->ns, 0, c->ns)) return -1;
    return finish();
}

static int vec_op_prologue(double *out_field, double *dev_out)
{
    /* the output keeps the entries the operator does not write */
    Context *c = ctx();
    return upload_field(out_field, dev_out, c->map_vec, c->nv, c->nv);
}

static int grad_parts(double *in_field, double *out_field, struct grid *grid, int parts)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    double *f = c->dev_tmp[0], *v = c->dev_tmp[1];
    if (upload_field(in_field, f, c->map_s, c->ns, c->ns)) return -1;
    if (vec_op_prologue(out_field, v)) return -1;
    op_grad(c, f, v, parts);
    if (download_field(out_field, v, c->map_vec, c->nv, c->nv, 0, c->nv)) return -1;
    return finish();
}

int grad_hor_cov(double *in_field, double *out_field, struct grid *grid)
{
    return grad_parts(in_field, out_field, grid, OP_GRAD_H);
}
int grad_vert_cov(double *in_field, double *out_field, struct grid *grid)
{
    return grad_parts(in_field, out_field, grid, OP_GRAD_V);
}
int grad_cov(double *in_field, double *out_field, struct grid *grid)
{
    return grad_parts(in_field, out_field, grid, OP_GRAD_H | OP_GRAD_V);
}
int grad(double *in_field, double *out_field, struct grid *grid)
{
    return grad_parts(in_field, out_field, grid, OP_GRAD_H | OP_GRAD_V | OP_GRAD_CON);
}
int grad_hor(double *in_field, double *out_field, struct grid *grid)
{
    if (grad(in_field, out_field, grid)) return -1;
    /* gradient_operators.c:76-91: vertical components set to zero */
    Context *c = ctx();
    const long long vpl = (long long)c->nc + c->ne;
    for (int k = 0; k <= c->nl; ++k) memset(out_field + k * vpl, 0, (size_t)c->nc * sizeof(double));
    return 0;
}

int vector_field_hor_cov_to_con(double *field, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    double *v = c->dev_tmp[1];
    if (upload_field(field, v, c->map_vec, c->nv, c->nv)) return -1;
    op_cov_to_con(c, v);
    if (download_field(field, v, c->map_vec, c->nv, c->nv, 0, c->nv)) return -1;
    return finish();
}

static int stv(double *s, double *vec, double *out, struct grid *grid, int parts)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    double *fs = c->dev_tmp[0], *fv = c->dev_tmp[1], *fo = c->dev_tmp[2];
    if (upload_field(s, fs, c->map_s, c->ns, c->ns)) return -1;
    if (upload_field(vec, fv, c->map_vec, c->nv, c->nv)) return -1;
    if (vec_op_prologue(out, fo)) return -1;
    op_scalar_times_vector(c, fs, fv, fo, parts);
    if (download_field(out, fo, c->map_vec, c->nv, c->nv, 0, c->nv)) return -1;
    return finish();
}

int scalar_times_vector(double *scalar_field, double *vector_field, double *out_field, struct grid *grid)
{
    return stv(scalar_field, vector_field, out_field, grid, OP_STV_H | OP_STV_V);
}
int scalar_times_vector_h(double *in_field_h, double *vector_field, double *out_field, struct grid *grid)
{
    return stv(in_field_h, vector_field, out_field, grid, OP_STV_H);
}
int scalar_times_vector_h_upstream(double *in_field_h, double *vector_field, double *out_field, struct grid *grid)
{
    return stv(in_field_h, vector_field, out_field, grid, OP_STV_H | OP_STV_UPSTREAM);
}
int scalar_times_vector_v(double *in_field_v, double *vector_field, double *out_field, struct grid *grid)
{
    return stv(in_field_v, vector_field, out_field, grid, OP_STV_V);
}

int divv_h(double *in_field, double *out_field, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    double *fv = c->dev_tmp[1], *fo = c->dev_tmp[0];
    if (upload_field(in_field, fv, c->map_vec, c->nv, c->nv)) return -1;
    op_divv(c, fv, nullptr, nullptr, fo, 0);
    if (download_field(out_field, fo, c->map_s, c->ns, c->ns, 0, c->ns)) return -1;
    return finish();
}

int divv_h_tracer(double *in_field, double *density_field, double *wind_field, double *out_field, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    double *fv = c->dev_tmp[1], *fd = c->dev_tmp[0], *fw = c->dev_tmp[2], *fo = c->dev_tmp[3];
    if (upload_field(in_field, fv, c->map_vec, c->nv, c->nv)) return -1;
    if (upload_field(density_field, fd, c->map_s, c->ns, c->ns)) return -1;
    if (upload_field(wind_field, fw, c->map_vec, c->nv, c->nv)) return -1;
    op_divv(c, fv, fd, fw, fo, 1);
    if (download_field(out_field, fo, c->map_s, c->ns, c->ns, 0, c->ns)) return -1;
    return finish();
}

int inner_product(double *in_field_0, double *in_field_1, double *out_field, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    double *a = c->dev_tmp[1], *b = c->dev_tmp[2], *o = c->dev_tmp[0];
    if (upload_field(in_field_0, a, c->map_vec, c->nv, c->nv)) return -1;
    if (upload_field(in_field_1, b, c->map_vec, c->nv, c->nv)) return -1;
    op_inner_product(c, a, b, o);
    if (download_field(out_field, o, c->map_s, c->ns, c->ns, 0, c->ns)) return -1;
    return finish();
}

static int rel_vort_common(double *velocity_field, double *density_field, struct diagnostics *diagnostics,
                           struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    const long long ntri = (long long)c->nl * c->nt;
    double *wind = c->dev_tmp[0], *rel = c->dev_tmp[1], *tri = c->dev_tmp[2], *pv = c->dev_tmp[3];
    if (upload_field(velocity_field, wind, c->map_vec, c->nv, c->nv)) return -1;
    op_rel_vort(c, wind, tri, rel);
    if (download_field(member<double>(diagnostics, GAME_DIAGNOSTICS, "rel_vort_on_triangles"), tri, c->map_tri, ntri,
                       ntri, 0, ntri)) return -1;
    CK(cudaStreamSynchronize(c->stream));
    if (download_field(member<double>(diagnostics, GAME_DIAGNOSTICS, "rel_vort"), rel, c->map_curl, c->ncurl,
                       c->ncurl, 0, c->ncurl)) return -1;
    if (density_field) {
        CK(cudaStreamSynchronize(c->stream));
        double *rho = wind; /* wind no longer needed */
        if (upload_field(density_field, rho, c->map_s, c->ns, c->ns)) return -1;
        op_pot_vort(c, rel, rho, pv);
        if (download_field(member<double>(diagnostics, GAME_DIAGNOSTICS, "pot_vort"), pv, c->map_curl, c->ncurl,
                           c->ncurl, 0, c->ncurl)) return -1;
    }
    return finish();
}

int calc_rel_vort(double *velocity_field, struct diagnostics *diagnostics, struct grid *grid, struct dualgrid *dualgrid)
{
    (void)dualgrid;
    return rel_vort_common(velocity_field, nullptr, diagnostics, grid);
}

int calc_pot_vort(double *velocity_field, double *density_field, struct diagnostics *diagnostics, struct grid *grid,
                  struct dualgrid *dualgrid)
{
    (void)dualgrid;
    return rel_vort_common(velocity_field, density_field, diagnostics, grid);
}

int add_f_to_rel_vort(double *rel_vort, double *out_field, struct dualgrid *dualgrid)
{
    if (check_ready(nullptr)) return -1;
    if (dualgrid != g_bound.dualgrid) return fail("dualgrid pointer differs from the one given to game_gpu_init");
    Context *c = ctx();
    double *rel = c->dev_tmp[1], *pv = c->dev_tmp[3];
    if (upload_field(rel_vort, rel, c->map_curl, c->ncurl, c->ncurl)) return -1;
    op_pot_vort(c, rel, nullptr, pv);
    if (download_field(out_field, pv, c->map_curl, c->ncurl, c->ncurl, 0, c->ncurl)) return -1;
    return finish();
}

int vorticity_flux(double *mass_flux_density, double *pot_vorticity, double *out_field, struct grid *grid,
                   struct dualgrid *dualgrid)
{
    (void)dualgrid;
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    double *fl = c->dev_tmp[0], *pv = c->dev_tmp[1], *o = c->dev_tmp[2];
    if (upload_field(mass_flux_density, fl, c->map_vec, c->nv, c->nv)) return -1;
    if (upload_field(pot_vorticity, pv, c->map_curl, c->ncurl, c->ncurl)) return -1;
    op_vorticity_flux(c, fl, pv, o);
    if (download_field(out_field, o, c->map_vec, c->nv, c->nv, 0, c->nv)) return -1;
    return finish();
}

/* ------------------------------------------------ integrals, surface pressure */
double global_scalar_integrator(double *density_gen, struct grid *grid)
{
    if (check_ready(grid)) return NAN;
    Context *c = ctx();
    if (cudaMemcpyAsync(c->staging, density_gen, (size_t)c->ns * sizeof(double), cudaMemcpyHostToDevice, c->stream) !=
        cudaSuccess) {
        fail("global_scalar_integrator: host-to-device copy failed");
        return NAN;
    }
    c->h2d_bytes += c->ns * (long long)sizeof(double);
    if (launch_integral(c->staging, 0, 1, c->ns, c->map_s, c->hg64.volume, c->red_partials, c->red_counters, c->red_out,
                        c->stream))
        return NAN;
    c->kernel_launches++;
    double r = NAN;
    if (cudaMemcpyAsync(&r, c->red_out, sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) {
        fail("global_scalar_integrator: device-to-host copy failed");
        return NAN;
    }
    c->d2h_bytes += (long long)sizeof(double);
    if (finish()) return NAN;
    return r;
}

/* the device mirror of a State for a read-only diagnostic: in resident mode
 * the mirror as it is, else a fresh upload of the host struct */
static StateMirror *diag_mirror(struct state *state)
{
    Context *c = ctx();
    if (c->resident) {
        StateMirror *m = mirror(state, 0);
        if (!m) fail("resident mode: this State has no device mirror (game_gpu_sync_to_device it first)");
        return m;
    }
    StateMirror *m = mirror(state, 1);
    if (m && upload_state(state, m)) return nullptr;
    return m;
}

int game_gpu_write_out_integral(struct state *state, int integral_id, double *result)
{
    if (check_ready(nullptr)) return -1;
    if (integral_id < 0 || integral_id > 2) return fail("integral_id must be 0 (masses), 1 (rho*theta_v) or 2 (energy)");
    Context *c = ctx();
    StateMirror *m = diag_mirror(state);
    if (!m) return -1;
    const long long ns = c->ns;
    int n_out = 1;
    if (integral_id == 0) {
        n_out = c->n_const;
        if (launch_integral(m->ds.rho, ns, n_out, ns, nullptr, c->hg64.volume, c->red_partials, c->red_counters,
                            c->red_out, c->stream))
            return -1;
    } else if (integral_id == 1) {
        if (launch_integral(m->ds.rhotheta_v, ns, 1, ns, nullptr, c->hg64.volume, c->red_partials, c->red_counters,
                            c->red_out, c->stream))
            return -1;
    } else {
        n_out = 3;
        if (!c->temperature_from_step && diag_temperature(c, m, c->temperature)) return -1;
        if (diag_energy_densities(c, m, c->temperature, c->energy_buf)) return -1;
        if (launch_integral(c->energy_buf, ns, 3, ns, nullptr, c->hg64.volume, c->red_partials, c->red_counters,
                            c->red_out, c->stream))
            return -1;
    }
    c->kernel_launches++;
    double r[INTEGRAL_MAX_FIELDS];
    CK(cudaMemcpyAsync(r, c->red_out, (size_t)n_out * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    c->d2h_bytes += n_out * (long long)sizeof(double);
    if (finish()) return -1;
    if (integral_id == 2) {
        result[0] = 0.5 * r[0];
        result[1] = r[1];
        result[2] = C_D_V * r[2];
    } else {
        for (int k = 0; k < n_out; ++k) result[k] = r[k];
    }
    return 0;
}

int game_gpu_surface_pressure(struct state *state, double *surface_p, double *mslp)
{
    if (check_ready(nullptr)) return -1;
    Context *c = ctx();
    StateMirror *m = diag_mirror(state);
    if (!m) return -1;
    double *ps = c->dev_tmp[0], *pm = c->dev_tmp[0] + c->nc;
    if (diag_surface_pressure(c, m, ps, mslp ? pm : nullptr)) return -1;
    if (download_field(surface_p, ps, c->map_s, c->nc, c->nc, 0, c->nc)) return -1;
    /* same stream: the second scatter into the staging buffer runs after the
     * first copy out of it */
    if (mslp && download_field(mslp, pm, c->map_s, c->nc, c->nc, 0, c->nc)) return -1;
    return finish();
}

/* -------------------------------------------------------- the sub-steps
 * Host-in/host-out in every residency mode, on private device buffers: they
 * never read or write the device mirrors or the lagged fields of the
 * device-resident step.  FP64 path, reference operation order.  Scratch
 * members of Diagnostics that the reference overwrites as work space
 * (scalar_field_placeholder, flux_density_divv, and flux_density inside
 * scalar_tendencies_expl) are not written. */
static double *vec_of(void *base, int sid, const char *name) { return member<double>(base, sid, name); }

static int up_vec(void *base, int sid, const char *name, double *dev)
{
    Context *c = ctx();
    return upload_field(vec_of(base, sid, name), dev, c->map_vec, c->nv, c->nv);
}
static int down_vec(void *base, int sid, const char *name, const double *dev)
{
    Context *c = ctx();
    return download_field(vec_of(base, sid, name), dev, c->map_vec, c->nv, c->nv, 0, c->nv);
}
static int up_scal(void *base, int sid, const char *name, double *dev, int n_fields = 1)
{
    Context *c = ctx();
    for (int k = 0; k < n_fields; ++k)
        if (upload_field(vec_of(base, sid, name) + (long long)k * c->ns, dev + (long long)k * c->ns, c->map_s, c->ns,
                         c->ns))
            return -1;
    return 0;
}
static int down_scal(void *base, int sid, const char *name, const double *dev)
{
    Context *c = ctx();
    return download_field(vec_of(base, sid, name), dev, c->map_s, c->ns, c->ns, 0, c->ns);
}

int manage_pressure_gradient(struct state *state, struct grid *grid, struct dualgrid *dualgrid,
                             struct diagnostics *diagnostics, struct forcings *forcings,
                             struct irreversible_quantities *irrev, struct config *config)
{
    (void)dualgrid;
    (void)diagnostics;
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    Context::SubBuffers &b = c->sub;
    double *nl = b.vec[0], *l = b.vec[1], *old = b.vec[2];
    if (upload_state(state, &b.sn)) return -1;
    if (up_vec(forcings, GAME_FORCINGS, "pressure_gradient_acc_neg_nl", nl)) return -1;
    if (up_vec(forcings, GAME_FORCINGS, "pressure_gradient_acc_neg_l", l)) return -1;
    if (up_vec(forcings, GAME_FORCINGS, "pgrad_acc_old", old)) return -1;
    StepParams p = params_from_config(c, config, 1.0);
    sub_pressure_gradient(c, p, &b.sn, nl, l, old, b.decel);
    if (down_vec(forcings, GAME_FORCINGS, "pgrad_acc_old", old)) return -1;
    if (down_vec(forcings, GAME_FORCINGS, "pressure_gradient_acc_neg_nl", nl)) return -1;
    if (down_vec(forcings, GAME_FORCINGS, "pressure_gradient_acc_neg_l", l)) return -1;
    if (down_scal(irrev, GAME_IRREV, "pressure_gradient_decel_factor", b.decel)) return -1;
    return finish();
}

int calc_pressure_grad_condensates_v(struct state *state, struct grid *grid, struct forcings *forcings,
                                     struct irreversible_quantities *irrev)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    Context::SubBuffers &b = c->sub;
    if (upload_state(state, &b.sn)) return -1;
    if (up_vec(forcings, GAME_FORCINGS, "pressure_grad_condensates_v", b.vec[0])) return -1;
    sub_condensates_v(c, &b.sn, b.decel, b.vec[0]);
    if (down_vec(forcings, GAME_FORCINGS, "pressure_grad_condensates_v", b.vec[0])) return -1;
    if (down_scal(irrev, GAME_IRREV, "pressure_gradient_decel_factor", b.decel)) return -1;
    return finish();
}

int vector_tendencies_expl(struct state *state, struct state *state_tendency, struct grid *grid,
                           struct dualgrid *dualgrid, struct diagnostics *diagnostics, struct forcings *forcings,
                           struct irreversible_quantities *irrev, struct config *config, int rk_step, double delta_t)
{
    (void)dualgrid;
    if (check_ready(grid)) return -1;
    if (check_config(config)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    Context::SubBuffers &b = c->sub;
    const long long ns = c->ns, ncurl = c->ncurl, ntri = (long long)c->nl * c->nt;
    double *pg_old = b.vec[0], *nl = b.vec[1], *l = b.vec[2], *cond_v = b.vec[3], *fric = b.vec[4];
    double *flux = b.vec[5], *pvt = b.vec[6], *v2g = b.vec[7], *rel = b.vec[8], *pv = b.vec[9];
    if (upload_state(state, &b.sn)) return -1;
    if (upload_state(state_tendency, &b.st)) return -1;
    if (up_vec(forcings, GAME_FORCINGS, "pgrad_acc_old", pg_old)) return -1;
    if (up_vec(forcings, GAME_FORCINGS, "pressure_gradient_acc_neg_nl", nl)) return -1;
    if (up_vec(forcings, GAME_FORCINGS, "pressure_gradient_acc_neg_l", l)) return -1;
    if (up_vec(forcings, GAME_FORCINGS, "pressure_grad_condensates_v", cond_v)) return -1;
    if (up_vec(irrev, GAME_IRREV, "friction_acc", fric)) return -1;
    if (up_vec(forcings, GAME_FORCINGS, "pot_vort_tend", pvt)) return -1;
    if (up_vec(forcings, GAME_FORCINGS, "v_squared_grad", v2g)) return -1;
    const int first = *member<int>(config, GAME_CONFIG, "totally_first_step_bool");
    if (rk_step == 1 || first == 1) {
        /* vector_tendencies_expl.c:24-35; entries the reference's operators
         * leave alone keep the caller's values */
        double *wind = b.sn.ds.w, *rho_gas = b.sn.ds.rho + (long long)c->n_cond * ns;
        if (up_vec(diagnostics, GAME_DIAGNOSTICS, "flux_density", flux)) return -1;
        op_scalar_times_vector(c, rho_gas, wind, flux, OP_STV_H | OP_STV_V);
        op_rel_vort(c, wind, b.tri, rel);
        op_pot_vort(c, rel, rho_gas, pv);
        op_vorticity_flux(c, flux, pv, pvt);
        op_inner_product(c, wind, wind, b.v2);
        op_grad(c, b.v2, v2g, OP_GRAD_H | OP_GRAD_V | OP_GRAD_CON);
        if (down_vec(diagnostics, GAME_DIAGNOSTICS, "flux_density", flux)) return -1;
        if (download_field(vec_of(diagnostics, GAME_DIAGNOSTICS, "rel_vort_on_triangles"), b.tri, c->map_tri, ntri,
                           ntri, 0, ntri))
            return -1;
        if (download_field(vec_of(diagnostics, GAME_DIAGNOSTICS, "rel_vort"), rel, c->map_curl, ncurl, ncurl, 0,
                           ncurl))
            return -1;
        if (download_field(vec_of(diagnostics, GAME_DIAGNOSTICS, "pot_vort"), pv, c->map_curl, ncurl, ncurl, 0, ncurl))
            return -1;
        if (down_scal(diagnostics, GAME_DIAGNOSTICS, "v_squared", b.v2)) return -1;
        if (down_vec(forcings, GAME_FORCINGS, "pot_vort_tend", pvt)) return -1;
        if (down_vec(forcings, GAME_FORCINGS, "v_squared_grad", v2g)) return -1;
    }
    StepParams p = params_from_config(c, config, delta_t);
    sub_vector_tendency(c, p, rk_step, b.st.ds.w, pg_old, nl, l, pvt, v2g, fric, cond_v);
    if (download_state(state_tendency, &b.st, 16)) return -1;
    return finish();
}

int scalar_tendencies_expl(struct state *state_old, struct state *state, struct state *state_tendency,
                           struct grid *grid, struct dualgrid *dualgrid, double delta_t,
                           struct diagnostics *diagnostics, struct forcings *forcings,
                           struct irreversible_quantities *irrev, struct config *config, int rk_step)
{
    (void)state_old;
    (void)dualgrid;
    (void)forcings;
    if (check_ready(grid)) return -1;
    if (check_config(config)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    Context::SubBuffers &b = c->sub;
    if (upload_state(state, &b.sn)) return -1;
    if (upload_state(state_tendency, &b.st)) return -1;
    if (c->moist) {
        if (up_scal(diagnostics, GAME_DIAGNOSTICS, "temperature", b.temperature)) return -1;
        sub_cp_tables(c, b.temperature, b.cp_ice, b.cp_water);
        if (up_scal(irrev, GAME_IRREV, "phase_trans_rates", b.pt_rates, c->n_cond + 1)) return -1;
        if (up_scal(irrev, GAME_IRREV, "phase_trans_heating_rate", b.pt_heat)) return -1;
        if (up_scal(irrev, GAME_IRREV, "condensates_sediment_heat", b.sed_heat)) return -1;
    }
    StepParams p = params_from_config(c, config, delta_t);
    sub_scalar_tendencies(c, p, &b.sn, &b.st, rk_step, b.theta, b.cp_ice, b.cp_water, b.pt_rates, b.pt_heat,
                          b.sed_heat);
    if (download_state(state_tendency, &b.st, 1 | 2)) return -1;
    return finish();
}

int three_band_solver_ver_waves(struct state *state_old, struct state *state_new, struct state *state_tendency,
                                struct diagnostics *diagnostics, struct forcings *forcings, struct config *config,
                                double delta_t, struct grid *grid, int rk_step)
{
    (void)diagnostics;
    (void)forcings;
    if (check_ready(grid)) return -1;
    if (check_config(config)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    Context::SubBuffers &b = c->sub;
    if (upload_state(state_old, &b.so)) return -1;
    if (upload_state(state_new, &b.sn)) return -1;
    if (upload_state(state_tendency, &b.st)) return -1;
    StepParams p = params_from_config(c, config, delta_t);
    if (sub_ver_waves(c, p, &b.so, &b.sn, &b.st, rk_step)) return -1;
    if (download_state(state_new, &b.sn, 1 | 2 | 4 | 8 | 16)) return -1;
    return finish();
}

int three_band_solver_gen_densities(struct state *state_old, struct state *state_new, struct state *state_tendency,
                                    struct diagnostics *diagnostics, struct irreversible_quantities *irrev,
                                    struct config *config, double delta_t, int rk_step, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    if (check_config(config)) return -1;
    Context *c = ctx();
    if (c->n_const <= 1) return finish();
    if (ensure_sub_buffers(c)) return -1;
    Context::SubBuffers &b = c->sub;
    if (upload_state(state_old, &b.so)) return -1;
    if (upload_state(state_new, &b.sn)) return -1;
    if (upload_state(state_tendency, &b.st)) return -1;
    if (up_scal(diagnostics, GAME_DIAGNOSTICS, "temperature", b.temperature)) return -1;
    sub_cp_tables(c, b.temperature, b.cp_ice, b.cp_water);
    if (up_scal(irrev, GAME_IRREV, "condensates_sediment_heat", b.sed_heat)) return -1;
    StepParams p = params_from_config(c, config, delta_t);
    sub_gen_densities(c, p, &b.so, &b.sn, &b.st, rk_step, b.temperature, b.cp_ice, b.cp_water, b.sed_heat);
    if (download_state(state_new, &b.sn, 1)) return -1;
    if (rk_step == 0 && down_scal(irrev, GAME_IRREV, "condensates_sediment_heat", b.sed_heat)) return -1;
    return finish();
}

/* ----------------------------------------------- adjoint / tangent-linear */
/* copy a device state block into a private mirror and download it */
static int adj_download(struct state *host, StateMirror *m, const double *blk)
{
    Context *c = ctx();
    if (blk != m->dev)
        CK(cudaMemcpyAsync(m->dev, blk, (size_t)adj_block_len(c) * sizeof(double), cudaMemcpyDeviceToDevice,
                           c->stream));
    if (download_state(host, m, 1 | 2 | 4 | 8 | 16)) return -1;
    return finish();
}

/* the window forward on the device: result in the sub-step mirror sn */
static int window_forward_dev(const char *who, struct state *state_init, struct grid *grid,
                              struct diagnostics *diagnostics, struct forcings *forcings,
                              struct irreversible_quantities *irrev, struct config *config, double delta_t,
                              int n_steps)
{
    if (check_ready(grid)) return -1;
    if (check_config(config)) return -1;
    Context *c = ctx();
    if (c->n_const != 1 && c->n_const != 6)
        return fail(std::string(who) + ": the adjoint model covers the dry build and the moist build of six "
                                       "constituents");
    if (ensure_sub_buffers(c)) return -1;
    Context::SubBuffers &b = c->sub;
    if (upload_state(state_init, &b.so)) return -1;
    StepParams p = params_from_config(c, config, delta_t);
    double *auxP = b.vec[0], *auxV = b.vec[1], *auxG = b.vec[2], *fl = b.vec[3];
    if (up_vec(diagnostics, GAME_DIAGNOSTICS, "flux_density", fl)) return -1;
    if (!p.first_step) {
        if (up_vec(forcings, GAME_FORCINGS, "pressure_gradient_acc_neg_nl", auxP)) return -1;
        if (up_vec(forcings, GAME_FORCINGS, "pressure_gradient_acc_neg_l", b.vec[4])) return -1;
        if (up_vec(forcings, GAME_FORCINGS, "pot_vort_tend", auxV)) return -1;
        if (up_vec(forcings, GAME_FORCINGS, "v_squared_grad", auxG)) return -1;
        adj_add_into(c, auxP, b.vec[4], c->nv); /* the step reads nl + l */
    }
    /* moist: the sedimentation heat the first substage reads */
    if (c->n_const > 1 && up_scal(irrev, GAME_IRREV, "condensates_sediment_heat", b.sed_heat)) return -1;
    return adj_window_forward(c, &b.so, p, n_steps, auxP, auxV, auxG, fl, c->n_const > 1 ? b.sed_heat : nullptr,
                              &b.sn);
}

int rkhevi_window_forward(struct state *state_init, struct state *state_final, struct grid *grid,
                          struct dualgrid *dualgrid, struct diagnostics *diagnostics, struct forcings *forcings,
                          struct irreversible_quantities *irrev, struct config *config, double delta_t, int n_steps)
{
    (void)dualgrid;
    if (window_forward_dev("rkhevi_window_forward", state_init, grid, diagnostics, forcings, irrev, config, delta_t,
                           n_steps))
        return -1;
    Context *c = ctx();
    return adj_download(state_final, &c->sub.sn, c->sub.sn.dev);
}

int manage_rkhevi_adj(struct state *state_old, struct state *state_new, struct grid *grid, struct dualgrid *dualgrid,
                      struct state *state_tendency, struct diagnostics *diagnostics, struct forcings *forcings,
                      struct irreversible_quantities *irrev, struct config *config, double delta_t,
                      double time_coordinate, struct state *state_new_bar, struct state *state_old_bar)
{
    (void)state_new;
    (void)dualgrid;
    (void)state_tendency;
    (void)time_coordinate;
    if (window_forward_dev("manage_rkhevi_adj", state_old, grid, diagnostics, forcings, irrev, config, delta_t, 1))
        return -1;
    Context *c = ctx();
    Context::SubBuffers &b = c->sub;
    if (upload_state(state_new_bar, &b.st)) return -1;
    if (adj_window_backward(c, b.st.dev, b.sn.dev)) return -1;
    return adj_download(state_old_bar, &b.sn, b.sn.dev);
}

int game_gpu_set_checkpoint_stride(int every)
{
    if (check_ready(nullptr)) return -1;
    if (every < 1) return fail("game_gpu_set_checkpoint_stride: a stride of at least 1 expected");
    ctx()->adj_ck_every = every;
    return 0;
}

int rkhevi_window_tl(struct state *state_init_dot, struct state *state_final_dot)
{
    if (check_ready(nullptr)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    Context::SubBuffers &b = c->sub;
    if (upload_state(state_init_dot, &b.st)) return -1;
    if (adj_window_tl(c, b.st.dev, b.sn.dev)) return -1;
    return adj_download(state_final_dot, &b.sn, b.sn.dev);
}

int rkhevi_window_backward(struct state *state_final_bar, struct state *state_init_bar)
{
    if (check_ready(nullptr)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    Context::SubBuffers &b = c->sub;
    if (upload_state(state_final_bar, &b.st)) return -1;
    if (adj_window_backward(c, b.st.dev, b.sn.dev)) return -1;
    return adj_download(state_init_bar, &b.sn, b.sn.dev);
}

int game_gpu_sfc_pressure_objective(struct state *state, const double *weights, double *objective,
                                    struct state *state_bar)
{
    if (check_ready(nullptr)) return -1;
    Context *c = ctx();
    if (c->n_const != 1 && c->n_const != 6)
        return fail("game_gpu_sfc_pressure_objective: dry build or moist build of six constituents");
    if (ensure_sub_buffers(c)) return -1;
    Context::SubBuffers &b = c->sub;
    double *w = adj_obj_weights(c);
    if (!w) return -1;
    if (upload_state(state, &b.st)) return -1;
    if (upload_field(weights, w, c->map_s, c->nc, c->nc)) return -1;
    if (adj_objective(c, &b.st, w, objective, state_bar ? b.sn.dev : nullptr)) return -1;
    if (state_bar) return adj_download(state_bar, &b.sn, b.sn.dev);
    return finish();
}

/* ------------------------------------------------- operator adjoints
 * Host arrays in the reference layout.  Bars of a forward's inputs are
 * accumulated (x_bar += (dy/dx)^T y_bar); bars of its outputs are read. */
static int up(const double *h, double *d, const int *map, long long n) { return upload_field(h, d, map, n, n); }
static int down(double *h, const double *d, const int *map, long long n) { return download_field(h, d, map, n, n, 0, n); }

int grad_adj(double *out_field_bar, double *in_field_bar, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    double *ob = c->sub.vec[0], *ib = c->sub.vec[1];
    if (up(out_field_bar, ob, c->map_vec, c->nv) || up(in_field_bar, ib, c->map_s, c->ns)) return -1;
    op_grad_adj(c, ob, ib);
    if (down(in_field_bar, ib, c->map_s, c->ns)) return -1;
    return finish();
}

int divv_h_adj(double *out_field_bar, double *in_field_bar, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    double *ob = c->sub.vec[0], *ib = c->sub.vec[1];
    if (up(out_field_bar, ob, c->map_s, c->ns) || up(in_field_bar, ib, c->map_vec, c->nv)) return -1;
    op_divv_adj(c, ob, ib);
    if (down(in_field_bar, ib, c->map_vec, c->nv)) return -1;
    return finish();
}

int scalar_times_vector_adj(double *scalar_field, double *vector_field, double *out_field_bar,
                            double *scalar_field_bar, double *vector_field_bar, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    double **v = c->sub.vec;
    if (up(scalar_field, v[0], c->map_s, c->ns) || up(vector_field, v[1], c->map_vec, c->nv)
        || up(out_field_bar, v[2], c->map_vec, c->nv) || up(scalar_field_bar, v[3], c->map_s, c->ns)
        || up(vector_field_bar, v[4], c->map_vec, c->nv))
        return -1;
    op_stv_adj(c, v[0], v[1], v[2], v[3], v[4]);
    if (down(scalar_field_bar, v[3], c->map_s, c->ns) || down(vector_field_bar, v[4], c->map_vec, c->nv)) return -1;
    return finish();
}

int inner_product_adj(double *in_field_0, double *in_field_1, double *out_field_bar, double *in_field_0_bar,
                      double *in_field_1_bar, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    double **v = c->sub.vec;
    if (up(in_field_0, v[0], c->map_vec, c->nv) || up(in_field_1, v[1], c->map_vec, c->nv)
        || up(out_field_bar, v[2], c->map_s, c->ns) || up(in_field_0_bar, v[3], c->map_vec, c->nv)
        || up(in_field_1_bar, v[4], c->map_vec, c->nv))
        return -1;
    op_inner_adj(c, v[0], v[1], v[2], v[3], v[4]);
    if (down(in_field_0_bar, v[3], c->map_vec, c->nv) || down(in_field_1_bar, v[4], c->map_vec, c->nv)) return -1;
    return finish();
}

int calc_pot_vort_adj(double *velocity_field, double *density_field, double *pot_vort_bar,
                      double *velocity_field_bar, double *density_field_bar, struct grid *grid,
                      struct dualgrid *dualgrid)
{
    (void)dualgrid;
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    double **v = c->sub.vec;
    double *wind = v[0], *rho = v[1], *rel = v[2], *pv = v[3], *pvb = v[4], *zero_u = v[5], *wb = v[6], *rb = v[7],
           *trib = v[8];
    if (up(velocity_field, wind, c->map_vec, c->nv) || up(density_field, rho, c->map_s, c->ns)) return -1;
    op_rel_vort(c, wind, c->sub.tri, rel);
    op_pot_vort(c, rel, rho, pv);
    if (up(pot_vort_bar, pvb, c->map_curl, c->ncurl) || up(velocity_field_bar, wb, c->map_vec, c->nv)
        || up(density_field_bar, rb, c->map_s, c->ns))
        return -1;
    CK(cudaMemsetAsync(zero_u, 0, (size_t)c->nl * c->ne * sizeof(double), c->stream));
    CK(cudaMemsetAsync(trib, 0, (size_t)c->nl * c->nt * sizeof(double), c->stream));
    op_pot_vort_adj(c, wind, rho, pv, pvb, zero_u, wb, rb, trib);
    if (down(velocity_field_bar, wb, c->map_vec, c->nv) || down(density_field_bar, rb, c->map_s, c->ns)) return -1;
    return finish();
}

int vorticity_flux_adj(double *mass_flux_density, double *pot_vorticity, double *out_field_bar,
                       double *mass_flux_density_bar, double *pot_vorticity_bar, struct grid *grid,
                       struct dualgrid *dualgrid)
{
    (void)dualgrid;
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    double **v = c->sub.vec;
    if (up(mass_flux_density, v[0], c->map_vec, c->nv) || up(pot_vorticity, v[1], c->map_curl, c->ncurl)
        || up(out_field_bar, v[2], c->map_vec, c->nv) || up(mass_flux_density_bar, v[3], c->map_vec, c->nv)
        || up(pot_vorticity_bar, v[4], c->map_curl, c->ncurl))
        return -1;
    op_vflux_adj(c, v[0], v[1], v[2], v[3], v[4]);
    if (down(mass_flux_density_bar, v[3], c->map_vec, c->nv) || down(pot_vorticity_bar, v[4], c->map_curl, c->ncurl))
        return -1;
    return finish();
}

int three_band_solver_ver_waves_adj(struct state *state_old, struct state *state_new, struct state *state_tendency,
                                    struct diagnostics *diagnostics, struct forcings *forcings, struct config *config,
                                    double delta_t, struct grid *grid, int rk_step, struct state *state_old_bar,
                                    struct state *state_new_bar, struct state *state_tendency_bar)
{
    (void)diagnostics;
    (void)forcings;
    if (check_ready(grid)) return -1;
    if (check_config(config)) return -1;
    Context *c = ctx();
    if (c->n_const != 1) return fail("three_band_solver_ver_waves_adj: dry build only (MOISTURE_ON = 0)");
    if (ensure_sub_buffers(c)) return -1;
    Context::SubBuffers &b = c->sub;
    if (upload_state(state_old, &b.so) || upload_state(state_new, &b.sn) || upload_state(state_tendency, &b.st))
        return -1;
    if (upload_state(state_old_bar, &b.bso) || upload_state(state_new_bar, &b.bsn)
        || upload_state(state_tendency_bar, &b.bst))
        return -1;
    StepParams p = params_from_config(c, config, delta_t);
    if (adj_waves_backward(c, &b.so, &b.sn, &b.st, p, rk_step, &b.bso, &b.bsn, &b.bst)) return -1;
    if (download_state(state_old_bar, &b.bso, 31) || download_state(state_new_bar, &b.bsn, 31)
        || download_state(state_tendency_bar, &b.bst, 31))
        return -1;
    return finish();
}

int divv_h_tracer_adj(double *in_field, double *density_field, double *wind_field, double *out_field_bar,
                      double *in_field_bar, double *density_field_bar, double *wind_field_bar, struct grid *grid)
{
    (void)in_field; /* the operator is linear in it */
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    if (ensure_sub_buffers(c)) return -1;
    double **v = c->sub.vec;
    if (up(density_field, v[0], c->map_s, c->ns) || up(wind_field, v[1], c->map_vec, c->nv)
        || up(out_field_bar, v[2], c->map_s, c->ns) || up(in_field_bar, v[3], c->map_vec, c->nv)
        || up(density_field_bar, v[4], c->map_s, c->ns) || up(wind_field_bar, v[5], c->map_vec, c->nv))
        return -1;
    op_divv_tracer_adj(c, v[0], v[1], v[2], v[3], v[4], v[5]);
    if (down(in_field_bar, v[3], c->map_vec, c->nv) || down(density_field_bar, v[4], c->map_s, c->ns)
        || down(wind_field_bar, v[5], c->map_vec, c->nv))
        return -1;
    return finish();
}

int three_band_solver_gen_densities_adj(struct state *state_old, struct state *state_new,
                                        struct state *state_tendency, struct diagnostics *diagnostics,
                                        struct irreversible_quantities *irrev, struct config *config, double delta_t,
                                        int rk_step, struct grid *grid, struct state *state_old_bar,
                                        struct state *state_new_bar, struct state *state_tendency_bar,
                                        struct diagnostics *diagnostics_bar,
                                        struct irreversible_quantities *irrev_bar)
{
    (void)irrev;
    if (check_ready(grid)) return -1;
    if (check_config(config)) return -1;
    Context *c = ctx();
    if (c->n_const <= 1) return finish();
    if (ensure_sub_buffers(c)) return -1;
    Context::SubBuffers &b = c->sub;
    double *t_b = b.vec[0], *sed_b = b.vec[1];
    if (upload_state(state_old, &b.so) || upload_state(state_new, &b.sn) || upload_state(state_tendency, &b.st))
        return -1;
    if (upload_state(state_old_bar, &b.bso) || upload_state(state_new_bar, &b.bsn)
        || upload_state(state_tendency_bar, &b.bst))
        return -1;
    if (up_scal(diagnostics, GAME_DIAGNOSTICS, "temperature", b.temperature)) return -1;
    if (up_scal(diagnostics_bar, GAME_DIAGNOSTICS, "temperature", t_b)) return -1;
    if (rk_step == 0 && up_scal(irrev_bar, GAME_IRREV, "condensates_sediment_heat", sed_b)) return -1;
    StepParams p = params_from_config(c, config, delta_t);
    if (adj_gen_densities(c, p, &b.so, &b.sn, &b.st, b.temperature, rk_step, sed_b, &b.bso, &b.bsn, &b.bst, t_b))
        return fail("three_band_solver_gen_densities_adj: more than 256 layers or a launch error");
    if (download_state(state_old_bar, &b.bso, 1 | 16) || download_state(state_new_bar, &b.bsn, 1 | 16)
        || download_state(state_tendency_bar, &b.bst, 1))
        return -1;
    if (down_scal(diagnostics_bar, GAME_DIAGNOSTICS, "temperature", t_b)) return -1;
    if (rk_step == 0 && down_scal(irrev_bar, GAME_IRREV, "condensates_sediment_heat", sed_b)) return -1;
    return finish();
}

/* ------------------------------------------------------ output diagnostics
 * The operators only output uses (host-in/host-out) and the fields of
 * write_out (output_f64.cu). */
int interpolate_to_ll(double in_field[], double out_field[], struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    double *f = c->dev_tmp[0];
    if (upload_field(in_field, f, c->map_s, c->nc, c->nc)) return -1;
    if (output_latlon_host(c, f, out_field)) return -1;
    return finish();
}

int edges_to_cells_lowest_layer(double in_field[], double out_field[], struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    double *e = c->dev_tmp[1], *o = c->dev_tmp[0];
    if (output_upload_edges(c, in_field, 1, e)) return -1;
    op_edges_to_cells_lowest(c, e, o);
    if (download_field(out_field, o, c->map_s, c->nc, c->nc, 0, c->nc)) return -1;
    return finish();
}

int epv_diagnostics(double *pot_vort, struct state *state, double *epv, struct grid *grid, struct dualgrid *dualgrid)
{
    if (check_ready(grid)) return -1;
    if (dualgrid != g_bound.dualgrid) return fail("dualgrid pointer differs from the one given to game_gpu_init");
    Context *c = ctx();
    double *pv = c->dev_tmp[1], *tvp = c->dev_tmp[2], *o = c->dev_tmp[0];
    double *host_tvp = member<double>(state, GAME_STATE, "theta_v_pert");
    if (upload_field(pot_vort, pv, c->map_curl, c->ncurl, c->ncurl)) return -1;
    if (upload_field(host_tvp, tvp, c->map_s, c->ns, c->ns)) return -1;
    DState s{};
    s.theta_v_pert = tvp;
    if (op_epv(c, pv, s, o)) return -1;
    if (download_field(epv, o, c->map_s, c->ns, c->ns, 0, c->ns)) return -1;
    /* the top layer of theta_v_pert as the reference leaves it */
    if (download_field(host_tvp, tvp, c->map_s, c->ns, c->ns, 0, c->nc)) return -1;
    return finish();
}

int inner_product_tangential(double *in_field_0, double *in_field_1, double *out_field, struct grid *grid,
                             struct dualgrid *dualgrid)
{
    if (check_ready(grid)) return -1;
    if (dualgrid != g_bound.dualgrid) return fail("dualgrid pointer differs from the one given to game_gpu_init");
    Context *c = ctx();
    double *a = c->dev_tmp[1], *b = c->dev_tmp[2], *o = c->dev_tmp[0];
    if (upload_field(in_field_0, a, c->map_vec, c->nv, c->nv)) return -1;
    if (upload_field(in_field_1, b, c->map_vec, c->nv, c->nv)) return -1;
    op_inner_product_tangential(c, a, b, o);
    if (download_field(out_field, o, c->map_s, c->ns, c->ns, 0, c->ns)) return -1;
    return finish();
}

int calc_uv_at_edge(double *in_field, double *out_field_u, double *out_field_v, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    const long long off = (long long)(c->nl + 1) * c->nc;
    double *in = c->dev_tmp[1], *u = c->dev_tmp[2], *v = c->dev_tmp[3];
    if (upload_field(in_field, in, c->map_vec, c->nv, c->nv)) return -1;
    if (vec_op_prologue(out_field_u, u) || vec_op_prologue(out_field_v, v)) return -1;
    op_uv_at_edge(c, in + off, u + off, v + off);
    if (download_field(out_field_u, u, c->map_vec, c->nv, c->nv, 0, c->nv)) return -1;
    if (download_field(out_field_v, v, c->map_vec, c->nv, c->nv, 0, c->nv)) return -1;
    return finish();
}

int curl_field_to_cells(double *in_field, double *out_field, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    double *in = c->dev_tmp[1], *o = c->dev_tmp[0];
    if (upload_field(in_field, in, c->map_curl, c->ncurl, c->ncurl)) return -1;
    op_curl_to_cells(c, in + (long long)(c->nl + 1) * c->ne, o);
    if (download_field(out_field, o, c->map_s, c->ns, c->ns, 0, c->ns)) return -1;
    return finish();
}

int edges_to_cells(double *in_field, double *out_field, struct grid *grid)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    double *in = c->dev_tmp[1], *o = c->dev_tmp[0];
    if (upload_field(in_field, in, c->map_vec, c->nv, c->nv)) return -1;
    op_edges_to_cells(c, in + (long long)(c->nl + 1) * c->nc, o);
    if (download_field(out_field, o, c->map_s, c->ns, c->ns, 0, c->ns)) return -1;
    return finish();
}

int game_gpu_write_out_fields(struct state *state_write_out, double wind_h_lowest_layer_array[],
                              int min_no_of_output_steps, struct diagnostics *diagnostics,
                              struct forcings *forcings, struct grid *grid, struct config *config,
                              struct game_gpu_output_fields *native, struct game_gpu_output_fields *latlon)
{
    if (check_ready(grid)) return -1;
    Context *c = ctx();
    if (latlon && !c->og.ll_ok) return fail("lat-lon output: the grid's latlon_interpol_indices are out of range");
    StateMirror *m = diag_mirror(state_write_out);
    if (!m) return -1;
    OutParams p{};
    p.n_cond = c->n_cond;
    p.moist = c->moist;
    p.n_const = c->n_const;
    p.prog_soil_temp = *member<int>(config, GAME_CONFIG, "prog_soil_temp");
    p.gust_turbulence = *member<int>(config, GAME_CONFIG, "sfc_sensible_heat_flux") == 1
                        || *member<int>(config, GAME_CONFIG, "sfc_phase_trans") == 1
                        || *member<int>(config, GAME_CONFIG, "pbl_scheme") == 1;
    p.n_wind_steps = min_no_of_output_steps;
    p.snow_velocity = *member<double>(config, GAME_CONFIG, "snow_velocity");
    p.rain_velocity = *member<double>(config, GAME_CONFIG, "rain_velocity");
    OutHost h{};
    h.sfc_sw_in = member<double>(forcings, GAME_FORCINGS, "sfc_sw_in");
    h.temperature_soil = member<double>(state_write_out, GAME_STATE, "temperature_soil");
    h.monin_obukhov_length = member<double>(diagnostics, GAME_DIAGNOSTICS, "monin_obukhov_length");
    h.roughness_velocity = member<double>(diagnostics, GAME_DIAGNOSTICS, "roughness_velocity");
    h.v_squared = member<double>(diagnostics, GAME_DIAGNOSTICS, "v_squared");
    h.wind_lowest = wind_h_lowest_layer_array;
    if (output_run(c, m, p, h, native, latlon)) return -1;
    if (finish()) return -1;
    if (!c->resident) {
        /* write_out leaves the top layer of theta_v_pert rounded as
         * (x + theta_v_bg) - theta_v_bg (spatial_ops_for_output.c:113-122) */
        double *tvp = member<double>(state_write_out, GAME_STATE, "theta_v_pert");
        const double *bg = member<double>(grid, GAME_GRID, "theta_v_bg");
        for (int i = 0; i < c->nc; ++i) {
            const double x = tvp[i] + bg[i];
            tvp[i] = x - bg[i];
        }
    }
    return 0;
}

int game_gpu_record_wind_lowest(struct state *state, int slot)
{
    if (check_ready(nullptr)) return -1;
    Context *c = ctx();
    StateMirror *m = diag_mirror(state);
    if (!m) return -1;
    if (output_record_wind(c, m, slot)) return -1;
    return finish();
}

/* ------------------------------------------------ write_out, write_out_integral
 * The reference's output entry points (src/io/io.h:10-11): the fields on the
 * GPU, the files on the host.  Config_io (src/game_types.h:240-258) has no
 * size that depends on the grid, so its layout is fixed. */
struct ConfigIoLayout {
    int grib_output_switch, netcdf_output_switch, pressure_level_output_switch, model_level_output_switch,
        surface_output_switch, write_out_interval, write_out_integrals, year, month, day, hour;
    char run_id[100], month_string[3], day_string[3], hour_string[3];
    int ideal_input_id;
};

int write_out(struct state *state_write_out, double wind_h_lowest_layer_array[], int min_no_of_output_steps,
              double t_init, double t_write, struct diagnostics *diagnostics, struct forcings *forcings,
              struct grid *grid, struct dualgrid *dualgrid, struct config_io *config_io, struct config *config,
              struct irreversible_quantities *irrev)
{
    if (check_ready(grid)) return -1;
    if (dualgrid != g_bound.dualgrid) return fail("dualgrid pointer differs from the one given to game_gpu_init");
    const ConfigIoLayout *io = (const ConfigIoLayout *)config_io;
    if (io->grib_output_switch == 1)
        return fail("write_out: GRIB output is not available in this library (set grib_output_switch = 0; the "
                    "lat-lon fields the GRIB path writes come from game_gpu_write_out_fields)");
    Context *c = ctx();
    const long long nc = c->nc, ns = c->ns, nv = c->nv;
    const int t_rel = (int)(t_write - t_init);
    const bool netcdf = io->netcdf_output_switch == 1;
    const bool surface = netcdf && io->surface_output_switch == 1;
    const bool plevels = netcdf && io->pressure_level_output_switch == 1;
    const bool model = (io->model_level_output_switch == 1 && netcdf)
                       || (io->ideal_input_id == -1 && t_rel == *member<int>(config, GAME_CONFIG, "time_to_next_analysis"));
    /* the fields, reference order */
    std::vector<double> sf(11 * nc), ml(6 * ns), pl(7 * 6 * nc);
    game_gpu_output_fields nat{};
    double *sp[11];
    for (int k = 0; k < 11; ++k) sp[k] = sf.data() + k * nc;
    nat.mslp = sp[0]; nat.surface_p = sp[1]; nat.t2 = sp[2]; nat.tcdc = sp[3]; nat.rprate = sp[4];
    nat.sprate = sp[5]; nat.cape = sp[6]; nat.sfc_sw_down = sp[7]; nat.u10 = sp[8]; nat.v10 = sp[9];
    nat.gusts = sp[10];
    nat.temperature = ml.data(); nat.rh = ml.data() + ns; nat.rel_vort = ml.data() + 2 * ns;
    nat.divv_h = ml.data() + 3 * ns; nat.u = ml.data() + 4 * ns; nat.v = ml.data() + 5 * ns;
    std::vector<double> epv(ns), pressure(ns);
    nat.epv = epv.data(); nat.pressure = pressure.data();
    double *pp[7];
    for (int k = 0; k < 7; ++k) pp[k] = pl.data() + k * 6 * nc;
    nat.geopotential_height = pp[0]; nat.t_pl = pp[1]; nat.rh_pl = pp[2]; nat.epv_pl = pp[3]; nat.u_pl = pp[4];
    nat.v_pl = pp[5]; nat.rel_vort_pl = pp[6];
    if (game_gpu_write_out_fields(state_write_out, wind_h_lowest_layer_array, min_no_of_output_steps, diagnostics,
                                  forcings, grid, config, &nat, nullptr))
        return -1;
    static const double levels[6] = {20000, 30000, 50000, 70000, 85000, 92500};
    ncw_output o{};
    o.n_cells = nc; o.n_scalars = ns; o.n_vectors = nv; o.n_densities = (long long)c->n_const * ns;
    o.n_h_vectors = (long long)c->nl * c->ne; o.n_v_vectors = (long long)(c->nl + 1) * nc; o.n_curl = c->ncurl;
    o.n_soil = (long long)c->dims.n_soil * nc;
    o.mslp = nat.mslp; o.surface_p = nat.surface_p; o.t2 = nat.t2; o.tcdc = nat.tcdc; o.rprate = nat.rprate;
    o.sprate = nat.sprate; o.cape = nat.cape; o.sfc_sw_down = nat.sfc_sw_down; o.u10 = nat.u10; o.v10 = nat.v10;
    o.gusts = nat.gusts; o.pressure_levels = levels;
    o.geopotential_height = nat.geopotential_height; o.t_pl = nat.t_pl; o.rh_pl = nat.rh_pl; o.epv_pl = nat.epv_pl;
    o.u_pl = nat.u_pl; o.v_pl = nat.v_pl; o.rel_vort_pl = nat.rel_vort_pl;
    o.temperature = nat.temperature; o.rh = nat.rh; o.rel_vort = nat.rel_vort; o.divv_h = nat.divv_h;
    /* the prognostic state, the soil temperature and the TKE as they are at
     * this point: the device copies where the library holds them */
    std::vector<double> state_copy, tke_copy;
    const double *rho = member<double>(state_write_out, GAME_STATE, "rho");
    const double *wind = member<double>(state_write_out, GAME_STATE, "wind");
    const double *t_soil = member<double>(state_write_out, GAME_STATE, "temperature_soil");
    const double *tke = member<double>(irrev, GAME_IRREV, "tke");
    if (model && c->resident) {
        StateMirror *m = mirror(state_write_out, 0);
        if (!m) return fail("resident mode: this State has no device mirror (game_gpu_sync_to_device it first)");
        /* a host image of the State block, filled from the mirror */
        state_copy.resize((size_t)c->state_len);
        const size_t off = c->off_state_rho;
        std::vector<char> img(off + state_copy.size() * sizeof(double));
        if (download_state(img.data(), m, 1 | 16 | 32) || finish()) return -1;
        std::memcpy(state_copy.data(), img.data() + off, state_copy.size() * sizeof(double));
        rho = state_copy.data();
        wind = state_copy.data() + (c->n_const + 3) * ns;
        t_soil = state_copy.data() + (c->n_const + 3) * ns + nv;
    }
    if (model && g_bound.diff_imported && c->dbuf) {
        tke_copy.resize((size_t)ns);
        if (download_field(tke_copy.data(), c->dbuf->tke, c->map_s, ns, ns, 0, ns) || finish()) return -1;
        tke = tke_copy.data();
    }
    o.densities = rho; o.wind = wind; o.t_soil = t_soil; o.tke = tke;
    char path[320];
    if (surface) {
        snprintf(path, sizeof path, "%s+%ds_surface.nc", io->run_id, t_rel);
        if (ncw_write_surface(path, &o)) return fail(std::string("write_out: ") + ncw_last_error());
    }
    if (plevels) {
        snprintf(path, sizeof path, "%s+%ds_pressure_levels.nc", io->run_id, t_rel);
        if (ncw_write_pressure_levels(path, &o)) return fail(std::string("write_out: ") + ncw_last_error());
    }
    if (model) {
        snprintf(path, sizeof path, "%s+%ds.nc", io->run_id, t_rel);
        if (ncw_write_model_levels(path, &o)) return fail(std::string("write_out: ") + ncw_last_error());
    }
    return 0;
}

int write_out_integral(struct state *state_write_out, double time_since_init, struct grid *grid,
                       struct dualgrid *dualgrid, struct diagnostics *diagnostics, int integral_id)
{
    (void)diagnostics;
    if (check_ready(grid)) return -1;
    if (dualgrid != g_bound.dualgrid) return fail("dualgrid pointer differs from the one given to game_gpu_init");
    double r[INTEGRAL_MAX_FIELDS];
    if (game_gpu_write_out_integral(state_write_out, integral_id, r)) return -1;
    static const char *names[3] = {"masses", "potential_temperature_density", "energy"};
    FILE *f = std::fopen(names[integral_id], "a");
    if (!f) return fail(std::string("write_out_integral: cannot open ") + names[integral_id]);
    /* write_output.c:1539-1592: "%lf" fields, tab-separated */
    if (integral_id == 0) {
        std::fprintf(f, "%lf\t", time_since_init);
        for (int k = 0; k < ctx()->n_const; ++k) std::fprintf(f, k == ctx()->n_const - 1 ? "%lf\n" : "%lf\t", r[k]);
    } else if (integral_id == 1) {
        std::fprintf(f, "%lf\t%lf\n", time_since_init, r[0]);
    } else {
        std::fprintf(f, "%lf\t%lf\t%lf\t%lf\n", time_since_init, r[0], r[1], r[2]);
    }
    std::fclose(f);
    return 0;
}

/* io.h:12 -> write_output.c:1670-1677: the State at t_write by linear
 * interpolation in time between state_0 at t_0 and state_p1 at t_p1 */
int interpolation_t(struct state *state_0, struct state *state_p1, struct state *state_write, double t_0,
                    double t_p1, double t_write, struct grid *grid)
{
    const double weight_p1 = (t_write - t_0) / (t_p1 - t_0);
    const double weight_0 = 1.0 - weight_p1;
    return linear_combine_two_states(state_0, state_p1, state_write, weight_0, weight_p1, grid);
}

}  // extern "C"
