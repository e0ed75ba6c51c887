/*
 * Library context: grid dimensions, struct layout, SFC permutation, device
 * tables, device mirrors of the caller's State structs and the work arrays
 * of the step.  One context per process (the reference runs one model per
 * process, src/coordinator.c:27).
 */
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "devgrid.cuh"
#include "layout.h"

struct game_gpu_health; /* include/game_gb300.h */

namespace game {

struct AdjState;

/* device buffer owned by the context */
struct DBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

/* precision mode of the step */
enum Precision { PREC_FP64 = 0, PREC_MIXED = 1 };

/* work arrays of the step in the horizontal precision R */
template <typename R>
struct Work {
    R *P_h, *P_v;           /* pressure-gradient sum nl + l   [L][Ne], [L+1][Nc] */
    R *pg_old_h;            /* previous step's pressure gradient, horizontal part */
    R *pvt_h, *pvt_v;       /* vorticity flux (pot_vort_tend) */
    R *v2g_h, *v2g_v;       /* kinetic-energy gradient */
    R *flux_h, *flux_v;     /* mass flux density */
    R *zh, *zv;             /* potential vorticity: tangential [L+1][Ne], rhombus [L][Ne] */
    R *tri_vort;            /* [L][Nt] */
    R *v2;                  /* kinetic energy [L][Nc] */
};

struct StateMirror {
    double *dev = nullptr;  /* device layout, (C+3)*S + Vt doubles */
    DState ds{};
};

struct Context {
    game_dims dims{};
    int nc = 0, ne = 0, nt = 0, nl = 0, n_oro = 0, n_const = 0, n_cond = 0, moist = 0;
    long long ns = 0, nv = 0, ndv = 0, ncurl = 0, state_len = 0;
    double radius = 0.0, toa = 0.0;
    int precision = PREC_FP64;
    int resident = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;                   /* second branch of the step */
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr; /* fork / join of the branches */
    /* recorded by the step once the tendency is final (after substage 1's
     * scalar tendencies), and after its copy to a pinned host State */
    cudaEvent_t ev_tend = nullptr, ev_tend_copied = nullptr;

    /* host struct offsets (bytes) */
    size_t off_grid_z_vector = 0;
    size_t off_state_rho = 0, off_state_wind = 0, off_state_rhotheta = 0, off_state_theta = 0, off_state_exner = 0;

    /* permutations: new -> old and old -> new */
    std::vector<int> c_n2o, c_o2n, e_n2o, e_o2n, t_n2o, t_o2n;

    /* device tables */
    HGrid<double> hg64{};
    HGrid<float> hg32{};
    VGrid vg{};
    std::vector<DBuf> owned;

    /* index maps device position -> reference position */
    int *map_state = nullptr;   /* state block, length state_len */
    int *imap_state = nullptr;  /* its inverse: reference position -> device position */
    int *map_s = nullptr;       /* scalar field, length S */
    int *map_vec = nullptr;     /* vector field: [w (L+1)*Nc][u L*Ne], length Vt */
    int *map_curl = nullptr;    /* curl field: [zh (L+1)*Ne][zv L*Ne], length NCURL */
    int *map_tri = nullptr;     /* triangle field, length L*Nt */
    double *staging = nullptr;  /* reference-layout staging, max field length */
    size_t staging_len = 0;
    double *dev_tmp[4] = {nullptr, nullptr, nullptr, nullptr}; /* device-layout scratch fields for operators */

    /* persistent step fields (device layout) */
    double *temperature = nullptr;    /* [L][Nc] */
    double *theta = nullptr;          /* rho*theta_v / rho_gas, [L][Nc] */
    double *pt_rates = nullptr;       /* [5][L][Nc] (moist) */
    double *pt_heat = nullptr;        /* [L][Nc] */
    double *sed_heat = nullptr;       /* [L][Nc] */
    double *cp_ice = nullptr, *cp_water = nullptr; /* c_p of ice / liquid water at T, [L][Nc] */
    /* mixed path: FP32 shadow of state_new and FP32 copies of per-step fields */
    float *shadow = nullptr;          /* [rho C*S][rhotheta S][theta' S][Pi' S][w (L+1)Nc][u L*Ne] */
    float *theta32 = nullptr, *cp32_ice = nullptr, *cp32_water = nullptr;
    /* mixed path: pressure-gradient factors of the step start per (layer,
     * cell): Pi', c_p theta_v, c_p theta_v', rho_gas / rho_total (k_pg_cells) */
    float4 *pg_cell = nullptr;
    double *gravity_potential = nullptr; /* [L][Nc] */
    /* global integrals: per-block (hi, lo) partial sums, one counter and one
     * result per field, and three energy-density fields [3][L][Nc] */
    double *red_partials = nullptr;
    unsigned *red_counters = nullptr;
    double *red_out = nullptr;
    double *energy_buf = nullptr;
    int temperature_from_step = 0;   /* temperature holds T(state_old) of the last step */
    double *inv_vol = nullptr;        /* 1 / volume [L][Nc] (mixed path) */
    double *inv_area_v = nullptr;     /* 1 / area of the interfaces [L+1][Nc] (mixed path) */
    /* vertical sound-wave solver: per-layer and per-interface work */
    double *wv_layer = nullptr;       /* 8 x [L][Nc] */
    double *wv_rows = nullptr;        /* 7 x [L-1][Nc] */
    Work<double> w64{};
    Work<float> w32{};

    std::map<const void *, StateMirror> states;

    /* adjoint / tangent-linear window state (adj_f64.cu), created on first use;
     * the windows store every adj_ck_every-th step start */
    struct AdjState *adj = nullptr;
    int adj_ck_every = 1;
    void (*adj_release)(Context *) = nullptr;

    /* private buffers of the sub-step entry points (three_band_solver_*,
     * *_tendencies_expl, ...), allocated on their first call; never the
     * mirrors or the lagged fields of the device-resident step */
    struct SubBuffers {
        bool ready = false;
        StateMirror so, sn, st;
        StateMirror bso, bsn, bst; /* bars of the adjoint entry points */
        double *vec[10] = {}; /* each max(Vt, curl field) */
        double *temperature = nullptr, *cp_ice = nullptr, *cp_water = nullptr, *theta = nullptr;
        double *pt_rates = nullptr; /* 5 S */
        double *pt_heat = nullptr, *sed_heat = nullptr, *decel = nullptr, *v2 = nullptr, *tri = nullptr;
    } sub;

    /* CUDA graphs of the device-side step, keyed by every value the launches
     * capture: the step parameters (time step, config values, first-step
     * flag), the precision and the three state mirrors */
    struct GraphKey {
        StepParams p;
        int prec, solver;
        const void *so, *sn, *st;
        bool operator<(const GraphKey &o) const;
    };
    struct GraphEntry {
        cudaGraphExec_t exec;
        int launches; /* kernels in the graph */
    };
    std::map<GraphKey, GraphEntry> graphs;
    /* Klemp damping coefficient of every inner interface [L-1][Nc] and
     * 1 / (1 + dt * coefficient) for the values in damp_key (start height,
     * maximum coefficient, dt) */
    double *damp_dc = nullptr, *damp_inv = nullptr;
    float2 *damp_inv_df = nullptr; /* damp_inv as double-float pairs */
    double damp_key[3] = {-1.0, -1.0, -1.0};
    /* grid terms of the mixed-path sound-wave rows [6][L-1][Nc] */
    double *wv_geo = nullptr;
    /* diffusion branch: tables, fields (allocated with the lagged fields on
     * their first import) and whether the tendencies add the irreversible
     * terms (set once a diffusion switch was on or an imported term was
     * nonzero) */
    DiffGrid<double> dg64{};
    DiffGrid<float> dg32{};
    DiffBufs *dbuf = nullptr;
    int irr_active = 0;
    /* Held-Suarez radiation: whether the reference's radiation blocks tile
     * the grid without overrunning radiation_tendency, and how many cells of
     * a layer (in reference numbering) they cover */
    int rad_blocks_ok = 0, rad_covered = 0;
    /* output diagnostics: tables, and work arrays allocated on first use */
    OutGrid og{};
    struct OutBufs *obuf = nullptr;
    void (*obuf_release)(Context *) = nullptr;
    int use_graphs = 1;
    int column_solver = 0; /* 0 by layer count, 1 per-thread sweeps, 2 warp cyclic reduction */
    /* arithmetic of the mixed path's vertical eliminations: 0 FP64, 1
     * double-float (default) */
    int double_float = 1;
    DfGrid dfg{};
    /* health check: device counters, and the step interval of the automatic
     * check in manage_rkhevi (0 off) */
    unsigned long long *health = nullptr;
    int health_every = 0;
    long long health_count = 0;
    int kernel_launches = 0;  /* launches of this library's kernels since the counter was reset */
    long long h2d_bytes = 0, d2h_bytes = 0;

    /* per-kernel timing: events around every step kernel while profiling */
    int profiling = 0;
    struct Pending {
        const char *name;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    std::map<std::string, std::pair<double, long long>> prof_totals; /* name -> (ms, launches) */
    std::vector<cudaEvent_t> user_events;
};

/* brackets one kernel launch with events while the context is profiling */
struct ProfScope {
    Context *c;
    cudaEvent_t b = nullptr;
    const char *name;
    ProfScope(Context *ctx_, const char *n) : c(ctx_), name(n)
    {
        if (c->profiling) {
            cudaEvent_t a;
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            cudaEventRecord(a, c->stream);
            c->pending.push_back({name, a, b});
        }
    }
    ~ProfScope()
    {
        if (c->profiling) cudaEventRecord(b, c->stream);
    }
};
int profile_flush(Context *c);

Context *ctx();
void set_error(const std::string &msg);
int fail(const std::string &msg);
#define CK(call)                                                                                \
    do {                                                                                        \
        cudaError_t _e = (call);                                                                \
        if (_e != cudaSuccess) return ::game::fail(std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

int init_context(int res_id, int n_layers, int moisture_on, const void *grid, const void *dualgrid);
int destroy_context();
StateMirror *mirror(const void *host_state, int create);
/* sets m.ds from m.dev (a state block of the context's layout) */
void set_mirror_views(Context *c, StateMirror &m);
int ensure_sub_buffers(Context *c);
int ensure_diff_buffers(Context *c);
/* the library's own pinned host allocations (game_gpu_host_alloc) and
 * their device addresses: States inside them are copied by kernels that read
 * and write host memory directly over NVLink-C2C */
void pinned_register(void *host, void *dev, size_t bytes);
void pinned_unregister(void *host);
int upload_state(const void *host_state, StateMirror *m);
int download_state(const void *host_state, StateMirror *m, int which_mask);
/* download_state on stream s for a State inside a pinned allocation of the
 * library (no staging array involved); 0 when the State is not in one */
int download_state_pinned(const void *host_state, StateMirror *m, int which_mask, cudaStream_t s);
int upload_field(const double *host, double *dev, const int *map, long long n, long long host_len);
int download_field(double *host, const double *dev, const int *map, long long n, long long host_len,
                   long long host_lo, long long host_hi);

/* the mixed step's lagged fields in its FP32 work arrays (aux.cu), from and to
 * device vector fields [w (L+1) Nc][u L Ne] of doubles: P the pressure
 * gradient nl + l, pvt the vorticity flux, v2g the kinetic-energy gradient,
 * flux the mass flux density (its levels 0 and L are read by the step);
 * P, pvt and v2g may be null on load (zeros) */
void aux_load_mixed(Context *c, const double *P, const double *pvt, const double *v2g, const double *flux);
void aux_store_mixed(Context *c, double *P, double *pvt, double *v2g);

/* health check of a State mirror (health.cu): 0 healthy, GAME_GPU_UNHEALTHY
 * with the message set, -1 on a CUDA error */
int check_mirror(Context *c, StateMirror *m, struct game_gpu_health *report, const char *what);

/* the step on device mirrors (step.cu templates) */
int run_step(Context *c, StateMirror *so, StateMirror *sn, StateMirror *st, const void *config, double dt);

/* gather / scatter kernels */
void launch_gather(double *dst, const double *src, const int *map, long long n, cudaStream_t s);
void launch_scatter(double *dst, const double *src, const int *map, long long n, cudaStream_t s);

}  // namespace game
