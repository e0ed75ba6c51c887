/*
 * Context set-up: reads the caller's Grid/Dualgrid (reference layout), builds
 * the Hilbert-curve renumbering of cells, edges and triangles, uploads the
 * renumbered tables in [slot][layer][entity] order, and owns the device
 * mirrors of State structs and the work arrays of the step.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <numeric>

#include "context.h"
#include "diag.h"

namespace game {

static Context *g_ctx = nullptr;
static std::string g_err;

Context *ctx() { return g_ctx; }
void set_error(const std::string &m) { g_err = m; }
int fail(const std::string &m)
{
    g_err = m;
    return -1;
}
const char *last_error() { return g_err.c_str(); }

bool Context::GraphKey::operator<(const GraphKey &o) const
{
    if (prec != o.prec) return prec < o.prec;
    if (solver != o.solver) return solver < o.solver;
    if (so != o.so) return so < o.so;
    if (sn != o.sn) return sn < o.sn;
    if (st != o.st) return st < o.st;
    /* StepParams is plain data, value-initialised before it is filled */
    return std::memcmp(&p, &o.p, sizeof(StepParams)) < 0;
}

/* ----------------------------------------------------------- gather/scatter */
__global__ void k_gather(double *dst, const double *src, const int *map, long long n)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[map[i]];
}
__global__ void k_scatter(double *dst, const double *src, const int *map, long long n)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[map[i]] = src[i];
}

/* State copies straight between the caller's pinned host struct and the
 * device mirror, without the staging array: host positions [lo, lo + n) are
 * read (upload) or written (download) in order, so the NVLink-C2C traffic is
 * sequential; the device side is addressed through the reference -> device
 * map of the state block. */
__global__ void k_state_from_host(double *dev, const double *host, const int *imap, long long lo, long long n)
{
    const long long j = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < lo + n) dev[imap[j]] = host[j];
}
__global__ void k_state_to_host(double *host, const double *dev, const int *imap, long long lo, long long n)
{
    const long long j = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < lo + n) host[j] = dev[imap[j]];
}

/* ------------------------------------------------- pinned host allocations
 * Allocations made through game_gpu_host_alloc, with the device address of
 * each: a State that lies entirely inside one of them is copied by the
 * kernels above. */
namespace {
struct PinnedAlloc {
    const char *host;
    char *dev;
    size_t bytes;
};
std::vector<PinnedAlloc> g_pinned;
}  // namespace

void pinned_register(void *host, void *dev, size_t bytes) { g_pinned.push_back({(const char *)host, (char *)dev, bytes}); }

void pinned_unregister(void *host)
{
    for (size_t i = 0; i < g_pinned.size(); ++i)
        if (g_pinned[i].host == host) {
            g_pinned.erase(g_pinned.begin() + (long)i);
            return;
        }
}

/* the device address of [host, host + bytes) if that range lies inside one
 * registered pinned allocation, else null */
static char *pinned_device_range(const void *host, size_t bytes)
{
    const char *h = (const char *)host;
    for (const PinnedAlloc &a : g_pinned)
        if (h >= a.host && h + bytes <= a.host + a.bytes) return a.dev + (h - a.host);
    return nullptr;
}
void launch_gather(double *dst, const double *src, const int *map, long long n, cudaStream_t s)
{
    if (n <= 0) return;
    k_gather<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dst, src, map, n);
    if (g_ctx) g_ctx->kernel_launches++;
}
void launch_scatter(double *dst, const double *src, const int *map, long long n, cudaStream_t s)
{
    if (n <= 0) return;
    k_scatter<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dst, src, map, n);
    if (g_ctx) g_ctx->kernel_launches++;
}

/* --------------------------------------------------------- Hilbert curve
 * 3-D Hilbert index of a point on the unit sphere (J. Skilling, "Programming
 * the Hilbert curve", AIP Conf. Proc. 707, 2004: axes -> transposed index). */
static uint64_t hilbert3(double x, double y, double z)
{
    const int bits = 20;
    uint32_t X[3];
    double v[3] = {x, y, z};
    for (int i = 0; i < 3; ++i) {
        double q = (v[i] + 1.0) * 0.5 * ((1u << bits) - 1);
        if (q < 0) q = 0;
        if (q > (double)((1u << bits) - 1)) q = (double)((1u << bits) - 1);
        X[i] = (uint32_t)q;
    }
    uint32_t M = 1u << (bits - 1), P, Q, t;
    for (Q = M; Q > 1; Q >>= 1) {
        P = Q - 1;
        for (int i = 0; i < 3; ++i) {
            if (X[i] & Q) {
                X[0] ^= P;
            } else {
                t = (X[0] ^ X[i]) & P;
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    for (int i = 1; i < 3; ++i) X[i] ^= X[i - 1];
    t = 0;
    for (Q = M; Q > 1; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1;
    for (int i = 0; i < 3; ++i) X[i] ^= t;
    uint64_t key = 0;
    for (int b = bits - 1; b >= 0; --b)
        for (int i = 0; i < 3; ++i) key = (key << 1) | ((X[i] >> b) & 1u);
    return key;
}

static std::vector<int> order_by_key(const std::vector<uint64_t> &key, int fixed_prefix)
{
    std::vector<int> n2o(key.size());
    std::iota(n2o.begin(), n2o.end(), 0);
    std::stable_sort(n2o.begin() + fixed_prefix, n2o.end(), [&](int a, int b) { return key[a] < key[b]; });
    return n2o;
}

static std::vector<int> invert(const std::vector<int> &n2o)
{
    std::vector<int> o2n(n2o.size());
    for (size_t i = 0; i < n2o.size(); ++i) o2n[n2o[i]] = (int)i;
    return o2n;
}

/* ------------------------------------------------------------ allocation */
template <typename T>
static T *dalloc(Context *c, size_t n)
{
    void *p = nullptr;
    if (n == 0) n = 1;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, n * sizeof(T));
    c->owned.push_back({p, n * sizeof(T)});
    return (T *)p;
}

template <typename T>
static T *dupload(Context *c, const std::vector<T> &h)
{
    T *p = dalloc<T>(c, h.size());
    if (p) cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return p;
}

template <typename T>
static std::vector<float> to_f32(const std::vector<T> &v)
{
    std::vector<float> r(v.size());
    for (size_t i = 0; i < v.size(); ++i) r[i] = (float)v[i];
    return r;
}

/* a double table uploaded in both precisions */
struct Dual {
    double *d = nullptr;
    float *f = nullptr;
};
static Dual dual_upload(Context *c, const std::vector<double> &h)
{
    Dual r;
    r.d = dupload(c, h);
    r.f = dupload(c, to_f32(h));
    return r;
}

/* --------------------------------------------------------------- set-up */
int init_context(int res_id, int n_layers, int moisture_on, const void *grid_p, const void *dual_p)
{
    if (g_ctx) destroy_context();
    Context *c = new Context();
    g_ctx = c;
    if (game_dims_init(&c->dims, res_id, n_layers, moisture_on) != 0) return fail("invalid (res_id, n_layers, moisture_on)");
    const game_dims &d = c->dims;
    c->nc = (int)d.n_cells;
    c->ne = (int)d.n_edges;
    c->nt = (int)d.n_triangles;
    c->nl = n_layers;
    c->n_const = d.n_constituents;
    c->n_cond = d.n_condensed;
    c->moist = moisture_on;
    c->ns = d.n_scalars;
    c->nv = d.n_vectors;
    c->ndv = d.n_dual_vectors;
    c->ncurl = d.n_curl;
    /* State members rho .. temperature_soil, contiguous in the reference struct */
    c->state_len = (long long)(c->n_const + 3) * c->ns + c->nv + (long long)d.n_soil * d.n_cells;
    if (n_layers > 256) return fail("more than 256 layers are not supported by the column solvers");
    const int NC = c->nc, NE = c->ne, NT = c->nt, L = n_layers;
    const long long VPL = (long long)NC + NE, DPL = (long long)NE + NT, NS = c->ns, NV = c->nv;

    auto gptr = [&](const char *name) -> const char * {
        size_t o = game_layout_offset(&c->dims, GAME_GRID, name);
        return o == (size_t)-1 ? nullptr : (const char *)grid_p + o;
    };
    auto dptr = [&](const char *name) -> const char * {
        size_t o = game_layout_offset(&c->dims, GAME_DUALGRID, name);
        return o == (size_t)-1 ? nullptr : (const char *)dual_p + o;
    };
#define GD(name) ((const double *)gptr(name))
#define GI(name) ((const int *)gptr(name))
#define DD(name) ((const double *)dptr(name))
#define DI(name) ((const int *)dptr(name))
    c->n_oro = *GI("no_of_oro_layers");
    c->radius = *GD("radius");
    c->toa = *GD("toa");
    if (c->n_oro < 1 || c->n_oro >= L) return fail("no_of_oro_layers must satisfy 1 <= no_of_oro_layers < NO_OF_LAYERS");
    c->off_grid_z_vector = game_layout_offset(&c->dims, GAME_GRID, "z_vector");
    c->off_state_rho = game_layout_offset(&c->dims, GAME_STATE, "rho");
    c->off_state_rhotheta = game_layout_offset(&c->dims, GAME_STATE, "rhotheta_v");
    c->off_state_theta = game_layout_offset(&c->dims, GAME_STATE, "theta_v_pert");
    c->off_state_exner = game_layout_offset(&c->dims, GAME_STATE, "exner_pert");
    c->off_state_wind = game_layout_offset(&c->dims, GAME_STATE, "wind");

    const int *from = GI("from_index"), *to = GI("to_index");
    const int *adj = GI("adjacent_vector_indices_h"), *adj_sign = GI("adjacent_signs_h");
    const int *trsk_i = GI("trsk_indices"), *trsk_m = GI("trsk_modified_curl_indices");
    const int *rh_i = GI("density_to_rhombi_indices");
    const int *dfrom = DI("from_index"), *dto = DI("to_index");
    const int *vi = DI("vorticity_indices_triangles"), *vs = DI("vorticity_signs_triangles");
    const double *lat = GD("latitude_scalar"), *lon = GD("longitude_scalar");
    /* ---- validation of every index table against its range */
    for (int e = 0; e < NE; ++e)
        if (from[e] < 0 || from[e] >= NC || to[e] < 0 || to[e] >= NC || dfrom[e] < 0 || dfrom[e] >= NT || dto[e] < 0
            || dto[e] >= NT)
            return fail("edge connectivity out of range");
    for (long long k = 0; k < 6LL * NC; ++k)
        if (adj[k] < 0 || adj[k] >= NE) return fail("adjacent_vector_indices_h out of range");
    for (long long k = 0; k < 10LL * NE; ++k)
        if (trsk_i[k] < 0 || trsk_i[k] >= NE || trsk_m[k] < 0 || trsk_m[k] >= NE) return fail("TRSK indices out of range");
    for (long long k = 0; k < 4LL * NE; ++k)
        if (rh_i[k] < 0 || rh_i[k] >= NC) return fail("density_to_rhombi_indices out of range");
    for (long long k = 0; k < 3LL * NT; ++k)
        if (vi[k] < 0 || vi[k] >= NE) return fail("vorticity_indices_triangles out of range");

    /* ---- Hilbert renumbering; pentagons keep 0..11 */
    std::vector<double> cx(NC), cy(NC), cz(NC);
    std::vector<uint64_t> key(NC);
    for (int i = 0; i < NC; ++i) {
        cx[i] = cos(lat[i]) * cos(lon[i]);
        cy[i] = cos(lat[i]) * sin(lon[i]);
        cz[i] = sin(lat[i]);
        key[i] = hilbert3(cx[i], cy[i], cz[i]);
    }
    c->c_n2o = order_by_key(key, N_PENT);
    c->c_o2n = invert(c->c_n2o);
    std::vector<uint64_t> ekey(NE);
    std::vector<double> ex(NE), ey(NE), ez(NE);
    for (int e = 0; e < NE; ++e) {
        ex[e] = 0.5 * (cx[from[e]] + cx[to[e]]);
        ey[e] = 0.5 * (cy[from[e]] + cy[to[e]]);
        ez[e] = 0.5 * (cz[from[e]] + cz[to[e]]);
        double n = sqrt(ex[e] * ex[e] + ey[e] * ey[e] + ez[e] * ez[e]);
        ekey[e] = hilbert3(ex[e] / n, ey[e] / n, ez[e] / n);
    }
    c->e_n2o = order_by_key(ekey, 0);
    c->e_o2n = invert(c->e_n2o);
    std::vector<uint64_t> tkey(NT);
    for (int t = 0; t < NT; ++t) {
        double x = 0, y = 0, z = 0;
        for (int j = 0; j < 3; ++j) {
            int e = vi[3 * t + j];
            x += ex[e]; y += ey[e]; z += ez[e];
        }
        double n = sqrt(x * x + y * y + z * z);
        tkey[t] = hilbert3(x / n, y / n, z / n);
    }
    c->t_n2o = order_by_key(tkey, 0);
    c->t_o2n = invert(c->t_n2o);
    const std::vector<int> &cn = c->c_n2o, &co = c->c_o2n, &en = c->e_n2o, &eo = c->e_o2n, &tn = c->t_n2o,
                           &to_ = c->t_o2n;

    /* ---- permuted tables */
    const double *nd = GD("normal_distance"), *vol = GD("volume"), *area = GD("area"), *zs = GD("z_scalar");
    const double *zv = GD("z_vector"), *gm = GD("gravity_m"), *slope = GD("slope"), *tbg = GD("theta_v_bg");
    const double *ebg = GD("exner_bg"), *ebgg = GD("exner_bg_grad"), *ipw = GD("inner_product_weights");
    const double *tw = GD("trsk_weights"), *rw = GD("density_to_rhombi_weights"), *gpot = GD("gravity_potential");
    const double *darea = DD("area"), *dz = DD("z_vector"), *fvec = DD("f_vec");

    auto cell_field = [&](const double *f) {  /* Scalar_field -> [L][Nc] */
        std::vector<double> r((size_t)L * NC);
        for (int l = 0; l < L; ++l)
            for (int i = 0; i < NC; ++i) r[(size_t)l * NC + i] = f[(size_t)l * NC + cn[i]];
        return r;
    };
    auto iface_field = [&](const double *f) {  /* Vector_field vertical part -> [L+1][Nc] */
        std::vector<double> r((size_t)(L + 1) * NC);
        for (int k = 0; k <= L; ++k)
            for (int i = 0; i < NC; ++i) r[(size_t)k * NC + i] = f[k * VPL + cn[i]];
        return r;
    };
    auto edge_field = [&](const double *f) {  /* Vector_field horizontal part -> [L][Ne] */
        std::vector<double> r((size_t)L * NE);
        for (int l = 0; l < L; ++l)
            for (int e = 0; e < NE; ++e) r[(size_t)l * NE + e] = f[NC + l * VPL + en[e]];
        return r;
    };

    std::vector<double> h_vol = cell_field(vol), h_zs = cell_field(zs), h_tbg = cell_field(tbg), h_ebg = cell_field(ebg);
    std::vector<double> h_ipw((size_t)8 * L * NC);
    for (int j = 0; j < 8; ++j)
        for (int l = 0; l < L; ++l)
            for (int i = 0; i < NC; ++i)
                h_ipw[((size_t)j * L + l) * NC + i] = ipw[8 * ((size_t)l * NC + cn[i]) + j];
    std::vector<int> h_adj((size_t)6 * NC), h_sign((size_t)6 * NC), h_nbr((size_t)6 * NC);
    for (int i = 0; i < NC; ++i) {
        int old = cn[i];
        for (int j = 0; j < 6; ++j) {
            int e = adj[6 * old + j];
            int s = adj_sign[6 * old + j];
            h_adj[(size_t)j * NC + i] = eo[e];
            h_sign[(size_t)j * NC + i] = s;
            int other = (from[e] == old) ? to[e] : from[e];
            h_nbr[(size_t)j * NC + i] = co[other];
        }
    }
    std::vector<double> h_ndv = iface_field(nd), h_areav = iface_field(area), h_zv = iface_field(zv);
    std::vector<double> h_ebggv = iface_field(ebgg), h_gmv = iface_field(gm);
    std::vector<int> h_from(NE), h_to(NE), h_dfrom(NE), h_dto(NE);
    for (int e = 0; e < NE; ++e) {
        int old = en[e];
        h_from[e] = co[from[old]];
        h_to[e] = co[to[old]];
        h_dfrom[e] = to_[dfrom[old]];
        h_dto[e] = to_[dto[old]];
    }
    std::vector<double> h_ndh = edge_field(nd), h_areah = edge_field(area), h_zh = edge_field(zv),
                        h_slope = edge_field(slope), h_ebggh = edge_field(ebgg);
    /* cells none of whose edges slopes in any layer: there every
     * terrain-following correction of the scalar tendencies vanishes, and the
     * mixed path skips it (the FP64 path keeps the reference's operations) */
    std::vector<int> h_tilt(NC, 0);
    for (int i = 0; i < NC; ++i) {
        const int n_edges = i < N_PENT ? 5 : 6;
        for (int j = 0; j < n_edges && !h_tilt[i]; ++j) {
            const int e = h_adj[(size_t)j * NC + i];
            for (int l = 0; l < L; ++l)
                if (h_slope[(size_t)l * NE + e] != 0.0) {
                    h_tilt[i] = 1;
                    break;
                }
        }
    }
    std::vector<double> h_tw((size_t)10 * NE), h_rw((size_t)4 * NE), h_fvec((size_t)2 * NE);
    std::vector<int> h_ti((size_t)10 * NE), h_tm((size_t)10 * NE), h_ri((size_t)4 * NE);
    for (int e = 0; e < NE; ++e) {
        int old = en[e];
        for (int j = 0; j < 10; ++j) {
            h_tw[(size_t)j * NE + e] = tw[10 * (size_t)old + j];
            h_ti[(size_t)j * NE + e] = eo[trsk_i[10 * (size_t)old + j]];
            h_tm[(size_t)j * NE + e] = eo[trsk_m[10 * (size_t)old + j]];
        }
        for (int j = 0; j < 4; ++j) {
            h_rw[(size_t)j * NE + e] = rw[4 * (size_t)old + j];
            h_ri[(size_t)j * NE + e] = co[rh_i[4 * (size_t)old + j]];
        }
        h_fvec[e] = fvec[old];
        h_fvec[NE + e] = fvec[NE + old];
    }
    std::vector<double> h_dah((size_t)(L + 1) * NE);
    for (int k = 0; k <= L; ++k)
        for (int e = 0; e < NE; ++e) h_dah[(size_t)k * NE + e] = darea[k * DPL + en[e]];
    /* height differences of calc_pot_vort's TOA/surface density extrapolation
     * (vorticities.c:48-79).  The reference indexes z_vector at
     * NO_OF_SCALARS + h (+ VPL) and NO_OF_SCALARS + (L-2 or L-1)*VPL + h; the
     * latter lies past the end of z_vector and reads the Grid members that
     * follow it in memory (gravity_potential, then gravity_m).  The same reads
     * are reproduced here so that results match the reference. */
    auto zx = [&](long long idx) -> double {
        if (idx < NV) return zv[idx];
        idx -= NV;
        if (idx < NS) return gpot[idx];
        idx -= NS;
        return gm[idx];
    };
    std::vector<double> h_pvz((size_t)4 * NE);
    for (int e = 0; e < NE; ++e) {
        long long h = en[e];
        int f = from[h], t = to[h];
        h_pvz[e] = zx(0) - zx(NS + h);                                   /* top: delta z */
        h_pvz[NE + e] = zx(NS + h) - zx(NS + VPL + h);                   /* top: gradient denominator */
        h_pvz[2 * (size_t)NE + e] = 0.5 * (zx(L * VPL + f) + zx(L * VPL + t)) - zx(NS + (L - 1) * VPL + h);
        h_pvz[3 * (size_t)NE + e] = zx(NS + (L - 2) * VPL + h) - zx(NS + (L - 1) * VPL + h);
    }
    std::vector<int> h_vi((size_t)3 * NT), h_vs((size_t)3 * NT);
    for (int t = 0; t < NT; ++t)
        for (int j = 0; j < 3; ++j) {
            h_vi[(size_t)j * NT + t] = eo[vi[3 * (size_t)tn[t] + j]];
            h_vs[(size_t)j * NT + t] = vs[3 * (size_t)tn[t] + j];
        }
    std::vector<double> h_dat((size_t)L * NT), h_dzt((size_t)L * NT);
    for (int l = 0; l < L; ++l)
        for (int t = 0; t < NT; ++t) {
            h_dat[(size_t)l * NT + t] = darea[NE + l * DPL + tn[t]];
            h_dzt[(size_t)l * NT + t] = dz[NE + l * DPL + tn[t]];
        }
    /* diffusion branch: layer thickness, the dual normal distances of the
     * triangle prisms and of the surface level's edges */
    {
        const double *dnd = DD("normal_distance");
        std::vector<double> h_lt = cell_field(GD("layer_thickness")), h_dndt((size_t)L * NT), h_dnds(NE);
        for (int l = 0; l < L; ++l)
            for (int t = 0; t < NT; ++t) h_dndt[(size_t)l * NT + t] = dnd[NE + l * DPL + tn[t]];
        for (int e = 0; e < NE; ++e) h_dnds[e] = dnd[(long long)L * DPL + en[e]];
        const Dual lt = dual_upload(c, h_lt), dndt = dual_upload(c, h_dndt), dnds = dual_upload(c, h_dnds),
                   zvi = dual_upload(c, iface_field(zv));
        /* Held-Suarez radiation: the reference's 18 radiation blocks take
         * (NS / 18) / L columns each, the first 18 * that cells of every layer
         * in its numbering (manage_radiation_calls.c:86-100) */
        const long long n_rad = NS / 18, per_block = n_rad / L;
        c->rad_blocks_ok = n_rad % L == 0;
        std::vector<double> h_lat(NC);
        std::vector<int> h_cov(NC);
        for (int i = 0; i < NC; ++i) {
            h_lat[i] = lat[cn[i]];
            h_cov[i] = cn[i] < 18 * per_block ? 1 : 0;
        }
        const Dual zsc = dual_upload(c, h_zs), lat_d = dual_upload(c, h_lat);
        const int *cov = dupload(c, h_cov);
        c->rad_covered = (int)(18 * per_block);
        c->dg64 = {lt.d, dndt.d, dnds.d, zvi.d, zsc.d, lat_d.d, cov, *GD("eff_hor_res"), *GD("mean_velocity_area")};
        c->dg32 = {lt.f, dndt.f, dnds.f, zvi.f, zsc.f, lat_d.f, cov, *GD("eff_hor_res"), *GD("mean_velocity_area")};
    }
    /* output diagnostics: edge directions, surface properties, the
     * permutations and the lat-lon interpolation tables ([5][N_ll], cells in
     * device numbering; an index outside the grid disables the lat-lon
     * output instead of failing the initialisation) */
    {
        const double *dir = GD("direction"), *rl = GD("roughness_length"), *alb = GD("sfc_albedo");
        const int *land = GI("is_land"), *lli = GI("latlon_interpol_indices");
        const double *llw = GD("latlon_interpol_weights");
        const long long NLL = c->dims.n_latlon;
        std::vector<double> h_dir(NE), h_rl(NC), h_alb(NC), h_llw((size_t)5 * NLL);
        std::vector<int> h_land(NC), h_lli((size_t)5 * NLL);
        for (int e = 0; e < NE; ++e) h_dir[e] = dir[en[e]];
        for (int i = 0; i < NC; ++i) {
            h_rl[i] = rl[cn[i]];
            h_alb[i] = alb[cn[i]];
            h_land[i] = land[cn[i]];
        }
        int ll_ok = 1;
        for (long long p = 0; p < NLL; ++p)
            for (int j = 0; j < 5; ++j) {
                const int ref = lli[5 * p + j];
                if (ref < 0 || ref >= NC) ll_ok = 0;
                h_lli[(size_t)j * NLL + p] = (ref >= 0 && ref < NC) ? co[ref] : 0;
                h_llw[(size_t)j * NLL + p] = llw[5 * p + j];
            }
        c->og.direction = dupload(c, h_dir);
        c->og.roughness_length = dupload(c, h_rl);
        c->og.sfc_albedo = dupload(c, h_alb);
        c->og.is_land = dupload(c, h_land);
        c->og.c_n2o = dupload(c, cn);
        c->og.e_n2o = dupload(c, en);
        c->og.ll_idx = dupload(c, h_lli);
        c->og.ll_w = dupload(c, h_llw);
        c->og.n_ll = NLL;
        c->og.ll_ok = ll_ok;
    }

    /* ---- upload */
    Dual t_vol = dual_upload(c, h_vol), t_ipw = dual_upload(c, h_ipw), t_ndv = dual_upload(c, h_ndv),
         t_areav = dual_upload(c, h_areav), t_ebggv = dual_upload(c, h_ebggv), t_gmv = dual_upload(c, h_gmv),
         t_ndh = dual_upload(c, h_ndh), t_areah = dual_upload(c, h_areah), t_zh = dual_upload(c, h_zh),
         t_slope = dual_upload(c, h_slope), t_ebggh = dual_upload(c, h_ebggh), t_tw = dual_upload(c, h_tw),
         t_rw = dual_upload(c, h_rw), t_fvec = dual_upload(c, h_fvec), t_dah = dual_upload(c, h_dah),
         t_pvz = dual_upload(c, h_pvz), t_dat = dual_upload(c, h_dat), t_dzt = dual_upload(c, h_dzt),
         t_tbg = dual_upload(c, h_tbg), t_ebg = dual_upload(c, h_ebg);
    int *d_adj = dupload(c, h_adj), *d_sign = dupload(c, h_sign), *d_nbr = dupload(c, h_nbr);
    int *d_from = dupload(c, h_from), *d_to = dupload(c, h_to), *d_ti = dupload(c, h_ti), *d_tm = dupload(c, h_tm);
    int *d_ri = dupload(c, h_ri), *d_dfrom = dupload(c, h_dfrom), *d_dto = dupload(c, h_dto);
    int *d_vi = dupload(c, h_vi), *d_vs = dupload(c, h_vs), *d_tilt = dupload(c, h_tilt);
    double *d_zs = dupload(c, h_zs), *d_tbg = t_tbg.d, *d_ebg = t_ebg.d, *d_zv = dupload(c, h_zv);

    auto fill = [&](auto &hg, auto pick) {
        hg.nc = NC; hg.ne = NE; hg.nt = NT; hg.nl = L; hg.n_oro = c->n_oro;
        hg.volume = pick(t_vol); hg.theta_v_bg = pick(t_tbg); hg.exner_bg = pick(t_ebg); hg.ipw = pick(t_ipw); hg.adj = d_adj; hg.adj_sign = d_sign; hg.adj_nbr = d_nbr;
        hg.nd_v = pick(t_ndv); hg.area_v = pick(t_areav); hg.exner_bg_grad_v = pick(t_ebggv); hg.gravity_m_v = pick(t_gmv);
        hg.from = d_from; hg.to = d_to; hg.nd_h = pick(t_ndh); hg.area_h = pick(t_areah); hg.z_h = pick(t_zh);
        hg.slope_h = pick(t_slope); hg.exner_bg_grad_h = pick(t_ebggh); hg.trsk_w = pick(t_tw); hg.trsk_i = d_ti;
        hg.trsk_m = d_tm; hg.rhombi_w = pick(t_rw); hg.rhombi_i = d_ri; hg.f_vec = pick(t_fvec);
        hg.dual_from = d_dfrom; hg.dual_to = d_dto; hg.dual_area_h = pick(t_dah); hg.pvz = pick(t_pvz);
        hg.vort_i = d_vi; hg.vort_s = d_vs; hg.dual_area_t = pick(t_dat); hg.dual_z_t = pick(t_dzt);
        hg.tilt = d_tilt;
    };
    fill(c->hg64, [](const Dual &x) { return (const double *)x.d; });
    c->hg64.radius = c->radius;
    fill(c->hg32, [](const Dual &x) { return (const float *)x.f; });
    c->hg32.radius = (float)c->radius;
    c->vg.nc = NC; c->vg.nl = L;
    c->vg.volume = t_vol.d; c->vg.z_scalar = d_zs; c->vg.exner_bg = d_ebg; c->vg.theta_v_bg = d_tbg;
    c->vg.area_v = t_areav.d; c->vg.z_v = d_zv;

    /* ---- index maps (device position -> reference position) */
    std::vector<int> m_s((size_t)NS), m_vec((size_t)NV), m_curl((size_t)c->ncurl), m_tri((size_t)L * NT);
    for (int l = 0; l < L; ++l)
        for (int i = 0; i < NC; ++i) m_s[(size_t)l * NC + i] = l * NC + cn[i];
    for (int k = 0; k <= L; ++k)
        for (int i = 0; i < NC; ++i) m_vec[(size_t)k * NC + i] = (int)(k * VPL + cn[i]);
    for (int l = 0; l < L; ++l)
        for (int e = 0; e < NE; ++e) m_vec[(size_t)(L + 1) * NC + (size_t)l * NE + e] = (int)(NC + l * VPL + en[e]);
    for (int k = 0; k <= L; ++k)
        for (int e = 0; e < NE; ++e) m_curl[(size_t)k * NE + e] = k * 2 * NE + en[e];
    for (int l = 0; l < L; ++l)
        for (int e = 0; e < NE; ++e) m_curl[(size_t)(L + 1) * NE + (size_t)l * NE + e] = NE + l * 2 * NE + en[e];
    for (int l = 0; l < L; ++l)
        for (int t = 0; t < NT; ++t) m_tri[(size_t)l * NT + t] = l * NT + tn[t];
    std::vector<int> m_state((size_t)c->state_len);
    {
        /* device state block: [rho C*S][rhotheta S][theta_pert S][exner_pert S][w (L+1)Nc][u L Ne];
         * reference State: rho, rhotheta_v, theta_v_pert, exner_pert, wind (contiguous) */
        size_t p = 0;
        for (int k = 0; k < c->n_const + 3; ++k)
            for (long long i = 0; i < NS; ++i) m_state[p++] = (int)(k * NS + m_s[i]);
        for (long long i = 0; i < NV; ++i) m_state[p++] = (int)((c->n_const + 3) * NS + m_vec[i]);
        /* soil temperature: kept in reference order (no kernel of the step reads it) */
        while (p < (size_t)c->state_len) {
            m_state[p] = (int)p;
            ++p;
        }
    }
    c->map_s = dupload(c, m_s);
    c->map_vec = dupload(c, m_vec);
    c->map_curl = dupload(c, m_curl);
    c->map_tri = dupload(c, m_tri);
    c->map_state = dupload(c, m_state);
    {
        std::vector<int> inv(m_state.size());
        for (size_t q = 0; q < m_state.size(); ++q) inv[(size_t)m_state[q]] = (int)q;
        c->imap_state = dupload(c, inv);
    }
    c->staging_len = (size_t)std::max<long long>(std::max<long long>(c->state_len, c->ncurl), 8 * NS);
    c->staging = dalloc<double>(c, c->staging_len);
    for (int k = 0; k < 4; ++k) c->dev_tmp[k] = dalloc<double>(c, (size_t)std::max<long long>(NV, c->ncurl));

    /* ---- persistent step fields and work arrays */
    c->temperature = dalloc<double>(c, NS);
    c->theta = dalloc<double>(c, NS);
    c->pt_rates = dalloc<double>(c, 5 * NS);
    c->pt_heat = dalloc<double>(c, NS);
    c->sed_heat = dalloc<double>(c, NS);
    c->cp_ice = dalloc<double>(c, NS);
    c->cp_water = dalloc<double>(c, NS);
    /* k_make_shadow moves element pairs: every field must start on an even
     * element (true of every icosahedral grid: 10 * 4^RES_ID + 2 cells,
     * 30 * 4^RES_ID edges) */
    if (NC % 2 != 0 || NE % 2 != 0) return fail("grid with an odd number of cells or edges");
    c->shadow = dalloc<float>(c, (size_t)(c->n_const + 3) * NS + (size_t)(L + 1) * NC + (size_t)L * NE);
    c->theta32 = dalloc<float>(c, NS);
    c->pg_cell = dalloc<float4>(c, NS);
    c->cp32_ice = dalloc<float>(c, NS);
    c->cp32_water = dalloc<float>(c, NS);
    c->gravity_potential = dupload(c, cell_field(gpot));
    c->red_partials = dalloc<double>(c, (size_t)2 * INTEGRAL_MAX_BLOCKS * INTEGRAL_MAX_FIELDS);
    c->red_counters = dalloc<unsigned>(c, INTEGRAL_MAX_FIELDS);
    c->red_out = dalloc<double>(c, INTEGRAL_MAX_FIELDS);
    c->energy_buf = dalloc<double>(c, 3 * (size_t)NS);
    c->wv_layer = dalloc<double>(c, 8 * (size_t)NS);
    c->wv_rows = dalloc<double>(c, 7 * (size_t)(L - 1) * NC);
    c->damp_dc = dalloc<double>(c, (size_t)(L - 1) * NC);
    c->damp_inv = dalloc<double>(c, (size_t)(L - 1) * NC);
    {
        std::vector<double> iv(h_vol.size()), ia(h_areav.size());
        for (size_t k = 0; k < iv.size(); ++k) iv[k] = 1.0 / h_vol[k];
        for (size_t k = 0; k < ia.size(); ++k) ia[k] = h_areav[k] != 0.0 ? 1.0 / h_areav[k] : 0.0;
        c->inv_vol = dupload(c, iv);
        c->inv_area_v = dupload(c, ia);
        /* double-float (hi, lo) pairs of the tracer solver's tables */
        auto df_pairs = [](const std::vector<double> &x) {
            std::vector<float> out(2 * x.size());
            for (size_t k = 0; k < x.size(); ++k) {
                const float hi = (float)x[k];
                out[2 * k] = hi;
                out[2 * k + 1] = (float)(x[k] - (double)hi);
            }
            return out;
        };
        c->dfg.area_v = (const float2 *)dupload(c, df_pairs(h_areav));
        c->dfg.inv_area_v = (const float2 *)dupload(c, df_pairs(ia));
        c->dfg.inv_vol = (const float2 *)dupload(c, df_pairs(iv));
        c->dfg.volume = (const float2 *)dupload(c, df_pairs(h_vol));
        c->dfg.exner_bg = (const float2 *)dupload(c, df_pairs(h_ebg));
        c->dfg.theta_v_bg = (const float2 *)dupload(c, df_pairs(h_tbg));
        /* mixed-path sound-wave rows: dz, H, G1, G2, Cz, Ez per inner interface */
        const size_t ni = (size_t)(L - 1) * NC;
        std::vector<double> geo(6 * ni);
        for (size_t q = 0; q < ni; ++q) {
            const size_t b = q, lo = q + NC, wi = q + NC;
            const double dz = h_zs[b] - h_zs[lo];
            geo[q] = dz;
            geo[ni + q] = 0.5 * (h_ebg[b] - h_ebg[lo]);
            geo[2 * ni + q] = 2.0 * ia[wi];
            geo[3 * ni + q] = 0.5 * (iv[lo] - iv[b]);
            geo[4 * ni + q] = dz * iv[b];
            geo[5 * ni + q] = dz * iv[lo];
        }
        c->wv_geo = dupload(c, geo);
        c->dfg.geo = (const float2 *)dupload(c, df_pairs(geo));
        c->damp_inv_df = dalloc<float2>(c, ni);
        c->dfg.damp_inv = c->damp_inv_df;
    }
    auto work = [&](auto &w, auto tag) {
        using R = decltype(tag);
        w.P_h = dalloc<R>(c, (size_t)L * NE); w.P_v = dalloc<R>(c, (size_t)(L + 1) * NC);
        w.pg_old_h = dalloc<R>(c, (size_t)L * NE);
        w.pvt_h = dalloc<R>(c, (size_t)L * NE); w.pvt_v = dalloc<R>(c, (size_t)(L + 1) * NC);
        w.v2g_h = dalloc<R>(c, (size_t)L * NE); w.v2g_v = dalloc<R>(c, (size_t)(L + 1) * NC);
        w.flux_h = dalloc<R>(c, (size_t)L * NE); w.flux_v = dalloc<R>(c, (size_t)(L + 1) * NC);
        w.zh = dalloc<R>(c, (size_t)(L + 1) * NE); w.zv = dalloc<R>(c, (size_t)L * NE);
        w.tri_vort = dalloc<R>(c, (size_t)L * NT); w.v2 = dalloc<R>(c, (size_t)L * NC);
    };
    work(c->w64, double(0));
    work(c->w32, float(0));
    for (auto &b : c->owned)
        if (!b.p) return fail("device allocation failed");
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_tend, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_tend_copied, cudaEventDisableTiming));
    CK(cudaDeviceSynchronize());
    CK(cudaGetLastError());
    return 0;
#undef GD
#undef GI
#undef DD
#undef DI
}

int profile_flush(Context *c)
{
    CK(cudaStreamSynchronize(c->stream));
    for (auto &p : c->pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.a, p.b);
        auto &t = c->prof_totals[p.name];
        t.first += ms;
        t.second += 1;
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    c->pending.clear();
    return 0;
}

int destroy_context()
{
    Context *c = g_ctx;
    if (!c) return 0;
    cudaDeviceSynchronize();
    profile_flush(c);
    for (auto e : c->user_events) cudaEventDestroy(e);
    if (c->adj_release) c->adj_release(c);
    if (c->obuf_release) c->obuf_release(c);
    for (auto &kv : c->graphs) cudaGraphExecDestroy(kv.second.exec);
    for (auto &kv : c->states) cudaFree(kv.second.dev);
    for (auto &b : c->owned) cudaFree(b.p);
    if (c->health) cudaFree(c->health);
    delete c->dbuf;
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->ev_tend) cudaEventDestroy(c->ev_tend);
    if (c->ev_tend_copied) cudaEventDestroy(c->ev_tend_copied);
    delete c;
    g_ctx = nullptr;
    return 0;
}

/* --------------------------------------------------------- state mirrors */
/* device layout pointers of a state block */
void set_mirror_views(Context *c, StateMirror &m)
{
    const long long ns = c->ns;
    m.ds.rho = m.dev;
    m.ds.rhotheta_v = m.dev + c->n_const * ns;
    m.ds.theta_v_pert = m.ds.rhotheta_v + ns;
    m.ds.exner_pert = m.ds.theta_v_pert + ns;
    m.ds.w = m.ds.exner_pert + ns;
    m.ds.u = m.ds.w + (long long)(c->nl + 1) * c->nc;
}

StateMirror *mirror(const void *host_state, int create)
{
    Context *c = g_ctx;
    auto it = c->states.find(host_state);
    if (it != c->states.end()) return &it->second;
    if (!create) return nullptr;
    StateMirror m;
    if (cudaMalloc(&m.dev, (size_t)c->state_len * sizeof(double)) != cudaSuccess) {
        fail("device allocation of a state mirror failed");
        return nullptr;
    }
    cudaMemset(m.dev, 0, (size_t)c->state_len * sizeof(double));
    set_mirror_views(c, m);
    c->states[host_state] = m;
    return &c->states[host_state];
}

int ensure_diff_buffers(Context *c)
{
    if (c->dbuf) return 0;
    const size_t S = (size_t)c->ns, C = (size_t)c->n_const, L = (size_t)c->nl;
    const size_t NC = (size_t)c->nc, NE = (size_t)c->ne, NT = (size_t)c->nt;
    DiffBufs *b = new DiffBufs();
    c->dbuf = b;
    struct Want {
        double **p;
        size_t n;
    } want[] = {
        {&b->tke, S}, {&b->visc, S}, {&b->hdiss, S}, {&b->fric, (size_t)c->nv}, {&b->mol, S}, {&b->n2, S},
        {&b->mdt, C * S}, {&b->tdh, S}, {&b->rad, S}, {&b->ph_tb, 2 * NC}, {&b->dvdz_top, NE},
        {&b->adv, S}, {&b->vint, S}, {&b->wdv, S}, {&b->tri, L * NT}, {&b->zt, L * NT}, {&b->zr, L * NE},
        {&b->s1, S}, {&b->s2, S}, {&b->s3, S}, {&b->flx, L * NE}, {&b->mch, S}, {&b->mcv, S}, {&b->tch, S},
        {&b->tcv, S}, {&b->fh, (C + 1) * L * NE}, {&b->fv, (C + 1) * (L + 1) * NC}, {&b->kvt, S},
        {&b->hs_p, S}, {&b->hs_ps, NC},
    };
    for (auto &w : want)
        if (!(*w.p = dalloc<double>(c, w.n))) return fail("device allocation of the diffusion fields failed");
    return 0;
}

int ensure_sub_buffers(Context *c)
{
    Context::SubBuffers &b = c->sub;
    if (b.ready) return 0;
    const size_t NS = (size_t)c->ns, nvec = (size_t)std::max<long long>(c->nv, c->ncurl);
    for (StateMirror *m : {&b.so, &b.sn, &b.st, &b.bso, &b.bsn, &b.bst}) {
        m->dev = dalloc<double>(c, (size_t)c->state_len);
        if (!m->dev) return fail("device allocation of the sub-step buffers failed");
        set_mirror_views(c, *m);
    }
    for (auto &v : b.vec)
        if (!(v = dalloc<double>(c, nvec))) return fail("device allocation of the sub-step buffers failed");
    double **scal[] = {&b.temperature, &b.cp_ice, &b.cp_water, &b.theta, &b.pt_heat, &b.sed_heat, &b.decel, &b.v2};
    for (double **p : scal)
        if (!(*p = dalloc<double>(c, NS))) return fail("device allocation of the sub-step buffers failed");
    if (!(b.pt_rates = dalloc<double>(c, 5 * NS))) return fail("device allocation of the sub-step buffers failed");
    if (!(b.tri = dalloc<double>(c, (size_t)c->nl * c->nt))) return fail("device allocation of the sub-step buffers failed");
    b.ready = true;
    return 0;
}

/* the State members rho .. wind are contiguous in the reference struct:
 * one copy of (C+3)*S + Vt doubles, then one gather into device order */
int upload_state(const void *host_state, StateMirror *m)
{
    Context *c = g_ctx;
    const double *h = (const double *)((const char *)host_state + c->off_state_rho);
    if (const char *hd = pinned_device_range(h, (size_t)c->state_len * sizeof(double))) {
        k_state_from_host<<<(unsigned)((c->state_len + 255) / 256), 256, 0, c->stream>>>(
            m->dev, (const double *)hd, c->imap_state, 0, c->state_len);
        c->kernel_launches++;
        c->h2d_bytes += (long long)c->state_len * (long long)sizeof(double);
        CK(cudaGetLastError());
        return 0;
    }
    CK(cudaMemcpyAsync(c->staging, h, (size_t)c->state_len * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    c->h2d_bytes += (long long)c->state_len * (long long)sizeof(double);
    launch_gather(m->dev, c->staging, c->map_state, c->state_len, c->stream);
    return 0;
}

/* which_mask bits: 1 rho, 2 rhotheta_v, 4 theta_v_pert, 8 exner_pert, 16 wind, 32 temperature_soil */
int download_state_pinned(const void *host_state, StateMirror *m, int which_mask, cudaStream_t s)
{
    Context *c = g_ctx;
    double *h = (double *)((char *)host_state + c->off_state_rho);
    char *hd = pinned_device_range(h, (size_t)c->state_len * sizeof(double));
    if (!hd) return 0;
    const long long ns = c->ns;
    const long long soil0 = (c->n_const + 3) * ns + c->nv;
    struct Part { int bit; long long lo, n; } parts[6] = {
        {1, 0, c->n_const * ns}, {2, c->n_const * ns, ns}, {4, (c->n_const + 1) * ns, ns},
        {8, (c->n_const + 2) * ns, ns}, {16, (c->n_const + 3) * ns, c->nv}, {32, soil0, c->state_len - soil0}};
    for (auto &p : parts)
        if ((which_mask & p.bit) && p.n > 0) {
            k_state_to_host<<<(unsigned)((p.n + 255) / 256), 256, 0, s>>>((double *)hd, m->dev, c->imap_state, p.lo,
                                                                       p.n);
            c->kernel_launches++;
            c->d2h_bytes += p.n * (long long)sizeof(double);
        }
    return 1;
}

int download_state(const void *host_state, StateMirror *m, int which_mask)
{
    Context *c = g_ctx;
    double *h = (double *)((char *)host_state + c->off_state_rho);
    const long long ns = c->ns;
    const long long soil0 = (c->n_const + 3) * ns + c->nv;
    struct Part { int bit; long long lo, n; } parts[6] = {
        {1, 0, c->n_const * ns}, {2, c->n_const * ns, ns}, {4, (c->n_const + 1) * ns, ns},
        {8, (c->n_const + 2) * ns, ns}, {16, (c->n_const + 3) * ns, c->nv}, {32, soil0, c->state_len - soil0}};
    if (download_state_pinned(host_state, m, which_mask, c->stream)) return 0;
    launch_scatter(c->staging, m->dev, c->map_state, c->state_len, c->stream);
    if (which_mask == 63) {
        CK(cudaMemcpyAsync(h, c->staging, (size_t)c->state_len * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        c->d2h_bytes += (long long)c->state_len * (long long)sizeof(double);
    } else {
        for (auto &p : parts)
            if (which_mask & p.bit) {
                CK(cudaMemcpyAsync(h + p.lo, c->staging + p.lo, (size_t)p.n * sizeof(double), cudaMemcpyDeviceToHost,
                                   c->stream));
                c->d2h_bytes += p.n * (long long)sizeof(double);
            }
    }
    return 0;
}

/* one reference-layout field: host -> staging -> device layout */
int upload_field(const double *host, double *dev, const int *map, long long n, long long host_len)
{
    Context *c = g_ctx;
    CK(cudaMemcpyAsync(c->staging, host, (size_t)host_len * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    c->h2d_bytes += host_len * (long long)sizeof(double);
    launch_gather(dev, c->staging, map, n, c->stream);
    return 0;
}

/* device layout -> staging -> host for reference positions [host_lo, host_hi);
 * the map is a bijection onto the field, so the scatter writes every staging
 * position of that range */
int download_field(double *host, const double *dev, const int *map, long long n, long long host_len,
                   long long host_lo, long long host_hi)
{
    Context *c = g_ctx;
    (void)host_len;
    launch_scatter(c->staging, dev, map, n, c->stream);
    CK(cudaMemcpyAsync(host + host_lo, c->staging + host_lo, (size_t)(host_hi - host_lo) * sizeof(double),
                       cudaMemcpyDeviceToHost, c->stream));
    c->d2h_bytes += (host_hi - host_lo) * (long long)sizeof(double);
    return 0;
}

}  // namespace game
