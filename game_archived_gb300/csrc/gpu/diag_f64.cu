/*
 * Global integrals and surface pressure on the device mirrors of a State
 * (compiled with --fmad=false: every pointwise product and sum is rounded as
 * in the reference C; the reductions below use explicit fma for their exact
 * product errors).
 *
 *   global_scalar_integrator   src/io/write_output.c:1659-1668
 *   write_out_integral values  src/io/write_output.c:1515-1596
 *   surface pressure, MSLP     src/io/write_output.c:105-121
 *
 * Reductions.  The reference sums field*volume serially.  Here every block
 * accumulates its share of the products as a double-word number: the exact
 * rounding error of each product (fma(a, b, -a*b)) and of each addition
 * (TwoSum) is carried in a second double, so the sum is exact to about 2^-100
 * relative before it is rounded once.  Block results go to a scratch array of
 * (hi, lo) pairs; the block that finishes last (an atomic counter per field)
 * merges them in block order, writes the result and sets the counter back to
 * zero.  The result does not depend on which block finishes last, so the
 * sum is deterministic for a given grid size.
 */
#include "context.h"
#include "diag.h"
#include "ops.h"

namespace game {
namespace {

struct DW {
    double hi, lo;
};

__device__ __forceinline__ DW dw_add(DW x, DW y)
{
    const double s = x.hi + y.hi;
    const double bp = s - x.hi;
    const double e = (x.hi - (s - bp)) + (y.hi - bp);
    const double l = e + (x.lo + y.lo);
    const double h = s + l;
    return {h, l - (h - s)};
}

/* acc += a*b with the product's rounding error kept */
__device__ __forceinline__ void dw_add_product(DW &acc, double a, double b)
{
    const double p = a * b;
    const double pe = fma(a, b, -p);
    const double s = acc.hi + p;
    const double bp = s - acc.hi;
    const double e = (acc.hi - (s - bp)) + (p - bp);
    acc.hi = s;
    acc.lo += e + pe;
}

/* fixed-order tree over the block; result valid in thread 0 */
__device__ DW block_reduce(DW v)
{
    __shared__ double sh_hi[32], sh_lo[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        DW w{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
        v = dw_add(v, w);
    }
    if (lane == 0) {
        sh_hi[warp] = v.hi;
        sh_lo[warp] = v.lo;
    }
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    if (warp == 0) {
        v = lane < nw ? DW{sh_hi[lane], sh_lo[lane]} : DW{0.0, 0.0};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            DW w{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
            v = dw_add(v, w);
        }
    }
    return v;
}

/* out[k] = sum_i f[k*fstride + idx(i)] * w[i], i < n, k = blockIdx.y, with
 * idx(i) = map[i] when a map is given (field in the reference's order,
 * weights in the device order), else i.  partials holds gridDim.x (hi, lo)
 * pairs per field, counters one zero-initialised counter per field. */
__global__ void __launch_bounds__(INTEGRAL_THREADS)
    k_integral(const double *f, long long fstride, long long n, const int *map, const double *w, double *partials,
               unsigned *counters, double *out)
{
    const int k = blockIdx.y;
    const double *fk = f + (long long)k * fstride;
    DW acc{0.0, 0.0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        dw_add_product(acc, map ? fk[map[i]] : fk[i], w[i]);
    acc = block_reduce(acc);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        double *pk = partials + 2 * ((long long)k * gridDim.x + blockIdx.x);
        pk[0] = acc.hi;
        pk[1] = acc.lo;
        __threadfence();
        last = atomicAdd(&counters[k], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    DW r{0.0, 0.0};
    const volatile double *pk = partials + 2 * (long long)k * gridDim.x;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) r = dw_add(r, DW{pk[2 * b], pk[2 * b + 1]});
    r = block_reduce(r);
    if (threadIdx.x == 0) {
        out[k] = r.hi + r.lo;
        counters[k] = 0u;
    }
}

/* temperature_diagnostics (src/constituents/derived_quantities.c:15-40) at
 * device cell index i */
__device__ __forceinline__ double temperature_at(const VGrid &vg, const DState &s, int n_cond, int moist, long long ns,
                                                 long long i)
{
    double t = (vg.theta_v_bg[i] + s.theta_v_pert[i]) * (vg.exner_bg[i] + s.exner_pert[i]);
    if (moist) t = t / (1.0 + s.rho[(n_cond + 1) * ns + i] / s.rho[n_cond * ns + i] * (M_D / M_V - 1.0));
    return t;
}

/* gas_constant_diagnostics (derived_quantities.c:42-61) */
__device__ __forceinline__ double gas_constant_at(const DState &s, int n_cond, int moist, long long ns, long long i)
{
    if (!moist) return R_D;
    double r = (s.rho[n_cond * ns + i] - s.rho[(n_cond + 1) * ns + i]) * R_D + s.rho[(n_cond + 1) * ns + i] * R_V;
    return r / s.rho[n_cond * ns + i];
}

__global__ void k_temperature(VGrid vg, DState s, int n_cond, int moist, double *t)
{
    const long long ns = (long long)vg.nl * vg.nc;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ns) t[i] = temperature_at(vg, s, n_cond, moist, ns, i);
}

/* energy densities of write_out_integral(..., 2): rho_g * |v|^2 (|v|^2 from
 * the inner product, already in e[0..ns)), rho_g * gravity potential,
 * rho_g * T; written to e[0], e[ns], e[2 ns] */
__global__ void k_energy_densities(long long ns, const double *rho_g, const double *gpot, const double *t, double *e)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ns) return;
    const double r = rho_g[i];
    e[i] = r * e[i];
    e[ns + i] = r * gpot[i];
    e[2 * ns + i] = r * t[i];
}

/* write_output.c:105-121 per column (device cell index i) */
__global__ void k_surface_pressure(VGrid vg, const double *gravity_m_v, DState s, int n_cond, int moist, double *p_sfc,
                                   double *mslp)
{
    const int nc = vg.nc, nl = vg.nl;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const long long ns = (long long)nl * nc, si = (long long)(nl - 1) * nc + i;
    const double lapse = 0.0065;
    const double t_low = temperature_at(vg, s, n_cond, moist, ns, si);
    const double rgas = gas_constant_at(s, n_cond, moist, ns, si);
    const double p = s.rho[n_cond * ns + si] * rgas * t_low;
    const double gm = gravity_m_v[(long long)(nl - 1) * nc + i];
    const double z = vg.z_scalar[si];
    if (mslp) {
        const double t_mslp = t_low + lapse * z;
        mslp[i] = p / pow(1 - (t_mslp - t_low) / t_mslp, gm / (rgas * lapse));
    }
    const double t_sfc = t_low + lapse * (z - vg.z_v[(long long)nl * nc + i]);
    p_sfc[i] = p / pow(1.0 - (t_sfc - t_low) / t_sfc, gm / (rgas * lapse));
}

inline unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace

int integral_blocks(long long n)
{
    long long b = (n + INTEGRAL_THREADS - 1) / INTEGRAL_THREADS;
    if (b < 1) b = 1;
    return (int)(b < INTEGRAL_MAX_BLOCKS ? b : INTEGRAL_MAX_BLOCKS);
}

int launch_integral(const double *f, long long fstride, int n_fields, long long n, const int *map, const double *w,
                    double *partials, unsigned *counters, double *out, cudaStream_t stream)
{
    if (n_fields < 1 || n_fields > INTEGRAL_MAX_FIELDS) return fail("integral: field count out of range");
    dim3 grid((unsigned)integral_blocks(n), (unsigned)n_fields);
    k_integral<<<grid, INTEGRAL_THREADS, 0, stream>>>(f, fstride, n, map, w, partials, counters, out);
    CK(cudaGetLastError());
    return 0;
}

int diag_temperature(Context *c, StateMirror *s, double *t)
{
    k_temperature<<<blocks_for(c->ns, 256), 256, 0, c->stream>>>(c->vg, s->ds, c->n_cond, c->moist, t);
    c->kernel_launches++;
    CK(cudaGetLastError());
    return 0;
}

int diag_energy_densities(Context *c, StateMirror *s, const double *temperature, double *e)
{
    /* |v|^2 at the cells (inner_product, src/spatial_operators/inner_product.c) */
    op_inner_product(c, s->ds.w, s->ds.w, e);
    k_energy_densities<<<blocks_for(c->ns, 256), 256, 0, c->stream>>>(c->ns, s->ds.rho + (long long)c->n_cond * c->ns,
                                                                       c->gravity_potential, temperature, e);
    c->kernel_launches += 2;
    CK(cudaGetLastError());
    return 0;
}

int diag_surface_pressure(Context *c, StateMirror *s, double *p_sfc, double *mslp)
{
    k_surface_pressure<<<blocks_for(c->nc, 128), 128, 0, c->stream>>>(c->vg, c->hg64.gravity_m_v, s->ds, c->n_cond,
                                                                       c->moist, p_sfc, mslp);
    c->kernel_launches++;
    CK(cudaGetLastError());
    return 0;
}

}  // namespace game
