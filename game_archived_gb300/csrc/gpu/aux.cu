/*
 * Import and export of the lagged fields the reference carries from one
 * manage_rkhevi call to the next (src/time_stepping/vector_tendencies_expl.c:24-35,
 * manage_pressure_gradient.c:25-32): the pressure gradient nl + l, the
 * vorticity flux, the kinetic-energy gradient and the boundary entries of the
 * mass flux density.  Device-layout vector fields: [w (L+1)][Nc] then [u L][Ne].
 */
#include "context.h"

namespace game {
namespace {

/* l_f may be null (nl_f then holds the sum); nl_f, pvt and v2g may all be
 * null, which imports zeros (a window that starts with the model's first
 * step reads none of them) */
template <typename R>
__global__ void k_import(int nc, int ne, int nl, const double *nl_f, const double *l_f, const double *pvt,
                         const double *v2g, const double *flux, Work<R> w)
{
    const long long nw = (long long)(nl + 1) * nc, nu = (long long)nl * ne;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nw + nu) return;
    const R P = nl_f ? R(l_f ? nl_f[i] + l_f[i] : nl_f[i]) : R(0);
    const R pv = pvt ? R(pvt[i]) : R(0), kg = v2g ? R(v2g[i]) : R(0);
    if (i < nw) {
        w.P_v[i] = P;
        w.pvt_v[i] = pv;
        w.v2g_v[i] = kg;
        w.flux_v[i] = R(flux[i]);
    } else {
        const long long j = i - nw;
        w.P_h[j] = P;
        w.pvt_h[j] = pv;
        w.v2g_h[j] = kg;
        w.flux_h[j] = R(flux[i]);
    }
}

template <typename R>
__global__ void k_export(int nc, int ne, int nl, Work<R> w, double *P, double *pvt, double *v2g)
{
    const long long nw = (long long)(nl + 1) * nc, nu = (long long)nl * ne;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nw) {
        P[i] = double(w.P_v[i]);
        pvt[i] = double(w.pvt_v[i]);
        v2g[i] = double(w.v2g_v[i]);
    } else if (i < nw + nu) {
        const long long j = i - nw;
        P[i] = double(w.P_h[j]);
        pvt[i] = double(w.pvt_h[j]);
        v2g[i] = double(w.v2g_h[j]);
    }
}

}  // namespace

void aux_sum_to_work(Context *c, const double *nl, const double *l, const double *pvt, const double *v2g,
                     const double *flux, const double *, const double *)
{
    const long long n = c->nv;
    const unsigned nb = (unsigned)((n + 255) / 256);
    k_import<double><<<nb, 256, 0, c->stream>>>(c->nc, c->ne, c->nl, nl, l, pvt, v2g, flux, c->w64);
    k_import<float><<<nb, 256, 0, c->stream>>>(c->nc, c->ne, c->nl, nl, l, pvt, v2g, flux, c->w32);
    c->kernel_launches += 2;
}

void aux_load_mixed(Context *c, const double *P, const double *pvt, const double *v2g, const double *flux)
{
    const long long n = c->nv;
    k_import<float><<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->nc, c->ne, c->nl, P, nullptr, pvt, v2g,
                                                                        flux, c->w32);
    c->kernel_launches++;
}

void aux_store_mixed(Context *c, double *P, double *pvt, double *v2g)
{
    const long long n = c->nv;
    k_export<float><<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->nc, c->ne, c->nl, c->w32, P, pvt, v2g);
    c->kernel_launches++;
}

int aux_export(Context *c, double *P, double *pvt, double *v2g)
{
    const long long n = c->nv;
    const unsigned nb = (unsigned)((n + 255) / 256);
    if (c->precision == PREC_FP64) k_export<double><<<nb, 256, 0, c->stream>>>(c->nc, c->ne, c->nl, c->w64, P, pvt, v2g);
    else k_export<float><<<nb, 256, 0, c->stream>>>(c->nc, c->ne, c->nl, c->w32, P, pvt, v2g);
    c->kernel_launches++;
    return 0;
}

}  // namespace game
