/*
 * Diffusion branch of the RKHEVI step: Brunt-Vaisala frequency, TKE update,
 * effective viscosities, horizontal and vertical momentum diffusion, the
 * dissipation rate, and temperature and mass diffusion
 * (src/subgrid_scale/effective_diff_coeffs.c, src/subgrid_scale/tke.c,
 * src/spatial_operators/momentum_diff_diss.c, called from
 * src/time_stepping/vector_tendencies_expl.c:41-69 and
 * scalar_tendencies_expl.c:44-88 at the first RK substep).
 *
 * Templated on the horizontal precision R like the other step kernels.
 * R = double (diff_f64.cu, --fmad=false): every expression in the
 * reference's operation order.  R = float (diff_mixed.cu): the same
 * operators on the FP32 tables and the FP32 shadow of state_new, with the
 * divergences of the diffusive mass fluxes summed as double-word FP32
 * pairs, each edge's flux entering both of its cells, so that diffusion
 * conserves mass like the advection does.  The fields carried between
 * steps (TKE, viscosity, friction, heating, mass tendency) are stored in
 * double on both paths; the scratch of one step is stored in R.
 *
 * The reference's sequence of whole-field operator calls (each writing a
 * placeholder field) becomes a few fused per-point kernels:
 *   kd_n2_adv        N^2 of every layer but the last (whose value the
 *                    reference never writes) and the TKE advection term
 *   kd_tke           TKE update
 *   kd_hor_visc      molecular + turbulent viscosity (and, for momentum
 *                    diffusion, viscosity times the wind divergence)
 *   k_tri_vort, kd_zt, kd_zr   relative vorticity on triangles and rhombi
 *                    times the viscosity averaged there
 *   kd_fric_h        horizontal friction: curl of the vorticity and gradient
 *                    of the divergence term, plus vertical diffusion of u
 *   kd_wdiff_a..d    vertical and horizontal diffusion of w
 *   kd_dissipation   heating_diss = -rho * (wind . friction)
 *   kd_sdiff_*       diffusion coefficients, diffusive fluxes of T and of
 *                    every density, their divergences
 * Device layout: scalar [L][Nc], vector [w (L+1)][Nc] then [u L][Ne],
 * triangle [L][Nt].
 */
#pragma once

#include "diff.h"
#include "kernels.cuh"

namespace game {
namespace {

constexpr double K_B_ = 1.380649e-23;
constexpr double PI_ = 3.14159265358979323846;
constexpr double EPS_SEC = 1e-10;

inline unsigned dnb(long long n, int bs = 256) { return (unsigned)((n + bs - 1) / bs); }

/* molecular diffusion coefficient from kinetic gas theory
 * (src/constituents/derived_quantities.c:117-134); pow(r, 2) is the product
 * r * r, which the reference's compiler folds it to */
template <typename R>
__device__ __forceinline__ R calc_diffusion_coeff(R temperature, R density)
{
    const R particle_radius = R(130e-12);
    const R particle_mass = R(M_D / N_A);
    const R thermal_velocity = sqrt(R(8.0 * K_B_) * temperature / R(PI_ * (M_D / N_A)));
    const R particle_density = density / particle_mass;
    const R cross_section = R(4.0 * PI_) * (particle_radius * particle_radius);
    const R mean_free_path = R(1) / (sqrt(R(2)) * particle_density * cross_section);
    return R(1.0 / 3.0) * thermal_velocity * mean_free_path;
}

/* effective_diff_coeffs.c:293-303 (x^0.5 as sqrt) */
template <typename R>
__device__ __forceinline__ R tke2hor(R tke, R effective_resolution)
{
    const R mean_velocity = sqrt(R(2) * tke);
    const R mean_free_path = effective_resolution / R(6);
    return R(1.0 / 6.0) * mean_free_path * mean_velocity;
}

/* effective_diff_coeffs.c:305-320 */
template <typename R>
__device__ __forceinline__ R tke2vert(R tke, R n_squared, R layer_thickness)
{
    const R tke_vert = R(3.0 * 1e-3) * tke;
    const R mean_velocity = sqrt(R(2) * tke_vert);
    const R n_used = sqrt(fmax(n_squared, R(1e-4)));
    R mean_free_path = sqrt(R(2) * tke_vert) / n_used;
    mean_free_path = fmin(mean_free_path, layer_thickness);
    return R(1.0 / 6.0) * mean_free_path * mean_velocity;
}

/* divv_h (divergences.c:14-64) at cell c of layer l of the edge field in_u
 * [L][Ne]; with R = float the edge terms are summed as a double-word pair */
template <typename R, typename F>
__device__ __forceinline__ double divv_h_cell(const HGrid<R> &g, const F *in_u, int l, int c)
{
    const int n_edges = c < N_PENT ? 5 : 6, nl = g.nl, n_oro = g.n_oro;
    const long long nc = g.nc;
    FluxSum<R> comp_h;
    for (int j = 0; j < n_edges; ++j) {
        const long long vi = (long long)l * g.ne + g.adj[j * nc + c];
        comp_h.add(R(in_u[vi]) * R(g.adj_sign[j * nc + c]) * g.area_h[vi]);
    }
    auto fin = [&](int ll, int j) { return R(in_u[(long long)ll * g.ne + g.adj[j * nc + c]]); };
    R comp_v = R(0);
    if (l == nl - n_oro - 1) {
        const R lo = contra_corr(g, l + 1, c, n_edges, fin);
        comp_v = -lo * g.area_v[(long long)(l + 1) * nc + c];
    } else if (l == nl - 1) {
        const R up = contra_corr(g, l, c, n_edges, fin);
        comp_v = up * g.area_v[(long long)l * nc + c];
    } else if (l > nl - n_oro - 1) {
        const R up = contra_corr(g, l, c, n_edges, fin);
        const R lo = contra_corr(g, l + 1, c, n_edges, fin);
        comp_v = up * g.area_v[(long long)l * nc + c] - lo * g.area_v[(long long)(l + 1) * nc + c];
    }
    return 1.0 / double(g.volume[(long long)l * nc + c]) * (comp_h.value() + double(comp_v));
}

/* ------------------------------------------------------------ momentum */

/* N^2 (effective_diff_coeffs.c:233-291) and the advection term of the TKE
 * update (tke.c:22-24: inner product of grad(tke) with the wind).  The
 * reference writes the last layer's N^2 past the end of n_squared, so that
 * layer keeps its value.  The TOA and surface vertical entries of the TKE
 * gradient are those the reference's placeholder field holds there (ph_tb):
 * grad leaves them unwritten. */
template <typename R>
__global__ void kd_n2_adv(HGrid<R> g, SView<R> sv, DiffBufs b, DiffScratch<R> s)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int nl = g.nl, l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const long long nc = g.nc;
    auto theta = [&](int ll) {
        const long long q = (long long)ll * nc + c;
        return g.theta_v_bg[q] + sv.theta_v_pert[q];
    };
    auto nsq = [&](int k) {
        const R tu = theta(k - 1), tl = theta(k);
        const R gr = (tu - tl) / g.nd_v[(long long)k * nc + c];
        const R scal = R(0.5) * (R(1) / tu + R(1) / tl);
        return g.gravity_m_v[(long long)k * nc + c] * (scal * gr);
    };
    if (l == 0)
        b.n2[i] = double(nsq(1));
    else if (l < nl - 1)
        b.n2[i] = double(ipw_at(g, 6, l, c) * nsq(l) + ipw_at(g, 7, l, c) * nsq(l + 1));
    /* advection of the TKE */
    const int n_edges = c < N_PENT ? 5 : 6;
    R r = R(0);
    for (int j = 0; j < n_edges; ++j) {
        const int e = g.adj[j * nc + c];
        r += ipw_at(g, j, l, c) * grad_h(g, b.tke, l, e) * sv.u[(long long)l * g.ne + e];
    }
    const R a_top = l >= 1 ? grad_v(g, b.tke, l, c) : R(b.ph_tb[c]);
    const R a_bot = l + 1 <= nl - 1 ? grad_v(g, b.tke, l + 1, c) : R(b.ph_tb[nc + c]);
    r += ipw_at(g, 6, l, c) * a_top * sv.w[i];
    r += ipw_at(g, 7, l, c) * a_bot * sv.w[i + nc];
    s.adv[i] = r;
}

/* TKE update (tke.c:26-58) */
template <typename R>
__global__ void kd_tke(long long ns, int gas, R dt, R mean_velocity_area, SView<R> sv, DiffBufs b, DiffScratch<R> s)
{
    const long long i = gtid();
    if (i >= ns) return;
    const R rg = sv.rho[gas * ns + i];
    const R decay = R(8.0 * (PI_ * PI_)) / mean_velocity_area * R(b.visc[i]) / rg;
    const R tke = R(b.tke[i]);
    R t = tke + dt * (-s.adv[i] + R(b.hdiss[i]) / rg - decay * tke);
    if (t < R(0)) t = R(0);
    b.tke[i] = double(t);
}

/* hor_viscosity (effective_diff_coeffs.c:19-112) at the cells: vint is the
 * molecular + turbulent value the rhombi and triangles average, visc the
 * final cell value (gas density times the turbulent part); with WDV also
 * visc times the divergence of the wind (momentum_diff_diss.c:29-40) */
template <typename R, bool WDV>
__global__ void kd_hor_visc(HGrid<R> g, R eff_hor_res, int gas, const double *temperature, SView<R> sv, DiffBufs b,
                            DiffScratch<R> s)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const R rg = sv.rho[gas * ns + i];
    const R tke = R(b.tke[i]);
    const R mol = calc_diffusion_coeff(R(temperature[i]), rg);
    b.mol[i] = double(mol);
    s.vint[i] = mol + tke2hor(tke, eff_hor_res);
    const R visc = rg * tke2hor(tke, eff_hor_res);
    b.visc[i] = double(visc);
    if (WDV) {
        const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
        s.wdv[i] = visc * R(divv_h_cell(g, sv.u, l, c));
    }
}

/* relative vorticity on the triangles times the viscosity averaged to them
 * (effective_diff_coeffs.c:67-103, momentum_diff_diss.c:54-57) */
template <typename R>
__global__ void kd_zt(HGrid<R> g, int gas, SView<R> sv, DiffScratch<R> s)
{
    const long long n = (long long)g.nl * g.nt, i = gtid();
    if (i >= n) return;
    const long long ns = (long long)g.nl * g.nc;
    const int l = (int)(i / g.nt), t = (int)(i - (long long)l * g.nt);
    const long long sb = (long long)l * g.nc;
    const int e0 = g.vort_i[t], e1 = g.vort_i[g.nt + t], e2 = g.vort_i[2 * g.nt + t];
    const R *v = s.vint, *rg = sv.rho + gas * ns;
    const R vt = R(1.0 / 6.0) * (v[sb + g.from[e0]] + v[sb + g.to[e0]] + v[sb + g.from[e1]] + v[sb + g.to[e1]]
                                 + v[sb + g.from[e2]] + v[sb + g.to[e2]]);
    const R dens = R(1.0 / 6.0) * (rg[sb + g.from[e0]] + rg[sb + g.to[e0]] + rg[sb + g.from[e1]] + rg[sb + g.to[e1]]
                                   + rg[sb + g.from[e2]] + rg[sb + g.to[e2]]);
    s.zt[i] = dens * vt * s.tri[i];
}

/* relative vorticity on the rhombi (vorticities.c:104-165) times the
 * viscosity averaged there (effective_diff_coeffs.c:44-65) */
template <typename R>
__global__ void kd_zr(HGrid<R> g, int gas, SView<R> sv, DiffScratch<R> s)
{
    const long long n = (long long)g.nl * g.ne, i = gtid();
    if (i >= n) return;
    const long long ns = (long long)g.nl * g.nc;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    const long long tf = (long long)l * g.nt + g.dual_from[e], tt = (long long)l * g.nt + g.dual_to[e];
    const R af = g.dual_area_t[tf], at = g.dual_area_t[tt];
    const R raw = (af * s.tri[tf] + at * s.tri[tt]) / (af + at);
    const long long f = (long long)l * g.nc + g.from[e], t = (long long)l * g.nc + g.to[e];
    const R *rg = sv.rho + gas * ns;
    R vr = R(0.5) * (s.vint[f] + s.vint[t]);
    vr = R(0.5) * (rg[f] + rg[t]) * vr;
    s.zr[i] = vr * raw;
}

/* hor_calc_curl_of_vorticity (momentum_diff_diss.c:207-294) at edge e of layer l */
template <typename R>
__device__ __forceinline__ R curl_of_vorticity(const HGrid<R> &g, const DiffGrid<R> &dg, const DiffScratch<R> &s,
                                               int l, int e)
{
    const int nt = g.nt, ne = g.ne, nl = g.nl;
    const int tt = g.dual_to[e], tf = g.dual_from[e];
    const R dnt = dg.dual_nd_t[(long long)l * nt + tt], dnf = dg.dual_nd_t[(long long)l * nt + tf];
    const R zto = s.zt[(long long)l * nt + tt], zfr = s.zt[(long long)l * nt + tf];
    const R cdw = fabs(zto - zfr) / (fabs(zto) + fabs(zfr) + R(EPS_SEC));
    const R *zr = s.zr + (long long)l * ne, *zh = g.z_h + (long long)l * ne;
    R out = R(0), delta_z = R(0);
    for (int j = 0; j < 3; ++j) {
        const int et = g.vort_i[j * nt + tt], ef = g.vort_i[j * nt + tf];
        out += +R(1.0 / 3.0) * (R(1) - cdw) * (dnt * zr[et] - dnf * zr[ef]);
        delta_z += R(1.0 / 3.0) * (zh[et] - zh[ef]);
    }
    out += cdw * (zto * dnt - zfr * dnf);
    out = out / g.area_h[(long long)l * ne + e];
    if (l >= nl - g.n_oro) {
        R delta_x = dg.dual_nd_sfc[e];
        delta_x = delta_x * (g.radius + zh[e]) / g.radius;
        const R tangential_slope = delta_z / delta_x;
        const int lu = l == 0 ? l : l - 1, ll = l == nl - 1 ? l : l + 1;
        const R delta_zeta = s.zr[(long long)lu * ne + e] - s.zr[(long long)ll * ne + e];
        delta_z = g.z_h[(long long)lu * ne + e] - g.z_h[(long long)ll * ne + e];
        const R dzeta_dz = delta_zeta / delta_z;
        out -= tangential_slope * dzeta_dz;
    }
    return out;
}

/* vertical-diffusion viscosity of u at half level k of edge e
 * (effective_diff_coeffs.c:114-168); the TOA and surface levels take the
 * values of the levels next to them */
template <typename R>
__device__ __forceinline__ R vert_hor_viscosity(const HGrid<R> &g, const DiffBufs &b, const DiffScratch<R> &s,
                                                const R *rg, int k, int e)
{
    if (k == 0) k = 1;
    if (k == g.nl) k = g.nl - 1;
    const long long nc = g.nc;
    const long long f0 = (long long)(k - 1) * nc + g.from[e], t0 = (long long)(k - 1) * nc + g.to[e];
    const long long f1 = (long long)k * nc + g.from[e], t1 = (long long)k * nc + g.to[e];
    const R *kv = s.kvt;
    R mdc = R(0.25) * (kv[f0] + kv[t0] + kv[f1] + kv[t1]);
    const R molecular_viscosity = R(0.25) * (R(b.mol[f0]) + R(b.mol[t0]) + R(b.mol[f1]) + R(b.mol[t1]));
    mdc += molecular_viscosity;
    return R(0.25) * (rg[f0] + rg[t0] + rg[f1] + rg[t1]) * mdc;
}

/* vertical shear of u at half level k (momentum_diff_diss.c:90-118); the TOA
 * row is never written by the reference and keeps the caller's values */
template <typename R>
__device__ __forceinline__ R dv_hdz(const HGrid<R> &g, const DiffGrid<R> &dg, const DiffBufs &b, const SView<R> &sv,
                                    int k, int e)
{
    const long long ne = g.ne;
    if (k == 0) return R(b.dvdz_top[e]);
    if (k == g.nl) {
        const long long q = (long long)(g.nl - 1) * ne + e, sfc = (long long)g.nl * g.nc;
        return sv.u[q] / (g.z_h[q] - R(0.5) * (dg.z_v[sfc + g.from[e]] + dg.z_v[sfc + g.to[e]]));
    }
    const long long qu = (long long)(k - 1) * ne + e, ql = (long long)k * ne + e;
    return (sv.u[qu] - sv.u[ql]) / (g.z_h[qu] - g.z_h[ql]);
}

/* friction acceleration of the horizontal wind: H, horizontal momentum
 * diffusion (momentum_diff_diss.c:59-79, replacing the value); V, vertical
 * diffusion of u (:120-135, added to it) */
template <typename R, bool H, bool V>
__global__ void kd_fric_h(HGrid<R> g, DiffGrid<R> dg, int n_const, int gas, SView<R> sv, DiffBufs b,
                          DiffScratch<R> s)
{
    const long long n = (long long)g.nl * g.ne, i = gtid();
    if (i >= n) return;
    const long long ns = (long long)g.nl * g.nc, nw = (long long)(g.nl + 1) * g.nc, nc = g.nc;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    const int fr = g.from[e], to = g.to[e];
    const long long f = (long long)l * nc + fr, t = (long long)l * nc + to;
    R fa;
    if (H) {
        const R gr = grad_h(g, s.wdv, l, e);
        const R cu = curl_of_vorticity(g, dg, s, l, e);
        fa = (gr - cu) / (R(0.5) * (density_total_r(sv.rho, n_const, ns, f) + density_total_r(sv.rho, n_const, ns, t)));
    } else {
        fa = R(b.fric[nw + i]);
    }
    if (V) {
        const R *rg = sv.rho + gas * ns;
        const R z_upper = R(0.5) * (dg.z_v[(long long)l * nc + fr] + dg.z_v[(long long)l * nc + to]);
        const R z_lower = R(0.5) * (dg.z_v[(long long)(l + 1) * nc + fr] + dg.z_v[(long long)(l + 1) * nc + to]);
        const R delta_z = z_upper - z_lower;
        fa += (vert_hor_viscosity(g, b, s, rg, l, e) * dv_hdz(g, dg, b, sv, l, e)
               - vert_hor_viscosity(g, b, s, rg, l + 1, e) * dv_hdz(g, dg, b, sv, l + 1, e))
              / delta_z
              / (R(0.5) * (density_total_r(sv.rho, n_const, ns, f) + density_total_r(sv.rho, n_const, ns, t)));
    }
    b.fric[nw + i] = double(fa);
}

/* diffusion of w, step a (momentum_diff_diss.c:137-150 and 153-166):
 * s1 = rho * viscosity * dw/dz, s2 = w averaged to the cell; also the
 * turbulent vertical diffusivity of the cell (kvt), which the vertical
 * diffusion of u averages to its half levels */
template <typename R>
__global__ void kd_wdiff_a(HGrid<R> g, DiffGrid<R> dg, int gas, SView<R> sv, DiffBufs b, DiffScratch<R> s)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int nl = g.nl, l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const long long nc = g.nc;
    const R up = l == 0 ? R(0) : sv.w[(long long)l * nc + c];
    const R lo = l == nl - 1 ? R(0) : sv.w[(long long)(l + 1) * nc + c];
    const R comp_v = up * g.area_v[(long long)l * nc + c] - lo * g.area_v[(long long)(l + 1) * nc + c];
    const R dwdz = R(0) + R(1) / g.volume[i] * comp_v;
    const R kv = tke2vert(R(b.tke[i]), R(b.n2[i]), dg.layer_thickness[i]);
    s.kvt[i] = kv;
    const R mdc = R(b.mol[i]) + kv;
    s.s1[i] = sv.rho[gas * ns + i] * mdc * dwdz;
    s.s2[i] = ipw_at(g, 6, l, c) * sv.w[(long long)l * nc + c] + ipw_at(g, 7, l, c) * sv.w[(long long)(l + 1) * nc + c];
}

/* step b (:167-182): viscosity at the edge times the horizontal gradient of s2 */
template <typename R>
__global__ void kd_wdiff_b(HGrid<R> g, DiffBufs b, DiffScratch<R> s)
{
    const long long n = (long long)g.nl * g.ne, i = gtid();
    if (i >= n) return;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    const long long o = (long long)l * g.nc;
    s.flx[i] = R(0.5) * (R(b.visc[o + g.from[e]]) + R(b.visc[o + g.to[e]])) * grad_h(g, s.s2, l, e);
}

/* step c (:184): divergence of the diffusive flux */
template <typename R>
__global__ void kd_wdiff_c(HGrid<R> g, DiffScratch<R> s)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    s.s3[i] = R(divv_h_cell(g, s.flx, l, c));
}

/* step d (:151 and :186-199) at the inner interfaces: second derivative of
 * s1, plus s3 averaged to the interface, divided by the density */
template <typename R>
__global__ void kd_wdiff_d(HGrid<R> g, int n_const, SView<R> sv, DiffBufs b, DiffScratch<R> s)
{
    const long long n = (long long)(g.nl - 1) * g.nc, i = gtid();
    if (i >= n) return;
    const long long ns = (long long)g.nl * g.nc, nc = g.nc;
    const int k = (int)(i / nc) + 1, c = (int)(i - (long long)(k - 1) * nc);
    const long long up = (long long)(k - 1) * nc + c, lo = (long long)k * nc + c;
    R fa = (s.s1[up] - s.s1[lo]) / g.nd_v[(long long)k * nc + c];
    fa += R(0.5) * (s.s3[up] + s.s3[lo]);
    fa = fa / (R(0.5) * (density_total_r(sv.rho, n_const, ns, up) + density_total_r(sv.rho, n_const, ns, lo)));
    b.fric[(long long)k * nc + c] = double(fa);
}

/* simple_dissipation_rate (momentum_diff_diss.c:296-310) */
template <typename R>
__global__ void kd_dissipation(HGrid<R> g, int n_const, SView<R> sv, DiffBufs b)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const long long nc = g.nc, nw = (long long)(g.nl + 1) * nc;
    const int n_edges = c < N_PENT ? 5 : 6;
    R r = R(0);
    for (int j = 0; j < n_edges; ++j) {
        const long long vi = (long long)l * g.ne + g.adj[j * nc + c];
        r += ipw_at(g, j, l, c) * sv.u[vi] * R(b.fric[nw + vi]);
    }
    r += ipw_at(g, 6, l, c) * sv.w[i] * R(b.fric[i]);
    r += ipw_at(g, 7, l, c) * sv.w[i + nc] * R(b.fric[i + nc]);
    b.hdiss[i] = double(-density_total_r(sv.rho, n_const, ns, i) * r);
}

/* ------------------------------------------------- Held-Suarez forcing */

/* boundary-layer friction of the Held-Suarez test
 * (src/subgrid_scale/planetary_boundary_layer.c:141-197), step a per cell:
 * the layer's pressure and, in the lowest layer, the surface pressure
 * extrapolated with the standard lapse rate; the reference evaluates both at
 * each edge's two cells, the same values */
template <typename R>
__global__ void kd_pbl_hs_cell(HGrid<R> g, DiffGrid<R> dg, int gas, int moist, const double *temperature, SView<R> sv,
                               DiffScratch<R> s)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int nl = g.nl, l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const R exner = g.exner_bg[i] + sv.exner_pert[i];
    const R p = R(P_0) * pow(exner, R(C_D_P / R_D));
    s.hs_p[i] = p;
    if (l == nl - 1) {
        const R lapse = R(0.0065);
        const R temp_lowest_layer = R(temperature[i]);
        const R temp_surface = temp_lowest_layer + lapse * (dg.z_scalar[i] - dg.z_v[(long long)nl * g.nc + c]);
        R gas_constant = R(R_D);
        if (moist) {
            const R rg = sv.rho[gas * ns + i], rv = sv.rho[(gas + 1) * ns + i];
            gas_constant = (rg - rv) * R(R_D) + rv * R(R_V);
            gas_constant = gas_constant / rg;
        }
        const R surface_p_factor = pow(R(1) - (temp_surface - temp_lowest_layer) / temp_surface,
                                       g.gravity_m_v[(long long)(nl - 1) * g.nc + c] / (gas_constant * lapse));
        s.hs_ps[c] = p / surface_p_factor;
    }
}

/* step b per edge: Rayleigh friction below sigma = 0.7, added to the
 * friction acceleration */
template <typename R>
__global__ void kd_pbl_hs(HGrid<R> g, SView<R> sv, DiffBufs b, DiffScratch<R> s)
{
    const long long n = (long long)g.nl * g.ne, i = gtid();
    if (i >= n) return;
    const long long nw = (long long)(g.nl + 1) * g.nc;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    const long long o = (long long)l * g.nc;
    const R pressure = R(0.5) * (s.hs_p[o + g.from[e]] + s.hs_p[o + g.to[e]]);
    const R pressure_sfc = R(0.5) * (s.hs_ps[g.from[e]] + s.hs_ps[g.to[e]]);
    const R sigma = pressure / pressure_sfc, sigma_b = R(0.7);
    const R fa = R(b.fric[nw + i]) + -R(1.0 / 86400.0) * fmax(R(0), (sigma - sigma_b) / (R(1) - sigma_b)) * sv.u[i];
    b.fric[nw + i] = double(fa);
}

/* Held-Suarez radiative forcing (src/radiation/held_suar.c:18-56), FP64 on
 * both paths (it is updated only every radiation time step), at the cells the
 * reference's radiation blocks reach */
__device__ __forceinline__ double hs_t_eq(double latitude, double pressure)
{
    const double delta_t_y = 60.0, delta_theta_v_z = 10.0, kappa = 2.0 / 7.0;
    double result = 315.0;
    result = result - delta_t_y * pow(sin(latitude), 2.0);
    result = result - delta_theta_v_z * log(pressure / P_0) * pow(cos(latitude), 2.0);
    result = result * pow(pressure / P_0, kappa);
    return fmax(200.0, result);
}

__device__ __forceinline__ double hs_k_t(double latitude, double pressure)
{
    const double k_a = 1.0 / 40.0 * 1.0 / 86400.0, k_s = 1.0 / 4.0 * 1.0 / 86400.0, sigma_b = 0.7;
    const double sigma = pressure / P_0;
    return k_a + (k_s - k_a) * fmax(0.0, (sigma - sigma_b) / (1.0 - sigma_b)) * pow(cos(latitude), 4.0);
}

__global__ void kd_hs_rad(long long ns, int nc, int gas, const double *lat, const int *cov, const double *temperature,
                          DState so, double *rad)
{
    const long long i = gtid();
    if (i >= ns) return;
    const int c = (int)(i % nc);
    if (!cov[c]) return;
    const double rg = so.rho[gas * ns + i], t = temperature[i];
    const double pressure = rg * R_D * t;
    double r = -hs_k_t(lat[c], pressure) * (t - hs_t_eq(lat[c], pressure));
    rad[i] = C_D_V * rg * r;
}

/* -------------------------------------------------------------- scalars */

/* scalar_diffusion_coeffs (effective_diff_coeffs.c:203-229); c_v as
 * c_v_mass_weighted_air (derived_quantities.c:97-115) */
template <typename R>
__global__ void kd_sdiff_coeff(long long ns, int n_cond, int moist, const R *lt, const R *cp_ice, const R *cp_water,
                               SView<R> sv, DiffBufs b, DiffScratch<R> s)
{
    const long long i = gtid();
    if (i >= ns) return;
    const R mch = R(b.visc[i]) / sv.rho[n_cond * ns + i];
    const R mcv = R(b.mol[i]) + tke2vert(R(b.tke[i]), R(b.n2[i]), lt[i]);
    s.mch[i] = mch;
    s.mcv[i] = mcv;
    R cv = R(0);
    for (int k = 0; k < n_cond; ++k) cv += sv.rho[k * ns + i] * ((k % 2 == 0) ? cp_ice[i] : cp_water[i]);
    cv += sv.rho[n_cond * ns + i] * R(C_D_V);
    if (moist) cv += sv.rho[(n_cond + 1) * ns + i] * R(C_V_V);
    s.tch[i] = cv * mch;
    s.tcv[i] = cv * mcv;
}

/* the fields a scalar-diffusion pass treats: temperature (stored in double)
 * and/or every density (read in R); inv_vol (mixed path) is 1 / volume */
template <typename R>
struct SFields {
    int nf;
    const void *f[8];   /* [L][Nc] */
    int f_double[8];
    const R *kh[8], *kv[8];
    int vert[8];
    double *out[8];     /* [L][Nc] */
    const double *inv_vol;
};

template <typename R>
__device__ __forceinline__ R sfield(const SFields<R> &sf, int q, long long idx)
{
    return sf.f_double[q] ? R(((const double *)sf.f[q])[idx]) : ((const R *)sf.f[q])[idx];
}

/* diffusive fluxes: one thread per edge of a layer (gradient with the
 * terrain-following correction, gradient_operators.c:66-74, times the
 * coefficient averaged to the edge, multiplications.c:45-66) or per inner
 * interface (vertical gradient times the coefficient averaged to the
 * interface, multiplications.c:98-117), for every field; the grid terms
 * are loaded once for all fields.  FP64 path: divisions as the reference;
 * mixed path: one reciprocal per distance, shared by the fields. */
template <typename R>
__global__ void kd_sdiff_flux(HGrid<R> g, SFields<R> sf, DiffScratch<R> s)
{
    constexpr bool EXACT = sizeof(R) == sizeof(double);
    auto quot = [](R x, R d, R rd) { return EXACT ? x / d : x * rd; };
    const long long nh = (long long)g.nl * g.ne, nv = (long long)(g.nl - 1) * g.nc, i = gtid();
    const long long nc = g.nc;
    const int nl = g.nl;
    if (i < nh) {
        const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
        const int fr = g.from[e], to = g.to[e];
        const long long o = (long long)l * nc;
        const R nd = g.nd_h[i];
        const bool oro = l >= nl - g.n_oro, below = l < nl - 1;
        R w6f = R(0), w6t = R(0), w7f = R(0), w7t = R(0), d6f = R(1), d6t = R(1), d7f = R(1), d7t = R(1), sl = R(0);
        if (oro) {
            w6f = ipw_at(g, 6, l, fr);
            w6t = ipw_at(g, 6, l, to);
            d6f = g.nd_v[o + fr];
            d6t = g.nd_v[o + to];
            if (below) {
                w7f = ipw_at(g, 7, l, fr);
                w7t = ipw_at(g, 7, l, to);
                d7f = g.nd_v[o + nc + fr];
                d7t = g.nd_v[o + nc + to];
            }
            sl = g.slope_h[i];
        }
        const R rnd = EXACT ? R(0) : R(1) / nd, r6f = EXACT ? R(0) : R(1) / d6f, r6t = EXACT ? R(0) : R(1) / d6t;
        const R r7f = EXACT ? R(0) : R(1) / d7f, r7t = EXACT ? R(0) : R(1) / d7t;
        for (int q = 0; q < sf.nf; ++q) {
            R gr = quot(sfield(sf, q, o + to) - sfield(sf, q, o + fr), nd, rnd);
            if (oro) {
                R cc = w6f * quot(sfield(sf, q, o - nc + fr) - sfield(sf, q, o + fr), d6f, r6f);
                cc += w6t * quot(sfield(sf, q, o - nc + to) - sfield(sf, q, o + to), d6t, r6t);
                if (below) {
                    cc += w7f * quot(sfield(sf, q, o + fr) - sfield(sf, q, o + nc + fr), d7f, r7f);
                    cc += w7t * quot(sfield(sf, q, o + to) - sfield(sf, q, o + nc + to), d7t, r7t);
                }
                cc = R(0.5) * cc;
                gr += -sl * cc;
            }
            const R sc = R(0.5) * (sf.kh[q][o + to] + sf.kh[q][o + fr]);
            s.fh[(long long)q * nh + i] = sc * gr;
        }
    } else if (i < nh + nv) {
        const long long rv = i - nh;
        const int k = (int)(rv / nc) + 1, c = (int)(rv - (long long)(k - 1) * nc);
        const long long up = (long long)(k - 1) * nc + c, lo = (long long)k * nc + c;
        const R nd = g.nd_v[lo], rnd = EXACT ? R(0) : R(1) / nd;
        for (int q = 0; q < sf.nf; ++q) {
            if (!sf.vert[q]) continue;
            const R sc = R(0.5) * (sf.kv[q][up] + sf.kv[q][lo]);
            const R gr = quot(sfield(sf, q, up) - sfield(sf, q, lo), nd, rnd);
            s.fv[(long long)q * (nl + 1) * nc + lo] = sc * gr;
        }
    }
}

/* their divergences, one thread per cell for every field: divv_h
 * (divergences.c:14-64) and add_vertical_divv (:150-185).  The cell's edges,
 * signs, face areas and terrain-correction weights are loaded once; the
 * terms are summed in the reference's order (FP64 path) or as double-word
 * pairs (mixed path), and the mixed path multiplies by 1 / volume */
template <typename R>
__global__ void kd_sdiff_div(HGrid<R> g, SFields<R> sf, DiffScratch<R> s)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int nl = g.nl, n_oro = g.n_oro, l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const long long nc = g.nc, ne = g.ne, nh = (long long)nl * ne;
    const int n_edges = c < N_PENT ? 5 : 6;
    int ej[6];
    R sg[6], ar[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        const bool on = j < n_edges;
        ej[j] = on ? g.adj[j * nc + c] : 0;
        sg[j] = on ? R(g.adj_sign[j * nc + c]) : R(0);
        ar[j] = on ? g.area_h[(long long)l * ne + ej[j]] : R(0);
    }
    /* terrain correction (averaging.c:41-95) at level l (up, from layers l-1
     * and l) and level l+1 (lo, from layers l and l+1) */
    const bool oro = l >= nl - n_oro - 1;
    const bool need_up = oro && l != nl - n_oro - 1, need_lo = oro && l != nl - 1;
    const bool up_prev = need_up && l > nl - n_oro, lo_prev = need_lo && l + 1 > nl - n_oro;
    R wu0[6], wu1[6], wl1[6];
    auto wcorr = [&](int ll, int j) { return R(-0.5) * ipw_at(g, j, ll, c) * g.slope_h[(long long)ll * ne + ej[j]]; };
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        const bool on = j < n_edges;
        wu0[j] = on && up_prev ? wcorr(l - 1, j) : R(0);
        wu1[j] = on && (need_up || lo_prev) ? wcorr(l, j) : R(0);
        wl1[j] = on && need_lo ? wcorr(l + 1, j) : R(0);
    }
    const R area_up = g.area_v[(long long)l * nc + c], area_lo = g.area_v[(long long)(l + 1) * nc + c];
    const bool exact = sizeof(R) == sizeof(double);
    const double iv = exact ? 0.0 : sf.inv_vol[i];
    for (int q = 0; q < sf.nf; ++q) {
        const R *fh = s.fh + (long long)q * nh;
        FluxSum<R> comp_h;
        for (int j = 0; j < n_edges; ++j) comp_h.add(fh[(long long)l * ne + ej[j]] * sg[j] * ar[j]);
        R up = R(0), lo = R(0);
        if (need_up) {
            if (up_prev)
                for (int j = 0; j < n_edges; ++j) up += wu0[j] * fh[(long long)(l - 1) * ne + ej[j]];
            for (int j = 0; j < n_edges; ++j) up += wu1[j] * fh[(long long)l * ne + ej[j]];
        }
        if (need_lo) {
            if (lo_prev)
                for (int j = 0; j < n_edges; ++j) lo += wu1[j] * fh[(long long)l * ne + ej[j]];
            for (int j = 0; j < n_edges; ++j) lo += wl1[j] * fh[(long long)(l + 1) * ne + ej[j]];
        }
        R comp_v = R(0);
        if (oro) {
            if (l == nl - n_oro - 1) comp_v = -lo * area_lo;
            else if (l == nl - 1) comp_v = up * area_up;
            else comp_v = up * area_up - lo * area_lo;
        }
        double out = exact ? 1.0 / double(g.volume[i]) * (comp_h.value() + double(comp_v))
                           : iv * (comp_h.value() + double(comp_v));
        if (sf.vert[q]) {
            const R *fv = s.fv + (long long)q * (nl + 1) * nc;
            const R vu = l == 0 ? R(0) : fv[(long long)l * nc + c];
            const R vl = l == nl - 1 ? R(0) : fv[(long long)(l + 1) * nc + c];
            const double cv = double(vu * area_up) - double(vl * area_lo);
            out += exact ? 1 / double(g.volume[i]) * cv : iv * cv;
        }
        sf.out[q][i] = out;
    }
}

/* the momentum part of the branch (vector_tendencies_expl.c:41-69) */
template <typename R>
void diffusion_momentum(Context *c, const StepParams &p, const HGrid<R> &g, const DiffGrid<R> &dg,
                        const SView<R> &sv)
{
    const bool any_h = p.diff & (DIFF_MOM_H | DIFF_TEMP_H | DIFF_MASS_H);
    const bool H = p.diff & DIFF_MOM_H, V = p.diff & DIFF_MOM_V, PBL = p.diff & DIFF_PBL_HS;
    if (!any_h && !V && !PBL) return;
    DiffBufs &b = *c->dbuf;
    const DiffScratch<R> s = diff_scratch<R>(b);
    const long long ns = c->ns, nh = (long long)c->nl * c->ne;
    const int gas = c->n_cond;
    cudaStream_t st = c->stream;
    if (any_h) {
        {
            ProfScope ps(c, "kd_n2_adv");
            kd_n2_adv<R><<<dnb(ns), 256, 0, st>>>(g, sv, b, s);
        }
        {
            ProfScope ps(c, "kd_tke");
            kd_tke<R><<<dnb(ns), 256, 0, st>>>(ns, gas, R(p.dt), R(dg.mean_velocity_area), sv, b, s);
        }
        c->kernel_launches += 2;
    }
    if (H) {
        {
            ProfScope ps(c, "kd_hor_visc");
            kd_hor_visc<R, true><<<dnb(ns), 256, 0, st>>>(g, R(dg.eff_hor_res), gas, c->temperature, sv, b, s);
        }
        {
            ProfScope ps(c, "kd_tri_vort");
            k_tri_vort<R><<<dnb((long long)c->nl * c->nt), 256, 0, st>>>(g, sv.u, s.tri);
        }
        {
            ProfScope ps(c, "kd_zt");
            kd_zt<R><<<dnb((long long)c->nl * c->nt), 256, 0, st>>>(g, gas, sv, s);
        }
        {
            ProfScope ps(c, "kd_zr");
            kd_zr<R><<<dnb(nh), 256, 0, st>>>(g, gas, sv, s);
        }
        c->kernel_launches += 4;
    }
    if (V) {
        ProfScope ps(c, "kd_wdiff_a");
        kd_wdiff_a<R><<<dnb(ns), 256, 0, st>>>(g, dg, gas, sv, b, s);
        c->kernel_launches++;
    }
    {
        ProfScope ps(c, "kd_fric_h");
        if (H && V) kd_fric_h<R, true, true><<<dnb(nh), 256, 0, st>>>(g, dg, c->n_const, gas, sv, b, s);
        else if (H) kd_fric_h<R, true, false><<<dnb(nh), 256, 0, st>>>(g, dg, c->n_const, gas, sv, b, s);
        else if (V) kd_fric_h<R, false, true><<<dnb(nh), 256, 0, st>>>(g, dg, c->n_const, gas, sv, b, s);
        if (H || V) c->kernel_launches++;
    }
    if (V) {
        {
            ProfScope ps(c, "kd_wdiff_b");
            kd_wdiff_b<R><<<dnb(nh), 256, 0, st>>>(g, b, s);
        }
        {
            ProfScope ps(c, "kd_wdiff_c");
            kd_wdiff_c<R><<<dnb(ns), 256, 0, st>>>(g, s);
        }
        {
            ProfScope ps(c, "kd_wdiff_d");
            kd_wdiff_d<R><<<dnb((long long)(c->nl - 1) * c->nc), 256, 0, st>>>(g, c->n_const, sv, b, s);
        }
        c->kernel_launches += 3;
    }
    if (PBL) {
        {
            ProfScope ps(c, "kd_pbl_hs_cell");
            kd_pbl_hs_cell<R><<<dnb(ns), 256, 0, st>>>(g, dg, gas, c->moist, c->temperature, sv, s);
        }
        {
            ProfScope ps(c, "kd_pbl_hs");
            kd_pbl_hs<R><<<dnb(nh), 256, 0, st>>>(g, sv, b, s);
        }
        c->kernel_launches += 2;
    }
    if (H || PBL) {
        ProfScope ps(c, "kd_dissipation");
        kd_dissipation<R><<<dnb(ns), 256, 0, st>>>(g, c->n_const, sv, b);
        c->kernel_launches++;
    }
    /* grad_hor (called by both momentum diffusions) zeroes the vertical
     * entries of the reference's placeholder field, TOA and surface included */
    if (H || V) cudaMemsetAsync(b.ph_tb, 0, (size_t)2 * c->nc * sizeof(double), st);
}

/* the scalar part (scalar_tendencies_expl.c:44-88) */
template <typename R>
void diffusion_scalar(Context *c, const StepParams &p, const HGrid<R> &g, const DiffGrid<R> &dg, const SView<R> &sv,
                      const R *cp_ice, const R *cp_water)
{
    const bool TH = p.diff & DIFF_TEMP_H, MH = p.diff & DIFF_MASS_H;
    if (!TH && !MH) return;
    DiffBufs &b = *c->dbuf;
    const DiffScratch<R> s = diff_scratch<R>(b);
    const long long ns = c->ns;
    const int gas = c->n_cond;
    cudaStream_t st = c->stream;
    if (!(p.diff & DIFF_MOM_H)) {
        ProfScope ps(c, "kd_hor_visc");
        kd_hor_visc<R, false><<<dnb(ns), 256, 0, st>>>(g, R(dg.eff_hor_res), gas, c->temperature, sv, b, s);
        c->kernel_launches++;
    }
    {
        ProfScope ps(c, "kd_sdiff_coeff");
        kd_sdiff_coeff<R><<<dnb(ns), 256, 0, st>>>(ns, c->n_cond, c->moist, dg.layer_thickness, cp_ice, cp_water, sv,
                                                     b, s);
        c->kernel_launches++;
    }
    SFields<R> sf{};
    if (TH) {
        sf.f[sf.nf] = c->temperature;
        sf.f_double[sf.nf] = 1;
        sf.kh[sf.nf] = s.tch;
        sf.kv[sf.nf] = s.tcv;
        sf.vert[sf.nf] = (p.diff & DIFF_TEMP_V) ? 1 : 0;
        sf.out[sf.nf] = b.tdh;
        ++sf.nf;
    }
    if (MH)
        for (int k = 0; k < c->n_const; ++k) {
            sf.f[sf.nf] = sv.rho + (long long)k * ns;
            sf.f_double[sf.nf] = sizeof(R) == sizeof(double);
            sf.kh[sf.nf] = s.mch;
            sf.kv[sf.nf] = s.mcv;
            sf.vert[sf.nf] = (p.diff & DIFF_MASS_V) ? 1 : 0;
            sf.out[sf.nf] = b.mdt + (long long)k * ns;
            ++sf.nf;
        }
    sf.inv_vol = c->inv_vol;
    const long long per = (long long)c->nl * c->ne + (long long)(c->nl - 1) * c->nc;
    {
        ProfScope ps(c, "kd_sdiff_flux");
        kd_sdiff_flux<R><<<dnb(per), 256, 0, st>>>(g, sf, s);
    }
    {
        ProfScope ps(c, "kd_sdiff_div");
        kd_sdiff_div<R><<<dnb(ns, 128), 128, 0, st>>>(g, sf, s);
    }
    c->kernel_launches += 2;
}

}  // namespace
}  // namespace game
