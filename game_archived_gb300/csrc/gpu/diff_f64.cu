/*
 * Diffusion branch of the RKHEVI step: Brunt-Vaisala frequency, TKE update,
 * effective viscosities, horizontal and vertical momentum diffusion, the
 * dissipation rate, and temperature and mass diffusion
 * (src/subgrid_scale/effective_diff_coeffs.c, src/subgrid_scale/tke.c,
 * src/spatial_operators/momentum_diff_diss.c, called from
 * src/time_stepping/vector_tendencies_expl.c:41-69 and
 * scalar_tendencies_expl.c:44-88 at the first RK substep).
 *
 * FP64 on both precision paths, compiled with --fmad=false, every
 * expression in the reference's operation order.  The reference's
 * sequence of whole-field operator calls (each writing a placeholder field)
 * becomes a few fused per-point kernels:
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
#include "diff.h"
#include "kernels.cuh"

namespace game {
namespace {

using G = HGrid<double>;

constexpr double K_B_ = 1.380649e-23;
constexpr double PI_ = 3.14159265358979323846;
constexpr double EPS_SEC = 1e-10;

inline unsigned nb(long long n, int bs = 256) { return (unsigned)((n + bs - 1) / bs); }

/* molecular diffusion coefficient from kinetic gas theory
 * (src/constituents/derived_quantities.c:117-134); pow(r, 2) is the product
 * r * r, which the reference's compiler folds it to */
__device__ __forceinline__ double calc_diffusion_coeff(double temperature, double density)
{
    const double particle_radius = 130e-12;
    const double particle_mass = M_D / N_A;
    const double thermal_velocity = sqrt(8.0 * K_B_ * temperature / (PI_ * particle_mass));
    const double particle_density = density / particle_mass;
    const double cross_section = 4.0 * PI_ * (particle_radius * particle_radius);
    const double mean_free_path = 1.0 / (sqrt(2.0) * particle_density * cross_section);
    return 1.0 / 3.0 * thermal_velocity * mean_free_path;
}

/* effective_diff_coeffs.c:293-303 (x^0.5 as sqrt) */
__device__ __forceinline__ double tke2hor(double tke, double effective_resolution)
{
    const double mean_velocity = sqrt(2.0 * tke);
    const double mean_free_path = effective_resolution / 6.0;
    return 1.0 / 6.0 * mean_free_path * mean_velocity;
}

/* effective_diff_coeffs.c:305-320 */
__device__ __forceinline__ double tke2vert(double tke, double n_squared, double layer_thickness)
{
    const double tke_vert = 3.0 * 1e-3 * tke;
    const double mean_velocity = sqrt(2.0 * tke_vert);
    const double n_used = sqrt(fmax(n_squared, 1e-4));
    double mean_free_path = sqrt(2.0 * tke_vert) / n_used;
    mean_free_path = fmin(mean_free_path, layer_thickness);
    return 1.0 / 6.0 * mean_free_path * mean_velocity;
}

/* divv_h (divergences.c:14-64) at cell c of layer l of the edge field in_u [L][Ne] */
__device__ __forceinline__ double divv_h_cell(const G &g, const double *in_u, int l, int c)
{
    const int n_edges = c < N_PENT ? 5 : 6, nl = g.nl, n_oro = g.n_oro;
    const long long nc = g.nc;
    double comp_h = 0.0;
    for (int j = 0; j < n_edges; ++j) {
        const long long vi = (long long)l * g.ne + g.adj[j * nc + c];
        comp_h += in_u[vi] * double(g.adj_sign[j * nc + c]) * g.area_h[vi];
    }
    auto fin = [&](int ll, int j) { return in_u[(long long)ll * g.ne + g.adj[j * nc + c]]; };
    double comp_v = 0.0;
    if (l == nl - n_oro - 1) {
        const double lo = contra_corr(g, l + 1, c, n_edges, fin);
        comp_v = -lo * g.area_v[(long long)(l + 1) * nc + c];
    } else if (l == nl - 1) {
        const double up = contra_corr(g, l, c, n_edges, fin);
        comp_v = up * g.area_v[(long long)l * nc + c];
    } else if (l > nl - n_oro - 1) {
        const double up = contra_corr(g, l, c, n_edges, fin);
        const double lo = contra_corr(g, l + 1, c, n_edges, fin);
        comp_v = up * g.area_v[(long long)l * nc + c] - lo * g.area_v[(long long)(l + 1) * nc + c];
    }
    return 1.0 / g.volume[(long long)l * nc + c] * (comp_h + comp_v);
}

/* ------------------------------------------------------------ momentum */

/* N^2 (effective_diff_coeffs.c:233-291) and the advection term of the TKE
 * update (tke.c:22-24: inner product of grad(tke) with the wind).  The
 * reference writes the last layer's N^2 past the end of n_squared, so that
 * layer keeps its value.  The TOA and surface vertical entries of the TKE
 * gradient are those the reference's placeholder field holds there (ph_tb):
 * grad leaves them unwritten. */
__global__ void kd_n2_adv(G g, DState sn, DiffBufs b)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int nl = g.nl, l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const long long nc = g.nc;
    auto theta = [&](int ll) {
        const long long q = (long long)ll * nc + c;
        return g.theta_v_bg[q] + sn.theta_v_pert[q];
    };
    auto nsq = [&](int k) {
        const double tu = theta(k - 1), tl = theta(k);
        const double gr = (tu - tl) / g.nd_v[(long long)k * nc + c];
        const double sv = 0.5 * (1.0 / tu + 1.0 / tl);
        return g.gravity_m_v[(long long)k * nc + c] * (sv * gr);
    };
    if (l == 0)
        b.n2[i] = nsq(1);
    else if (l < nl - 1)
        b.n2[i] = ipw_at(g, 6, l, c) * nsq(l) + ipw_at(g, 7, l, c) * nsq(l + 1);
    /* advection of the TKE */
    const int n_edges = c < N_PENT ? 5 : 6;
    double r = 0;
    for (int j = 0; j < n_edges; ++j) {
        const int e = g.adj[j * nc + c];
        r += ipw_at(g, j, l, c) * grad_h(g, b.tke, l, e) * sn.u[(long long)l * g.ne + e];
    }
    const double a_top = l >= 1 ? grad_v(g, b.tke, l, c) : b.ph_tb[c];
    const double a_bot = l + 1 <= nl - 1 ? grad_v(g, b.tke, l + 1, c) : b.ph_tb[nc + c];
    r += ipw_at(g, 6, l, c) * a_top * sn.w[i];
    r += ipw_at(g, 7, l, c) * a_bot * sn.w[i + nc];
    b.adv[i] = r;
}

/* TKE update (tke.c:26-58) */
__global__ void kd_tke(long long ns, int gas, double dt, double mean_velocity_area, DState sn, DiffBufs b)
{
    const long long i = gtid();
    if (i >= ns) return;
    const double rg = sn.rho[gas * ns + i];
    const double decay = 8.0 * (PI_ * PI_) / mean_velocity_area * b.visc[i] / rg;
    double t = b.tke[i] + dt * (-b.adv[i] + b.hdiss[i] / rg - decay * b.tke[i]);
    if (t < 0.0) t = 0.0;
    b.tke[i] = t;
}

/* hor_viscosity (effective_diff_coeffs.c:19-112) at the cells: vint is the
 * molecular + turbulent value the rhombi and triangles average, visc the
 * final cell value (gas density times the turbulent part); with WDV also
 * visc times the divergence of the wind (momentum_diff_diss.c:29-40) */
template <bool WDV>
__global__ void kd_hor_visc(G g, double eff_hor_res, int gas, const double *temperature, DState sn, DiffBufs b)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const double rg = sn.rho[gas * ns + i];
    const double mol = calc_diffusion_coeff(temperature[i], rg);
    b.mol[i] = mol;
    b.vint[i] = mol + tke2hor(b.tke[i], eff_hor_res);
    const double visc = rg * tke2hor(b.tke[i], eff_hor_res);
    b.visc[i] = visc;
    if (WDV) {
        const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
        b.wdv[i] = visc * divv_h_cell(g, sn.u, l, c);
    }
}

/* relative vorticity on the triangles times the viscosity averaged to them
 * (effective_diff_coeffs.c:67-103, momentum_diff_diss.c:54-57) */
__global__ void kd_zt(G g, int gas, DState sn, DiffBufs b)
{
    const long long n = (long long)g.nl * g.nt, i = gtid();
    if (i >= n) return;
    const long long ns = (long long)g.nl * g.nc;
    const int l = (int)(i / g.nt), t = (int)(i - (long long)l * g.nt);
    const long long sb = (long long)l * g.nc;
    const int e0 = g.vort_i[t], e1 = g.vort_i[g.nt + t], e2 = g.vort_i[2 * g.nt + t];
    const double *v = b.vint, *rg = sn.rho + gas * ns;
    const double vt = 1.0 / 6.0 * (v[sb + g.from[e0]] + v[sb + g.to[e0]] + v[sb + g.from[e1]] + v[sb + g.to[e1]]
                                   + v[sb + g.from[e2]] + v[sb + g.to[e2]]);
    const double dens = 1.0 / 6.0 * (rg[sb + g.from[e0]] + rg[sb + g.to[e0]] + rg[sb + g.from[e1]] + rg[sb + g.to[e1]]
                                     + rg[sb + g.from[e2]] + rg[sb + g.to[e2]]);
    b.zt[i] = dens * vt * b.tri[i];
}

/* relative vorticity on the rhombi (vorticities.c:104-165) times the
 * viscosity averaged there (effective_diff_coeffs.c:44-65) */
__global__ void kd_zr(G g, int gas, DState sn, DiffBufs b)
{
    const long long n = (long long)g.nl * g.ne, i = gtid();
    if (i >= n) return;
    const long long ns = (long long)g.nl * g.nc;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    const long long tf = (long long)l * g.nt + g.dual_from[e], tt = (long long)l * g.nt + g.dual_to[e];
    const double af = g.dual_area_t[tf], at = g.dual_area_t[tt];
    const double raw = (af * b.tri[tf] + at * b.tri[tt]) / (af + at);
    const long long f = (long long)l * g.nc + g.from[e], t = (long long)l * g.nc + g.to[e];
    const double *rg = sn.rho + gas * ns;
    double vr = 0.5 * (b.vint[f] + b.vint[t]);
    vr = 0.5 * (rg[f] + rg[t]) * vr;
    b.zr[i] = vr * raw;
}

/* hor_calc_curl_of_vorticity (momentum_diff_diss.c:207-294) at edge e of layer l */
__device__ __forceinline__ double curl_of_vorticity(const G &g, const DiffGrid &dg, const DiffBufs &b, int l, int e)
{
    const int nt = g.nt, ne = g.ne, nl = g.nl;
    const int tt = g.dual_to[e], tf = g.dual_from[e];
    const double dnt = dg.dual_nd_t[(long long)l * nt + tt], dnf = dg.dual_nd_t[(long long)l * nt + tf];
    const double zto = b.zt[(long long)l * nt + tt], zfr = b.zt[(long long)l * nt + tf];
    const double cdw = fabs(zto - zfr) / (fabs(zto) + fabs(zfr) + EPS_SEC);
    const double *zr = b.zr + (long long)l * ne, *zh = g.z_h + (long long)l * ne;
    double out = 0.0, delta_z = 0.0;
    for (int j = 0; j < 3; ++j) {
        const int et = g.vort_i[j * nt + tt], ef = g.vort_i[j * nt + tf];
        out += +1.0 / 3.0 * (1.0 - cdw) * (dnt * zr[et] - dnf * zr[ef]);
        delta_z += 1.0 / 3.0 * (zh[et] - zh[ef]);
    }
    out += cdw * (zto * dnt - zfr * dnf);
    out = out / g.area_h[(long long)l * ne + e];
    if (l >= nl - g.n_oro) {
        double delta_x = dg.dual_nd_sfc[e];
        delta_x = delta_x * (g.radius + zh[e]) / g.radius;
        const double tangential_slope = delta_z / delta_x;
        const int lu = l == 0 ? l : l - 1, ll = l == nl - 1 ? l : l + 1;
        const double delta_zeta = b.zr[(long long)lu * ne + e] - b.zr[(long long)ll * ne + e];
        delta_z = g.z_h[(long long)lu * ne + e] - g.z_h[(long long)ll * ne + e];
        const double dzeta_dz = delta_zeta / delta_z;
        out -= tangential_slope * dzeta_dz;
    }
    return out;
}

/* vertical-diffusion viscosity of u at half level k of edge e
 * (effective_diff_coeffs.c:114-168); the TOA and surface levels take the
 * values of the levels next to them */
__device__ __forceinline__ double vert_hor_viscosity(const G &g, const DiffGrid &dg, const DiffBufs &b,
                                                     const double *rg, int k, int e)
{
    if (k == 0) k = 1;
    if (k == g.nl) k = g.nl - 1;
    const long long nc = g.nc;
    const long long f0 = (long long)(k - 1) * nc + g.from[e], t0 = (long long)(k - 1) * nc + g.to[e];
    const long long f1 = (long long)k * nc + g.from[e], t1 = (long long)k * nc + g.to[e];
    const double *lt = dg.layer_thickness;
    double mdc = 0.25 * (tke2vert(b.tke[f0], b.n2[f0], lt[f0]) + tke2vert(b.tke[t0], b.n2[t0], lt[t0])
                         + tke2vert(b.tke[f1], b.n2[f1], lt[f1]) + tke2vert(b.tke[t1], b.n2[t1], lt[t1]));
    const double molecular_viscosity = 0.25 * (b.mol[f0] + b.mol[t0] + b.mol[f1] + b.mol[t1]);
    mdc += molecular_viscosity;
    return 0.25 * (rg[f0] + rg[t0] + rg[f1] + rg[t1]) * mdc;
}

/* vertical shear of u at half level k (momentum_diff_diss.c:90-118); the TOA
 * row is never written by the reference and keeps the caller's values */
__device__ __forceinline__ double dv_hdz(const G &g, const VGrid &vg, const DiffBufs &b, const DState &sn, int k, int e)
{
    const long long ne = g.ne;
    if (k == 0) return b.dvdz_top[e];
    if (k == g.nl) {
        const long long q = (long long)(g.nl - 1) * ne + e, s = (long long)g.nl * g.nc;
        return sn.u[q] / (g.z_h[q] - 0.5 * (vg.z_v[s + g.from[e]] + vg.z_v[s + g.to[e]]));
    }
    const long long qu = (long long)(k - 1) * ne + e, ql = (long long)k * ne + e;
    return (sn.u[qu] - sn.u[ql]) / (g.z_h[qu] - g.z_h[ql]);
}

/* friction acceleration of the horizontal wind: H, horizontal momentum
 * diffusion (momentum_diff_diss.c:59-79, replacing the value); V, vertical
 * diffusion of u (:120-135, added to it) */
template <bool H, bool V>
__global__ void kd_fric_h(G g, VGrid vg, DiffGrid dg, int n_const, int gas, DState sn, DiffBufs b)
{
    const long long n = (long long)g.nl * g.ne, i = gtid();
    if (i >= n) return;
    const long long ns = (long long)g.nl * g.nc, nw = (long long)(g.nl + 1) * g.nc, nc = g.nc;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    const int fr = g.from[e], to = g.to[e];
    const long long f = (long long)l * nc + fr, t = (long long)l * nc + to;
    double fa;
    if (H) {
        const double gr = grad_h(g, b.wdv, l, e);
        const double cu = curl_of_vorticity(g, dg, b, l, e);
        fa = (gr - cu) / (0.5 * (density_total(sn.rho, n_const, ns, f) + density_total(sn.rho, n_const, ns, t)));
    } else {
        fa = b.fric[nw + i];
    }
    if (V) {
        const double *rg = sn.rho + gas * ns;
        const double z_upper = 0.5 * (vg.z_v[(long long)l * nc + fr] + vg.z_v[(long long)l * nc + to]);
        const double z_lower = 0.5 * (vg.z_v[(long long)(l + 1) * nc + fr] + vg.z_v[(long long)(l + 1) * nc + to]);
        const double delta_z = z_upper - z_lower;
        fa += (vert_hor_viscosity(g, dg, b, rg, l, e) * dv_hdz(g, vg, b, sn, l, e)
               - vert_hor_viscosity(g, dg, b, rg, l + 1, e) * dv_hdz(g, vg, b, sn, l + 1, e))
              / delta_z
              / (0.5 * (density_total(sn.rho, n_const, ns, f) + density_total(sn.rho, n_const, ns, t)));
    }
    b.fric[nw + i] = fa;
}

/* diffusion of w, step a (momentum_diff_diss.c:137-150 and 153-166):
 * s1 = rho * viscosity * dw/dz, s2 = w averaged to the cell */
__global__ void kd_wdiff_a(G g, DiffGrid dg, int gas, DState sn, DiffBufs b)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int nl = g.nl, l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const long long nc = g.nc;
    const double up = l == 0 ? 0.0 : sn.w[(long long)l * nc + c];
    const double lo = l == nl - 1 ? 0.0 : sn.w[(long long)(l + 1) * nc + c];
    const double comp_v = up * g.area_v[(long long)l * nc + c] - lo * g.area_v[(long long)(l + 1) * nc + c];
    const double dwdz = 0.0 + 1 / g.volume[i] * comp_v;
    const double mdc = b.mol[i] + tke2vert(b.tke[i], b.n2[i], dg.layer_thickness[i]);
    b.s1[i] = sn.rho[gas * ns + i] * mdc * dwdz;
    b.s2[i] = ipw_at(g, 6, l, c) * sn.w[(long long)l * nc + c] + ipw_at(g, 7, l, c) * sn.w[(long long)(l + 1) * nc + c];
}

/* step b (:167-182): viscosity at the edge times the horizontal gradient of s2 */
__global__ void kd_wdiff_b(G g, DiffBufs b)
{
    const long long n = (long long)g.nl * g.ne, i = gtid();
    if (i >= n) return;
    const int l = (int)(i / g.ne), e = (int)(i - (long long)l * g.ne);
    const long long o = (long long)l * g.nc;
    b.flx[i] = 0.5 * (b.visc[o + g.from[e]] + b.visc[o + g.to[e]]) * grad_h(g, b.s2, l, e);
}

/* step c (:184): divergence of the diffusive flux */
__global__ void kd_wdiff_c(G g, DiffBufs b)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    b.s3[i] = divv_h_cell(g, b.flx, l, c);
}

/* step d (:151 and :186-199) at the inner interfaces: second derivative of
 * s1, plus s3 averaged to the interface, divided by the density */
__global__ void kd_wdiff_d(G g, int n_const, DState sn, DiffBufs b)
{
    const long long n = (long long)(g.nl - 1) * g.nc, i = gtid();
    if (i >= n) return;
    const long long ns = (long long)g.nl * g.nc, nc = g.nc;
    const int k = (int)(i / nc) + 1, c = (int)(i - (long long)(k - 1) * nc);
    const long long up = (long long)(k - 1) * nc + c, lo = (long long)k * nc + c;
    double fa = (b.s1[up] - b.s1[lo]) / g.nd_v[(long long)k * nc + c];
    fa += 0.5 * (b.s3[up] + b.s3[lo]);
    fa = fa / (0.5 * (density_total(sn.rho, n_const, ns, up) + density_total(sn.rho, n_const, ns, lo)));
    b.fric[(long long)k * nc + c] = fa;
}

/* simple_dissipation_rate (momentum_diff_diss.c:296-310) */
__global__ void kd_dissipation(G g, int n_const, DState sn, DiffBufs b)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= ns) return;
    const int l = (int)(i / g.nc), c = (int)(i - (long long)l * g.nc);
    const long long nc = g.nc, nw = (long long)(g.nl + 1) * nc;
    const int n_edges = c < N_PENT ? 5 : 6;
    double r = 0;
    for (int j = 0; j < n_edges; ++j) {
        const long long vi = (long long)l * g.ne + g.adj[j * nc + c];
        r += ipw_at(g, j, l, c) * sn.u[vi] * b.fric[nw + vi];
    }
    r += ipw_at(g, 6, l, c) * sn.w[i] * b.fric[i];
    r += ipw_at(g, 7, l, c) * sn.w[i + nc] * b.fric[i + nc];
    b.hdiss[i] = -density_total(sn.rho, n_const, ns, i) * r;
}

/* -------------------------------------------------------------- scalars */

/* scalar_diffusion_coeffs (effective_diff_coeffs.c:203-229) */
__global__ void kd_sdiff_coeff(long long ns, int n_cond, int moist, const double *lt, const double *cp_ice,
                               const double *cp_water, DState sn, DiffBufs b)
{
    const long long i = gtid();
    if (i >= ns) return;
    const double mch = b.visc[i] / sn.rho[n_cond * ns + i];
    const double mcv = b.mol[i] + tke2vert(b.tke[i], b.n2[i], lt[i]);
    b.mch[i] = mch;
    b.mcv[i] = mcv;
    const double cv = c_v_mass_weighted(sn.rho, n_cond, moist, ns, i, cp_ice[i], cp_water[i]);
    b.tch[i] = cv * mch;
    b.tcv[i] = cv * mcv;
}

/* the fields a scalar-diffusion pass treats: temperature and/or every density */
struct SFields {
    int nf;
    const double *f[8];      /* [L][Nc] */
    const double *kh[8], *kv[8];
    int vert[8];
    double *out[8];          /* [L][Nc] */
};

/* diffusive fluxes: horizontal at every edge (grad + scalar_times_vector_h),
 * vertical at the inner interfaces (scalar_times_vector_v), of field q */
__global__ void kd_sdiff_flux(G g, SFields sf, DiffBufs b)
{
    const long long nh = (long long)g.nl * g.ne, nv = (long long)(g.nl - 1) * g.nc;
    const long long per = nh + nv, i = gtid();
    if (i >= (long long)sf.nf * per) return;
    const int q = (int)(i / per);
    const long long r = i - (long long)q * per;
    const long long nc = g.nc;
    if (r < nh) {
        const int l = (int)(r / g.ne), e = (int)(r - (long long)l * g.ne);
        const long long o = (long long)l * nc;
        const double sv = 0.5 * (sf.kh[q][o + g.to[e]] + sf.kh[q][o + g.from[e]]);
        b.fh[(long long)q * nh + r] = sv * grad_h(g, sf.f[q], l, e);
    } else if (sf.vert[q]) {
        const long long rv = r - nh;
        const int k = (int)(rv / nc) + 1, c = (int)(rv - (long long)(k - 1) * nc);
        const double sv = 0.5 * (sf.kv[q][(long long)(k - 1) * nc + c] + sf.kv[q][(long long)k * nc + c]);
        b.fv[(long long)q * (g.nl + 1) * nc + (long long)k * nc + c] = sv * grad_v(g, sf.f[q], k, c);
    }
}

/* their divergences: divv_h, then add_vertical_divv (divergences.c:150-185) */
__global__ void kd_sdiff_div(G g, SFields sf, DiffBufs b)
{
    const long long ns = (long long)g.nl * g.nc, i = gtid();
    if (i >= (long long)sf.nf * ns) return;
    const int q = (int)(i / ns);
    const long long s = i - (long long)q * ns;
    const int nl = g.nl, l = (int)(s / g.nc), c = (int)(s - (long long)l * g.nc);
    const long long nc = g.nc;
    double out = divv_h_cell(g, b.fh + (long long)q * nl * g.ne, l, c);
    if (sf.vert[q]) {
        const double *fv = b.fv + (long long)q * (nl + 1) * nc;
        const double up = l == 0 ? 0.0 : fv[(long long)l * nc + c];
        const double lo = l == nl - 1 ? 0.0 : fv[(long long)(l + 1) * nc + c];
        const double comp_v = up * g.area_v[(long long)l * nc + c] - lo * g.area_v[(long long)(l + 1) * nc + c];
        out += 1 / g.volume[s] * comp_v;
    }
    sf.out[q][s] = out;
}

}  // namespace

void launch_diffusion_momentum(Context *c, const StepParams &p, const DState &sn)
{
    const bool any_h = p.diff & (DIFF_MOM_H | DIFF_TEMP_H | DIFF_MASS_H);
    const bool H = p.diff & DIFF_MOM_H, V = p.diff & DIFF_MOM_V;
    if (!any_h && !V) return;
    const G &g = c->hg64;
    DiffBufs &b = *c->dbuf;
    const long long ns = c->ns, nh = (long long)c->nl * c->ne;
    const int gas = c->n_cond;
    cudaStream_t s = c->stream;
    if (any_h) {
        {
            ProfScope ps(c, "kd_n2_adv");
            kd_n2_adv<<<nb(ns), 256, 0, s>>>(g, sn, b);
        }
        {
            ProfScope ps(c, "kd_tke");
            kd_tke<<<nb(ns), 256, 0, s>>>(ns, gas, p.dt, c->dg.mean_velocity_area, sn, b);
        }
        c->kernel_launches += 2;
    }
    if (H) {
        {
            ProfScope ps(c, "kd_hor_visc");
            kd_hor_visc<true><<<nb(ns), 256, 0, s>>>(g, c->dg.eff_hor_res, gas, c->temperature, sn, b);
        }
        {
            ProfScope ps(c, "k_tri_vort");
            k_tri_vort<double><<<nb((long long)c->nl * c->nt), 256, 0, s>>>(g, sn.u, b.tri);
        }
        {
            ProfScope ps(c, "kd_zt");
            kd_zt<<<nb((long long)c->nl * c->nt), 256, 0, s>>>(g, gas, sn, b);
        }
        {
            ProfScope ps(c, "kd_zr");
            kd_zr<<<nb(nh), 256, 0, s>>>(g, gas, sn, b);
        }
        c->kernel_launches += 4;
    }
    {
        ProfScope ps(c, "kd_fric_h");
        if (H && V) kd_fric_h<true, true><<<nb(nh), 256, 0, s>>>(g, c->vg, c->dg, c->n_const, gas, sn, b);
        else if (H) kd_fric_h<true, false><<<nb(nh), 256, 0, s>>>(g, c->vg, c->dg, c->n_const, gas, sn, b);
        else if (V) kd_fric_h<false, true><<<nb(nh), 256, 0, s>>>(g, c->vg, c->dg, c->n_const, gas, sn, b);
        if (H || V) c->kernel_launches++;
    }
    if (V) {
        {
            ProfScope ps(c, "kd_wdiff_a");
            kd_wdiff_a<<<nb(ns), 256, 0, s>>>(g, c->dg, gas, sn, b);
        }
        {
            ProfScope ps(c, "kd_wdiff_b");
            kd_wdiff_b<<<nb(nh), 256, 0, s>>>(g, b);
        }
        {
            ProfScope ps(c, "kd_wdiff_c");
            kd_wdiff_c<<<nb(ns), 256, 0, s>>>(g, b);
        }
        {
            ProfScope ps(c, "kd_wdiff_d");
            kd_wdiff_d<<<nb((long long)(c->nl - 1) * c->nc), 256, 0, s>>>(g, c->n_const, sn, b);
        }
        c->kernel_launches += 4;
    }
    if (H) {
        ProfScope ps(c, "kd_dissipation");
        kd_dissipation<<<nb(ns), 256, 0, s>>>(g, c->n_const, sn, b);
        c->kernel_launches++;
    }
    /* grad_hor (called by both momentum diffusions) zeroes the vertical
     * entries of the reference's placeholder field, TOA and surface included */
    if (H || V) cudaMemsetAsync(b.ph_tb, 0, (size_t)2 * c->nc * sizeof(double), s);
}

void launch_diffusion_scalar(Context *c, const StepParams &p, const DState &sn)
{
    const bool TH = p.diff & DIFF_TEMP_H, MH = p.diff & DIFF_MASS_H;
    if (!TH && !MH) return;
    const G &g = c->hg64;
    DiffBufs &b = *c->dbuf;
    const long long ns = c->ns;
    const int gas = c->n_cond;
    cudaStream_t s = c->stream;
    if (!(p.diff & DIFF_MOM_H)) {
        ProfScope ps(c, "kd_hor_visc");
        kd_hor_visc<false><<<nb(ns), 256, 0, s>>>(g, c->dg.eff_hor_res, gas, c->temperature, sn, b);
        c->kernel_launches++;
    }
    {
        ProfScope ps(c, "kd_sdiff_coeff");
        kd_sdiff_coeff<<<nb(ns), 256, 0, s>>>(ns, c->n_cond, c->moist, c->dg.layer_thickness, c->cp_ice, c->cp_water,
                                                sn, b);
        c->kernel_launches++;
    }
    SFields sf{};
    if (TH) {
        sf.f[sf.nf] = c->temperature;
        sf.kh[sf.nf] = b.tch;
        sf.kv[sf.nf] = b.tcv;
        sf.vert[sf.nf] = (p.diff & DIFF_TEMP_V) ? 1 : 0;
        sf.out[sf.nf] = b.tdh;
        ++sf.nf;
    }
    if (MH)
        for (int k = 0; k < c->n_const; ++k) {
            sf.f[sf.nf] = sn.rho + (long long)k * ns;
            sf.kh[sf.nf] = b.mch;
            sf.kv[sf.nf] = b.mcv;
            sf.vert[sf.nf] = (p.diff & DIFF_MASS_V) ? 1 : 0;
            sf.out[sf.nf] = b.mdt + (long long)k * ns;
            ++sf.nf;
        }
    const long long per = (long long)c->nl * c->ne + (long long)(c->nl - 1) * c->nc;
    {
        ProfScope ps(c, "kd_sdiff_flux");
        kd_sdiff_flux<<<nb(sf.nf * per), 256, 0, s>>>(g, sf, b);
    }
    {
        ProfScope ps(c, "kd_sdiff_div");
        kd_sdiff_div<<<nb(sf.nf * ns), 256, 0, s>>>(g, sf, b);
    }
    c->kernel_launches += 2;
}

}  // namespace game
