/*
 * ORACLE -- test infrastructure only (see game_oracle.h).
 *
 * CPU restatement of the GAME RKHEVI step with run-time grid sizes.  Every
 * function keeps the reference's order of floating-point operations; build
 * with -ffp-contract=off.  The diffusion branch (momentum, temperature and
 * mass diffusion with the TKE scheme) is restated; PBL, surface fluxes, soil
 * and radiation are not: the step returns -1 if their switches are on.
 */
#include "game_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* src/game_constants.h:10-27 */
#define T_0 273.15
#define N_A (6.02214076e23)
#define P_0 100000.0
#define C_D_V 717.942189
#define C_V_V 1396.475121
#define C_D_P 1005.0
#define M_D (N_A * 0.004810e-23)
#define M_V (N_A * 0.002991e-23)
#define R_D 287.057811
#define R_V 461.524879
#define N_PENT 12
/* column arrays of the solvers (the reference sizes them NO_OF_LAYERS) */
#define ORC_MAX_L 256

#define NC (g->nc)
#define NE (g->ne)
#define NT (g->nt)
#define NL (g->nl)
#define VPL ((long)g->nc + g->ne)
#define DPL ((long)g->ne + g->nt)
#define NS ((long)g->nl * g->nc)
#define NV ((long)g->nl * VPL + g->nc)
#define NCURL ((long)g->nl * 2 * g->ne + g->ne)
#define COND (g->n_cond)

/* the loops the reference runs as OpenMP parallel loops; none is a reduction,
 * so results do not depend on the thread count */
#ifdef _OPENMP
#define ORC_PAR _Pragma("omp parallel for schedule(static)")
#else
#define ORC_PAR
#endif

/* ------------------------------------------------------------ gradients
 * src/spatial_operators/gradient_operators.c */
int orc_grad_hor_cov(const orc_grid *g, const double *in, double *out)
{
    /* :14-33 */
    ORC_PAR
    for (long e = 0; e < NE; ++e)
        for (long l = 0; l < NL; ++l) {
            long vi = NC + l * VPL + e;
            out[vi] = (in[g->to[e] + l * NC] - in[g->from[e] + l * NC]) / g->normal_distance[vi];
        }
    return 0;
}

int orc_grad_vert_cov(const orc_grid *g, const double *in, double *out)
{
    /* :35-54 (inner interfaces only; TOA and surface entries are left as they are) */
    ORC_PAR
    for (long i = NC; i < (long)(NL + 1) * NC - NC; ++i) {
        long layer = i / NC, h = i - layer * NC;
        long lower = h + layer * NC, upper = h + (layer - 1) * NC, vi = h + layer * VPL;
        out[vi] = (in[upper] - in[lower]) / g->normal_distance[vi];
    }
    return 0;
}

int orc_grad_cov(const orc_grid *g, const double *in, double *out)
{
    /* :56-64 */
    orc_grad_hor_cov(g, in, out);
    orc_grad_vert_cov(g, in, out);
    return 0;
}

int orc_grad(const orc_grid *g, const double *in, double *out)
{
    /* :66-74 */
    orc_grad_cov(g, in, out);
    orc_vector_field_hor_cov_to_con(g, out);
    return 0;
}

int orc_grad_hor(const orc_grid *g, const double *in, double *out)
{
    /* :76-91 */
    orc_grad(g, in, out);
    ORC_PAR
    for (long i = 0; i < (long)(NL + 1) * NC; ++i) {
        long layer = i / NC, h = i - layer * NC;
        out[h + layer * VPL] = 0;
    }
    return 0;
}

/* --------------------------------------------------------------- averaging
 * src/spatial_operators/averaging.c */
static double remap_verpri2horpri_vector(const orc_grid *g, const double *f, long layer, long e)
{
    /* :14-39 */
    long fr = g->from[e], to = g->to[e];
    double c = g->ipw[8 * (layer * NC + fr) + 6] * f[layer * VPL + fr];
    c += g->ipw[8 * (layer * NC + to) + 6] * f[layer * VPL + to];
    if (layer < NL - 1) {
        c += g->ipw[8 * (layer * NC + fr) + 7] * f[(layer + 1) * VPL + fr];
        c += g->ipw[8 * (layer * NC + to) + 7] * f[(layer + 1) * VPL + to];
    }
    c = 0.5 * c;
    return c;
}

static double vertical_contravariant_corr(const orc_grid *g, const double *f, long layer, long h)
{
    /* :41-95 */
    double r = 0;
    int n_edges = h < N_PENT ? 5 : 6;
    if (layer >= NL - g->n_oro) {
        if (layer == NL - g->n_oro) {
            for (int j = 0; j < n_edges; ++j) {
                long si = layer * NC + h, vi = NC + layer * VPL + g->adj[6 * h + j];
                r += -0.5 * g->ipw[8 * si + j] * g->slope[vi] * f[vi];
            }
        } else {
            for (int j = 0; j < n_edges; ++j) {
                long si = (layer - 1) * NC + h, vi = NC + (layer - 1) * VPL + g->adj[6 * h + j];
                r += -0.5 * g->ipw[8 * si + j] * g->slope[vi] * f[vi];
            }
            for (int j = 0; j < n_edges; ++j) {
                long si = layer * NC + h, vi = NC + layer * VPL + g->adj[6 * h + j];
                r += -0.5 * g->ipw[8 * si + j] * g->slope[vi] * f[vi];
            }
        }
    }
    return r;
}

static double horizontal_covariant(const orc_grid *g, const double *f, long layer, long e)
{
    /* :97-111 */
    long vi = NC + layer * VPL + e;
    double r = f[vi];
    if (layer >= NL - g->n_oro) {
        double vc = remap_verpri2horpri_vector(g, f, layer, e);
        r += g->slope[vi] * vc;
    }
    return r;
}

int orc_vector_field_hor_cov_to_con(const orc_grid *g, double *f)
{
    /* :113-133 */
    ORC_PAR
    for (long i = 0; i < (long)g->n_oro * NE; ++i) {
        long li = i / NE, e = i - li * NE;
        double vg = remap_verpri2horpri_vector(g, f, li + (NL - g->n_oro), e);
        long vi = NC + (NL - g->n_oro + li) * VPL + e;
        f[vi] += -g->slope[vi] * vg;
    }
    return 0;
}

/* ------------------------------------------------------------- divergences
 * src/spatial_operators/divergences.c */
int orc_divv_h(const orc_grid *g, const double *in, double *out)
{
    /* :14-64 */
    ORC_PAR
    for (long h = 0; h < NC; ++h) {
        int n_edges = h < N_PENT ? 5 : 6;
        for (long l = 0; l < NL; ++l) {
            long i = l * NC + h;
            double comp_h = 0.0;
            for (int j = 0; j < n_edges; ++j) {
                long vi = NC + l * VPL + g->adj[6 * h + j];
                comp_h += in[vi] * g->adj_sign[6 * h + j] * g->area[vi];
            }
            double comp_v = 0.0;
            if (l == NL - g->n_oro - 1) {
                double lo = vertical_contravariant_corr(g, in, l + 1, h);
                comp_v = -lo * g->area[h + (l + 1) * VPL];
            } else if (l == NL - 1) {
                double up = vertical_contravariant_corr(g, in, l, h);
                comp_v = up * g->area[h + l * VPL];
            } else if (l > NL - g->n_oro - 1) {
                double up = vertical_contravariant_corr(g, in, l, h);
                double lo = vertical_contravariant_corr(g, in, l + 1, h);
                comp_v = up * g->area[h + l * VPL] - lo * g->area[h + (l + 1) * VPL];
            }
            out[i] = 1.0 / g->volume[i] * (comp_h + comp_v);
        }
    }
    return 0;
}

int orc_divv_h_tracer(const orc_grid *g, const double *in, const double *density, const double *wind, double *out)
{
    /* :66-148 */
    ORC_PAR
    for (long h = 0; h < NC; ++h) {
        int n_edges = h < N_PENT ? 5 : 6;
        for (long l = 0; l < NL; ++l) {
            long i = l * NC + h;
            double comp_h = 0.0;
            for (int j = 0; j < n_edges; ++j) {
                long vi = NC + l * VPL + g->adj[6 * h + j];
                comp_h += in[vi] * g->adj_sign[6 * h + j] * g->area[vi];
            }
            double comp_v = 0.0, d_up, d_lo;
            if (l == NL - g->n_oro - 1) {
                double lo = vertical_contravariant_corr(g, wind, l + 1, h);
                d_lo = lo <= 0.0 ? density[i] : density[i + NC];
                comp_v = -d_lo * lo * g->area[h + (l + 1) * VPL];
            } else if (l == NL - 1) {
                double up = vertical_contravariant_corr(g, wind, l, h);
                d_up = up <= 0.0 ? density[i - NC] : density[i];
                comp_v = d_up * up * g->area[h + l * VPL];
            } else if (l > NL - g->n_oro - 1) {
                double up = vertical_contravariant_corr(g, wind, l, h);
                d_up = up <= 0.0 ? density[i - NC] : density[i];
                double lo = vertical_contravariant_corr(g, wind, l + 1, h);
                d_lo = lo <= 0.0 ? density[i] : density[i + NC];
                comp_v = d_up * up * g->area[h + l * VPL] - d_lo * lo * g->area[h + (l + 1) * VPL];
            }
            out[i] = 1.0 / g->volume[i] * (comp_h + comp_v);
        }
    }
    return 0;
}

/* -------------------------------------------------------- multiplications
 * src/spatial_operators/multiplications.c */
int orc_scalar_times_vector_h(const orc_grid *g, const double *s, const double *v, double *out)
{
    /* :45-66 */
    ORC_PAR
    for (long e = 0; e < NE; ++e)
        for (long l = 0; l < NL; ++l) {
            long vi = NC + l * VPL + e;
            double sv = 0.5 * (s[g->to[e] + l * NC] + s[g->from[e] + l * NC]);
            out[vi] = sv * v[vi];
        }
    return 0;
}

int orc_scalar_times_vector_h_upstream(const orc_grid *g, const double *s, const double *v, double *out)
{
    /* :68-96 */
    ORC_PAR
    for (long e = 0; e < NE; ++e)
        for (long l = 0; l < NL; ++l) {
            long vi = NC + l * VPL + e;
            double sv = v[vi] >= 0.0 ? s[g->from[e] + l * NC] : s[g->to[e] + l * NC];
            out[vi] = sv * v[vi];
        }
    return 0;
}

int orc_scalar_times_vector_v(const orc_grid *g, const double *s, const double *v, double *out)
{
    /* :98-117 (inner interfaces only) */
    ORC_PAR
    for (long h = 0; h < NC; ++h)
        for (long l = 1; l < NL; ++l) {
            long i = l * VPL + h;
            double sv = 0.5 * (s[h + (l - 1) * NC] + s[h + l * NC]);
            out[i] = sv * v[i];
        }
    return 0;
}

int orc_scalar_times_vector(const orc_grid *g, const double *s, const double *v, double *out)
{
    /* :35-43 */
    orc_scalar_times_vector_h(g, s, v, out);
    orc_scalar_times_vector_v(g, s, v, out);
    return 0;
}

/* ------------------------------------------------------------ inner product
 * src/spatial_operators/inner_product.c:13-43 */
int orc_inner_product(const orc_grid *g, const double *a, const double *b, double *out)
{
    ORC_PAR
    for (long h = 0; h < NC; ++h) {
        int n_edges = h < N_PENT ? 5 : 6;
        for (long l = 0; l < NL; ++l) {
            long i = l * NC + h, base = 8 * i;
            out[i] = 0;
            for (int j = 0; j < n_edges; ++j) {
                long vi = NC + l * VPL + g->adj[6 * h + j];
                out[i] += g->ipw[base + j] * a[vi] * b[vi];
            }
            out[i] += g->ipw[base + 6] * a[h + l * VPL] * b[h + l * VPL];
            out[i] += g->ipw[base + 7] * a[h + (l + 1) * VPL] * b[h + (l + 1) * VPL];
        }
    }
    return 0;
}

/* ------------------------------------------------------------- vorticities
 * src/spatial_operators/vorticities.c */
int orc_calc_rel_vort_on_triangles(const orc_grid *g, const double *w, double *out)
{
    /* :167-222 */
    ORC_PAR
    for (long i = 0; i < (long)NL * NT; ++i) {
        long layer = i / NT, h = i - layer * NT;
        out[i] = 0;
        for (int j = 0; j < 3; ++j) {
            long vi = NC + layer * VPL + g->vort_idx[3 * h + j];
            double vel = w[vi];
            double rescale = 1;
            if (layer >= NL - g->n_oro) {
                long dvi = NE + layer * DPL + h;
                rescale = (g->radius + g->dual_z_vector[dvi]) / (g->radius + g->z_vector[vi]);
                double dz = g->dual_z_vector[dvi] - g->z_vector[vi];
                long vgi;
                if (dz > 0) vgi = vi - VPL;
                else if (layer == NL - 1) vgi = vi - VPL;
                else vgi = vi + VPL;
                double vgrad = (w[vi] - w[vgi]) / (g->z_vector[vi] - g->z_vector[vgi]);
                vel += dz * vgrad;
            }
            out[i] += rescale * g->normal_distance[vi] * g->vort_sign[3 * h + j] * vel;
        }
        out[i] = out[i] / g->dual_area[NE + layer * DPL + h];
    }
    return 0;
}

int orc_calc_rel_vort(const orc_grid *g, const double *w, orc_diag *d)
{
    /* :104-165 */
    orc_calc_rel_vort_on_triangles(g, w, d->rel_vort_on_triangles);
    ORC_PAR
    for (long i = NE; i < NCURL; ++i) {
        long layer = i / (2 * NE), h = i - layer * 2 * NE;
        if (h >= NE) {
            long base = NE + layer * DPL, e = h - NE;
            long tf = g->dual_from[e], tt = g->dual_to[e];
            d->rel_vort[i] = (g->dual_area[base + tf] * d->rel_vort_on_triangles[layer * NT + tf]
                              + g->dual_area[base + tt] * d->rel_vort_on_triangles[layer * NT + tt])
                             / (g->dual_area[base + tf] + g->dual_area[base + tt]);
        } else {
            long base = layer * VPL;
            if (layer == NL) {
                long i2 = base - NE + h;
                double c2 = horizontal_covariant(g, w, layer - 1, h);
                d->rel_vort[i] = 1 / g->dual_area[h + layer * DPL] * g->normal_distance[i2] * c2;
            } else {
                long i0 = base + NC + h, i1 = base + g->from[h], i2 = base - NE + h, i3 = base + g->to[h];
                double c0 = horizontal_covariant(g, w, layer, h);
                double c2 = horizontal_covariant(g, w, layer - 1, h);
                d->rel_vort[i] = 1 / g->dual_area[h + layer * DPL]
                                 * (-g->normal_distance[i0] * c0 + g->normal_distance[i1] * w[i1]
                                    + g->normal_distance[i2] * c2 - g->normal_distance[i3] * w[i3]);
            }
        }
    }
    for (long i = 0; i < NE; ++i) d->rel_vort[i] = d->rel_vort[i + 2 * NE];
    return 0;
}

int orc_add_f_to_rel_vort(const orc_grid *g, const double *rel, double *out)
{
    /* :87-102 */
    ORC_PAR
    for (long i = 0; i < NCURL; ++i) {
        long layer = i / (2 * NE), h = i - layer * 2 * NE;
        out[i] = rel[i] + g->f_vec[h];
    }
    return 0;
}

/* Grid::z_vector read at index idx, as the reference's calc_pot_vort reads it.
 * At the surface level it indexes z_vector[NO_OF_SCALARS + (layer - 2)*VPL + h]
 * (vorticities.c:55-56), which lies past the end of z_vector for the standard
 * sizes; the read then lands in the members that follow z_vector in the Grid
 * struct (gravity_potential, then gravity_m), and results depend on them. */
static double zv_ext(const orc_grid *g, long idx)
{
    if (idx < NV) return g->z_vector[idx];
    idx -= NV;
    if (idx < NS) return g->gravity_potential[idx];
    return g->gravity_m[idx - NS];
}

int orc_calc_pot_vort(const orc_grid *g, const double *w, const double *rho, orc_diag *d)
{
    /* :18-85 */
    orc_calc_rel_vort(g, w, d);
    orc_add_f_to_rel_vort(g, d->rel_vort, d->pot_vort);
    ORC_PAR
    for (long i = 0; i < NCURL; ++i) {
        long layer = i / (2 * NE), h = i - layer * 2 * NE;
        double dens;
        if (h >= NE) {
            long e = h - NE;
            dens = 0;
            for (int j = 0; j < 4; ++j)
                dens += g->rhombi_weights[4 * e + j] * rho[layer * NC + g->rhombi_idx[4 * e + j]];
        } else {
            long fr = g->from[h], to = g->to[h];
            if (layer == 0) {
                dens = 0.5 * (rho[fr] + rho[to])
                       + (0.5 * (rho[fr] + rho[to]) - 0.5 * (rho[fr + NC] + rho[to + NC]))
                             / (zv_ext(g, NS + h) - zv_ext(g, NS + VPL + h)) * (zv_ext(g, 0) - zv_ext(g, NS + h));
            } else if (layer == NL) {
                long a = (layer - 1) * NC, b = (layer - 2) * NC;
                dens = 0.5 * (rho[a + fr] + rho[a + to])
                       + (0.5 * (rho[b + fr] + rho[b + to]) - 0.5 * (rho[a + fr] + rho[a + to]))
                             / (zv_ext(g, NS + (layer - 2) * VPL + h) - zv_ext(g, NS + (layer - 1) * VPL + h))
                             * (0.5 * (zv_ext(g, layer * VPL + fr) + zv_ext(g, layer * VPL + to))
                                - zv_ext(g, NS + (layer - 1) * VPL + h));
            } else {
                long uf = (layer - 1) * NC + fr, ut = (layer - 1) * NC + to;
                dens = 0.25 * (rho[uf] + rho[ut] + rho[uf + NC] + rho[ut + NC]);
            }
        }
        d->pot_vort[i] = d->pot_vort[i] / dens;
    }
    return 0;
}

/* ---------------------------------------------------------- vorticity flux
 * src/spatial_operators/vorticity_flux.c:16-187 */
int orc_vorticity_flux(const orc_grid *g, const double *mf, const double *pv, double *out)
{
    ORC_PAR
    for (long h = 0; h < VPL; ++h) {
        for (long l = 0; l < NL + 1; ++l) {
            long i = l * VPL + h;
            if (h >= NC && l < NL) {
                out[i] = 0;
                long e = h - NC, mb = NC + l * VPL, pb = NE + l * 2 * NE;
                const double *tw = &g->trsk_weights[10 * e];
                const int *ti = &g->trsk_indices[10 * e], *tm = &g->trsk_mci[10 * e];
                if (g->from[e] < N_PENT) {
                    for (int j = 0; j < 4; ++j) out[i] += tw[j] * mf[mb + ti[j]] * pv[pb + tm[j]];
                } else {
                    for (int j = 0; j < 5; ++j) {
                        if (j == 2) out[i] += tw[j] * mf[mb + ti[j]] * 0.5 * (pv[pb + tm[j]] + pv[pb + e]);
                        else out[i] += tw[j] * mf[mb + ti[j]] * pv[pb + tm[j]];
                    }
                }
                if (g->to[e] < N_PENT) {
                    for (int j = 5; j < 9; ++j) out[i] += tw[j] * mf[mb + ti[j]] * pv[pb + tm[j]];
                } else {
                    for (int j = 5; j < 10; ++j) {
                        if (j == 7) out[i] += tw[j] * mf[mb + ti[j]] * 0.5 * (pv[pb + tm[j]] + pv[pb + e]);
                        else out[i] += tw[j] * mf[mb + ti[j]] * pv[pb + tm[j]];
                    }
                }
                long fr = g->from[e], to = g->to[e];
                out[i] -= 0.5 * g->ipw[8 * (l * NC + fr) + 6] * mf[l * VPL + fr] * pv[e + l * 2 * NE];
                out[i] -= 0.5 * g->ipw[8 * (l * NC + to) + 6] * mf[l * VPL + to] * pv[e + l * 2 * NE];
                out[i] -= 0.5 * g->ipw[8 * (l * NC + fr) + 7] * mf[(l + 1) * VPL + fr] * pv[e + (l + 1) * 2 * NE];
                out[i] -= 0.5 * g->ipw[8 * (l * NC + to) + 7] * mf[(l + 1) * VPL + to] * pv[e + (l + 1) * 2 * NE];
            } else if (h < NC) {
                out[i] = 0;
                int n_edges = h < N_PENT ? 5 : 6;
                double vw = (l == 0 || l == NL) ? 1 : 0.5;
                if (l >= 1)
                    for (int j = 0; j < n_edges; ++j) {
                        long a = g->adj[6 * h + j];
                        out[i] += vw * g->ipw[8 * ((l - 1) * NC + h) + j] * mf[NC + (l - 1) * VPL + a] * pv[l * 2 * NE + a];
                    }
                if (l <= NL - 1)
                    for (int j = 0; j < n_edges; ++j) {
                        long a = g->adj[6 * h + j];
                        out[i] += vw * g->ipw[8 * (l * NC + h) + j] * mf[NC + l * VPL + a] * pv[l * 2 * NE + a];
                    }
            }
        }
    }
    return 0;
}

/* -------------------------------------------------------- state blending
 * src/spatial_operators/linear_combine_two_states.c:14-43 */
int orc_linear_combine_two_states(const orc_grid *g, const orc_state *s0, const orc_state *s1, orc_state *o,
                                  double c0, double c1)
{
    ORC_PAR
    for (long i = 0; i < NS; ++i) {
        for (int j = 0; j < g->n_const; ++j)
            o->rho[j * NS + i] = c0 * s0->rho[j * NS + i] + c1 * s1->rho[j * NS + i];
        o->rhotheta_v[i] = c0 * s0->rhotheta_v[i] + c1 * s1->rhotheta_v[i];
        o->theta_v_pert[i] = o->rhotheta_v[i] / o->rho[COND * NS + i] - g->theta_v_bg[i];
        o->exner_pert[i] = c0 * s0->exner_pert[i] + c1 * s1->exner_pert[i];
    }
    ORC_PAR
    for (long i = 0; i < NV; ++i) o->wind[i] = c0 * s0->wind[i] + c1 * s1->wind[i];
    return 0;
}

/* ------------------------------------------------------- thermodynamics
 * src/constituents/derived_quantities.c, dictionary.c */
int orc_temperature_diagnostics(const orc_grid *g, const orc_state *s, orc_diag *d)
{
    /* derived_quantities.c:15-40 */
    if (!g->moisture_on) {
        for (long i = 0; i < NS; ++i)
            d->temperature[i] = (g->theta_v_bg[i] + s->theta_v_pert[i]) * (g->exner_bg[i] + s->exner_pert[i]);
    } else {
        for (long i = 0; i < NS; ++i)
            d->temperature[i] = (g->theta_v_bg[i] + s->theta_v_pert[i]) * (g->exner_bg[i] + s->exner_pert[i])
                                / (1.0 + s->rho[(COND + 1) * NS + i] / s->rho[COND * NS + i] * (M_D / M_V - 1.0));
    }
    return 0;
}

static double density_total(const orc_grid *g, const orc_state *s, long i)
{
    /* derived_quantities.c:83-95 */
    double r = 0.0;
    for (int k = 0; k < g->n_const; ++k) r += s->rho[k * NS + i];
    return r;
}

static double c_p_ice(double t)
{
    /* dictionary.c:111-131 */
    if (t > T_0) t = T_0;
    if (t < 20.0) t = 20.0;
    double r = -2.0572 + 0.14644 * t + 0.06163 * t * exp(-pow(t / 125.1, 2));
    return r / M_V;
}

static double c_p_water(double t)
{
    /* dictionary.c:133-171 */
    double tc = t - T_0, r;
    if (tc >= 0.0) {
        if (tc > 35.0) tc = 35.0;
        r = 0.9979 + 3.1e-6 * pow(tc - 35.0, 2) + 3.8e-9 * pow(tc - 35.0, 4);
    } else {
        if (tc < -37.0) tc = -37.0;
        r = 1.000938 - 2.7052e-3 * tc - 2.3235e-5 * pow(tc, 2) + 4.3778e-6 * pow(tc, 3) + 2.7136e-7 * pow(tc, 4);
    }
    return 4186.8 * r;
}

static double c_p_cond(int id, double t)
{
    /* dictionary.c:173-190 */
    return fmod(id, 2) == 0 ? c_p_ice(t) : c_p_water(t);
}

static double enthalpy_evaporation(double t)
{
    /* dictionary.c:221-254 */
    double r;
    if (t < T_0) {
        if (t < 30.0) t = 30.0;
        r = 56579.0 - 42.212 * t + exp(0.1149 * (281.6 - t));
        r = r / M_V;
    } else {
        if (t > T_0 + 100.0) t = T_0 + 100.0;
        r = 3151378.0 - 2386.0 * t;
    }
    return r;
}

static double enthalpy_sublimation(double t)
{
    /* dictionary.c:256-279 */
    if (t < 30.0) t = 30.0;
    if (t > T_0) t = T_0;
    double r = 46782.5 + 35.8925 * t - 0.07414 * pow(t, 2) + 541.5 * exp(-pow(t / 123.75, 2));
    return r / M_V;
}

static double phase_trans_heat(int dir, double t)
{
    /* dictionary.c:192-219 */
    double r = 0.0;
    if (dir == 0) r = enthalpy_evaporation(t);
    if (dir == 1) r = enthalpy_sublimation(t);
    if (dir == 2) r = enthalpy_sublimation(t) - enthalpy_evaporation(t);
    return r;
}

static double saturation_pressure_over_water(double t)
{
    /* dictionary.c:281-323 */
    double tc = t - T_0, r;
    if (tc > 100.0) tc = 100.0;
    if (tc > 0.0) {
        r = exp(34.494 - 4924.99 / (tc + 237.1)) / pow(tc + 105.0, 1.57);
    } else {
        if (tc < -50.0) tc = -50.0;
        r = 6.107799961 + 4.436518521e-1 * tc + 1.428945805e-2 * pow(tc, 2) + 2.650648471e-4 * pow(tc, 3)
            + 3.031240396e-6 * pow(tc, 4) + 2.034080948e-8 * pow(tc, 5) + 6.136820929e-11 * pow(tc, 6);
        r = 100.0 * r;
    }
    return r;
}

static double dsaturation_pressure_over_water_dT(double t)
{
    /* dictionary.c:325-349 */
    double tc = t - T_0;
    if (tc > 100.0) tc = 100.0;
    if (tc < 0.0) tc = 0.0;
    return saturation_pressure_over_water(t) * (4924.99 / pow(tc + 237.1, 2.0) - 1.57 / (tc + 105.0));
}

static double saturation_pressure_over_ice(double t)
{
    /* dictionary.c:351-372 */
    double tc = t - T_0;
    if (tc < -80.0) tc = -80.0;
    if (tc > 0.0) tc = 0.0;
    return exp(43.494 - 6545.8 / (tc + 278.0)) / pow(tc + 868.0, 2);
}

static double dsaturation_pressure_over_ice_dT(double t)
{
    /* dictionary.c:374-398 */
    double tc = t - T_0;
    if (tc < -80.0) tc = -80.0;
    if (tc > 0.0) tc = 0.0;
    return saturation_pressure_over_ice(t) * (6545.8 / pow(tc + 278.0, 2.0) - 2.0 / (tc + 868.0));
}

static double enhancement_factor_over_water(double p) { return 1.00071 * exp(0.000000045 * p); } /* :400-410 */
static double enhancement_factor_over_ice(double p) { return 0.99882 * exp(0.00000008 * p); }    /* :412-424 */

static double c_v_mass_weighted_air(const orc_grid *g, const orc_state *s, const orc_diag *d, long i)
{
    /* derived_quantities.c:97-115 */
    double r = 0.0;
    for (int k = 0; k < COND; ++k) r += s->rho[k * NS + i] * c_p_cond(k, d->temperature[i]);
    r += s->rho[COND * NS + i] * C_D_V;
    if (g->moisture_on) r += s->rho[(COND + 1) * NS + i] * C_V_V;
    return r;
}

/* src/constituents/phase_trans.c:16-311 (surface effects off) */
int orc_calc_h2otracers_source_rates(const orc_grid *g, const orc_state *s, orc_diag *d, const orc_config *c,
                                     orc_irrev *ir, double dt)
{
    const double max_cloud_water = 0.2e-3;
    double *pr = ir->phase_trans_rates;
    if (c->sfc_phase_trans) return -1;
    ORC_PAR
    for (long i = 0; i < NS; ++i) {
        double T = d->temperature[i], sat, wvp, dry, air, a, b, cc, p, q, ef, diff, ptd;
        sat = T >= T_0 ? saturation_pressure_over_water(T) : saturation_pressure_over_ice(T);
        wvp = s->rho[(COND + 1) * NS + i] * R_V * T;
        dry = (s->rho[COND * NS + i] - s->rho[(COND + 1) * NS + i]) * R_D * T;
        air = dry + wvp;
        ef = T >= T_0 ? enhancement_factor_over_water(air) : enhancement_factor_over_ice(air);
        sat = ef * sat;
        int dir = T >= T_0 ? 0 : 1;
        a = -R_V * phase_trans_heat(dir, T) / c_v_mass_weighted_air(g, s, d, i);
        b = R_V * T - R_V * s->rho[(COND + 1) * NS + i] * phase_trans_heat(dir, T) / c_v_mass_weighted_air(g, s, d, i)
            + ef * (dir == 0 ? dsaturation_pressure_over_water_dT(T) : dsaturation_pressure_over_ice_dT(T))
                  * phase_trans_heat(dir, T) / c_v_mass_weighted_air(g, s, d, i);
        cc = wvp - sat;
        p = b / a;
        q = cc / a;
        diff = -0.5 * p - pow(0.25 * pow(p, 2) - q, 0.5);
        if (sat >= wvp) {
            if (T >= T_0) {
                pr[2 * NS + i] = -s->rho[2 * NS + i] / dt;
                ptd = fmin(s->rho[3 * NS + i], diff);
                pr[4 * NS + i] = ptd / dt;
                pr[3 * NS + i] = s->rho[2 * NS + i] / dt - ptd / dt;
                ir->phase_trans_heating_rate[i] = pr[2 * NS + i] * phase_trans_heat(2, T) - ptd * phase_trans_heat(0, T) / dt;
            } else {
                pr[3 * NS + i] = -s->rho[3 * NS + i] / dt;
                ptd = fmin(s->rho[2 * NS + i], diff);
                pr[4 * NS + i] = ptd / dt;
                pr[2 * NS + i] = s->rho[3 * NS + i] / dt - ptd / dt;
                ir->phase_trans_heating_rate[i] = -pr[3 * NS + i] * phase_trans_heat(2, T) - ptd * phase_trans_heat(1, T) / dt;
            }
        } else {
            if (T >= T_0) {
                pr[2 * NS + i] = -s->rho[2 * NS + i] / dt;
                pr[4 * NS + i] = diff / dt;
                pr[3 * NS + i] = s->rho[2 * NS + i] / dt - diff / dt;
                ir->phase_trans_heating_rate[i] = pr[2 * NS + i] * phase_trans_heat(2, T) - diff * phase_trans_heat(0, T) / dt;
            } else {
                pr[3 * NS + i] = -s->rho[3 * NS + i] / dt;
                pr[4 * NS + i] = diff / dt;
                pr[2 * NS + i] = s->rho[3 * NS + i] / dt - diff / dt;
                ir->phase_trans_heating_rate[i] = -pr[3 * NS + i] * phase_trans_heat(2, T) - diff * phase_trans_heat(1, T) / dt;
            }
        }
        pr[i] = 0.0;
        pr[NS + i] = 0.0;
        if (T < T_0) {
            pr[i] = fmax(s->rho[2 * NS + i] - max_cloud_water * s->rho[4 * NS + i], 0.0) / 1000.0;
            pr[2 * NS + i] -= pr[i];
        } else if (T >= T_0) {
            pr[NS + i] = fmax(s->rho[3 * NS + i] - max_cloud_water * s->rho[4 * NS + i], 0.0) / 1000.0;
            pr[3 * NS + i] -= pr[NS + i];
        }
        if (T >= T_0 && s->rho[i] > 0.0) {
            pr[i] = -s->rho[i] / dt;
            pr[NS + i] -= pr[i];
            ir->phase_trans_heating_rate[i] += pr[i] * phase_trans_heat(2, T);
        }
        if (T < T_0 && s->rho[NS + i] > 0.0) {
            pr[NS + i] = -s->rho[NS + i] / dt;
            pr[i] -= pr[NS + i];
            ir->phase_trans_heating_rate[i] += -pr[NS + i] * phase_trans_heat(2, T);
        }
    }
    return 0;
}

/* ------------------------------------------------------ pressure gradient
 * src/time_stepping/manage_pressure_gradient.c */
int orc_manage_pressure_gradient(const orc_grid *g, const orc_state *s, orc_diag *d, orc_forcings *f,
                                 orc_irrev *ir, const orc_config *c)
{
    /* :17-72 */
    if (c->totally_first_step_bool == 0)
        for (long i = 0; i < NV; ++i) f->pgrad_acc_old[i] = -f->pgrad_nl[i] - f->pgrad_l[i];
    ORC_PAR
    for (long i = 0; i < NS; ++i) d->scalar_field_placeholder[i] = C_D_P * (g->theta_v_bg[i] + s->theta_v_pert[i]);
    orc_grad(g, s->exner_pert, f->pgrad_nl);
    orc_scalar_times_vector(g, d->scalar_field_placeholder, f->pgrad_nl, f->pgrad_nl);
    ORC_PAR
    for (long i = 0; i < NS; ++i) d->scalar_field_placeholder[i] = C_D_P * s->theta_v_pert[i];
    orc_scalar_times_vector(g, d->scalar_field_placeholder, g->exner_bg_grad, f->pgrad_l);
    ORC_PAR
    for (long i = 0; i < NS; ++i)
        ir->pressure_gradient_decel_factor[i] = s->rho[COND * NS + i] / density_total(g, s, i);
    orc_scalar_times_vector(g, ir->pressure_gradient_decel_factor, f->pgrad_nl, f->pgrad_nl);
    orc_scalar_times_vector(g, ir->pressure_gradient_decel_factor, f->pgrad_l, f->pgrad_l);
    if (c->totally_first_step_bool == 1)
        for (long i = 0; i < NV; ++i) f->pgrad_acc_old[i] = -f->pgrad_nl[i] - f->pgrad_l[i];
    return 0;
}

int orc_calc_pressure_grad_condensates_v(const orc_grid *g, const orc_state *s, orc_forcings *f, orc_irrev *ir)
{
    /* :74-87 */
    ORC_PAR
    for (long i = 0; i < NS; ++i)
        ir->pressure_gradient_decel_factor[i] = s->rho[COND * NS + i] / density_total(g, s, i) - 1.0;
    orc_scalar_times_vector_v(g, ir->pressure_gradient_decel_factor, g->gravity_m, f->pgrad_condensates_v);
    return 0;
}

/* ------------------------------------------------------ diffusion branch
 * run at the first RK substep when a diffusion switch is on
 * (vector_tendencies_expl.c:37-69, scalar_tendencies_expl.c:44-88) */
#define K_B (1.380649e-23)
#define EPSILON_SECURITY (1e-10)
#define ORC_PI 3.14159265358979323846
#define NDV ((long)(g->nl + 1) * g->ne + (long)g->nl * g->nt)

/* src/spatial_operators/divergences.c:150-185 */
int orc_add_vertical_divv(const orc_grid *g, const double *in, double *out)
{
    ORC_PAR
    for (long h = 0; h < NC; ++h)
        for (long l = 0; l < NL; ++l) {
            long i = l * NC + h;
            double up, lo;
            if (l == 0) {
                up = 0;
                lo = in[h + (l + 1) * VPL];
            } else if (l == NL - 1) {
                up = in[h + l * VPL];
                lo = 0;
            } else {
                up = in[h + l * VPL];
                lo = in[h + (l + 1) * VPL];
            }
            double comp_v = up * g->area[h + l * VPL] - lo * g->area[h + (l + 1) * VPL];
            out[i] += 1 / g->volume[i] * comp_v;
        }
    return 0;
}

/* molecular diffusion coefficient from kinetic gas theory
 * (src/constituents/derived_quantities.c:117-134) */
static double calc_diffusion_coeff(double temperature, double density)
{
    double particle_radius = 130e-12;
    double particle_mass = M_D / N_A;
    double thermal_velocity = sqrt(8.0 * K_B * temperature / (ORC_PI * particle_mass));
    double particle_density = density / particle_mass;
    double cross_section = 4.0 * ORC_PI * pow(particle_radius, 2.0);
    double mean_free_path = 1.0 / (sqrt(2.0) * particle_density * cross_section);
    return 1.0 / 3.0 * thermal_velocity * mean_free_path;
}

/* src/subgrid_scale/effective_diff_coeffs.c:293-303 */
static double tke2hor_diff_coeff(double tke, double effective_resolution)
{
    double mean_velocity = pow(2.0 * tke, 0.5);
    double mean_free_path = effective_resolution / 6.0;
    return 1.0 / 6.0 * mean_free_path * mean_velocity;
}

/* src/subgrid_scale/effective_diff_coeffs.c:305-320 */
static double tke2vert_diff_coeff(double tke, double n_squared, double layer_thickness)
{
    double tke_vert = 3.0 * 1e-3 * tke;
    double mean_velocity = pow(2.0 * tke_vert, 0.5);
    double n_used = pow(fmax(n_squared, 1e-4), 0.5);
    double mean_free_path = pow(2.0 * tke_vert, 0.5) / n_used;
    mean_free_path = fmin(mean_free_path, layer_thickness);
    return 1.0 / 6.0 * mean_free_path * mean_velocity;
}

/* src/subgrid_scale/effective_diff_coeffs.c:233-291.  For the last layer the
 * reference writes n_squared[NO_OF_SCALARS - NO_OF_SCALARS_H + i] from
 * vector_field_placeholder[NO_OF_VECTORS - NO_OF_VECTORS_PER_LAYER -
 * NO_OF_SCALARS_H + i], both past the ends of their arrays: the read lands in
 * the Diagnostics members after vector_field_placeholder, the write in those
 * after n_squared, and the last layer of n_squared keeps its value.  The
 * same accesses are made here on the same struct. */
int orc_update_n_squared(const orc_grid *g, const orc_state *s, orc_diag *d)
{
    double *ph = d->scalar_field_placeholder, *vph = d->vector_field_placeholder;
    ORC_PAR
    for (long i = 0; i < NS; ++i) ph[i] = g->theta_v_bg[i] + s->theta_v_pert[i];
    orc_grad_vert_cov(g, ph, vph);
    ORC_PAR
    for (long i = 0; i < NS; ++i) ph[i] = 1.0 / ph[i];
    orc_scalar_times_vector_v(g, ph, vph, vph);
    ORC_PAR
    for (long i = NC; i < (long)(NL + 1) * NC - NC; ++i) {
        long layer = i / NC, h = i - layer * NC, vi = h + layer * VPL;
        vph[vi] = g->gravity_m[vi] * vph[vi];
    }
    ORC_PAR
    for (long i = 0; i < NS; ++i) {
        long layer = i / NC, h = i - layer * NC;
        if (layer == 0)
            d->n_squared[i] = vph[VPL + i];
        else if (layer == NL - 1)
            d->n_squared[NS - NC + i] = vph[NV - VPL - NC + i];
        else
            d->n_squared[i] = g->ipw[8 * i + 6] * vph[h + layer * VPL] + g->ipw[8 * i + 7] * vph[h + (layer + 1) * VPL];
    }
    return 0;
}

/* src/subgrid_scale/tke.c:16-60 */
int orc_tke_update(const orc_grid *g, orc_irrev *ir, double dt, const orc_state *s, orc_diag *d)
{
    orc_grad(g, ir->tke, d->vector_field_placeholder);
    orc_inner_product(g, d->vector_field_placeholder, s->wind, d->scalar_field_placeholder);
    ORC_PAR
    for (long i = 0; i < NS; ++i) {
        double decay = 8.0 * pow(ORC_PI, 2.0) / g->mean_velocity_area * ir->viscosity[i] / s->rho[COND * NS + i];
        ir->tke[i] += dt * (-d->scalar_field_placeholder[i] + ir->heating_diss[i] / s->rho[COND * NS + i]
                            - decay * ir->tke[i]);
        if (ir->tke[i] < 0.0) ir->tke[i] = 0.0;
    }
    return 0;
}

/* src/subgrid_scale/effective_diff_coeffs.c:19-112: molecular + turbulent
 * viscosity, averaged to rhombi and triangles and multiplied by the gas
 * density; the cell values are then replaced by density times the turbulent
 * part alone */
int orc_hor_viscosity(const orc_grid *g, const orc_state *s, orc_irrev *ir, const orc_diag *d)
{
    const double *rg = &s->rho[COND * NS];
    ORC_PAR
    for (long i = 0; i < NS; ++i) {
        ir->molecular_diffusion_coeff[i] = calc_diffusion_coeff(d->temperature[i], rg[i]);
        ir->viscosity[i] = ir->molecular_diffusion_coeff[i];
        ir->viscosity[i] += tke2hor_diff_coeff(ir->tke[i], g->eff_hor_res);
    }
    ORC_PAR
    for (long e = 0; e < NE; ++e)
        for (long l = 0; l < NL; ++l) {
            long vi = NC + l * VPL + e, f = l * NC + g->from[e], t = l * NC + g->to[e];
            ir->viscosity_rhombi[vi] = 0.5 * (ir->viscosity[f] + ir->viscosity[t]);
            ir->viscosity_rhombi[vi] = 0.5 * (rg[f] + rg[t]) * ir->viscosity_rhombi[vi];
        }
    ORC_PAR
    for (long i = 0; i < (long)NL * NT; ++i) {
        long layer = i / NT, h = i - layer * NT, sb = layer * NC;
        const int *vt = &g->vort_idx[3 * h];
        const double *v = ir->viscosity;
        ir->viscosity_triangles[i] = 1.0 / 6.0 * (v[sb + g->from[vt[0]]] + v[sb + g->to[vt[0]]] + v[sb + g->from[vt[1]]]
                                                  + v[sb + g->to[vt[1]]] + v[sb + g->from[vt[2]]] + v[sb + g->to[vt[2]]]);
        double dens = 1.0 / 6.0 * (rg[sb + g->from[vt[0]]] + rg[sb + g->to[vt[0]]] + rg[sb + g->from[vt[1]]]
                                   + rg[sb + g->to[vt[1]]] + rg[sb + g->from[vt[2]]] + rg[sb + g->to[vt[2]]]);
        ir->viscosity_triangles[i] = dens * ir->viscosity_triangles[i];
    }
    ORC_PAR
    for (long i = 0; i < NS; ++i) ir->viscosity[i] = rg[i] * tke2hor_diff_coeff(ir->tke[i], g->eff_hor_res);
    return 0;
}

/* src/spatial_operators/momentum_diff_diss.c:207-294 */
static void hor_calc_curl_of_vorticity(const orc_grid *g, const double *vort, const double *zt, double *out)
{
    ORC_PAR
    for (long i = 0; i < (long)NL * NE; ++i) {
        long layer = i / NE, h = i - layer * NE, vi = NC + layer * VPL + h;
        long tt = g->dual_to[h], tf = g->dual_from[h], base = NE + layer * DPL;
        const double *dn = g->dual_normal_distance;
        out[vi] = 0.0;
        double delta_z = 0.0;
        double zto = zt[layer * NT + tt], zfr = zt[layer * NT + tf];
        double cdw = fabs(zto - zfr) / (fabs(zto) + fabs(zfr) + EPSILON_SECURITY);
        for (int j = 0; j < 3; ++j) {
            out[vi] += +1.0 / 3.0 * (1.0 - cdw)
                       * (dn[base + tt] * vort[NE + layer * 2 * NE + g->vort_idx[3 * tt + j]]
                          - dn[base + tf] * vort[NE + layer * 2 * NE + g->vort_idx[3 * tf + j]]);
            delta_z += 1.0 / 3.0 * (g->z_vector[NC + layer * VPL + g->vort_idx[3 * tt + j]]
                                    - g->z_vector[NC + layer * VPL + g->vort_idx[3 * tf + j]]);
        }
        out[vi] += cdw * (zto * dn[base + tt] - zfr * dn[base + tf]);
        out[vi] = out[vi] / g->area[vi];
        if (layer >= NL - g->n_oro) {
            double delta_x = dn[NDV - NE + h];
            delta_x = delta_x * (g->radius + g->z_vector[vi]) / g->radius;
            double tangential_slope = delta_z / delta_x;
            long uz = NC + (layer - 1) * VPL + h, lz = NC + (layer + 1) * VPL + h;
            long uzeta = NE + (layer - 1) * 2 * NE + h, lzeta = NE + (layer + 1) * 2 * NE + h;
            if (layer == 0) {
                uz = NC + layer * VPL + h;
                uzeta = NE + layer * 2 * NE + h;
            }
            if (layer == NL - 1) {
                lz = NC + layer * VPL + h;
                lzeta = NE + layer * 2 * NE + h;
            }
            double delta_zeta = vort[uzeta] - vort[lzeta];
            delta_z = g->z_vector[uz] - g->z_vector[lz];
            double dzeta_dz = delta_zeta / delta_z;
            out[vi] -= tangential_slope * dzeta_dz;
        }
    }
}

/* src/spatial_operators/momentum_diff_diss.c:22-80 */
int orc_hor_momentum_diffusion(const orc_grid *g, const orc_state *s, orc_diag *d, orc_irrev *ir)
{
    orc_divv_h(g, s->wind, d->wind_divv);
    orc_calc_rel_vort(g, s->wind, d);
    orc_hor_viscosity(g, s, ir, d);
    ORC_PAR
    for (long i = 0; i < NS; ++i) d->wind_divv[i] = ir->viscosity[i] * d->wind_divv[i];
    orc_grad_hor(g, d->wind_divv, d->vector_field_placeholder);
    ORC_PAR
    for (long h = 0; h < NE; ++h)
        for (long l = 0; l < NL; ++l) {
            long ci = NE + 2 * l * NE + h;
            d->rel_vort[ci] = ir->viscosity_rhombi[NC + l * VPL + h] * d->rel_vort[ci];
        }
    ORC_PAR
    for (long i = 0; i < (long)NL * NT; ++i)
        d->rel_vort_on_triangles[i] = ir->viscosity_triangles[i] * d->rel_vort_on_triangles[i];
    hor_calc_curl_of_vorticity(g, d->rel_vort, d->rel_vort_on_triangles, d->curl_of_vorticity);
    ORC_PAR
    for (long h = 0; h < NE; ++h)
        for (long l = 0; l < NL; ++l) {
            long vi = NC + l * VPL + h, f = l * NC + g->from[h], t = l * NC + g->to[h];
            ir->friction_acc[vi] = (d->vector_field_placeholder[vi] - d->curl_of_vorticity[vi])
                                   / (0.5 * (density_total(g, s, f) + density_total(g, s, t)));
        }
    return 0;
}

/* src/subgrid_scale/effective_diff_coeffs.c:114-168 */
static void vert_hor_mom_viscosity(const orc_grid *g, const orc_state *s, const orc_diag *d, orc_irrev *ir)
{
    const double *rg = &s->rho[COND * NS], *n2 = d->n_squared, *lt = g->layer_thickness, *tke = ir->tke;
    const double *mol = ir->molecular_diffusion_coeff;
    ORC_PAR
    for (long i = 0; i < (long)NL * NE - NE; ++i) {
        long layer = i / NE, h = i - layer * NE;
        long f0 = layer * NC + g->from[h], t0 = layer * NC + g->to[h];
        long f1 = (layer + 1) * NC + g->from[h], t1 = (layer + 1) * NC + g->to[h];
        double mdc = 0.25 * (tke2vert_diff_coeff(tke[f0], n2[f0], lt[f0]) + tke2vert_diff_coeff(tke[t0], n2[t0], lt[t0])
                             + tke2vert_diff_coeff(tke[f1], n2[f1], lt[f1]) + tke2vert_diff_coeff(tke[t1], n2[t1], lt[t1]));
        double molecular_viscosity = 0.25 * (mol[f0] + mol[t0] + mol[f1] + mol[t1]);
        mdc += molecular_viscosity;
        ir->vert_hor_viscosity[i + NE] = 0.25 * (rg[f0] + rg[t0] + rg[f1] + rg[t1]) * mdc;
    }
    ORC_PAR
    for (long i = 0; i < NE; ++i) ir->vert_hor_viscosity[i] = ir->vert_hor_viscosity[i + NE];
    ORC_PAR
    for (long i = (long)NL * NE; i < (long)NL * NE + NE; ++i) ir->vert_hor_viscosity[i] = ir->vert_hor_viscosity[i - NE];
}

/* src/subgrid_scale/effective_diff_coeffs.c:170-193 */
static void vert_vert_mom_viscosity(const orc_grid *g, const orc_state *s, orc_diag *d, const orc_irrev *ir)
{
    ORC_PAR
    for (long h = 0; h < NC; ++h)
        for (long l = 0; l < NL; ++l) {
            long i = l * NC + h;
            double mdc = ir->molecular_diffusion_coeff[i]
                         + tke2vert_diff_coeff(ir->tke[i], d->n_squared[i], g->layer_thickness[i]);
            d->scalar_field_placeholder[i] = s->rho[COND * NS + i] * mdc * d->scalar_field_placeholder[i];
        }
}

/* src/spatial_operators/momentum_diff_diss.c:82-205.  The TOA row of dv_hdz
 * is never written (the branch meant for it cannot be reached) and keeps its
 * values. */
int orc_vert_momentum_diffusion(const orc_grid *g, const orc_state *s, orc_diag *d, orc_irrev *ir)
{
    const double *zv = g->z_vector, *w = s->wind;
    /* 1. vertical diffusion of horizontal velocity */
    ORC_PAR
    for (long i = NE; i < (long)NL * NE + NE; ++i) {
        long layer = i / NE, h = i - layer * NE, vi = NC + h + (layer - 1) * VPL;
        if (layer == NL)
            d->dv_hdz[i] = w[vi] / (zv[vi] - 0.5 * (zv[NV - NC + g->from[h]] + zv[NV - NC + g->to[h]]));
        else if (layer >= 1)
            d->dv_hdz[i] = (w[vi] - w[vi + VPL]) / (zv[vi] - zv[vi + VPL]);
    }
    vert_hor_mom_viscosity(g, s, d, ir);
    ORC_PAR
    for (long i = 0; i < (long)NL * NE; ++i) {
        long layer = i / NE, h = i - layer * NE, vi = NC + layer * VPL + h;
        double z_upper = 0.5 * (zv[layer * VPL + g->from[h]] + zv[layer * VPL + g->to[h]]);
        double z_lower = 0.5 * (zv[(layer + 1) * VPL + g->from[h]] + zv[(layer + 1) * VPL + g->to[h]]);
        double delta_z = z_upper - z_lower;
        ir->friction_acc[vi] += (ir->vert_hor_viscosity[i] * d->dv_hdz[i] - ir->vert_hor_viscosity[i + NE] * d->dv_hdz[i + NE])
                                / delta_z
                                / (0.5 * (density_total(g, s, layer * NC + g->from[h])
                                          + density_total(g, s, layer * NC + g->to[h])));
    }
    /* 2. vertical diffusion of vertical velocity */
    ORC_PAR
    for (long i = 0; i < NS; ++i) d->scalar_field_placeholder[i] = 0.0;
    orc_add_vertical_divv(g, w, d->scalar_field_placeholder);
    vert_vert_mom_viscosity(g, s, d, ir);
    orc_grad_vert_cov(g, d->scalar_field_placeholder, ir->friction_acc);
    /* 3. horizontal diffusion of vertical velocity */
    ORC_PAR
    for (long h = 0; h < NC; ++h)
        for (long l = 0; l < NL; ++l) {
            long i = l * NC + h;
            d->scalar_field_placeholder[i] = g->ipw[8 * i + 6] * w[h + l * VPL] + g->ipw[8 * i + 7] * w[h + (l + 1) * VPL];
        }
    orc_grad_hor(g, d->scalar_field_placeholder, d->vector_field_placeholder);
    ORC_PAR
    for (long h = 0; h < NE; ++h)
        for (long l = 0; l < NL; ++l) {
            long vi = NC + h + l * VPL;
            d->vector_field_placeholder[vi] = 0.5 * (ir->viscosity[l * NC + g->from[h]] + ir->viscosity[l * NC + g->to[h]])
                                              * d->vector_field_placeholder[vi];
        }
    orc_divv_h(g, d->vector_field_placeholder, d->scalar_field_placeholder);
    ORC_PAR
    for (long i = 0; i < (long)(NL + 1) * NC - 2 * NC; ++i) {
        long layer = i / NC, h = i - layer * NC, vi = h + (layer + 1) * VPL;
        ir->friction_acc[vi] += 0.5 * (d->scalar_field_placeholder[h + layer * NC]
                                       + d->scalar_field_placeholder[h + (layer + 1) * NC]);
        ir->friction_acc[vi] = ir->friction_acc[vi] / (0.5 * (density_total(g, s, h + layer * NC)
                                                              + density_total(g, s, h + (layer + 1) * NC)));
    }
    return 0;
}

/* src/spatial_operators/momentum_diff_diss.c:296-310 */
int orc_simple_dissipation_rate(const orc_grid *g, const orc_state *s, orc_irrev *ir)
{
    orc_inner_product(g, s->wind, ir->friction_acc, ir->heating_diss);
    ORC_PAR
    for (long i = 0; i < NS; ++i) ir->heating_diss[i] = -density_total(g, s, i) * ir->heating_diss[i];
    return 0;
}

/* src/subgrid_scale/effective_diff_coeffs.c:195-231 */
int orc_scalar_diffusion_coeffs(const orc_grid *g, const orc_state *s, const orc_config *c, orc_irrev *ir,
                                orc_diag *d)
{
    if (c->momentum_diff_h == 0) orc_hor_viscosity(g, s, ir, d);
    ORC_PAR
    for (long i = 0; i < NS; ++i) {
        ir->mass_diffusion_coeff_numerical_h[i] = ir->viscosity[i] / s->rho[COND * NS + i];
        ir->mass_diffusion_coeff_numerical_v[i] = ir->molecular_diffusion_coeff[i]
                                                  + tke2vert_diff_coeff(ir->tke[i], d->n_squared[i], g->layer_thickness[i]);
        ir->temp_diffusion_coeff_numerical_h[i] = c_v_mass_weighted_air(g, s, d, i) * ir->mass_diffusion_coeff_numerical_h[i];
        ir->temp_diffusion_coeff_numerical_v[i] = c_v_mass_weighted_air(g, s, d, i) * ir->mass_diffusion_coeff_numerical_v[i];
    }
    return 0;
}

/* ------------------------------------------------- Held-Suarez forcing
 * (rad_on = 2, pbl_scheme = 2) */
#define P_HS_0 100000.0

/* src/radiation/held_suar.c:34-46 */
static double hs_t_eq(double latitude, double pressure)
{
    double delta_t_y = 60.0, delta_theta_v_z = 10.0, kappa = 2.0 / 7.0, result = 315.0;
    result = result - delta_t_y * pow(sin(latitude), 2.0);
    result = result - delta_theta_v_z * log(pressure / P_HS_0) * pow(cos(latitude), 2.0);
    result = result * pow(pressure / P_HS_0, kappa);
    result = fmax(200.0, result);
    return result;
}

/* src/radiation/held_suar.c:48-56 */
static double hs_k_T(double latitude, double pressure)
{
    double k_a = 1.0 / 40.0 * 1.0 / 86400.0, k_s = 1.0 / 4.0 * 1.0 / 86400.0, sigma_b = 0.7;
    double sigma = pressure / P_HS_0;
    return k_a + (k_s - k_a) * fmax(0.0, (sigma - sigma_b) / (1.0 - sigma_b)) * pow(cos(latitude), 4.0);
}

/* src/radiation/held_suar.c:18-32 through call_radiation
 * (manage_radiation_calls.c:22-78).  The reference cuts the scalar points
 * into NO_OF_RAD_BLOCKS = 18 blocks of NO_OF_SCALARS/18 points, reshaped into
 * (NO_OF_SCALARS/18)/NO_OF_LAYERS columns each; every point's tendency
 * depends on its own values only, so the blocks just select the points: the
 * first 18 * columns-per-block cells of every layer.  When NO_OF_SCALARS/18
 * is not a multiple of the layer count the reference's loops run into a
 * layer NO_OF_LAYERS and write past the end of radiation_tendency; such grids
 * are refused (-1).  The blocks' surface fluxes, which Held-Suarez leaves at
 * zero, are copied back for the covered cells. */
int orc_held_suarez_radiation(const orc_grid *g, const orc_state *s, const orc_diag *d, orc_forcings *f)
{
    const long n_rad = NS / 18, per_layer = n_rad / NL, covered = 18 * per_layer;
    if (n_rad % NL != 0) return -1;
    ORC_PAR
    for (long i = 0; i < NS; ++i) {
        long layer = i / NC, h = i - layer * NC;
        if (h >= covered) continue;
        double rg = s->rho[COND * NS + i], t = d->temperature[i];
        double pressure = rg * R_D * t;
        f->radiation_tendency[i] = -hs_k_T(g->latitude_scalar[h], pressure) * (t - hs_t_eq(g->latitude_scalar[h], pressure));
        f->radiation_tendency[i] = C_D_V * rg * f->radiation_tendency[i];
    }
    for (long h = 0; h < covered; ++h) f->sfc_sw_in[h] = f->sfc_lw_out[h] = 0.0;
    return 0;
}

/* src/constituents/derived_quantities.c:42-61 */
static double gas_constant_diagnostics(const orc_grid *g, const orc_state *s, long i)
{
    double result = 0.0;
    if (!g->moisture_on) result = R_D;
    if (g->moisture_on) {
        result = (s->rho[COND * NS + i] - s->rho[(COND + 1) * NS + i]) * R_D + s->rho[(COND + 1) * NS + i] * R_V;
        result = result / s->rho[COND * NS + i];
    }
    return result;
}

/* boundary-layer friction of the Held-Suarez test
 * (src/subgrid_scale/planetary_boundary_layer.c:141-197), added to the
 * friction acceleration of every horizontal wind point */
int orc_pbl_held_suarez(const orc_grid *g, const orc_state *s, const orc_diag *d, orc_irrev *ir)
{
    const double bndr_lr_visc_max = 1.0 / 86400.0, sigma_b = 0.7, lapse = 0.0065;
    ORC_PAR
    for (long i = 0; i < (long)NL * NE; ++i) {
        long layer = i / NE, h = i - layer * NE, vi = NC + layer * VPL + h;
        long f = g->from[h], t = g->to[h];
        double exner_from = g->exner_bg[layer * NC + f] + s->exner_pert[layer * NC + f];
        double exner_to = g->exner_bg[layer * NC + t] + s->exner_pert[layer * NC + t];
        double pressure_from = P_HS_0 * pow(exner_from, C_D_P / R_D);
        double pressure_to = P_HS_0 * pow(exner_to, C_D_P / R_D);
        double pressure = 0.5 * (pressure_from + pressure_to);
        double psfc[2];
        for (int side = 0; side < 2; ++side) {
            long c = side == 0 ? f : t, lo = (NL - 1) * NC + c;
            double temp_lowest_layer = d->temperature[lo];
            double exner = g->exner_bg[lo] + s->exner_pert[lo];
            double pressure_value_lowest_layer = P_HS_0 * pow(exner, C_D_P / R_D);
            double temp_surface = temp_lowest_layer + lapse * (g->z_scalar[c + (NL - 1) * NC] - g->z_vector[NV - NC + c]);
            double surface_p_factor = pow(1.0 - (temp_surface - temp_lowest_layer) / temp_surface,
                                          g->gravity_m[(NL - 1) * VPL + c] / (gas_constant_diagnostics(g, s, lo) * lapse));
            psfc[side] = pressure_value_lowest_layer / surface_p_factor;
        }
        double pressure_sfc = 0.5 * (psfc[0] + psfc[1]);
        double sigma = pressure / pressure_sfc;
        ir->friction_acc[vi] += -bndr_lr_visc_max * fmax(0.0, (sigma - sigma_b) / (1.0 - sigma_b)) * s->wind[vi];
    }
    return 0;
}

/* ------------------------------------------------- explicit tendencies
 * src/time_stepping/vector_tendencies_expl.c:18-133 */
int orc_vector_tendencies_expl(const orc_grid *g, const orc_state *s, orc_state *tend, orc_diag *d,
                               orc_forcings *f, orc_irrev *ir, const orc_config *c, int rk_step, double dt)
{
    if (rk_step == 1 || c->totally_first_step_bool == 1) {
        orc_scalar_times_vector(g, &s->rho[COND * NS], s->wind, d->flux_density);
        orc_calc_pot_vort(g, s->wind, &s->rho[COND * NS], d);
        orc_vorticity_flux(g, d->flux_density, d->pot_vort, f->pot_vort_tend);
        orc_inner_product(g, s->wind, s->wind, d->v_squared);
        orc_grad(g, d->v_squared, f->v_squared_grad);
    }
    /* momentum diffusion and dissipation (:37-69) */
    if (rk_step == 0) {
        if (c->momentum_diff_h || c->mass_diff_h || c->temperature_diff_h) {
            orc_update_n_squared(g, s, d);
            orc_tke_update(g, ir, dt, s, d);
        }
        if (c->momentum_diff_h) orc_hor_momentum_diffusion(g, s, d, ir);
        if (c->momentum_diff_v) orc_vert_momentum_diffusion(g, s, d, ir);
        if (c->pbl_scheme == 1) return -1;
        if (c->pbl_scheme == 2) orc_pbl_held_suarez(g, s, d, ir);
        if (c->momentum_diff_h || c->pbl_scheme > 0) orc_simple_dissipation_rate(g, s, ir);
    }
    double new_w = rk_step == 1 ? 0.5 : 1.0, old_w = 1.0 - new_w;
    double cur_hor = 0.5 + c->impl_thermo_weight, old_hor = 1.0 - cur_hor, cur_ver = 1.0 - c->impl_thermo_weight;
    ORC_PAR
    for (long i = 0; i < NV; ++i) {
        long layer = i / VPL, h = i - layer * VPL;
        if (i < NC || i >= NV - NC) {
            tend->wind[i] = 0.0;
        } else if (h >= NC) {
            tend->wind[i] = old_w * tend->wind[i]
                            + new_w * (old_hor * f->pgrad_acc_old[i] - cur_hor * (f->pgrad_nl[i] + f->pgrad_l[i])
                                       + f->pot_vort_tend[i] - 0.5 * f->v_squared_grad[i] + ir->friction_acc[i]);
        } else {
            tend->wind[i] = old_w * tend->wind[i]
                            + new_w * (-cur_ver * (f->pgrad_nl[i] + f->pgrad_l[i]) + f->pot_vort_tend[i]
                                       - 0.5 * f->v_squared_grad[i] + ir->friction_acc[i] + f->pgrad_condensates_v[i]);
        }
    }
    return 0;
}

/* src/time_stepping/scalar_tendencies_expl.c:17-181 */
int orc_scalar_tendencies_expl(const orc_grid *g, const orc_state *s_old, const orc_state *s, orc_state *tend,
                               double dt, orc_diag *d, orc_forcings *f, orc_irrev *ir, const orc_config *c,
                               int rk_step)
{
    (void)s_old; (void)dt;
    double old_w[8], new_w[8];
    for (int k = 0; k < g->n_const; ++k) {
        new_w[k] = 1.0;
        if (rk_step == 1 && k != COND) new_w[k] = 0.5;
        old_w[k] = 1.0 - new_w[k];
    }
    /* diffusion coefficients, temperature and mass diffusion (:44-88) */
    if (rk_step == 0 && (c->mass_diff_h || c->temperature_diff_h)) orc_scalar_diffusion_coeffs(g, s, c, ir, d);
    if (c->temperature_diff_h && rk_step == 0) {
        orc_grad(g, d->temperature, d->vector_field_placeholder);
        orc_scalar_times_vector_h(g, ir->temp_diffusion_coeff_numerical_h, d->vector_field_placeholder,
                                  d->flux_density);
        orc_divv_h(g, d->flux_density, ir->temperature_diffusion_heating);
        if (c->temperature_diff_v) {
            orc_scalar_times_vector_v(g, ir->temp_diffusion_coeff_numerical_v, d->vector_field_placeholder,
                                      d->flux_density);
            orc_add_vertical_divv(g, d->flux_density, ir->temperature_diffusion_heating);
        }
    }
    if (c->mass_diff_h && rk_step == 0) {
        for (int k = 0; k < g->n_const; ++k) {
            long shift = k * NS;
            orc_grad(g, &s->rho[shift], d->vector_field_placeholder);
            orc_scalar_times_vector_h(g, ir->mass_diffusion_coeff_numerical_h, d->vector_field_placeholder,
                                      d->vector_field_placeholder);
            orc_divv_h(g, d->vector_field_placeholder, &ir->mass_diff_tendency[shift]);
            if (c->mass_diff_v) {
                orc_scalar_times_vector_v(g, ir->mass_diffusion_coeff_numerical_v, d->vector_field_placeholder,
                                          d->vector_field_placeholder);
                orc_add_vertical_divv(g, d->vector_field_placeholder, &ir->mass_diff_tendency[shift]);
            }
        }
    }
    for (int k = 0; k < g->n_const; ++k) {
        long shift = k * NS, shift_pt = shift;
        if (g->moisture_on && k == COND + 1) shift_pt = shift - NS;
        if (k == COND) {
            orc_scalar_times_vector_h(g, &s->rho[shift], s->wind, d->flux_density);
            orc_divv_h(g, d->flux_density, d->flux_density_divv);
        } else {
            orc_scalar_times_vector_h_upstream(g, &s->rho[shift], s->wind, d->flux_density);
            orc_divv_h_tracer(g, d->flux_density, &s->rho[shift], s->wind, d->flux_density_divv);
        }
        ORC_PAR
        for (long j = 0; j < NS; ++j) {
            long si = shift + j;
            tend->rho[si] = old_w[k] * tend->rho[si]
                            + new_w[k] * (-d->flux_density_divv[j] + ir->mass_diff_tendency[shift + j]
                                          + ir->phase_trans_rates[shift_pt + j]);
        }
        if (k == COND) {
            for (long j = 0; j < NS; ++j) d->scalar_field_placeholder[j] = s->rhotheta_v[j] / s->rho[shift + j];
            orc_scalar_times_vector_h(g, d->scalar_field_placeholder, d->flux_density, d->flux_density);
            orc_divv_h(g, d->flux_density, d->flux_density_divv);
            for (long j = 0; j < NS; ++j) {
                tend->rhotheta_v[j] = old_w[k] * tend->rhotheta_v[j]
                    + new_w[k] * (-d->flux_density_divv[j]
                                  + C_D_V * s->rho[shift + j] / c_v_mass_weighted_air(g, s, d, j)
                                        * (ir->heating_diss[j] + ir->temperature_diffusion_heating[j]
                                           + f->radiation_tendency[j] + ir->phase_trans_heating_rate[j]
                                           + ir->condensates_sediment_heat[j])
                                        / (C_D_P * (g->exner_bg[j] + s->exner_pert[j]))
                                  + (ir->phase_trans_rates[shift + j] + ir->mass_diff_tendency[shift + j])
                                        * d->scalar_field_placeholder[j]);
            }
        }
    }
    return 0;
}

/* --------------------------------------------------------- column solvers
 * src/time_stepping/column_solvers.c */
static void thomas(const double *cv, const double *dv, const double *ev, const double *rv, double *x, int n)
{
    /* :641-669 */
    double ep[ORC_MAX_L], rp[ORC_MAX_L];
    ep[0] = ev[0] / dv[0];
    for (int j = 1; j < n - 1; ++j) ep[j] = ev[j] / (dv[j] - ep[j - 1] * cv[j - 1]);
    rp[0] = rv[0] / dv[0];
    for (int j = 1; j < n; ++j) rp[j] = (rv[j] - rp[j - 1] * cv[j - 1]) / (dv[j] - ep[j - 1] * cv[j - 1]);
    x[n - 1] = rp[n - 1];
    for (int j = n - 2; j >= 0; --j) x[j] = rp[j] - ep[j] * x[j + 1];
}

int orc_three_band_solver_ver_waves(const orc_grid *g, const orc_state *so, orc_state *sn, const orc_state *st,
                                    const orc_config *c, double dt, int rk_step)
{
    /* :19-383 (sensible heat flux and soil off) */
    if (c->sfc_sensible_heat_flux || c->prog_soil_temp) return -1;
    if (NL > ORC_MAX_L) return -2;
    const double iw = c->impl_thermo_weight;
    const double damp_start = c->damping_start_height_over_toa * g->z_vector[0];
    const double pdw = 0.5;
    const long gp = COND * NS;
    ORC_PAR
    for (long i = 0; i < NC; ++i) {
        double cvec[ORC_MAX_L], dvec[ORC_MAX_L], evec[ORC_MAX_L], rvec[ORC_MAX_L], rho_expl[ORC_MAX_L], rt_expl[ORC_MAX_L], tp_expl[ORC_MAX_L], ep_expl[ORC_MAX_L];
        double th_int[ORC_MAX_L], sol[ORC_MAX_L], rho_io[ORC_MAX_L], rho_ie[ORC_MAX_L], alpha[ORC_MAX_L], beta[ORC_MAX_L], gam[ORC_MAX_L];
        for (long j = 0; j < NL; ++j) {
            long b = i + j * NC;
            rho_expl[j] = so->rho[gp + b] + dt * st->rho[gp + b];
            rt_expl[j] = so->rhotheta_v[b] + dt * st->rhotheta_v[b];
            if (rk_step == 0) {
                alpha[j] = -so->rhotheta_v[b] / pow(so->rho[gp + b], 2) / g->volume[b];
                beta[j] = 1.0 / so->rho[gp + b] / g->volume[b];
                gam[j] = R_D / (C_D_V * so->rhotheta_v[b]) * (g->exner_bg[b] + so->exner_pert[b]) / g->volume[b];
            } else {
                double ao = -so->rhotheta_v[b] / pow(so->rho[gp + b], 2);
                double bo = 1.0 / so->rho[gp + b];
                double go = R_D / (C_D_V * so->rhotheta_v[b]) * (g->exner_bg[b] + so->exner_pert[b]);
                double an = -sn->rhotheta_v[b] / pow(sn->rho[gp + b], 2);
                double bn = 1.0 / sn->rho[gp + b];
                double gn = R_D / (C_D_V * sn->rhotheta_v[b]) * (g->exner_bg[b] + sn->exner_pert[b]);
                alpha[j] = ((1.0 - pdw) * ao + pdw * an) / g->volume[b];
                beta[j] = ((1.0 - pdw) * bo + pdw * bn) / g->volume[b];
                gam[j] = ((1.0 - pdw) * go + pdw * gn) / g->volume[b];
            }
            tp_expl[j] = so->theta_v_pert[b] + dt * g->volume[b] * (alpha[j] * st->rho[gp + b] + beta[j] * st->rhotheta_v[b]);
            ep_expl[j] = so->exner_pert[b] + dt * g->volume[b] * gam[j] * st->rhotheta_v[b];
        }
        for (long j = 0; j < NL - 1; ++j) {
            long b = i + j * NC, lo = i + (j + 1) * NC;
            rho_io[j] = 0.5 * (so->rho[gp + b] + so->rho[gp + lo]);
            rho_ie[j] = 0.5 * (rho_expl[j] + rho_expl[j + 1]);
            th_int[j] = 0.5 * (sn->rhotheta_v[b] / sn->rho[gp + b] + sn->rhotheta_v[lo] / sn->rho[gp + lo]);
        }
        for (long j = 0; j < NL - 1; ++j) {
            long b = i + j * NC, lo = i + (j + 1) * NC, wi = i + (j + 1) * VPL;
            dvec[j] = -pow(th_int[j], 2) * (gam[j] + gam[j + 1])
                      + 0.5 * (g->exner_bg[b] - g->exner_bg[lo]) * (alpha[j + 1] - alpha[j] + th_int[j] * (beta[j + 1] - beta[j]))
                      - (g->z_scalar[b] - g->z_scalar[lo]) / (iw * pow(dt, 2) * C_D_P * rho_io[j])
                            * (2.0 / g->area[wi] + dt * so->wind[wi] * 0.5 * (-1.0 / g->volume[b] + 1.0 / g->volume[lo]));
            rvec[j] = -(so->wind[wi] + dt * st->wind[wi]) * (g->z_scalar[b] - g->z_scalar[lo]) / (iw * pow(dt, 2) * C_D_P)
                      + th_int[j] * (ep_expl[j] - ep_expl[j + 1]) / dt
                      + 0.5 / dt * (tp_expl[j] + tp_expl[j + 1]) * (g->exner_bg[b] - g->exner_bg[lo])
                      - (g->z_scalar[b] - g->z_scalar[lo]) / (iw * pow(dt, 2) * C_D_P) * so->wind[wi] * rho_ie[j] / rho_io[j];
        }
        for (long j = 0; j < NL - 2; ++j) {
            long b = i + j * NC, lo = i + (j + 1) * NC, lo2 = (j + 2) * NC + i;
            cvec[j] = th_int[j + 1] * gam[j + 1] * th_int[j]
                      + 0.5 * (g->exner_bg[lo] - g->exner_bg[lo2]) * (alpha[j + 1] + beta[j + 1] * th_int[j])
                      - (g->z_scalar[lo] - g->z_scalar[lo2]) / (iw * dt * C_D_P) * 0.5 * so->wind[i + (j + 2) * VPL]
                            / (g->volume[lo] * rho_io[j + 1]);
            evec[j] = th_int[j] * gam[j + 1] * th_int[j + 1]
                      - 0.5 * (g->exner_bg[b] - g->exner_bg[lo]) * (alpha[j + 1] + beta[j + 1] * th_int[j + 1])
                      + (g->z_scalar[b] - g->z_scalar[lo]) / (iw * dt * C_D_P) * 0.5 * so->wind[i + (j + 1) * VPL]
                            / (g->volume[lo] * rho_io[j]);
        }
        thomas(cvec, dvec, evec, rvec, sol, (int)NL - 1);
        for (long j = 0; j < NL - 1; ++j) {
            double zad = g->z_vector[i + (j + 1) * VPL] - damp_start, dc;
            if (zad < 0.0) dc = 0.0;
            else dc = c->damping_coeff_max * pow(sin(0.5 * M_PI * zad / (g->z_vector[0] - damp_start)), 2);
            sol[j] = sol[j] / (1.0 + dt * dc);
        }
        for (long j = 0; j < NL; ++j) {
            long b = i + j * NC;
            if (j == 0) sn->rho[gp + b] = rho_expl[j] + dt * (sol[j]) / g->volume[b];
            else if (j == NL - 1) sn->rho[gp + b] = rho_expl[j] + dt * (-sol[j - 1]) / g->volume[b];
            else sn->rho[gp + b] = rho_expl[j] + dt * (-sol[j - 1] + sol[j]) / g->volume[b];
        }
        for (long j = 0; j < NL; ++j) {
            long b = i + j * NC;
            if (j == 0) sn->rhotheta_v[b] = rt_expl[j] + dt * (th_int[j] * sol[j]) / g->volume[b];
            else if (j == NL - 1) sn->rhotheta_v[b] = rt_expl[j] + dt * (-th_int[j - 1] * sol[j - 1]) / g->volume[b];
            else sn->rhotheta_v[b] = rt_expl[j] + dt * (-th_int[j - 1] * sol[j - 1] + th_int[j] * sol[j]) / g->volume[b];
        }
        for (long j = 0; j < NL - 1; ++j) {
            long b = i + j * NC, wi = i + (j + 1) * VPL;
            double dint = 0.5 * (sn->rho[gp + b] + sn->rho[gp + i + (j + 1) * NC]);
            sn->wind[wi] = (2.0 * sol[j] / g->area[wi] - dint * so->wind[wi]) / rho_io[j];
        }
        for (long j = 0; j < NL; ++j) {
            long b = i + j * NC;
            sn->theta_v_pert[b] = sn->rhotheta_v[b] / sn->rho[gp + b] - g->theta_v_bg[b];
        }
        for (long j = 0; j < NL; ++j) {
            long b = i + j * NC;
            sn->exner_pert[b] = so->exner_pert[b] + g->volume[b] * gam[j] * (sn->rhotheta_v[b] - so->rhotheta_v[b]);
        }
    }
    return 0;
}

int orc_three_band_solver_gen_densities(const orc_grid *g, const orc_state *so, orc_state *sn, const orc_state *st,
                                        const orc_diag *d, orc_irrev *ir, const orc_config *c, double dt, int rk_step)
{
    /* :385-639 */
    const double iw = 0.5, ew = 1.0 - iw;
    if (NL > ORC_MAX_L) return -2;
    double *sh = ir->condensates_sediment_heat;
    for (int k = 0; k < g->n_const; ++k) {
        if (k == COND) continue;
        /* sink velocity of the constituent: snow, rain, cloud particles, none for vapour */
        double vsink = 0.0;
        int has_sink = 0;
        if (k < COND / 4) { vsink = c->snow_velocity; has_sink = 1; }
        else if (k < COND / 2) { vsink = c->rain_velocity; has_sink = 1; }
        else if (k < COND) { vsink = c->cloud_droplets_velocity; has_sink = 1; }
        ORC_PAR
        for (long i = 0; i < NC; ++i) {
            double cvec[ORC_MAX_L], dvec[ORC_MAX_L], evec[ORC_MAX_L], rvec[ORC_MAX_L], fi[ORC_MAX_L], fr[ORC_MAX_L], fe[ORC_MAX_L], sol[ORC_MAX_L];
            for (long j = 0; j < NL - 1; ++j) {
                if (rk_step == 0 && k == 0) sh[j * NC + i] = 0.0;
                long b = i + j * NC, lo = i + (j + 1) * NC, up = b;
                fi[j] = so->wind[i + (j + 1) * VPL];
                fr[j] = sn->wind[i + (j + 1) * VPL];
                if (has_sink) { fi[j] -= vsink; fr[j] -= vsink; }
                double a = g->area[i + (j + 1) * VPL];
                fi[j] = a * fi[j];
                fr[j] = a * fr[j];
                double dio, tio;
                if (fr[j] >= 0.0) { dio = so->rho[k * NS + lo]; tio = d->temperature[lo]; }
                else { dio = so->rho[k * NS + up]; tio = d->temperature[up]; }
                fr[j] = dio * fr[j];
                fe[j] = c_p_cond(k, tio) * tio * fr[j];
            }
            if (rk_step == 0 && k == 0) sh[(NL - 1) * NC + i] = 0.0;
            for (long j = 0; j < NL - 1; ++j) {
                long b = i + j * NC;
                if (fi[j] >= 0.0) { cvec[j] = 0.0; evec[j] = -iw * dt / g->volume[b] * fi[j]; }
                else { cvec[j] = iw * dt / g->volume[i + (j + 1) * NC] * fi[j]; evec[j] = 0.0; }
            }
            const long bot = i + NS - NC;
            const double a_sfc = g->area[i + NV - NC];
            for (long j = 0; j < NL; ++j) {
                long b = i + j * NC;
                if (j == 0) {
                    if (fi[0] >= 0.0) dvec[j] = 1.0;
                    else dvec[j] = 1.0 - iw * dt / g->volume[b] * fi[0];
                } else if (j == NL - 1) {
                    if (fi[j - 1] >= 0.0) dvec[j] = 1.0 + iw * dt / g->volume[b] * fi[j - 1];
                    else dvec[j] = 1.0;
                    if (has_sink) dvec[j] += iw * vsink * dt * a_sfc / g->volume[b];
                } else {
                    dvec[j] = 1.0;
                    if (fi[j - 1] >= 0.0) dvec[j] += iw * dt / g->volume[b] * fi[j - 1];
                    if (fi[j] < 0.0) dvec[j] -= iw * dt / g->volume[b] * fi[j];
                }
                rvec[j] = so->rho[k * NS + b] + dt * st->rho[k * NS + b];
                if (j == 0) {
                    rvec[j] += ew * dt * fr[j] / g->volume[b];
                    if (rk_step == 0 && k < COND) sh[b] += fe[j] / g->volume[b];
                } else if (j == NL - 1) {
                    rvec[j] += -ew * dt * fr[j - 1] / g->volume[b];
                    if (rk_step == 0 && k < COND) sh[b] += -fe[j - 1] / g->volume[b];
                    if (has_sink) {
                        rvec[j] += -ew * vsink * dt * so->rho[k * NS + bot] * a_sfc / g->volume[b];
                        if (rk_step == 0)
                            sh[b] += -vsink * d->temperature[bot] * c_p_cond(k, d->temperature[bot])
                                     * so->rho[k * NS + bot] * a_sfc / g->volume[b];
                    }
                } else {
                    rvec[j] += ew * dt * (-fr[j - 1] + fr[j]) / g->volume[b];
                    if (rk_step == 0 && k < COND) sh[b] += (-fe[j - 1] + fe[j]) / g->volume[b];
                }
            }
            thomas(cvec, dvec, evec, rvec, sol, (int)NL);
            for (long j = 0; j < NL; ++j) if (sol[j] < 0.0) sol[j] = 0.0;
            for (long j = 0; j < NL; ++j) sn->rho[k * NS + i + j * NC] = sol[j];
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ step
 * src/time_stepping/manage_rkhevi.c:20-100 */
int orc_manage_rkhevi(const orc_grid *g, const orc_state *so, orc_state *sn, orc_state *st, orc_diag *d,
                      orc_forcings *f, orc_irrev *ir, const orc_config *c, double dt, double t)
{
    (void)t;
    if (c->sfc_sensible_heat_flux || c->sfc_phase_trans || c->pbl_scheme == 1 || c->pbl_scheme > 2 || c->rad_on == 1
        || c->rad_on > 2 || c->prog_soil_temp)
        return -1;
    orc_temperature_diagnostics(g, so, d);
    if (g->moisture_on) orc_calc_h2otracers_source_rates(g, so, d, c, ir, dt);
    for (int rk = 0; rk < 2; ++rk) {
        if (rk == 0) orc_manage_pressure_gradient(g, sn, d, f, ir, c);
        orc_calc_pressure_grad_condensates_v(g, sn, f, ir);
        orc_vector_tendencies_expl(g, sn, st, d, f, ir, c, rk, dt);
        ORC_PAR
        for (long e = 0; e < NE; ++e)
            for (long l = 0; l < NL; ++l) {
                long vi = NC + l * VPL + e;
                sn->wind[vi] = so->wind[vi] + dt * st->wind[vi];
            }
        /* radiation: the Held-Suarez forcing, on state_old (manage_rkhevi.c:80-84) */
        if (c->rad_on == 2 && c->rad_update == 1 && rk == 0)
            if (orc_held_suarez_radiation(g, so, d, f)) return -1;
        if (orc_scalar_tendencies_expl(g, so, sn, st, dt, d, f, ir, c, rk)) return -1;
        if (orc_three_band_solver_ver_waves(g, so, sn, st, c, dt, rk)) return -1;
        if (g->n_const > 1) orc_three_band_solver_gen_densities(g, so, sn, st, d, ir, c, dt, rk);
    }
    return 0;
}

/* --------------------------------------------------------------- metrics */
double orc_global_scalar_integrator(const orc_grid *g, const double *field)
{
    /* src/io/write_output.c:1659-1668 (serial sum, kept in its order) */
    double r = 0.0;
    for (long i = 0; i < NS; ++i) r += field[i] * g->volume[i];
    return r;
}

int orc_surface_pressure(const orc_grid *g, const orc_state *s, const double *temperature, double *p_sfc,
                         double *mslp)
{
    /* src/io/write_output.c:105-121 with gas_constant_diagnostics
     * (src/constituents/derived_quantities.c:42-61) */
    const double lapse = 0.0065;
    ORC_PAR
    for (long i = 0; i < NC; ++i) {
        long si = (NL - 1) * NC + i;
        double rgas;
        if (!g->moisture_on) rgas = R_D;
        else {
            rgas = (s->rho[COND * NS + si] - s->rho[(COND + 1) * NS + si]) * R_D + s->rho[(COND + 1) * NS + si] * R_V;
            rgas = rgas / s->rho[COND * NS + si];
        }
        double t_low = temperature[si];
        double p = s->rho[COND * NS + si] * rgas * t_low;
        if (mslp) {
            double t_mslp = t_low + lapse * g->z_scalar[i + (NL - 1) * NC];
            mslp[i] = p / pow(1 - (t_mslp - t_low) / t_mslp, g->gravity_m[(NL - 1) * VPL + i] / (rgas * lapse));
        }
        double t_sfc = t_low + lapse * (g->z_scalar[i + (NL - 1) * NC] - g->z_vector[NV - NC + i]);
        double fac = pow(1.0 - (t_sfc - t_low) / t_sfc, g->gravity_m[(NL - 1) * VPL + i] / (rgas * lapse));
        p_sfc[i] = p / fac;
    }
    return 0;
}

/* ------------------------------------------------------------ output
 * The operators only output uses and the fields write_out computes
 * (src/io/write_output.c:51-1513, src/io/spatial_ops_for_output.c,
 * src/spatial_operators/averaging.c:135-234), without the writers. */
#define G_MEAN_SFC_ABS 9.80616

static double tangential_wind(const orc_grid *g, const double *in, long layer, long h)
{
    /* averaging.c:135-150 */
    double component = 0;
    for (int i = 0; i < 10; ++i)
        component += g->trsk_weights[10 * h + i] * in[NC + layer * VPL + g->trsk_indices[10 * h + i]];
    return component;
}

static void passive_turn(double u_in, double v_in, double turn_angle, double *u_out, double *v_out)
{
    /* geodesy.c:206-223: the active turn by -turn_angle */
    const double a = -turn_angle;
    *u_out = cos(a) * u_in - sin(a) * v_in;
    *v_out = sin(a) * u_in + cos(a) * v_in;
}

static int find_min_index(const double *v, int n)
{
    /* index_helpers.c:13-28: first index of the minimum */
    int r = 0;
    double cur = v[0];
    for (int i = 1; i < n; ++i)
        if (v[i] < cur) {
            cur = v[i];
            r = i;
        }
    return r;
}

int orc_calc_uv_at_edge(const orc_grid *g, const double *in, double *u, double *v)
{
    /* averaging.c:152-174 */
    ORC_PAR
    for (long i = 0; i < (long)NL * NE; ++i) {
        long layer = i / NE, h = i - layer * NE;
        double w0 = in[NC + layer * VPL + h];
        double w1 = tangential_wind(g, in, layer, h);
        passive_turn(w0, w1, -g->direction[h], &u[NC + layer * VPL + h], &v[NC + layer * VPL + h]);
    }
    return 0;
}

int orc_curl_field_to_cells(const orc_grid *g, const double *in, double *out)
{
    /* averaging.c:176-204 */
    ORC_PAR
    for (long i = 0; i < NS; ++i) {
        long layer = i / NC, h = i - layer * NC;
        out[i] = 0;
        int n_edges = h < N_PENT ? 5 : 6;
        for (int j = 0; j < n_edges; ++j)
            out[i] += 0.5 * g->ipw[8 * i + j] * in[NE + layer * 2 * NE + g->adj[6 * h + j]];
    }
    return 0;
}

int orc_edges_to_cells(const orc_grid *g, const double *in, double *out)
{
    /* averaging.c:206-234 */
    ORC_PAR
    for (long i = 0; i < NS; ++i) {
        long layer = i / NC, h = i - layer * NC;
        out[i] = 0;
        int n_edges = h < N_PENT ? 5 : 6;
        for (int j = 0; j < n_edges; ++j)
            out[i] += 0.5 * g->ipw[8 * i + j] * in[NC + layer * VPL + g->adj[6 * h + j]];
    }
    return 0;
}

int orc_edges_to_cells_lowest_layer(const orc_grid *g, const double *in, double *out)
{
    /* spatial_ops_for_output.c:199-225 */
    ORC_PAR
    for (long i = 0; i < NC; ++i) {
        out[i] = 0;
        int n_edges = i < N_PENT ? 5 : 6;
        for (int j = 0; j < n_edges; ++j)
            out[i] += 0.5 * g->ipw[8 * (NS - NC + i) + j] * in[g->adj[6 * i + j]];
    }
    return 0;
}

int orc_inner_product_tangential(const orc_grid *g, const double *in0, const double *in1, double *out)
{
    /* spatial_ops_for_output.c:137-166: all six edge slots, also for
     * pentagons (whose sixth slot has weight 0) */
    ORC_PAR
    for (long i = 0; i < NS; ++i) {
        long layer = i / NC, h = i - layer * NC;
        out[i] = 0;
        for (int j = 0; j < 6; ++j) {
            double tw = tangential_wind(g, in1, layer, g->adj[6 * h + j]);
            out[i] += g->ipw[8 * i + j] * in0[NC + layer * VPL + g->adj[6 * h + j]] * tw;
        }
        out[i] += g->ipw[8 * i + 6] * in0[h + layer * VPL] * in1[h + layer * VPL];
        out[i] += g->ipw[8 * i + 7] * in0[h + (layer + 1) * VPL] * in1[h + (layer + 1) * VPL];
    }
    return 0;
}

int orc_epv_diagnostics(const orc_grid *g, const double *pot_vort, orc_state *s, double *epv)
{
    /* spatial_ops_for_output.c:17-135 */
    /* zero-initialised like the reference's calloc: the gradient leaves the
     * surface and top levels of its output untouched */
    double *pv = calloc((size_t)NV, sizeof(double)), *grad_pt = calloc((size_t)NV, sizeof(double));
    if (!pv || !grad_pt) {
        free(pv);
        free(grad_pt);
        return -1;
    }
    const double *zv = g->z_vector;
    ORC_PAR
    for (long i = 0; i < NV; ++i) {
        long layer = i / VPL, h = i - layer * VPL;
        if (h >= NC) {
            long e = h - NC, f = g->from[e], t = g->to[e];
            double lt = 0.5 * (zv[layer * VPL + f] + zv[layer * VPL + t])
                        - 0.5 * (zv[(layer + 1) * VPL + f] + zv[(layer + 1) * VPL + t]);
            double upper, lower;
            if (layer == 0) upper = (0.5 * (zv[layer * VPL + f] + zv[layer * VPL + t]) - zv[i]) / lt;
            else upper = 0.5 * (zv[i - VPL] - zv[i]) / lt;
            if (layer == NL - 1) lower = (zv[i] - 0.5 * (zv[(layer + 1) * VPL + f] + zv[(layer + 1) * VPL + t])) / lt;
            else lower = 0.5 * (zv[i] - zv[i + VPL]) / lt;
            pv[i] = upper * pot_vort[layer * 2 * NE + e] + lower * pot_vort[(layer + 1) * 2 * NE + e];
        } else {
            pv[i] = 0;
            if (layer == 0) {
                for (int j = 0; j < 6; ++j)
                    pv[i] += 0.5 * g->ipw[8 * h + j] * pot_vort[NE + layer * 2 * NE + g->adj[6 * h + j]];
            } else if (layer == NL) {
                long si = (long)(NL - 1) * NC + h;
                for (int j = 0; j < 6; ++j)
                    pv[i] += 0.5 * g->ipw[8 * si + j] * pot_vort[NE + (layer - 1) * 2 * NE + g->adj[6 * h + j]];
            } else {
                long su = (layer - 1) * NC + h, sl = layer * NC + h;
                for (int j = 0; j < 6; ++j)
                    pv[i] += 0.25 * g->ipw[8 * su + j] * pot_vort[NE + (layer - 1) * 2 * NE + g->adj[6 * h + j]];
                for (int j = 0; j < 6; ++j)
                    pv[i] += 0.25 * g->ipw[8 * sl + j] * pot_vort[NE + layer * 2 * NE + g->adj[6 * h + j]];
            }
        }
    }
    /* the gradient of theta_v' with the background added in the top layer
     * only (:113-122) */
    for (long i = 0; i < NC; ++i) s->theta_v_pert[i] += g->theta_v_bg[i];
    orc_grad(g, s->theta_v_pert, grad_pt);
    for (long i = 0; i < NC; ++i) s->theta_v_pert[i] -= g->theta_v_bg[i];
    orc_inner_product_tangential(g, pv, grad_pt, epv);
    free(pv);
    free(grad_pt);
    return 0;
}

int orc_interpolate_to_ll(const orc_grid *g, const double *in, double *out)
{
    /* spatial_ops_for_output.c:168-197 */
    ORC_PAR
    for (long i = 0; i < g->n_latlon; ++i) {
        out[i] = 0;
        for (int j = 0; j < 5; ++j) {
            double v = in[g->latlon_indices[5 * i + j]];
            if (v != 9999) {
                out[i] += g->latlon_weights[5 * i + j] * v;
            } else {
                out[i] = 9999;
                break;
            }
        }
    }
    return 0;
}

static double rel_humidity(double abs_humidity, double temperature)
{
    /* derived_quantities.c:63-81 */
    double vapour_pressure = abs_humidity * R_V * temperature;
    double saturation_pressure = 0.0;
    if (temperature > T_0) saturation_pressure = saturation_pressure_over_water(temperature);
    if (temperature <= T_0) saturation_pressure = saturation_pressure_over_ice(temperature);
    return vapour_pressure / saturation_pressure;
}

static double pseudopotential_temperature(const orc_grid *g, const orc_state *s, const orc_diag *d, long i)
{
    /* write_output.c:1680-1736 (Bolton 1980 in the moist case) */
    if (!g->moisture_on) return g->theta_v_bg[i] + s->theta_v_pert[i];
    const double T = d->temperature[i];
    double r = s->rho[(COND + 1) * NS + i] / (s->rho[COND * NS + i] - s->rho[(COND + 1) * NS + i]);
    double alpha_1 = 0.2854 * (1.0 - 0.28e-3 * r);
    double alpha_3 = r * (1.0 + 0.81e-3 * r);
    double pressure = P_0 * pow(g->exner_bg[i] + s->exner_pert[i], C_D_P / R_D);
    double saturation_pressure;
    if (T >= T_0) saturation_pressure = saturation_pressure_over_water(T);
    else saturation_pressure = saturation_pressure_over_ice(T);
    double vapour_pressure = s->rho[(COND + 1) * NS + i] * R_V * T;
    double rel_hum = vapour_pressure / saturation_pressure;
    double t_lcl = 1.0 / (1.0 / (T - 55.0) - log(rel_hum) / 2840.0) + 55.0;
    double alpha_2 = 3.376 / t_lcl - 0.00254;
    return T * pow(P_0 / pressure, alpha_1) * exp(alpha_2 * alpha_3);
}

/* wind speed at a height above the surface by linear inter-/extrapolation of
 * sqrt(v_squared) between the two layers nearest to it (write_output.c:310-340) */
static double speed_at_height(const orc_grid *g, const double *v_squared, long i, double height)
{
    const double *zs = g->z_scalar, *zv = g->z_vector;
    double vtm[ORC_MAX_L];
    for (int j = 0; j < NL; ++j) vtm[j] = fabs(zs[j * NC + i] - (zv[NV - NC + i] + height));
    int closest = find_min_index(vtm, NL);
    int second = closest - 1;
    if (closest < NL - 1 && zs[closest * NC + i] - zv[NV - NC + i] > height) second = closest + 1;
    return pow(v_squared[i + closest * NC], 0.5)
           + (pow(v_squared[i + closest * NC], 0.5) - pow(v_squared[i + second * NC], 0.5))
                 / (zs[i + closest * NC] - zs[i + second * NC]) * (zv[NV - NC + i] + height - zs[i + closest * NC]);
}

int orc_write_out_fields(const orc_grid *g, orc_state *s, const double *temperature_soil, const double *wind_lowest,
                         int n_wind_steps, orc_diag *d, const double *sfc_sw_in, const orc_config *c, orc_output *o)
{
    const double *zs = g->z_scalar, *zv = g->z_vector;
    orc_temperature_diagnostics(g, s, d);
    /* surface fields (:90-211) */
    const double lapse = 0.0065, z_tropopause = 12e3;
    const double min_precip_rate = 0.01 / (1000.0 * 3600.0 / 1024.0);
    ORC_PAR
    for (long i = 0; i < NC; ++i) {
        const long lo = (long)(NL - 1) * NC + i;
        double t_low = d->temperature[lo];
        double rgas = gas_constant_diagnostics(g, s, lo);
        double p = s->rho[COND * NS + lo] * rgas * t_low;
        double gm = g->gravity_m[(NL - 1) * VPL + i];
        double t_mslp = t_low + lapse * zs[lo];
        o->mslp[i] = p / pow(1 - (t_mslp - t_low) / t_mslp, gm / (rgas * lapse));
        double t_sfc = t_low + lapse * (zs[lo] - zv[NV - NC + i]);
        o->surface_p[i] = p / pow(1.0 - (t_sfc - t_low) / t_sfc, gm / (rgas * lapse));
        /* 2 m temperature */
        double vtm[ORC_MAX_L];
        for (int j = 0; j < NL; ++j) vtm[j] = fabs(zv[(long)NL * VPL + i] + 2 - zs[i + j * NC]);
        int closest = find_min_index(vtm, NL);
        double temp_closest = d->temperature[closest * NC + i];
        double delta_z_temp = zv[(long)NL * VPL + i] + 2 - zs[i + closest * NC];
        double gradient;
        if (c->prog_soil_temp == 1) {
            gradient = (temp_closest - temperature_soil[i]) / (zs[i + closest * NC] - zv[(long)NL * VPL + i]);
        } else {
            int second = closest - 1;
            if (zs[i + closest * NC] > zv[(long)NL * VPL + i] + 2 && closest < NL - 1) second = closest + 1;
            gradient = (temp_closest - d->temperature[second * NC + i]) / (zs[i + closest * NC] - zs[i + second * NC]);
        }
        o->t2[i] = temp_closest + delta_z_temp * gradient;
        /* CAPE; stops at the top layer where the reference would read above
         * the model top (a model top below the tropopause) */
        o->cape[i] = 0.0;
        int layer = NL - 1;
        double z_height = zs[layer * NC + i];
        double theta_e = pseudopotential_temperature(g, s, d, layer * NC + i);
        while (z_height < z_tropopause) {
            double theta_v = g->theta_v_bg[layer * NC + i] + s->theta_v_pert[layer * NC + i];
            double delta_z = g->layer_thickness[layer * NC + i];
            double integrand = g->gravity_m[layer * VPL + i] * (theta_e - theta_v) / theta_v;
            if (integrand > 0.0) o->cape[i] += integrand * delta_z;
            --layer;
            if (layer < 0) break;
            z_height = zs[layer * NC + i];
        }
        o->sfc_sw_down[i] = sfc_sw_in[i] / (1.0 - g->sfc_albedo[i] + EPSILON_SECURITY);
        if (COND == 4) {
            double cwc = 0.0;
            for (int k = 0; k < NL; ++k)
                if (zs[k * NC + i] < z_tropopause)
                    cwc += (s->rho[2 * NS + k * NC + i] + s->rho[3 * NS + k * NC + i])
                           * (zv[i + k * VPL] - zv[i + (k + 1) * VPL]);
            o->tcdc[i] = fmin(10.0 * cwc, 1.0);
            o->tcdc[i] = 100.0 * o->tcdc[i];
            if (o->tcdc[i] < 0.5) o->tcdc[i] = 0.0;
        } else {
            o->tcdc[i] = 0.0;
        }
        o->sprate[i] = 0.0;
        if (COND == 4) o->sprate[i] = c->snow_velocity * s->rho[lo];
        o->rprate[i] = 0.0;
        if (COND == 4) o->rprate[i] = c->rain_velocity * s->rho[NS + lo];
        if (o->rprate[i] < min_precip_rate) o->rprate[i] = 0.0;
        if (o->sprate[i] < min_precip_rate) o->sprate[i] = 0.0;
    }
    /* 10 m wind (:213-292) */
    double *u = malloc((size_t)NE * sizeof(double)), *v = malloc((size_t)NE * sizeof(double));
    if (!u || !v) {
        free(u);
        free(v);
        return -1;
    }
    ORC_PAR
    for (long h = 0; h < NE; ++h) {
        double mu = 0.0, mv = 0.0;
        for (int t = 0; t < n_wind_steps; ++t) {
            double wt = 0.0;
            for (int k = 0; k < 10; ++k)
                wt += g->trsk_weights[10 * h + k] * wind_lowest[(long)t * NE + g->trsk_indices[10 * h + k]];
            mu += 1.0 / n_wind_steps * wind_lowest[(long)t * NE + h];
            mv += 1.0 / n_wind_steps * wt;
        }
        passive_turn(mu, mv, -g->direction[h], &u[h], &v[h]);
        long f = g->from[h], to = g->to[h];
        double actual = 0.5 * (g->roughness_length[f] + g->roughness_length[to]);
        double extrapolation = 0.02;
        if (g->is_land[f] == 0) extrapolation = actual;
        double z_sfc = 0.5 * (zv[NV - NC + f] + zv[NV - NC + to]);
        double z_agl = zv[NV - VPL + h] - z_sfc;
        double rescale = log(10.0 / extrapolation) / log(z_agl / actual);
        u[h] = rescale * u[h];
        v[h] = rescale * v[h];
    }
    orc_edges_to_cells_lowest_layer(g, u, o->u10);
    orc_edges_to_cells_lowest_layer(g, v, o->v10);
    free(u);
    free(v);
    /* gusts (:294-350).  The reference's loop shares its work array
     * vector_to_minimize between OpenMP threads, so with several threads its
     * result depends on the schedule; this is its one-thread result. */
    const double h850 = 8000.0 * log(1000.0 / 850.0), h950 = 8000.0 * log(1000.0 / 950.0);
    ORC_PAR
    for (long i = 0; i < NC; ++i) {
        double speed = pow(pow(o->u10[i], 2) + pow(o->v10[i], 2), 0.5);
        if ((c->sfc_sensible_heat_flux == 1 || c->sfc_phase_trans == 1 || c->pbl_scheme == 1)
            && fabs(d->monin_obukhov_length[i]) > EPSILON_SECURITY) {
            o->gusts[i] = speed + 7.71 * d->roughness_velocity[i]
                                      * pow(fmax(1.0 - 0.5 / 12.0 * 1000.0 / d->monin_obukhov_length[i], 0.0), 1.0 / 3.0);
            double u850 = speed_at_height(g, d->v_squared, i, h850);
            double u950 = speed_at_height(g, d->v_squared, i, h950);
            o->gusts[i] += 0.6 * fmax(0.0, u850 - u950);
            o->gusts[i] = fmin(o->gusts[i], 3.0 * speed);
        } else {
            o->gusts[i] = 1.67 * speed;
        }
    }
    /* model-layer fields (:718-749) */
    orc_divv_h(g, s->wind, o->divv_h);
    orc_calc_rel_vort(g, s->wind, d);
    orc_curl_field_to_cells(g, d->rel_vort, o->rel_vort);
    orc_calc_uv_at_edge(g, s->wind, d->u_at_edge, d->v_at_edge);
    orc_edges_to_cells(g, d->u_at_edge, d->u_at_cell);
    orc_edges_to_cells(g, d->v_at_edge, d->v_at_cell);
    ORC_PAR
    for (long i = 0; i < NS; ++i) {
        if (g->n_const >= 4) o->rh[i] = 100.0 * rel_humidity(s->rho[(COND + 1) * NS + i], d->temperature[i]);
        else o->rh[i] = 0.0;
        o->pressure[i] = s->rho[COND * NS + i] * gas_constant_diagnostics(g, s, i) * d->temperature[i];
    }
    ORC_PAR
    for (long i = 0; i < NS; ++i) d->scalar_field_placeholder[i] = s->rho[COND * NS + i];
    orc_calc_pot_vort(g, s->wind, d->scalar_field_placeholder, d);
    if (orc_epv_diagnostics(g, d->pot_vort, s, o->epv)) return -1;
    /* pressure levels (:751-826) */
    static const double levels[ORC_N_PRESSURE_LEVELS] = {20000, 30000, 50000, 70000, 85000, 92500};
    ORC_PAR
    for (long i = 0; i < NC; ++i) {
        double vtm[ORC_MAX_L];
        for (int j = 0; j < ORC_N_PRESSURE_LEVELS; ++j) {
            for (int k = 0; k < NL; ++k) vtm[k] = fabs(log(levels[j] / o->pressure[k * NC + i]));
            int closest = find_min_index(vtm, NL);
            int second = closest + 1;
            if (levels[j] < o->pressure[closest * NC + i]) second = closest - 1;
            long k = i * ORC_N_PRESSURE_LEVELS + j;
            if ((closest == NL - 1 && second == NL) || (closest < 0 || second < 0)) {
                o->geopotential_height[k] = o->t_pl[k] = o->rh_pl[k] = o->epv_pl[k] = 9999;
                o->rel_vort_pl[k] = o->u_pl[k] = o->v_pl[k] = 9999;
            } else {
                long a = closest * NC + i, b = second * NC + i;
                double w = 1 - vtm[closest] / (fabs(log(o->pressure[a] / o->pressure[b])) + EPSILON_SECURITY);
                o->geopotential_height[k] = w * g->gravity_potential[a] + (1 - w) * g->gravity_potential[b];
                o->geopotential_height[k] = o->geopotential_height[k] / G_MEAN_SFC_ABS;
                o->t_pl[k] = w * d->temperature[a] + (1 - w) * d->temperature[b];
                o->rh_pl[k] = w * o->rh[a] + (1 - w) * o->rh[b];
                o->epv_pl[k] = w * o->epv[a] + (1 - w) * o->epv[b];
                o->rel_vort_pl[k] = w * o->rel_vort[a] + (1 - w) * o->rel_vort[b];
                o->u_pl[k] = w * d->u_at_cell[a] + (1 - w) * d->u_at_cell[b];
                o->v_pl[k] = w * d->v_at_cell[a] + (1 - w) * d->v_at_cell[b];
            }
        }
    }
    return 0;
}
