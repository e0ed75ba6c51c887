/*
 * Device-resident grid tables and fields of the RKHEVI step.
 *
 * Layout in HBM (all arrays structure-of-arrays, renumbered along a 3-D
 * Hilbert curve so that neighbour gathers stay local; the 12 pentagons keep
 * cell numbers 0..11):
 *   cell fields       [layer][cell]          (Nc fastest)
 *   interface fields  [level][cell]          (w, vertical metric, L+1 levels)
 *   edge fields       [layer][edge]          (u, horizontal metric)
 *   tangential curl   [level][edge]          (L+1 levels)
 *   rhombus curl      [layer][edge]
 *   triangle fields   [layer][triangle]
 *   per-entity tables [slot][entity]         (slot-major, e.g. TRSK [10][Ne])
 * so a warp's 32 consecutive threads read 32 consecutive entities of one
 * layer: every streamed field access is coalesced.
 */
#pragma once

#include <cstdint>

namespace game {

constexpr int N_PENT = 12;

/* physical constants of GAME (src/game_constants.h:10-27) */
constexpr double T_0 = 273.15;
constexpr double N_A = 6.02214076e23;
constexpr double P_0 = 100000.0;
constexpr double C_D_V = 717.942189;
constexpr double C_V_V = 1396.475121;
constexpr double C_D_P = 1005.0;
constexpr double M_D = N_A * 0.004810e-23;
constexpr double M_V = N_A * 0.002991e-23;
constexpr double R_D = 287.057811;
constexpr double R_V = 461.524879;

/* horizontal-operator tables, element type R (double on the FP64 path,
 * float on the mixed path) */
template <typename R>
struct HGrid {
    int nc, ne, nt, nl, n_oro;
    R radius;
    /* cells */
    const R *volume;        /* [L][Nc] */
    const R *theta_v_bg;    /* [L][Nc] background virtual potential temperature */
    const R *exner_bg;      /* [L][Nc] background Exner pressure */
    const R *ipw;           /* [8][L][Nc] inner-product weights */
    const int *adj;         /* [6][Nc] edges of the cell, reference order */
    const int *adj_sign;    /* [6][Nc] +1 cell is the edge's from cell, -1 to cell, 0 none */
    const int *adj_nbr;     /* [6][Nc] cell on the other side of edge j */
    const int *tilt;        /* [Nc] 1 where an edge of the cell has a nonzero slope in some layer */
    /* interfaces */
    const R *nd_v;          /* [L+1][Nc] vertical normal distance */
    const R *area_v;        /* [L+1][Nc] */
    const R *exner_bg_grad_v; /* [L+1][Nc] */
    const R *gravity_m_v;   /* [L+1][Nc] */
    /* edges */
    const int *from, *to;   /* [Ne] */
    const R *nd_h;          /* [L][Ne] */
    const R *area_h;        /* [L][Ne] */
    const R *z_h;           /* [L][Ne] */
    const R *slope_h;       /* [L][Ne] */
    const R *exner_bg_grad_h; /* [L][Ne] */
    const R *trsk_w;        /* [10][Ne] */
    const int *trsk_i;      /* [10][Ne] */
    const int *trsk_m;      /* [10][Ne] modified curl indices */
    const R *rhombi_w;      /* [4][Ne] */
    const int *rhombi_i;    /* [4][Ne] */
    const R *f_vec;         /* [2][Ne] */
    const int *dual_from, *dual_to; /* [Ne] */
    const R *dual_area_h;   /* [L+1][Ne] */
    const R *pvz;           /* [4][Ne] height differences of the TOA/surface density extrapolation */
    /* triangles */
    const int *vort_i;      /* [3][Nt] */
    const int *vort_s;      /* [3][Nt] */
    const R *dual_area_t;   /* [L][Nt] */
    const R *dual_z_t;      /* [L][Nt] */
};

/* device tables of the output pass, built at initialisation (device order
 * unless stated) */
struct OutGrid {
    const double *direction;        /* [Ne] */
    const double *roughness_length; /* [Nc] */
    const double *sfc_albedo;       /* [Nc] */
    const int *is_land;             /* [Nc] */
    const int *c_n2o;               /* [Nc] device cell -> reference cell */
    const int *e_n2o;               /* [Ne] device edge -> reference edge */
    const int *ll_idx;              /* [5][N_ll] device cells of each lat-lon point (lat-lon order) */
    const double *ll_w;             /* [5][N_ll] */
    long long n_ll;
    int ll_ok;                      /* the caller's lat-lon indices were all in range */
};

/* vertical-solver tables (always double) */
struct VGrid {
    int nc, nl;
    const double *volume, *z_scalar, *exner_bg, *theta_v_bg; /* [L][Nc] */
    const double *area_v, *z_v;                             /* [L+1][Nc] */
};

/* one State in device layout (always double: the prognostic variables) */
struct DState {
    double *rho;          /* [C][L][Nc] */
    double *rhotheta_v;   /* [L][Nc] */
    double *theta_v_pert; /* [L][Nc] */
    double *exner_pert;   /* [L][Nc] */
    double *w;            /* [L+1][Nc] */
    double *u;            /* [L][Ne] */
};

/* read view of the state in the horizontal precision R: the FP64 state itself
 * on the FP64 path, its FP32 shadow on the mixed path */
template <typename R>
struct SView {
    const R *rho, *rhotheta_v, *theta_v_pert, *exner_pert, *w, *u;
};

/* double-float copies (hi, lo) of vertical-solver tables, for the mixed
 * path's double-float eliminations */
struct DfGrid {
    const float2 *area_v;     /* [L+1][Nc] */
    const float2 *inv_area_v; /* [L+1][Nc] (0 where the area is 0) */
    const float2 *inv_vol;    /* [L][Nc] */
    const float2 *volume;     /* [L][Nc] */
    const float2 *exner_bg;   /* [L][Nc] */
    const float2 *theta_v_bg; /* [L][Nc] */
    /* grid terms of the sound-wave rows [6][L-1][Nc] (as the FP64 table
     * wv_geo: dz, H, G1, G2, Cz, Ez) */
    const float2 *geo;
    /* 1 / (1 + dt * Klemp coefficient) of the inner interfaces [L-1][Nc],
     * for the time step the damping table was last made for */
    const float2 *damp_inv;
};

/* FP32 shadow of state_new (mixed path); kernels that write the FP64 state
 * also write the shadow.  All pointers null on the FP64 path. */
struct Shadow {
    float *rho, *rhotheta_v, *theta_v_pert, *exner_pert, *w, *u;
};

/* run configuration of one step (no padding: compared bytewise as a key) */
struct StepParams {
    int n_const, n_cond, moist, first_step;
    /* diffusion switches (DIFF_* bits) and whether the step adds the
     * irreversible terms (friction, dissipative and diffusive heating,
     * radiation, mass diffusion) to its tendencies; dfloat: the mixed path's
     * vertical eliminations run in double-float arithmetic (dfloat.cuh)
     * instead of FP64 */
    int diff, irr, dfloat, pad_i1;
    double dt;
    double impl_thermo_weight, damping_start_height, damping_coeff_max, toa;
    double snow_velocity, rain_velocity, cloud_velocity;
    /* derived on the host for the mixed path: 1/dt, 1/(w dt^2 c_p), 0.5/(w dt c_p)
     * with w the implicit thermodynamic weight */
    double inv_dt, k_rows, k_rows2;
    /* pressure-gradient weights of the momentum tendencies
     * (vector_tendencies_expl.c:79-83): 0.5 + w, 1 - (0.5 + w), 1 - w, in
     * double and rounded to float */
    double cur_hor, old_hor, cur_ver;
    float cur_hor_f, old_hor_f, cur_ver_f, pad_f;
};
static_assert(sizeof(StepParams) == 8 * sizeof(int) + 14 * sizeof(double) + 4 * sizeof(float),
              "StepParams has padding");

/* config switches of the diffusion branch (StepParams::diff) */
enum {
    DIFF_MOM_H = 1, DIFF_MOM_V = 2, DIFF_TEMP_H = 4, DIFF_TEMP_V = 8, DIFF_MASS_H = 16, DIFF_MASS_V = 32,
    /* Held-Suarez forcing: boundary-layer friction (pbl_scheme = 2) and the
     * radiation relaxation updated in this step (rad_on = 2, rad_update = 1) */
    DIFF_PBL_HS = 64, DIFF_RAD_HS = 128
};

/* tables of the diffusion branch in the horizontal precision R */
template <typename R>
struct DiffGrid {
    const R *layer_thickness; /* [L][Nc] */
    const R *dual_nd_t;       /* [L][Nt] vertical extent of the triangle prisms (dual normal distance) */
    const R *dual_nd_sfc;     /* [Ne] dual normal distance of the surface level's edges */
    const R *z_v;             /* [L+1][Nc] height of the interfaces */
    const R *z_scalar;        /* [L][Nc] height of the cell centres */
    const R *lat;             /* [Nc] latitude */
    const int *rad_cov;       /* [Nc] 1 where the reference's radiation blocks reach the cell */
    double eff_hor_res, mean_velocity_area;
};

/* fields of the diffusion branch, device layout.  Persistent between steps
 * (imported from and exported to the caller's structs): tke, visc (viscosity),
 * hdiss (heating_diss), fric (friction_acc, vector layout), mol
 * (molecular_diffusion_coeff), n2 (n_squared), mdt (mass_diff_tendency,
 * [C][L][Nc]), tdh (temperature_diffusion_heating), rad (radiation_tendency),
 * ph_tb (TOA and surface vertical entries of vector_field_placeholder,
 * [2][Nc]) and dvdz_top (TOA row of dv_hdz, [Ne]).  The rest is scratch of
 * one step. */
struct DiffBufs {
    double *tke, *visc, *hdiss, *fric, *mol, *n2, *mdt, *tdh, *rad, *ph_tb, *dvdz_top;
    double *adv, *vint, *wdv, *tri, *zt, *zr, *s1, *s2, *s3, *flx;
    double *mch, *mcv, *tch, *tcv; /* mass / temperature diffusion coefficients, h and v */
    double *fh, *fv;               /* diffusive fluxes of T and the C densities: [C+1][L][Ne], [C+1][L+1][Nc] */
    double *kvt;                   /* turbulent vertical diffusivity of the cells [L][Nc] */
    double *hs_p, *hs_ps;          /* Held-Suarez boundary layer: pressure [L][Nc], surface pressure [Nc] */
};

/* the scratch part of DiffBufs in precision R (on the mixed path the double
 * allocations hold float arrays of the same length) */
template <typename R>
struct DiffScratch {
    R *adv, *vint, *wdv, *tri, *zt, *zr, *s1, *s2, *s3, *flx, *mch, *mcv, *tch, *tcv, *fh, *fv, *kvt, *hs_p, *hs_ps;
};
template <typename R>
inline DiffScratch<R> diff_scratch(const DiffBufs &b)
{
    return {(R *)b.adv, (R *)b.vint, (R *)b.wdv, (R *)b.tri, (R *)b.zt, (R *)b.zr, (R *)b.s1, (R *)b.s2,
            (R *)b.s3, (R *)b.flx, (R *)b.mch, (R *)b.mcv, (R *)b.tch, (R *)b.tcv, (R *)b.fh, (R *)b.fv,
            (R *)b.kvt, (R *)b.hs_p, (R *)b.hs_ps};
}

}  // namespace game
