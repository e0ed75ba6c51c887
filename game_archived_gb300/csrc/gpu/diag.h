/* global integrals and surface pressure on the device mirrors (diag_f64.cu) */
#pragma once

#include "context.h"

namespace game {

/* reduction launch shape: threads per block, at most 4 blocks per SM of a
 * 152-SM GB300, at most 8 fields per launch */
constexpr int INTEGRAL_THREADS = 256;
constexpr int INTEGRAL_MAX_BLOCKS = 608;
constexpr int INTEGRAL_MAX_FIELDS = 8;

/* blocks per field of a reduction over n points */
int integral_blocks(long long n);
/* out[k] = sum_i f[k*fstride + (map ? map[i] : i)] * w[i] for k < n_fields,
 * compensated; partials holds 2*INTEGRAL_MAX_BLOCKS doubles per field and
 * counters one unsigned per field, zero before the launch and zero again
 * after it */
int launch_integral(const double *f, long long fstride, int n_fields, long long n, const int *map, const double *w,
                    double *partials, unsigned *counters, double *out, cudaStream_t stream);
/* temperature_diagnostics of a mirror into t [L][Nc] */
int diag_temperature(Context *c, StateMirror *s, double *t);
/* e[0..3*ns): rho_g |v|^2, rho_g * gravity potential, rho_g * T */
int diag_energy_densities(Context *c, StateMirror *s, const double *temperature, double *e);
/* surface pressure and MSLP (nullable) per column, device cell order */
int diag_surface_pressure(Context *c, StateMirror *s, double *p_sfc, double *mslp);

}  // namespace game
