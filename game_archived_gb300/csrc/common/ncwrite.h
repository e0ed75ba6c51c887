/*
 * A writer of netCDF classic files (the format the reference's output code
 * creates with nc_create(..., NC_CLOBBER, ...)): fixed-size dimensions,
 * double variables, one text attribute ("units") per variable, no record
 * dimension.  Written from the published format description ("The NetCDF
 * Classic Format Specification", Unidata): big-endian header of dimensions,
 * global attributes and variables with their offsets, then each variable's
 * values in definition order.  Files whose data end below 2^31 bytes use
 * the classic format (CDF-1); larger ones the 64-bit-offset format (CDF-2).
 */
#ifndef GAME_NCWRITE_H
#define GAME_NCWRITE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ncw_file ncw_file;

/* a new file description; nothing is written before ncw_write */
ncw_file *ncw_create(void);
/* returns the dimension id, or -1 */
int ncw_def_dim(ncw_file *f, const char *name, long long len);
/* a double variable over ndims dimensions (outermost first) with the text
 * attribute units (NULL: none); returns the variable id, or -1 */
int ncw_def_var(ncw_file *f, const char *name, int ndims, const int *dimids, const char *units);
/* the values of variable varid (not copied: they must stay valid until
 * ncw_write returns) */
int ncw_put_var(ncw_file *f, int varid, const double *values);
/* writes the file (every variable must have values); 0 on success */
int ncw_write(ncw_file *f, const char *path);
void ncw_free(ncw_file *f);
const char *ncw_last_error(void);

/* The three netCDF files the reference's write_out creates
 * (src/io/write_output.c:353-441, :829-907, :1417-1513), with its dimension
 * and variable names, shapes, units and order.  Every array is in the
 * reference's order; the pressure-level fields are [NO_OF_SCALARS_H][6]. */
typedef struct ncw_output {
    long long n_cells, n_scalars, n_vectors, n_densities, n_h_vectors, n_v_vectors, n_curl, n_soil;
    const double *mslp, *surface_p, *t2, *tcdc, *rprate, *sprate, *cape, *sfc_sw_down, *u10, *v10, *gusts;
    const double *pressure_levels; /* [6] */
    const double *geopotential_height, *t_pl, *rh_pl, *epv_pl, *u_pl, *v_pl, *rel_vort_pl;
    const double *densities, *temperature, *wind, *rh, *rel_vort, *divv_h, *tke, *t_soil;
} ncw_output;
int ncw_write_surface(const char *path, const ncw_output *o);
int ncw_write_pressure_levels(const char *path, const ncw_output *o);
int ncw_write_model_levels(const char *path, const ncw_output *o);

#ifdef __cplusplus
}
#endif
#endif
