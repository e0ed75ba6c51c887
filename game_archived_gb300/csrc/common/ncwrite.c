/* netCDF classic writer (see ncwrite.h). */
#include "ncwrite.h"

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define NCW_MAX_DIMS 32
#define NCW_MAX_VARS 96
#define NCW_NAME 128

enum { NC_DIMENSION = 10, NC_VARIABLE = 11, NC_ATTRIBUTE = 12, NC_CHAR = 2, NC_DOUBLE = 6 };

typedef struct {
    char name[NCW_NAME];
    long long len;
} ncw_dim;

typedef struct {
    char name[NCW_NAME];
    char units[NCW_NAME];
    int has_units, ndims, dimids[NCW_MAX_DIMS];
    long long n;             /* values */
    const double *values;
    long long begin;
} ncw_var;

struct ncw_file {
    int n_dims, n_vars;
    ncw_dim dims[NCW_MAX_DIMS];
    ncw_var vars[NCW_MAX_VARS];
};

static char g_err[256];
const char *ncw_last_error(void) { return g_err; }

ncw_file *ncw_create(void) { return calloc(1, sizeof(ncw_file)); }
void ncw_free(ncw_file *f) { free(f); }

int ncw_def_dim(ncw_file *f, const char *name, long long len)
{
    if (f->n_dims == NCW_MAX_DIMS || strlen(name) >= NCW_NAME || len < 0) return -1;
    ncw_dim *d = &f->dims[f->n_dims];
    strcpy(d->name, name);
    d->len = len;
    return f->n_dims++;
}

int ncw_def_var(ncw_file *f, const char *name, int ndims, const int *dimids, const char *units)
{
    if (f->n_vars == NCW_MAX_VARS || strlen(name) >= NCW_NAME || ndims < 0 || ndims > NCW_MAX_DIMS) return -1;
    if (units && strlen(units) >= NCW_NAME) return -1;
    ncw_var *v = &f->vars[f->n_vars];
    memset(v, 0, sizeof *v);
    strcpy(v->name, name);
    if (units) {
        strcpy(v->units, units);
        v->has_units = 1;
    }
    v->ndims = ndims;
    v->n = 1;
    for (int i = 0; i < ndims; ++i) {
        if (dimids[i] < 0 || dimids[i] >= f->n_dims) return -1;
        v->dimids[i] = dimids[i];
        v->n *= f->dims[dimids[i]].len;
    }
    return f->n_vars++;
}

int ncw_put_var(ncw_file *f, int varid, const double *values)
{
    if (varid < 0 || varid >= f->n_vars) return -1;
    f->vars[varid].values = values;
    return 0;
}

/* ---------------------------------------------------------- header bytes */
typedef struct {
    unsigned char *p;
    size_t n, cap;
} buf;

static int put(buf *b, const void *src, size_t n)
{
    if (b->n + n > b->cap) {
        size_t cap = b->cap ? 2 * b->cap : 4096;
        while (cap < b->n + n) cap *= 2;
        unsigned char *q = realloc(b->p, cap);
        if (!q) return -1;
        b->p = q;
        b->cap = cap;
    }
    memcpy(b->p + b->n, src, n);
    b->n += n;
    return 0;
}

static int put_u32(buf *b, uint32_t x)
{
    unsigned char c[4] = {(unsigned char)(x >> 24), (unsigned char)(x >> 16), (unsigned char)(x >> 8), (unsigned char)x};
    return put(b, c, 4);
}

static int put_u64(buf *b, uint64_t x)
{
    return put_u32(b, (uint32_t)(x >> 32)) || put_u32(b, (uint32_t)x);
}

/* nelems, characters, zero padding to a multiple of 4 */
static int put_name(buf *b, const char *s)
{
    const size_t n = strlen(s);
    static const unsigned char zero[4] = {0, 0, 0, 0};
    return put_u32(b, (uint32_t)n) || put(b, s, n) || put(b, zero, (4 - n % 4) % 4);
}

static int header(const ncw_file *f, int version, buf *b)
{
    static const unsigned char magic[3] = {'C', 'D', 'F'};
    const unsigned char v = (unsigned char)version;
    if (put(b, magic, 3) || put(b, &v, 1) || put_u32(b, 0)) return -1; /* numrecs: no record dimension */
    if (f->n_dims) {
        if (put_u32(b, NC_DIMENSION) || put_u32(b, (uint32_t)f->n_dims)) return -1;
        for (int i = 0; i < f->n_dims; ++i)
            if (put_name(b, f->dims[i].name) || put_u32(b, (uint32_t)f->dims[i].len)) return -1;
    } else if (put_u32(b, 0) || put_u32(b, 0)) {
        return -1;
    }
    if (put_u32(b, 0) || put_u32(b, 0)) return -1; /* no global attributes */
    if (f->n_vars) {
        if (put_u32(b, NC_VARIABLE) || put_u32(b, (uint32_t)f->n_vars)) return -1;
        for (int i = 0; i < f->n_vars; ++i) {
            const ncw_var *v = &f->vars[i];
            if (put_name(b, v->name) || put_u32(b, (uint32_t)v->ndims)) return -1;
            for (int d = 0; d < v->ndims; ++d)
                if (put_u32(b, (uint32_t)v->dimids[d])) return -1;
            if (v->has_units) {
                static const unsigned char zero[4] = {0, 0, 0, 0};
                const size_t n = strlen(v->units);
                if (put_u32(b, NC_ATTRIBUTE) || put_u32(b, 1) || put_name(b, "units") || put_u32(b, NC_CHAR)
                    || put_u32(b, (uint32_t)n) || put(b, v->units, n) || put(b, zero, (4 - n % 4) % 4))
                    return -1;
            } else if (put_u32(b, 0) || put_u32(b, 0)) {
                return -1;
            }
            /* vsize: the bytes of the values (a multiple of 8), clamped as
             * the format prescribes for sizes that do not fit */
            const unsigned long long bytes = (unsigned long long)v->n * 8ull;
            const uint32_t vsize = bytes > 0xfffffffcull ? 0xffffffffu : (uint32_t)bytes;
            if (put_u32(b, NC_DOUBLE) || put_u32(b, vsize)) return -1;
            if (version == 1 ? put_u32(b, (uint32_t)v->begin) : put_u64(b, (uint64_t)v->begin)) return -1;
        }
    } else if (put_u32(b, 0) || put_u32(b, 0)) {
        return -1;
    }
    return 0;
}

/* the header size of a version: the offsets do not change its length */
static long long header_size(ncw_file *f, int version)
{
    buf b = {0};
    long long n = header(f, version, &b) ? -1 : (long long)b.n;
    free(b.p);
    return n;
}

int ncw_write(ncw_file *f, const char *path)
{
    for (int i = 0; i < f->n_vars; ++i)
        if (!f->vars[i].values) {
            snprintf(g_err, sizeof g_err, "variable %s has no values", f->vars[i].name);
            return -1;
        }
    int version = 1;
    long long total = 0;
    for (int pass = 0; pass < 2; ++pass) {
        long long at = header_size(f, version);
        if (at < 0) {
            snprintf(g_err, sizeof g_err, "out of memory");
            return -1;
        }
        for (int i = 0; i < f->n_vars; ++i) {
            f->vars[i].begin = at;
            at += f->vars[i].n * 8;
        }
        total = at;
        if (version == 1 && total > 0x7fffffffll) version = 2;
        else break;
    }
    buf h = {0};
    if (header(f, version, &h)) {
        free(h.p);
        snprintf(g_err, sizeof g_err, "out of memory");
        return -1;
    }
    FILE *fp = fopen(path, "wb");
    if (!fp) {
        free(h.p);
        snprintf(g_err, sizeof g_err, "cannot create %s", path);
        return -1;
    }
    int err = fwrite(h.p, 1, h.n, fp) != h.n;
    free(h.p);
    enum { CHUNK = 1 << 16 };
    unsigned char *out = malloc((size_t)CHUNK * 8);
    if (!out) err = 1;
    for (int i = 0; i < f->n_vars && !err; ++i) {
        const ncw_var *v = &f->vars[i];
        for (long long k0 = 0; k0 < v->n && !err; k0 += CHUNK) {
            const long long k1 = k0 + CHUNK < v->n ? k0 + CHUNK : v->n;
            for (long long k = k0; k < k1; ++k) {
                uint64_t x;
                memcpy(&x, &v->values[k], 8);
                unsigned char *o = out + (k - k0) * 8;
                for (int j = 0; j < 8; ++j) o[j] = (unsigned char)(x >> (56 - 8 * j));
            }
            err = fwrite(out, 8, (size_t)(k1 - k0), fp) != (size_t)(k1 - k0);
        }
    }
    free(out);
    if (fclose(fp)) err = 1;
    if (err) snprintf(g_err, sizeof g_err, "writing %s failed", path);
    (void)total;
    return err ? -1 : 0;
}

/* ------------------------------------------------------ write_out's files */
typedef struct {
    const char *name, *units;
    const double *values;
} ncw_field;

static int write_1d(const char *path, const char *dim, long long n, const ncw_field *fields, int n_fields)
{
    ncw_file *f = ncw_create();
    if (!f) return -1;
    int d = ncw_def_dim(f, dim, n), err = d < 0;
    for (int i = 0; i < n_fields && !err; ++i) {
        int v = ncw_def_var(f, fields[i].name, 1, &d, fields[i].units);
        err = v < 0 || ncw_put_var(f, v, fields[i].values);
    }
    if (!err) err = ncw_write(f, path);
    ncw_free(f);
    return err ? -1 : 0;
}

int ncw_write_surface(const char *path, const ncw_output *o)
{
    /* write_output.c:353-441 */
    const ncw_field fields[] = {
        {"mslp", "Pa", o->mslp}, {"surface_p", "Pa", o->surface_p}, {"t2", "K", o->t2}, {"tcdc", "%", o->tcdc},
        {"rprate", "kg/(m^2s)", o->rprate}, {"sprate", "kg/(m^2s)", o->sprate}, {"cape", "J/kg", o->cape},
        {"sfc_sw_down", "W/m^2", o->sfc_sw_down}, {"10u", "m/s", o->u10}, {"10v", "m/s", o->v10},
        {"10gusts", "m/s", o->gusts}};
    return write_1d(path, "scalar_index_h", o->n_cells, fields, (int)(sizeof fields / sizeof fields[0]));
}

int ncw_write_pressure_levels(const char *path, const ncw_output *o)
{
    /* write_output.c:829-907 */
    ncw_file *f = ncw_create();
    if (!f) return -1;
    const int dh = ncw_def_dim(f, "scalar_index_h", o->n_cells), dl = ncw_def_dim(f, "level_index", 6);
    const int d2[2] = {dh, dl};
    const ncw_field fields[] = {
        {"geopotential_height", "gpm", o->geopotential_height}, {"temperature", "K", o->t_pl},
        {"relative_humidity", "%", o->rh_pl}, {"ertels_potential_vorticity", "Km^2/(kgs)", o->epv_pl},
        {"wind_u", "m/s", o->u_pl}, {"wind_v", "m/s", o->v_pl}, {"relative_vorticity", "1/s", o->rel_vort_pl}};
    int v = ncw_def_var(f, "pressure_levels", 1, &dl, "Pa");
    int err = dh < 0 || dl < 0 || v < 0 || ncw_put_var(f, v, o->pressure_levels);
    for (size_t i = 0; i < sizeof fields / sizeof fields[0] && !err; ++i) {
        v = ncw_def_var(f, fields[i].name, 2, d2, fields[i].units);
        err = v < 0 || ncw_put_var(f, v, fields[i].values);
    }
    if (!err) err = ncw_write(f, path);
    ncw_free(f);
    return err ? -1 : 0;
}

int ncw_write_model_levels(const char *path, const ncw_output *o)
{
    /* write_output.c:1417-1513: every dimension of the reference's file,
     * used or not */
    ncw_file *f = ncw_create();
    if (!f) return -1;
    const int d_scalar = ncw_def_dim(f, "scalar_index", o->n_scalars);
    const int d_soil = ncw_def_dim(f, "soil_index", o->n_soil);
    const int d_vector = ncw_def_dim(f, "vector_index", o->n_vectors);
    const int d_dens = ncw_def_dim(f, "densities_index", o->n_densities);
    int err = ncw_def_dim(f, "vector_index_h", o->n_h_vectors) < 0 || ncw_def_dim(f, "vector_index_v", o->n_v_vectors) < 0
              || ncw_def_dim(f, "curl_point_index", o->n_curl) < 0 || ncw_def_dim(f, "single_double_dimid_index", 1) < 0;
    const struct {
        const char *name, *units;
        int dim;
        const double *values;
    } fields[] = {{"densities", "kg/m^3", d_dens, o->densities},
                  {"temperature", "K", d_scalar, o->temperature},
                  {"wind", "m/s", d_vector, o->wind},
                  {"rh", "%", d_scalar, o->rh},
                  {"rel_vort", "1/s", d_scalar, o->rel_vort},
                  {"divv_h_all_layers", "1/s", d_scalar, o->divv_h},
                  {"tke", "J/kg", d_scalar, o->tke},
                  {"t_soil", "K", d_soil, o->t_soil}};
    for (size_t i = 0; i < sizeof fields / sizeof fields[0] && !err; ++i) {
        const int v = ncw_def_var(f, fields[i].name, 1, &fields[i].dim, fields[i].units);
        err = fields[i].dim < 0 || v < 0 || ncw_put_var(f, v, fields[i].values);
    }
    if (!err) err = ncw_write(f, path);
    ncw_free(f);
    return err ? -1 : 0;
}
