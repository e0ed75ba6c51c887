/*
 * Test-infrastructure definitions of the netCDF and ecCodes calls made by the
 * reference's output code (src/io/write_output.c), linked into the reference
 * harness in place of the two libraries, which are not installed here.
 *
 * No file is written.  Every array the reference hands to nc_put_var_double
 * or nc_put_var_int (its output fields on the native grid, the grid
 * generator's tables) and every array it sets as the
 * "values" of a GRIB message (the same fields interpolated to the lat-lon
 * grid) is copied into an in-memory list together with what identifies it:
 * the output file name and the variable name (netCDF), or the file name and
 * the message's parameterCategory, parameterNumber, typeOfFirstFixedSurface
 * and level keys (GRIB).  ref_io_count / ref_io_record read the list back.
 */
#include <stdlib.h>
#include <string.h>

#include "ref_stubs/eccodes.h"
#include "ref_stubs/netcdf.h"

typedef struct {
    char file[320];
    char name[64];
    long category, number, surface_type, level;
    long n;
    double *data;
} io_record;

static io_record *g_rec;
static int g_n_rec, g_cap_rec;

static io_record *new_record(const char *file, const char *name, const double *data, long n)
{
    if (g_n_rec == g_cap_rec) {
        int cap = g_cap_rec ? 2 * g_cap_rec : 64;
        io_record *grown = realloc(g_rec, (size_t)cap * sizeof(io_record));
        if (!grown) abort();
        g_rec = grown;
        g_cap_rec = cap;
    }
    io_record *r = &g_rec[g_n_rec++];
    memset(r, 0, sizeof *r);
    strncpy(r->file, file, sizeof r->file - 1);
    strncpy(r->name, name, sizeof r->name - 1);
    r->category = r->number = r->surface_type = r->level = -1;
    r->n = n;
    r->data = malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
    if (!r->data) abort();
    memcpy(r->data, data, (size_t)n * sizeof(double));
    return r;
}

void ref_io_reset(void)
{
    for (int i = 0; i < g_n_rec; ++i) free(g_rec[i].data);
    g_n_rec = 0;
}

int ref_io_count(void) { return g_n_rec; }

int ref_io_record(int k, const char **file, const char **name, long *meta, long *n, const double **data)
{
    if (k < 0 || k >= g_n_rec) return 1;
    io_record *r = &g_rec[k];
    *file = r->file;
    *name = r->name;
    meta[0] = r->category;
    meta[1] = r->number;
    meta[2] = r->surface_type;
    meta[3] = r->level;
    *n = r->n;
    *data = r->data;
    return 0;
}

/* ------------------------------------------------- netCDF file structure
 * Every dimension and variable definition, in call order: kind 'D' with the
 * dimension's length, or 'V' with its dimensions' names joined by commas and
 * the "units" attribute given to it. */
typedef struct {
    char file[320];
    char kind;
    char name[64];
    char dims[256];
    char units[64];
    long long len;
} nc_def_record;

static nc_def_record *g_def;
static int g_n_def, g_cap_def;

static nc_def_record *new_def(void)
{
    if (g_n_def == g_cap_def) {
        int cap = g_cap_def ? 2 * g_cap_def : 64;
        nc_def_record *grown = realloc(g_def, (size_t)cap * sizeof(nc_def_record));
        if (!grown) abort();
        g_def = grown;
        g_cap_def = cap;
    }
    nc_def_record *r = &g_def[g_n_def++];
    memset(r, 0, sizeof *r);
    return r;
}

int ref_nc_def_count(void) { return g_n_def; }
void ref_nc_def_reset(void) { g_n_def = 0; }

int ref_nc_def_get(int k, const char **file, char *kind, const char **name, const char **dims, const char **units,
                   long long *len)
{
    if (k < 0 || k >= g_n_def) return 1;
    *file = g_def[k].file;
    *kind = g_def[k].kind;
    *name = g_def[k].name;
    *dims = g_def[k].dims;
    *units = g_def[k].units;
    *len = g_def[k].len;
    return 0;
}

/* ------------------------------------------------------------------ netCDF */
#define NC_MAX_FILES 8
#define NC_MAX_DIMS 32
#define NC_MAX_VARS 96

static struct {
    int open;
    char path[320];
    int n_dims, n_vars;
    size_t dim_len[NC_MAX_DIMS];
    char dim_name[NC_MAX_DIMS][64];
    int var_def[NC_MAX_VARS]; /* index of the variable's definition record */
    char var_name[NC_MAX_VARS][64];
    long var_len[NC_MAX_VARS];
} g_nc[NC_MAX_FILES];

int nc_create(const char *path, int cmode, int *ncidp)
{
    (void)cmode;
    for (int i = 0; i < NC_MAX_FILES; ++i)
        if (!g_nc[i].open) {
            memset(&g_nc[i], 0, sizeof g_nc[i]);
            g_nc[i].open = 1;
            strncpy(g_nc[i].path, path, sizeof g_nc[i].path - 1);
            *ncidp = i;
            return 0;
        }
    return 1;
}

int nc_def_dim(int ncid, const char *name, size_t len, int *idp)
{
    if (ncid < 0 || ncid >= NC_MAX_FILES || g_nc[ncid].n_dims == NC_MAX_DIMS) return 1;
    g_nc[ncid].dim_len[g_nc[ncid].n_dims] = len;
    strncpy(g_nc[ncid].dim_name[g_nc[ncid].n_dims], name, 63);
    nc_def_record *r = new_def();
    strncpy(r->file, g_nc[ncid].path, sizeof r->file - 1);
    r->kind = 'D';
    strncpy(r->name, name, sizeof r->name - 1);
    r->len = (long long)len;
    *idp = g_nc[ncid].n_dims++;
    return 0;
}

int nc_def_var(int ncid, const char *name, nc_type xtype, int ndims, const int *dimidsp, int *varidp)
{
    (void)xtype;
    if (ncid < 0 || ncid >= NC_MAX_FILES || g_nc[ncid].n_vars == NC_MAX_VARS) return 1;
    int v = g_nc[ncid].n_vars++;
    strncpy(g_nc[ncid].var_name[v], name, 63);
    long len = 1;
    nc_def_record *r = new_def();
    strncpy(r->file, g_nc[ncid].path, sizeof r->file - 1);
    r->kind = 'V';
    strncpy(r->name, name, sizeof r->name - 1);
    for (int d = 0; d < ndims; ++d) {
        len *= (long)g_nc[ncid].dim_len[dimidsp[d]];
        if (d) strncat(r->dims, ",", sizeof r->dims - strlen(r->dims) - 1);
        strncat(r->dims, g_nc[ncid].dim_name[dimidsp[d]], sizeof r->dims - strlen(r->dims) - 1);
    }
    r->len = len;
    g_nc[ncid].var_def[v] = g_n_def - 1;
    g_nc[ncid].var_len[v] = len;
    *varidp = v;
    return 0;
}

int nc_put_att_text(int ncid, int varid, const char *name, size_t len, const char *op)
{
    if (ncid < 0 || ncid >= NC_MAX_FILES || varid < 0 || varid >= g_nc[ncid].n_vars) return 1;
    if (!strcmp(name, "units")) {
        nc_def_record *r = &g_def[g_nc[ncid].var_def[varid]];
        const size_t n = len < sizeof r->units - 1 ? len : sizeof r->units - 1;
        memcpy(r->units, op, n);
        r->units[n] = 0;
    }
    return 0;
}

int nc_enddef(int ncid)
{
    (void)ncid;
    return 0;
}

int nc_put_var_double(int ncid, int varid, const double *op)
{
    if (ncid < 0 || ncid >= NC_MAX_FILES || varid < 0 || varid >= g_nc[ncid].n_vars) return 1;
    new_record(g_nc[ncid].path, g_nc[ncid].var_name[varid], op, g_nc[ncid].var_len[varid]);
    return 0;
}

int nc_put_var_int(int ncid, int varid, const int *op)
{
    /* recorded as doubles (exact for every index and sign the tables hold) */
    if (ncid < 0 || ncid >= NC_MAX_FILES || varid < 0 || varid >= g_nc[ncid].n_vars) return 1;
    const long n = g_nc[ncid].var_len[varid];
    double *tmp = malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
    if (!tmp) abort();
    for (long i = 0; i < n; ++i) tmp[i] = (double)op[i];
    new_record(g_nc[ncid].path, g_nc[ncid].var_name[varid], tmp, n);
    free(tmp);
    return 0;
}

int nc_open(const char *path, int mode, int *ncidp)
{
    (void)path; (void)mode; (void)ncidp;
    return 2;
}

int nc_inq_varid(int ncid, const char *name, int *varidp)
{
    (void)ncid; (void)name; (void)varidp;
    return 2;
}

int nc_get_var_double(int ncid, int varid, double *ip)
{
    (void)ncid; (void)varid; (void)ip;
    return 2;
}

int nc_get_var_int(int ncid, int varid, int *ip)
{
    (void)ncid; (void)varid; (void)ip;
    return 2;
}

int nc_close(int ncid)
{
    if (ncid < 0 || ncid >= NC_MAX_FILES) return 1;
    g_nc[ncid].open = 0;
    return 0;
}

const char *nc_strerror(int ncerr)
{
    (void)ncerr;
    return "netCDF stand-in error";
}

/* ------------------------------------------------------------------ ecCodes */
struct grib_handle {
    long category, number, surface_type, level;
    char short_name[64];
    double *values;
    long n_values;
};

codes_handle *codes_handle_new_from_file(codes_context *c, FILE *f, ProductKind product, int *error)
{
    (void)c; (void)f; (void)product;
    codes_handle *h = calloc(1, sizeof *h);
    if (!h) abort();
    h->category = h->number = h->surface_type = h->level = -1;
    *error = 0;
    return h;
}

int codes_handle_delete(codes_handle *h)
{
    if (h) free(h->values);
    free(h);
    return 0;
}

int codes_set_long(codes_handle *h, const char *key, long val)
{
    if (!strcmp(key, "parameterCategory")) h->category = val;
    else if (!strcmp(key, "parameterNumber")) h->number = val;
    else if (!strcmp(key, "typeOfFirstFixedSurface")) h->surface_type = val;
    else if (!strcmp(key, "level")) h->level = val;
    return 0;
}

int codes_set_double(codes_handle *h, const char *key, double val)
{
    (void)h; (void)key; (void)val;
    return 0;
}

int codes_set_string(codes_handle *h, const char *key, const char *mesg, size_t *length)
{
    (void)length;
    if (!strcmp(key, "shortName")) strncpy(h->short_name, mesg, sizeof h->short_name - 1);
    return 0;
}

int codes_set_double_array(codes_handle *h, const char *key, const double *vals, size_t length)
{
    if (strcmp(key, "values")) return 0;
    free(h->values);
    h->values = malloc((length ? length : 1) * sizeof(double));
    if (!h->values) abort();
    memcpy(h->values, vals, length * sizeof(double));
    h->n_values = (long)length;
    return 0;
}

int codes_write_message(const codes_handle *h, const char *file, const char *mode)
{
    (void)mode;
    io_record *r = new_record(file, h->short_name, h->values, h->n_values);
    r->category = h->category;
    r->number = h->number;
    r->surface_type = h->surface_type;
    r->level = h->level;
    return 0;
}
