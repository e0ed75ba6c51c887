/*
 * Test-infrastructure stand-in for the ecCodes header (the library is not
 * installed where the reference harness is built).  It declares the ecCodes
 * calls that the reference's output code makes, with ecCodes' public
 * signatures; the definitions in ../ref_io_stubs.c write no GRIB message but
 * record, per message, the keys that identify the field and the array set as
 * "values" (the field interpolated to the regular lat-lon grid).
 */
#ifndef REF_STUB_ECCODES_H
#define REF_STUB_ECCODES_H
#include <stdio.h>
typedef struct grib_handle codes_handle;
typedef struct grib_context codes_context;
typedef enum { PRODUCT_ANY, PRODUCT_GRIB } ProductKind;
codes_handle *codes_handle_new_from_file(codes_context *c, FILE *f, ProductKind product, int *error);
int codes_handle_delete(codes_handle *h);
int codes_set_long(codes_handle *h, const char *key, long val);
int codes_set_double(codes_handle *h, const char *key, double val);
int codes_set_string(codes_handle *h, const char *key, const char *mesg, size_t *length);
int codes_set_double_array(codes_handle *h, const char *key, const double *vals, size_t length);
int codes_write_message(const codes_handle *h, const char *file, const char *mode);
#endif
