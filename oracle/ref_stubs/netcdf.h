/*
 * Test-infrastructure stand-in for the netCDF C library's header (the library
 * is not installed where the reference harness is built).  It declares the
 * netCDF calls that the reference's output code makes, with netCDF's public
 * signatures; the definitions in ../ref_io_stubs.c write no file but record
 * every array handed to nc_put_var_double / nc_put_var_int, so that the
 * fields and tables the reference computes for its output can be compared
 * with other implementations.  Reading files is not available.
 */
#ifndef REF_STUB_NETCDF_H
#define REF_STUB_NETCDF_H
#include <stddef.h>
typedef int nc_type;
#define NC_NOWRITE 0
#define NC_CLOBBER 0
#define NC_INT 4
#define NC_DOUBLE 6
int nc_create(const char *path, int cmode, int *ncidp);
int nc_def_dim(int ncid, const char *name, size_t len, int *idp);
int nc_def_var(int ncid, const char *name, nc_type xtype, int ndims, const int *dimidsp, int *varidp);
int nc_put_att_text(int ncid, int varid, const char *name, size_t len, const char *op);
int nc_enddef(int ncid);
int nc_put_var_double(int ncid, int varid, const double *op);
int nc_put_var_int(int ncid, int varid, const int *op);
/* reading is not available: these return an error */
int nc_open(const char *path, int mode, int *ncidp);
int nc_inq_varid(int ncid, const char *name, int *varidp);
int nc_get_var_double(int ncid, int varid, double *ip);
int nc_get_var_int(int ncid, int varid, int *ip);
int nc_close(int ncid);
const char *nc_strerror(int ncerr);
#endif
