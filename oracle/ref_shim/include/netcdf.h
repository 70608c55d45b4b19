/*
 * netCDF stand-in so the reference's init/export translation units
 * (src/ibm3d_init.c, src/ibm3d_export.c) compile without libnetcdf.
 * Test infrastructure only: writers record each variable's payload into
 * $IBM3D_NC_DUMP_DIR/<variable>.bin when that is set (and discard it
 * otherwise); readers fail with an error code (the reference then aborts,
 * src/ibm3d_init.c:223).
 */
#ifndef ORACLE_SHIM_NETCDF_H
#define ORACLE_SHIM_NETCDF_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int nc_type;
#define NC_NOERR 0
#define NC_ENOTNC (-51)
#define NC_CLOBBER 0
#define NC_NOWRITE 0
#define NC_INT ((nc_type)4)
#define NC_FLOAT ((nc_type)5)
#define NC_DOUBLE ((nc_type)6)

int nc_create(const char *path, int cmode, int *ncidp);
int nc_open(const char *path, int mode, int *ncidp);
int nc_close(int ncid);
int nc_enddef(int ncid);
int nc_def_dim(int ncid, const char *name, size_t len, int *idp);
int nc_def_var(int ncid, const char *name, nc_type xtype, int ndims, const int *dimidsp, int *varidp);
int nc_put_att_text(int ncid, int varid, const char *name, size_t len, const char *op);
int nc_put_var_double(int ncid, int varid, const double *op);
int nc_put_var_float(int ncid, int varid, const float *op);
int nc_put_var_int(int ncid, int varid, const int *op);
int nc_inq_varid(int ncid, const char *name, int *varidp);
int nc_get_var_double(int ncid, int varid, double *ip);
int nc_get_var_float(int ncid, int varid, float *ip);
int nc_get_var_int(int ncid, int varid, int *ip);
const char *nc_strerror(int ncerr);

#ifdef __cplusplus
}
#endif

#endif
