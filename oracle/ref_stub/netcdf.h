/* No-op stand-in for the NetCDF header so that the reference's driver
 * (exp_bloch2d.c, whose output writers are called unconditionally) builds
 * in a container without NetCDF.  The output file is outside the
 * eigensolver path; every function here succeeds and writes nothing. */
#ifndef ORACLE_REF_STUB_NETCDF_H
#define ORACLE_REF_STUB_NETCDF_H
#include <stddef.h>
#define NC_NOERR 0
#define NC_DOUBLE 6
#define NC_CLOBBER 0
#define NC_64BIT_DATA 0x20
static inline int nc_create(const char *path, int mode, int *id) { (void) path; (void) mode; *id = 0; return NC_NOERR; }
static inline int nc_def_dim(int id, const char *name, size_t len, int *dim)
{ (void) id; (void) name; (void) len; *dim = 0; return NC_NOERR; }
static inline int nc_def_var(int id, const char *name, int type, int ndims, const int *dims, int *var)
{ (void) id; (void) name; (void) type; (void) ndims; (void) dims; *var = 0; return NC_NOERR; }
static inline int nc_enddef(int id) { (void) id; return NC_NOERR; }
static inline int nc_put_var1_double(int id, int var, const size_t *index, const double *v)
{ (void) id; (void) var; (void) index; (void) v; return NC_NOERR; }
static inline int nc_put_vara_double(int id, int var, const size_t *start, const size_t *count, const double *v)
{ (void) id; (void) var; (void) start; (void) count; (void) v; return NC_NOERR; }
static inline int nc_close(int id) { (void) id; return NC_NOERR; }
#endif
