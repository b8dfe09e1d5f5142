/* Empty stand-in for <hdf5.h>, used only to compile the reference unbinding
 * sources in a one-process oracle build (test infrastructure).  The
 * unbinding path does no file I/O; these declarations only let the shared
 * headers parse.  Every call fails with -1. */
#ifndef HBTG_ORACLE_STUB_HDF5_H
#define HBTG_ORACLE_STUB_HDF5_H

typedef long hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
typedef int htri_t;

#define H5P_DEFAULT 0
#define H5S_ALL 0
#define H5S_SELECT_SET 0
#define H5T_STR_NULLTERM 0
#define H5T_STRING 0
#define H5T_NATIVE_DOUBLE 0
#define H5T_NATIVE_FLOAT 0
#define H5T_NATIVE_INT 0
#define H5T_NATIVE_LONG 0

#include <stddef.h>
static inline herr_t H5Aclose(hid_t) { return -1; }
static inline hid_t H5Aget_type(hid_t) { return -1; }
static inline hid_t H5Aopen_by_name(hid_t, const char *, const char *, hid_t, hid_t) { return -1; }
static inline herr_t H5Aread(hid_t, hid_t, void *) { return -1; }
static inline herr_t H5Dclose(hid_t) { return -1; }
static inline hid_t H5Dget_space(hid_t) { return -1; }
static inline hid_t H5Dopen2(hid_t, const char *, hid_t) { return -1; }
static inline herr_t H5Dread(hid_t, hid_t, hid_t, hid_t, hid_t, void *) { return -1; }
static inline herr_t H5Dvlen_reclaim(hid_t, hid_t, hid_t, void *) { return -1; }
static inline long H5Fget_name(hid_t, char *name, size_t) { if (name) name[0] = 0; return -1; }
static inline long H5Iget_name(hid_t, char *name, size_t) { if (name) name[0] = 0; return -1; }
static inline htri_t H5Iis_valid(hid_t) { return 0; }
static inline herr_t H5Sclose(hid_t) { return -1; }
static inline hid_t H5Screate_simple(int, const hsize_t *, const hsize_t *) { return -1; }
static inline int H5Sget_simple_extent_dims(hid_t, hsize_t *, hsize_t *) { return -1; }
static inline int H5Sget_simple_extent_ndims(hid_t) { return -1; }
static inline herr_t H5Sselect_hyperslab(hid_t, int, const hsize_t *, const hsize_t *, const hsize_t *, const hsize_t *) { return -1; }
static inline herr_t H5Tclose(hid_t) { return -1; }
static inline hid_t H5Tcreate(int, size_t) { return -1; }
static inline herr_t H5Tset_strpad(hid_t, int) { return -1; }

#endif
