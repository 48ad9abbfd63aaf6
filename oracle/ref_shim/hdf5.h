/* Stand-in for HDF5.  The hot-path sources include it without calling it; the snapshot header
 * writer (src/header.c) calls the group, dataspace and attribute functions declared here, which
 * ref_shim.c implements by recording every attribute written (group, name, type, values), so the
 * attribute values can be compared without an HDF5 library. */
#ifndef ORC_SHIM_HDF5_H
#define ORC_SHIM_HDF5_H
#include <stdint.h>
typedef int64_t hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;

#define H5P_DEFAULT ((hid_t)0)
#define H5T_NATIVE_DOUBLE ((hid_t)1)
#define H5T_NATIVE_INT ((hid_t)2)
#define H5T_NATIVE_LONG ((hid_t)3)

hid_t H5Gcreate(hid_t loc, const char *name, hid_t lcpl, hid_t gcpl, hid_t gapl);
herr_t H5Gclose(hid_t grp);
hid_t H5Screate_simple(int rank, const hsize_t *dims, const hsize_t *maxdims);
herr_t H5Sset_extent_simple(hid_t space, int rank, const hsize_t *dims, const hsize_t *maxdims);
herr_t H5Sclose(hid_t space);
hid_t H5Acreate1(hid_t loc, const char *name, hid_t type, hid_t space, hid_t acpl);
herr_t H5Awrite(hid_t attr, hid_t type, const void *buf);
herr_t H5Aclose(hid_t attr);
#endif
