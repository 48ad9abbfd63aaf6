/* Type-only stand-in for HDF5: the hot-path sources include it but call none of it. */
#ifndef ORC_SHIM_HDF5_H
#define ORC_SHIM_HDF5_H
#include <stdint.h>
typedef int64_t hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
#endif
