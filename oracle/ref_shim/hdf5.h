/* ORACLE build shim: declarations of the HDF5 C API names that
 * components/common/include/basis_io_h5.hpp mentions, so the reference's
 * operator.cpp compiles without libhdf5.  Every call fails at run time; the
 * oracle loads bases from arrays, never from HDF5 through this path. */
#pragma once
#include <stdint.h>
typedef int64_t hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
#define H5F_ACC_TRUNC 0u
#define H5F_ACC_RDONLY 0u
#define H5P_DEFAULT ((hid_t)0)
#define H5S_ALL ((hid_t)0)
#define H5T_NATIVE_UINT64 ((hid_t)0)
#define H5T_NATIVE_DOUBLE ((hid_t)0)
static inline hid_t H5Fcreate(const char*, unsigned, hid_t, hid_t) { return -1; }
static inline hid_t H5Fopen(const char*, unsigned, hid_t) { return -1; }
static inline herr_t H5Fclose(hid_t) { return -1; }
static inline hid_t H5Screate_simple(int, const hsize_t*, const hsize_t*) { return -1; }
static inline herr_t H5Sclose(hid_t) { return -1; }
static inline hid_t H5Dcreate(hid_t, const char*, hid_t, hid_t, hid_t, hid_t, hid_t) { return -1; }
static inline hid_t H5Dcreate2(hid_t, const char*, hid_t, hid_t, hid_t, hid_t, hid_t) { return -1; }
static inline hid_t H5Dopen(hid_t, const char*, hid_t) { return -1; }
static inline herr_t H5Dclose(hid_t) { return -1; }
static inline herr_t H5Dwrite(hid_t, hid_t, hid_t, hid_t, hid_t, const void*) { return -1; }
static inline herr_t H5Dread(hid_t, hid_t, hid_t, hid_t, hid_t, void*) { return -1; }
static inline hid_t H5Dget_space(hid_t) { return -1; }
static inline int H5Sget_simple_extent_ndims(hid_t) { return -1; }
static inline int H5Sget_simple_extent_dims(hid_t, hsize_t*, hsize_t*) { return -1; }
