/* Declaration-only stand-in for <hdf5.h>: lets the oracle's pinning build
 * include reference headers that mention HDF5 types.  No HDF5 call is made
 * by the oracle; every function here aborts (test infrastructure only). */
#ifndef ORACLE_SHIM_HDF5_H
#define ORACLE_SHIM_HDF5_H
#include <cstdio>
#include <cstdlib>
typedef long long hid_t;
typedef unsigned long long hsize_t;
typedef long long hssize_t;
typedef int herr_t;
typedef int htri_t;
#define H5P_DEFAULT 0
#define H5P_DATASET_CREATE 1
#define H5T_NATIVE_DOUBLE 2
#define H5T_NATIVE_FLOAT 3
#define H5T_NATIVE_INT 4
#define H5S_ALL 0
#define H5S_SELECT_SET 0
#define H5F_ACC_RDONLY 0
#define H5F_ACC_RDWR 1
#define H5F_ACC_TRUNC 2
static inline hid_t oracle_h5_abort() { fprintf(stderr, "oracle: HDF5 not available\n"); abort(); return -1; }
static inline herr_t H5Dclose(hid_t) { return (herr_t)oracle_h5_abort(); }
static inline hid_t H5Dopen2(hid_t, const char*, hid_t) { return oracle_h5_abort(); }
static inline herr_t H5Pclose(hid_t) { return (herr_t)oracle_h5_abort(); }
static inline hid_t H5Pcreate(hid_t) { return oracle_h5_abort(); }
static inline herr_t H5Pset_chunk(hid_t, int, const hsize_t*) { return (herr_t)oracle_h5_abort(); }
static inline hid_t H5Screate_simple(int, const hsize_t*, const hsize_t*) { return oracle_h5_abort(); }
#endif
