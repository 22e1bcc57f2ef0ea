/* No-op HDF5 stand-in: the serial oracle never writes HDF5 output
 * (only the Cp dump uses it, and the oracle driver does not call it). */
#pragma once
typedef long long hid_t;
typedef unsigned long long hsize_t;
typedef int herr_t;
#define H5P_DEFAULT 0
#define H5P_FILE_ACCESS 0
#define H5F_ACC_RDWR 0
#define H5F_ACC_TRUNC 0
#define H5S_ALL 0
#define H5S_SELECT_SET 0
#define H5T_NATIVE_DOUBLE 0
static inline hid_t H5Pcreate(int) { return 0; }
static inline herr_t H5Pset_fapl_mpio(hid_t, int, int) { return 0; }
static inline herr_t H5Pclose(hid_t) { return 0; }
static inline hid_t H5Fcreate(const char*, int, int, hid_t) { return 0; }
static inline hid_t H5Fopen(const char*, int, hid_t) { return 0; }
static inline herr_t H5Fclose(hid_t) { return 0; }
static inline hid_t H5Screate_simple(int, const hsize_t*, const hsize_t*) { return 0; }
static inline herr_t H5Sclose(hid_t) { return 0; }
static inline herr_t H5Sselect_hyperslab(hid_t, int, const hsize_t*, const hsize_t*, const hsize_t*, const hsize_t*) { return 0; }
static inline hid_t H5Dcreate(hid_t, const char*, int, hid_t, int, int, int) { return 0; }
static inline hid_t H5Dopen(hid_t, const char*, int) { return 0; }
static inline hid_t H5Dget_space(hid_t) { return 0; }
static inline herr_t H5Dread(hid_t, int, hid_t, hid_t, int, void*) { return 0; }
static inline herr_t H5Dwrite(hid_t, int, hid_t, hid_t, int, const void*) { return 0; }
static inline herr_t H5Dclose(hid_t) { return 0; }
#define H5T_NATIVE_INT 0
static inline hid_t H5Gcreate(hid_t, const char*, int, int, hid_t) { return 0; }
static inline herr_t H5Gclose(hid_t) { return 0; }
