/*
 * No-op stand-in for <hdf5.h>, used ONLY to compile the SCORE reference sources
 * as a CPU oracle (test infrastructure; never linked into the product).
 * HDF5 is output-only in the reference and is not on the growth path; every call
 * here does nothing and reports success.
 */
#ifndef SCORE_ORACLE_STUB_HDF5_H
#define SCORE_ORACLE_STUB_HDF5_H

typedef long long hid_t;
typedef int herr_t;
typedef int htri_t;
typedef unsigned long long hsize_t;
typedef int hbool_t;
typedef struct { int dummy; } H5G_stat_t;

#define H5P_DEFAULT 0
#define H5S_ALL 0
#define H5F_ACC_TRUNC 2
#define H5F_ACC_RDWR 1
#define H5T_STD_U8LE 1
#define H5T_STD_U32LE 2
#define H5T_STD_I32LE 3
#define H5T_IEEE_F32LE 4
#define H5T_IEEE_F64LE 5
#define H5T_NATIVE_UCHAR 6
#define H5T_NATIVE_UINT 7
#define H5T_NATIVE_INT 8
#define H5T_NATIVE_FLOAT 9
#define H5T_NATIVE_DOUBLE 10

static inline hid_t H5Fcreate(const char*, unsigned, hid_t, hid_t) { return 1; }
static inline hid_t H5Fopen(const char*, unsigned, hid_t) { return 1; }
static inline herr_t H5Fclose(hid_t) { return 0; }
static inline hid_t H5Gcreate2(hid_t, const char*, hid_t, hid_t, hid_t) { return 1; }
static inline herr_t H5Gclose(hid_t) { return 0; }
static inline herr_t H5Gget_objinfo(hid_t, const char*, hbool_t, H5G_stat_t*) { return 0; }
static inline hid_t H5Screate_simple(int, const hsize_t*, const hsize_t*) { return 1; }
static inline herr_t H5Sclose(hid_t) { return 0; }
static inline hid_t H5Dcreate2(hid_t, const char*, hid_t, hid_t, hid_t, hid_t, hid_t) { return 1; }
#define H5Dcreate H5Dcreate2
static inline herr_t H5Dwrite(hid_t, hid_t, hid_t, hid_t, hid_t, const void*) { return 0; }
static inline herr_t H5Dclose(hid_t) { return 0; }
static inline herr_t H5Eset_auto(void*, void*, void*) { return 0; }

#endif
