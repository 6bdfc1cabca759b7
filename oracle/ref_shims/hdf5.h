/* Build shim for compiling the CIFlow reference sources as a test oracle.
 * HDF5 is not installed; the oracle never reads or writes HDF5 files, so every
 * call is a stub that fails with -1. Only the names the reference uses exist. */
#pragma once
#include <stddef.h>
typedef long long hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
#define H5P_DEFAULT 0
#define H5S_ALL 0
#define H5S_SCALAR 0
#define H5F_ACC_RDONLY 0
#define H5F_ACC_RDWR 1
#define H5F_ACC_TRUNC 2
#define H5T_NATIVE_INT 0
#define H5T_NATIVE_UINT 0
#define H5T_NATIVE_DOUBLE 0
#define H5T_NATIVE_LLONG 0
#define H5T_STD_I32LE 0
#define H5T_STD_I64LE 0
#define H5T_STD_U64LE 0
#define H5T_IEEE_F64LE 0
#define CIGPU_H5_STUB(name) template <typename... A> static inline long long name(A...) { return -1; }
CIGPU_H5_STUB(H5Fcreate) CIGPU_H5_STUB(H5Fopen) CIGPU_H5_STUB(H5Fclose)
CIGPU_H5_STUB(H5Gcreate) CIGPU_H5_STUB(H5Gopen) CIGPU_H5_STUB(H5Gclose)
CIGPU_H5_STUB(H5Dcreate) CIGPU_H5_STUB(H5Dopen) CIGPU_H5_STUB(H5Dclose)
CIGPU_H5_STUB(H5Dread) CIGPU_H5_STUB(H5Dwrite)
CIGPU_H5_STUB(H5Screate) CIGPU_H5_STUB(H5Screate_simple) CIGPU_H5_STUB(H5Sclose)
CIGPU_H5_STUB(H5Acreate) CIGPU_H5_STUB(H5Aopen) CIGPU_H5_STUB(H5Aopen_by_name)
CIGPU_H5_STUB(H5Aread) CIGPU_H5_STUB(H5Awrite) CIGPU_H5_STUB(H5Aclose)
#undef CIGPU_H5_STUB
