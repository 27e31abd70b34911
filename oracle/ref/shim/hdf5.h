// Stand-in for <hdf5.h>, used ONLY to compile the unmodified reference headers
// into the test oracle under oracle/_ref/.  Test infrastructure, not product
// code: the harness never opens a file, so every call fails with -1.
#pragma once
typedef long long hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
#define H5F_ACC_RDONLY 0u
#define H5F_ACC_RDWR 1u
#define H5F_ACC_TRUNC 2u
#define H5P_DEFAULT ((hid_t)0)
#define H5S_ALL ((hid_t)0)
#define H5T_NATIVE_CHAR ((hid_t)1)
#define H5T_NATIVE_DOUBLE ((hid_t)2)
#define H5T_NATIVE_FLOAT ((hid_t)3)
#define H5T_NATIVE_INT ((hid_t)4)
#define H5T_NATIVE_LDOUBLE ((hid_t)5)
#define H5T_NATIVE_LONG ((hid_t)6)
#define H5T_NATIVE_UINT ((hid_t)7)
#define H5T_NATIVE_ULONG ((hid_t)8)
template <class... A> static inline hid_t H5Fcreate(A...) { return -1; }
template <class... A> static inline hid_t H5Fopen(A...) { return -1; }
template <class... A> static inline herr_t H5Fclose(A...) { return -1; }
template <class... A> static inline hid_t H5Dcreate(A...) { return -1; }
template <class... A> static inline hid_t H5Dopen(A...) { return -1; }
template <class... A> static inline hid_t H5Dopen1(A...) { return -1; }
template <class... A> static inline hid_t H5Dcreate2(A...) { return -1; }
template <class... A> static inline herr_t H5Dread(A...) { return -1; }
template <class... A> static inline herr_t H5Dwrite(A...) { return -1; }
template <class... A> static inline herr_t H5Dclose(A...) { return -1; }
template <class... A> static inline hid_t H5Screate_simple(A...) { return -1; }
template <class... A> static inline herr_t H5Sclose(A...) { return -1; }
template <class... A> static inline herr_t H5Tclose(A...) { return -1; }
template <class... A> static inline hid_t H5Tcopy(A...) { return -1; }
