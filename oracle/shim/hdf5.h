// Stand-in for the HDF5 1.10 C API names that the reference's
// SimData::write_state calls.  HDF5 is not installed here; state output is not
// part of the time-stepping path, so every call is a no-op that reports
// success and nothing is written.  Oracle-only test infrastructure.
#ifndef PLB_ORACLE_SHIM_HDF5_H_
#define PLB_ORACLE_SHIM_HDF5_H_

#include <cstdint>

typedef int64_t hid_t;
typedef unsigned long long hsize_t;
typedef int herr_t;

#define H5F_ACC_TRUNC 0x0002u
#define H5P_DEFAULT ((hid_t)0)
#define H5S_ALL ((hid_t)0)
#define H5T_NATIVE_FLOAT ((hid_t)0)

static inline hid_t H5Fcreate(const char*, unsigned, hid_t, hid_t) { return 1; }
static inline hid_t H5Screate_simple(int, const hsize_t*, const hsize_t*) { return 1; }
static inline hid_t H5Dcreate2(hid_t, const char*, hid_t, hid_t, hid_t, hid_t, hid_t) { return 1; }
static inline herr_t H5Dwrite(hid_t, hid_t, hid_t, hid_t, hid_t, const void*) { return 0; }
static inline herr_t H5Dclose(hid_t) { return 0; }
static inline herr_t H5Sclose(hid_t) { return 0; }
static inline herr_t H5Fclose(hid_t) { return 0; }

#endif  // PLB_ORACLE_SHIM_HDF5_H_
