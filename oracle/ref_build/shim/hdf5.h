/*
 * Test infrastructure (oracle build only): a stand-in for the subset of the
 * HDF5 C API that xpcs-eigen's `corr` calls, so the reference can be built
 * from its unmodified sources where no libhdf5 is installed.
 *
 * Datasets live in an in-memory store that is loaded from, and written back
 * to, a flat "XH5C" container file (format in fakeh5.cpp).  Groups are
 * implicit path prefixes.  Only what configuration.cpp, h5_result.cpp and
 * io/hdf5.cpp use is declared.
 */
#ifndef XPCS_ORACLE_FAKE_HDF5_H
#define XPCS_ORACLE_FAKE_HDF5_H

#include <stddef.h>
#include <stdint.h>

typedef int64_t hid_t;
typedef int herr_t;
typedef int htri_t;
typedef unsigned long long hsize_t;

/* Element type codes of the container; also used as the type ids. */
enum {
  XH5C_I32 = 1,
  XH5C_I64 = 2,
  XH5C_F32 = 3,
  XH5C_F64 = 4,
  XH5C_STR = 5,
  XH5C_U32 = 6,
  XH5C_I16 = 7,
  XH5C_U16 = 8
};

#define H5P_DEFAULT ((hid_t)0)
#define H5S_ALL ((hid_t)0)
#define H5E_DEFAULT 0
#define H5F_ACC_RDONLY 0u
#define H5F_ACC_RDWR 1u
#define H5P_DATASET_CREATE 0
#define H5T_DIR_ASCEND 0
#define H5S_SELECT_SET 0
#define H5T_VARIABLE ((size_t)-1)

#define H5T_NATIVE_INT ((hid_t)XH5C_I32)
#define H5T_NATIVE_LONG ((hid_t)XH5C_I64)
#define H5T_NATIVE_FLOAT ((hid_t)XH5C_F32)
#define H5T_NATIVE_DOUBLE ((hid_t)XH5C_F64)
#define H5T_NATIVE_UINT32 ((hid_t)XH5C_U32)
#define H5T_NATIVE_SHORT ((hid_t)XH5C_I16)
#define H5T_NATIVE_USHORT ((hid_t)XH5C_U16)

hid_t H5Fopen(const char *name, unsigned flags, hid_t fapl);
herr_t H5Fclose(hid_t file);

hid_t H5Gopen2(hid_t loc, const char *name, hid_t gapl);
hid_t H5Gcreate(hid_t loc, const char *name, hid_t lcpl, hid_t gcpl, hid_t gapl);
herr_t H5Gclose(hid_t group);

hid_t H5Dopen(hid_t loc, const char *name, hid_t dapl);
hid_t H5Dopen2(hid_t loc, const char *name, hid_t dapl);
hid_t H5Dcreate(hid_t loc, const char *name, hid_t type, hid_t space, hid_t lcpl, hid_t dcpl,
                hid_t dapl);
hid_t H5Dcreate2(hid_t loc, const char *name, hid_t type, hid_t space, hid_t lcpl, hid_t dcpl,
                 hid_t dapl);
herr_t H5Dclose(hid_t dset);
hid_t H5Dget_space(hid_t dset);
hid_t H5Dget_type(hid_t dset);
hsize_t H5Dget_storage_size(hid_t dset);
herr_t H5Dread(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t xfer,
               void *buf);
herr_t H5Dwrite(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t xfer,
                const void *buf);

hid_t H5Screate_simple(int rank, const hsize_t *dims, const hsize_t *maxdims);
herr_t H5Sclose(hid_t space);
int H5Sget_simple_extent_dims(hid_t space, hsize_t *dims, hsize_t *maxdims);
int H5Sget_simple_extent_ndims(hid_t space);
herr_t H5Sselect_hyperslab(hid_t space, int op, const hsize_t *start, const hsize_t *stride,
                           const hsize_t *count, const hsize_t *block);

htri_t H5Tis_variable_str(hid_t type);
hid_t H5Tget_native_type(hid_t type, int direction);
htri_t H5Tequal(hid_t a, hid_t b);
size_t H5Tget_size(hid_t type);

herr_t H5Eset_auto(int estack, void *func, void *client_data);

hid_t H5Pcreate(int cls);
herr_t H5Pset_chunk(hid_t plist, int rank, const hsize_t *dims);
herr_t H5Pset_deflate(hid_t plist, unsigned level);

#endif
