/*
 * hdf5.h -- a recording stand-in for the part of the HDF5 C API that a
 * hydroFV snapshot writer calls.  TEST INFRASTRUCTURE ONLY.
 *
 * Neither build machine has the HDF5 library, so the snapshot writer's
 * HDF5 branch is compiled against these declarations and linked with
 * fake_hdf5.c, which records every group and dataset written and, when the
 * file is closed, stores a text listing of them (one line per object,
 * sorted by path) in place of the .h5 file.  The reference's own writer is
 * compiled against the same stand-in, so the two listings can be compared:
 * same groups, dataset names, element types, shapes and values.
 *
 * Names follow the HDF5 API (H5Fcreate, H5Gcreate, H5Dcreate, H5Dwrite,
 * H5Screate, H5Screate_simple, H5Tcopy, H5Tset_size and the close calls);
 * the macros H5Gcreate and H5Dcreate take the argument lists of the
 * library's version-2 calls.
 */
#ifndef HYDRO_TEST_FAKE_HDF5_H
#define HYDRO_TEST_FAKE_HDF5_H

#include <stddef.h>

typedef long long hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;

#define H5I_INVALID_HID ((hid_t) -1)
#define H5P_DEFAULT ((hid_t) 0)
#define H5S_ALL ((hid_t) 0)
#define H5F_ACC_TRUNC 2u
#define H5T_VARIABLE ((size_t) -1)

typedef enum { H5S_SCALAR = 0, H5S_SIMPLE = 1 } H5S_class_t;

/* predefined types */
#define H5T_NATIVE_DOUBLE ((hid_t) 1001)
#define H5T_NATIVE_LLONG ((hid_t) 1002)
#define H5T_NATIVE_INT ((hid_t) 1003)
#define H5T_C_S1 ((hid_t) 1004)

hid_t H5Fcreate(const char *name, unsigned flags, hid_t fcpl, hid_t fapl);
herr_t H5Fclose(hid_t file);
hid_t H5Gcreate2(hid_t loc, const char *name, hid_t lcpl, hid_t gcpl, hid_t gapl);
herr_t H5Gclose(hid_t group);
hid_t H5Screate(H5S_class_t type);
hid_t H5Screate_simple(int rank, const hsize_t dims[], const hsize_t maxdims[]);
herr_t H5Sclose(hid_t space);
hid_t H5Tcopy(hid_t type);
herr_t H5Tset_size(hid_t type, size_t size);
herr_t H5Tclose(hid_t type);
hid_t H5Dcreate2(hid_t loc, const char *name, hid_t type, hid_t space, hid_t lcpl, hid_t dcpl, hid_t dapl);
herr_t H5Dwrite(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t xfer, const void *buf);
herr_t H5Dclose(hid_t dset);

#define H5Gcreate H5Gcreate2
#define H5Dcreate H5Dcreate2

#endif
