/* No-op stand-in for the HDF5 API, used only to compile the reference sources
 * into the pinning library under oracle/_ref (libhdf5 is absent from this
 * image).  Every call succeeds and transfers nothing; the pinning harness
 * never calls the reference's file readers or writers.
 * Test infrastructure: never linked into the product library. */
#ifndef ORACLE_STUB_HDF5_H
#define ORACLE_STUB_HDF5_H
#include <stdio.h>
#include <stddef.h>
#include "mpi.h"
typedef long long hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
#define HOFFSET(s, m) offsetof(s, m)
#define H5P_DEFAULT 0
#define H5T_COMPOUND 6
#define H5T_NATIVE_DOUBLE 1
#define H5T_NATIVE_FLOAT 2
#define H5T_IEEE_F64BE 3
#define H5S_SELECT_SET 0
#define H5P_FILE_ACCESS 1
#define H5P_DATASET_XFER 2
#define H5FD_MPIO_COLLECTIVE 1
#define H5F_ACC_TRUNC 1
#define H5F_ACC_RDONLY 0
#define H5F_ACC_RDWR 2
static inline hid_t oracle_h5_nop(void) { return 0; }
#define H5Tcreate(...) oracle_h5_nop()
#define H5Tinsert(...) oracle_h5_nop()
#define H5Tclose(...) oracle_h5_nop()
#define H5Sclose(...) oracle_h5_nop()
#define H5Screate_simple(...) oracle_h5_nop()
#define H5Sselect_hyperslab(...) oracle_h5_nop()
#define H5Dclose(...) oracle_h5_nop()
#define H5Dwrite(...) oracle_h5_nop()
#define H5Dread(...) oracle_h5_nop()
#define H5Dget_space(...) oracle_h5_nop()
#define H5Dcreate(...) oracle_h5_nop()
#define H5Dopen(...) oracle_h5_nop()
#define H5Pcreate(...) oracle_h5_nop()
#define H5Pclose(...) oracle_h5_nop()
#define H5Pset_fapl_mpio(...) oracle_h5_nop()
#define H5Pset_dxpl_mpio(...) oracle_h5_nop()
#define H5Gclose(...) oracle_h5_nop()
#define H5Gopen1(...) oracle_h5_nop()
#define H5Gcreate(...) oracle_h5_nop()
#define H5Fclose(...) oracle_h5_nop()
#define H5Fopen(...) oracle_h5_nop()
#define H5Fcreate(...) oracle_h5_nop()
#endif
