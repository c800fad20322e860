/*
 * hdf5.h — ORACLE test infrastructure: the two HDF5 handle types that the
 * reference's Solver/src/data_types.h:244-248 and hdf5_funcs.h:21-26 name.
 * No HDF5 routine is provided: the parity harness compiles solver.c and
 * utils.c only and stands in for the three hdf5_funcs.c writers solver.c
 * calls (oracle/ref_harness.c).
 */
#ifndef NS3D_REF_SHIM_HDF5_H
#define NS3D_REF_SHIM_HDF5_H
typedef long long hid_t;
typedef unsigned long long hsize_t;
typedef int herr_t;
#endif
