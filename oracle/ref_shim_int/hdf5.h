/* ORACLE (test infrastructure only): the HDF5 name that
 * source/gravitational_waves.h declares a member function with. */
#ifndef SH_REF_SHIM_INT_HDF5_H_
#define SH_REF_SHIM_INT_HDF5_H_
typedef long long hid_t;
#endif
