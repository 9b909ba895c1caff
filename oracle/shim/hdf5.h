/* Stand-in for HDF5's header (declarations only), written for this project so
 * that the reference's emc_helper.cpp compiles for the oracle build.  Its HDF5
 * reader (read_images_from_models) is never called by the oracle; the
 * definitions in ref_helper_harness.cpp fail every call.  Test infrastructure;
 * not part of the product. */
#ifndef EMC_SHIM_HDF5_H
#define EMC_SHIM_HDF5_H
#ifdef __cplusplus
extern "C" {
#endif
typedef long long hid_t;
typedef int herr_t;
#define H5F_ACC_RDWR 1u
#define H5P_DEFAULT ((hid_t)0)
#define H5S_ALL ((hid_t)0)
#define H5T_NATIVE_FLOAT ((hid_t)1)
#define H5T_NATIVE_DOUBLE ((hid_t)2)
hid_t H5Fopen(const char* name, unsigned flags, hid_t access);
hid_t H5Dopen(hid_t file, const char* name, hid_t access);
herr_t H5Dread(hid_t dset, hid_t mem_type, hid_t mem_space, hid_t file_space, hid_t xfer,
               void* buf);
herr_t H5Dclose(hid_t dset);
herr_t H5Fclose(hid_t file);
#ifdef __cplusplus
}
#endif
#endif
