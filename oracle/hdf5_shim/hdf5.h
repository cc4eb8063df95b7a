/*
 * ORACLE -- test infrastructure.  A stand-in for <hdf5.h> that lets the
 * reference's serial build (phasefield.c with USE_MPI 0) compile and run
 * without libhdf5.  It declares exactly the calls that path makes
 * (phasefield.c:996-1109): H5Fopen/H5Fcreate/H5Fclose, H5Dopen2/
 * H5Dcreate2/H5Dclose/H5Dget_space/H5Dread/H5Dwrite, H5Screate_simple/
 * H5Sselect_hyperslab/H5Sclose.  h5shim.c implements them on top of the
 * oracle's own HDF5 subset (h5ref.h), so files read and written by the
 * reference build are real HDF5 files and no product code is involved.
 *
 * Like libhdf5, identifiers are never reused: an operation on a closed
 * identifier fails (returns a negative value) and leaves the buffer alone.
 * That is what makes the reference's read of /etaL through the closed
 * /etaS identifier (phasefield.c:1032) a no-op, as it is with libhdf5.
 */
#ifndef PPF_HDF5_SHIM_H
#define PPF_HDF5_SHIM_H

typedef long long hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;

#define H5F_ACC_RDONLY 0u
#define H5F_ACC_TRUNC 2u
#define H5P_DEFAULT ((hid_t)0)
#define H5S_SELECT_SET 0
#define H5T_IEEE_F64LE ((hid_t)-64)

hid_t H5Fopen(const char *name, unsigned flags, hid_t fapl);
hid_t H5Fcreate(const char *name, unsigned flags, hid_t fcpl, hid_t fapl);
herr_t H5Fclose(hid_t file);
hid_t H5Dopen2(hid_t loc, const char *name, hid_t dapl);
hid_t H5Dcreate2(hid_t loc, const char *name, hid_t type, hid_t space, hid_t lcpl, hid_t dcpl,
                 hid_t dapl);
herr_t H5Dclose(hid_t dset);
hid_t H5Dget_space(hid_t dset);
herr_t H5Dread(hid_t dset, hid_t memtype, hid_t memspace, hid_t filespace, hid_t xfer, void *buf);
herr_t H5Dwrite(hid_t dset, hid_t memtype, hid_t memspace, hid_t filespace, hid_t xfer,
                const void *buf);
hid_t H5Screate_simple(int rank, const hsize_t *dims, const hsize_t *maxdims);
herr_t H5Sselect_hyperslab(hid_t space, int op, const hsize_t *start, const hsize_t *stride,
                           const hsize_t *count, const hsize_t *block);
herr_t H5Sclose(hid_t space);

#endif
