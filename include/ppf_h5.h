/*
 * ppf_h5.h -- the HDF5 file subset that `ppf` reads and writes.
 *
 * The reference program does all of its I/O through libhdf5
 * (phasefield.c:996-1049 read_hdf5, :1052-1109 write_hdf5, and the MPI-IO
 * variants :481-547 / :550-624).  Only three things ever cross that boundary:
 * the 3-D datasets /etaS, /etaL and /c, stored as IEEE float64 little endian,
 * C order [z][y][x] (phasefield.c:504-514, 574).  This library implements
 * exactly that subset of the HDF5 format in plain C so that the GPU program
 * stays a drop-in without a libhdf5 dependency:
 *
 *   reading:  superblock v0/v1/v2/v3 (with or without a user block),
 *             object headers v1 and v2 (with continuation blocks),
 *             groups stored as symbol tables (v1 B-tree + local heap) or as
 *             compact link messages, dataspaces v1/v2, IEEE float32/float64
 *             of either byte order, layouts v1-v4: contiguous, compact,
 *             chunked with a v1 B-tree index (v3 layout, as written by the
 *             reference's MPI build, phasefield.c:577-582) and the v4
 *             single-chunk and implicit indexes.  Filters (compression) are
 *             rejected with an error.
 *   writing:  superblock v0, a symbol-table root group, v1 object headers,
 *             contiguous datasets (serial reference layout, :1067-1072) or
 *             chunked datasets with a v1 B-tree index (MPI reference layout,
 *             chunk = one subdomain, :574-582).
 *
 * All functions return 0 on success and a negative code on failure;
 * ppf_h5_last_error() then gives a message (thread local).
 */
#ifndef PPF_H5_H
#define PPF_H5_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PPF_H5_F64 0   /* H5T_IEEE_F64LE: the reference's only datatype */
#define PPF_H5_F32 1   /* H5T_IEEE_F32LE */

#define PPF_H5_EIO      (-1)  /* open/read/write failed or file truncated */
#define PPF_H5_EFORMAT  (-2)  /* not HDF5, or a structure outside the subset */
#define PPF_H5_ENOTFOUND (-3) /* no dataset of that name */
#define PPF_H5_EDIMS    (-4)  /* rank is not 3, or a size does not fit */
#define PPF_H5_ETYPE    (-5)  /* datatype is not IEEE float32/float64 */
#define PPF_H5_EARG     (-6)  /* bad argument */
#define PPF_H5_ENOMEM   (-7)

/* Dimensions of a rank-3 dataset `name` ("/etaS" or "etaS"), C order. */
int ppf_h5_dims(const char *path, const char *name, int64_t dims[3]);

/* Read the whole rank-3 dataset `name` converted to double.  `out` holds
 * dims[0]*dims[1]*dims[2] values (C order); `capacity` is its length in
 * elements.  `dims` receives the dataset dimensions. */
int ppf_h5_read3d(const char *path, const char *name, int64_t dims[3],
                  double *out, int64_t capacity);

/* Write a new file (truncating any old one) holding `n` rank-3 datasets of
 * identical dims, in the order given.  `dtype` is PPF_H5_F64 or PPF_H5_F32
 * (values are converted from double).  `chunk` NULL gives contiguous
 * storage; otherwise the datasets are chunked with those chunk dims. */
int ppf_h5_write3d(const char *path, int n, const char *const *names,
                   const double *const *data, const int64_t dims[3],
                   int dtype, const int64_t *chunk);

/* Same, plus one float64 dataset `meta_name` of shape (1, 1, nmeta) holding
 * `meta` (contiguous, little-endian host doubles); used for the program's
 * restart record.  Readers that look datasets up by name are unaffected. */
int ppf_h5_write3d_meta(const char *path, int n, const char *const *names, const double *const *data,
                        const int64_t dims[3], int dtype, const int64_t *chunk, const char *meta_name,
                        const double *meta, int nmeta);

const char *ppf_h5_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* PPF_H5_H */
