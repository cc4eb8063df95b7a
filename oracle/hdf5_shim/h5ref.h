/*
 * ORACLE -- test infrastructure.  A second, self-contained implementation of
 * the HDF5 file subset that the reference's serial I/O uses
 * (phasefield.c:996-1109: rank-3 IEEE float64 datasets /etaS, /etaL, /c in
 * C order), written from the HDF5 file-format specification for the oracle
 * side only: the reference build's <hdf5.h> stand-in (h5shim.c) and the
 * oracle's Python helpers use it, so that nothing on the reference side
 * depends on the product's HDF5 code.
 *
 * Files written: superblock version 0 (8-byte offsets and lengths), a root
 * group stored as a symbol table (version-1 B-tree of group nodes + local
 * heap), version-1 object headers, datasets with dataspace v1, IEEE float
 * datatype, fill value v2 and layout v3 -- contiguous, or chunked with a
 * version-1 B-tree chunk index (full-size edge chunks, as the reference's
 * MPI writer produces with chunk = subdomain, phasefield.c:574-582).
 * Files read: superblock versions 0/1 (user block allowed), symbol-table
 * groups, version-1 object headers with continuation blocks, dataspace
 * v1/v2, IEEE float32/float64 of either byte order, layouts v1-v3
 * contiguous and compact, and v3 chunked (version-1 B-tree, unfiltered).
 */
#ifndef H5REF_H
#define H5REF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* All return 0 on success, negative on failure (message: h5ref_error()). */
int h5ref_write(const char *path, int n, const char *const *names, const double *const *data,
                const int64_t dims[3], int as_float32, const int64_t *chunk /* NULL: contiguous */);
int h5ref_dims(const char *path, const char *name, int64_t dims[3]);
int h5ref_read(const char *path, const char *name, double *out, int64_t capacity);
/* Number of objects in the root group and the name/rank/first two dims of
 * object i (a structural probe; rank -1 for objects that are not datasets). */
int h5ref_list(const char *path, int i, char *name, int name_cap, int *rank, int64_t dims[3]);
/* A rank 1-3 contiguous or compact float dataset, as stored (structural
 * checks of files written by other HDF5 implementations). */
int h5ref_read_any(const char *path, const char *name, double *out, int64_t capacity, int *rank, int64_t dims[3]);
const char *h5ref_error(void);

#ifdef __cplusplus
}
#endif
#endif
