/*
 * ORACLE -- test infrastructure.  Implementation of the <hdf5.h> stand-in
 * (see hdf5.h here) over the oracle's own HDF5 subset (h5ref.c, independent
 * of the product's HDF5 code).  Supports the rank-3, float64, unit-stride
 * hyperslab transfers of phasefield.c:996-1109.
 */
#include "hdf5.h"

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "h5ref.h"

enum { K_FREE = 0, K_FILE, K_DSET, K_SPACE };

#define MAXDS 8

typedef struct {
    int kind;
    int closed;
    /* file */
    char path[1024];
    int writing;
    int nds;
    char dsname[MAXDS][64];
    double *dsdata[MAXDS];
    int64_t dsdims[MAXDS][3];
    /* dataset */
    hid_t file;
    int slot;          /* index into the file's dataset list (write) */
    char name[64];
    int64_t dims[3];
    /* dataspace */
    int rank;
    int64_t sdims[3], start[3], count[3];
} obj;

static obj *g_obj;
static hid_t g_n, g_cap;

static hid_t new_obj(int kind)
{
    if (g_n + 1 >= g_cap) {
        g_cap = g_cap ? 2 * g_cap : 64;
        g_obj = (obj *)realloc(g_obj, (size_t)g_cap * sizeof(obj));
    }
    hid_t id = ++g_n;              /* ids start at 1 and are never reused */
    memset(&g_obj[id], 0, sizeof(obj));
    g_obj[id].kind = kind;
    return id;
}

static obj *get(hid_t id, int kind, const char *fn)
{
    if (id <= 0 || id > g_n || g_obj[id].kind != kind || g_obj[id].closed) {
        fprintf(stderr, "HDF5-DIAG (shim): %s: invalid identifier %lld\n", fn, (long long)id);
        return NULL;
    }
    return &g_obj[id];
}

hid_t H5Fopen(const char *name, unsigned flags, hid_t fapl)
{
    (void)flags; (void)fapl;
    FILE *f = fopen(name, "rb");
    if (!f) { fprintf(stderr, "HDF5-DIAG (shim): H5Fopen: cannot open %s\n", name); return -1; }
    fclose(f);
    hid_t id = new_obj(K_FILE);
    snprintf(g_obj[id].path, sizeof g_obj[id].path, "%s", name);
    return id;
}

hid_t H5Fcreate(const char *name, unsigned flags, hid_t fcpl, hid_t fapl)
{
    (void)flags; (void)fcpl; (void)fapl;
    hid_t id = new_obj(K_FILE);
    snprintf(g_obj[id].path, sizeof g_obj[id].path, "%s", name);
    g_obj[id].writing = 1;
    return id;
}

herr_t H5Fclose(hid_t file)
{
    obj *f = get(file, K_FILE, "H5Fclose");
    if (!f) return -1;
    herr_t rc = 0;
    if (f->writing && f->nds > 0) {
        const char *names[MAXDS];
        const double *data[MAXDS];
        for (int i = 0; i < f->nds; ++i) { names[i] = f->dsname[i]; data[i] = f->dsdata[i]; }
        if (h5ref_write(f->path, f->nds, names, data, f->dsdims[0], 0, NULL) != 0) {
            fprintf(stderr, "HDF5-DIAG (shim): H5Fclose: %s\n", h5ref_error());
            rc = -1;
        }
    }
    for (int i = 0; i < f->nds; ++i) free(f->dsdata[i]);
    f->closed = 1;
    return rc;
}

hid_t H5Dopen2(hid_t loc, const char *name, hid_t dapl)
{
    (void)dapl;
    obj *f = get(loc, K_FILE, "H5Dopen2");
    if (!f) return -1;
    int64_t dims[3];
    if (h5ref_dims(f->path, name, dims) != 0) {
        fprintf(stderr, "HDF5-DIAG (shim): H5Dopen2: %s\n", h5ref_error());
        return -1;
    }
    hid_t id = new_obj(K_DSET);
    obj *d = &g_obj[id];
    d->file = loc;
    d->slot = -1;
    snprintf(d->name, sizeof d->name, "%s", name);
    memcpy(d->dims, dims, sizeof dims);
    return id;
}

hid_t H5Dcreate2(hid_t loc, const char *name, hid_t type, hid_t space, hid_t lcpl, hid_t dcpl,
                 hid_t dapl)
{
    (void)type; (void)lcpl; (void)dcpl; (void)dapl;
    obj *f = get(loc, K_FILE, "H5Dcreate2");
    obj *s = get(space, K_SPACE, "H5Dcreate2");
    if (!f || !s || !f->writing || f->nds == MAXDS || s->rank != 3) return -1;
    int slot = f->nds++;
    snprintf(f->dsname[slot], sizeof f->dsname[slot], "%s", name);
    memcpy(f->dsdims[slot], s->sdims, sizeof s->sdims);
    size_t n = (size_t)(s->sdims[0] * s->sdims[1] * s->sdims[2]);
    f->dsdata[slot] = (double *)calloc(n, sizeof(double));
    hid_t id = new_obj(K_DSET);
    obj *d = &g_obj[id];                 /* g_obj may have moved: re-fetch */
    d->file = loc;
    d->slot = slot;
    snprintf(d->name, sizeof d->name, "%s", name);
    memcpy(d->dims, g_obj[loc].dsdims[slot], sizeof d->dims);
    return id;
}

herr_t H5Dclose(hid_t dset)
{
    obj *d = get(dset, K_DSET, "H5Dclose");
    if (!d) return -1;
    d->closed = 1;
    return 0;
}

hid_t H5Screate_simple(int rank, const hsize_t *dims, const hsize_t *maxdims)
{
    (void)maxdims;
    if (rank != 3) return -1;
    hid_t id = new_obj(K_SPACE);
    obj *s = &g_obj[id];
    s->rank = 3;
    for (int i = 0; i < 3; ++i) { s->sdims[i] = (int64_t)dims[i]; s->start[i] = 0; s->count[i] = (int64_t)dims[i]; }
    return id;
}

hid_t H5Dget_space(hid_t dset)
{
    obj *d = get(dset, K_DSET, "H5Dget_space");
    if (!d) return -1;
    hsize_t dims[3] = {(hsize_t)d->dims[0], (hsize_t)d->dims[1], (hsize_t)d->dims[2]};
    return H5Screate_simple(3, dims, NULL);
}

herr_t H5Sselect_hyperslab(hid_t space, int op, const hsize_t *start, const hsize_t *stride,
                           const hsize_t *count, const hsize_t *block)
{
    obj *s = get(space, K_SPACE, "H5Sselect_hyperslab");
    if (!s || op != H5S_SELECT_SET) return -1;
    for (int i = 0; i < 3; ++i) {
        if ((stride && stride[i] != 1) || (block && block[i] != 1)) return -1;
        if (start[i] + count[i] > (hsize_t)s->sdims[i]) return -1;
        s->start[i] = (int64_t)start[i];
        s->count[i] = (int64_t)count[i];
    }
    return 0;
}

herr_t H5Sclose(hid_t space)
{
    obj *s = get(space, K_SPACE, "H5Sclose");
    if (!s) return -1;
    s->closed = 1;
    return 0;
}

/* copy the box `count` from src (dims sd, start ss) to dst (dims dd, start ds) */
static void copy_box(const double *src, const int64_t sd[3], const int64_t ss[3], double *dst,
                     const int64_t dd[3], const int64_t ds[3], const int64_t cnt[3])
{
    for (int64_t i = 0; i < cnt[0]; ++i)
        for (int64_t j = 0; j < cnt[1]; ++j)
            memcpy(dst + ((ds[0] + i) * dd[1] + ds[1] + j) * dd[2] + ds[2],
                   src + ((ss[0] + i) * sd[1] + ss[1] + j) * sd[2] + ss[2],
                   (size_t)cnt[2] * sizeof(double));
}

herr_t H5Dread(hid_t dset, hid_t memtype, hid_t memspace, hid_t filespace, hid_t xfer, void *buf)
{
    (void)xfer;
    obj *d = get(dset, K_DSET, "H5Dread");
    obj *ms = get(memspace, K_SPACE, "H5Dread");
    obj *fs = get(filespace, K_SPACE, "H5Dread");
    if (!d || !ms || !fs || memtype != H5T_IEEE_F64LE) return -1;
    for (int i = 0; i < 3; ++i)
        if (ms->count[i] != fs->count[i]) return -1;
    obj *f = get(d->file, K_FILE, "H5Dread");
    if (!f) return -1;
    size_t n = (size_t)(d->dims[0] * d->dims[1] * d->dims[2]);
    double *tmp = (double *)malloc(n * sizeof(double));
    if (!tmp) return -1;
    if (h5ref_read(f->path, d->name, tmp, (int64_t)n) != 0) {
        fprintf(stderr, "HDF5-DIAG (shim): H5Dread: %s\n", h5ref_error());
        free(tmp);
        return -1;
    }
    copy_box(tmp, d->dims, fs->start, (double *)buf, ms->sdims, ms->start, ms->count);
    free(tmp);
    return 0;
}

herr_t H5Dwrite(hid_t dset, hid_t memtype, hid_t memspace, hid_t filespace, hid_t xfer,
                const void *buf)
{
    (void)xfer;
    obj *d = get(dset, K_DSET, "H5Dwrite");
    obj *ms = get(memspace, K_SPACE, "H5Dwrite");
    obj *fs = get(filespace, K_SPACE, "H5Dwrite");
    if (!d || !ms || !fs || memtype != H5T_IEEE_F64LE || d->slot < 0) return -1;
    for (int i = 0; i < 3; ++i)
        if (ms->count[i] != fs->count[i]) return -1;
    obj *f = get(d->file, K_FILE, "H5Dwrite");
    if (!f) return -1;
    copy_box((const double *)buf, ms->sdims, ms->start, f->dsdata[d->slot], f->dsdims[d->slot],
             fs->start, fs->count);
    return 0;
}
