/*
 * h5lite.c -- the HDF5 subset behind ppf_h5.h (format notes in that header).
 *
 * Written from the public HDF5 File Format Specification (superblock,
 * object header, symbol table, local heap, v1 B-tree, layout, dataspace
 * and datatype message layouts).  The reference's I/O call sites it
 * replaces are phasefield.c:996-1049 (read_hdf5), :1052-1109 (write_hdf5),
 * :481-547 / :550-624 (MPI-IO read/write; chunk = subdomain at :577-579).
 * Plain C99, no dependency beyond libc; addresses are 64-bit throughout.
 */
#define _FILE_OFFSET_BITS 64
#define _POSIX_C_SOURCE 200809L
#include "ppf_h5.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/types.h>

#define UNDEF_ADDR 0xffffffffffffffffULL
/* libhdf5's "end of free list" value in a local heap: offsets are 8-byte
 * aligned, so the odd value 1 can never be a real block. */
#define HEAP_FREE_NULL 1ULL

static __thread char g_err[512];

static int fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

const char *ppf_h5_last_error(void) { return g_err; }

static uint64_t get_le(const uint8_t *p, int n)
{
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}

static void put_le(uint8_t *p, uint64_t v, int n)
{
    for (int i = 0; i < n; ++i) { p[i] = (uint8_t)(v & 0xff); v >>= 8; }
}

/* ------------------------------------------------------------------ */
/* reader                                                             */
/* ------------------------------------------------------------------ */

typedef struct {
    FILE *f;
    uint64_t base;   /* absolute position of the superblock */
    uint64_t fsize;
    int so, sl;      /* size of offsets / lengths */
    uint64_t root;   /* root group object header (relative) */
} rd_t;

static int rd_at(rd_t *r, uint64_t addr, void *buf, size_t n)
{
    if (addr == UNDEF_ADDR || r->base + addr < r->base ||
        r->base + addr + n > r->fsize)
        return fail(PPF_H5_EIO, "h5: read of %zu bytes at address %llu is beyond the end of the file",
                    n, (unsigned long long)addr);
    if (fseeko(r->f, (off_t)(r->base + addr), SEEK_SET) != 0)
        return fail(PPF_H5_EIO, "h5: seek failed");
    if (n && fread(buf, 1, n, r->f) != n)
        return fail(PPF_H5_EIO, "h5: short read");
    return 0;
}

static const uint8_t H5SIG[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};

static int rd_open(rd_t *r, const char *path)
{
    memset(r, 0, sizeof *r);
    r->f = fopen(path, "rb");
    if (!r->f) return fail(PPF_H5_EIO, "h5: cannot open '%s'", path);
    fseeko(r->f, 0, SEEK_END);
    r->fsize = (uint64_t)ftello(r->f);
    /* the superblock sits at 0 or after a user block of 512, 1024, ... */
    uint8_t sb[128];
    uint64_t pos = 0;
    for (;;) {
        if (pos + 8 > r->fsize) return fail(PPF_H5_EFORMAT, "h5: '%s' is not an HDF5 file", path);
        memset(sb, 0, sizeof sb);
        fseeko(r->f, (off_t)pos, SEEK_SET);
        size_t got = fread(sb, 1, sizeof sb, r->f);
        if (got >= 8 && memcmp(sb, H5SIG, 8) == 0) break;
        pos = pos ? pos * 2 : 512;
    }
    r->base = pos;
    int ver = sb[8];
    uint64_t eof = 0;
    if (ver == 0 || ver == 1) {
        r->so = sb[13];
        r->sl = sb[14];
        if ((r->so != 4 && r->so != 8) || (r->sl != 4 && r->sl != 8))
            return fail(PPF_H5_EFORMAT, "h5: unsupported offset/length sizes %d/%d", r->so, r->sl);
        int p = 24 + (ver == 1 ? 4 : 0);
        eof = get_le(sb + p + 2 * r->so, r->so);
        p += 4 * r->so;                       /* base, free-space, EOF, driver */
        /* root group symbol table entry: name offset, object header address */
        r->root = get_le(sb + p + r->so, r->so);
    } else if (ver == 2 || ver == 3) {
        r->so = sb[9];
        r->sl = sb[10];
        if ((r->so != 4 && r->so != 8) || (r->sl != 4 && r->sl != 8))
            return fail(PPF_H5_EFORMAT, "h5: unsupported offset/length sizes %d/%d", r->so, r->sl);
        eof = get_le(sb + 12 + 2 * r->so, r->so);
        int p = 12 + 3 * r->so;               /* base, extension, EOF */
        r->root = get_le(sb + p, r->so);
    } else {
        return fail(PPF_H5_EFORMAT, "h5: unsupported superblock version %d", ver);
    }
    /* like libhdf5, refuse a file shorter than its recorded end of file
     * (the address is relative to the superblock; some writers store it
     * absolute, so only a file shorter than both readings is truncated) */
    if (eof > r->fsize) return fail(PPF_H5_EIO, "h5: '%s' is truncated (%llu of %llu bytes)", path,
                                    (unsigned long long)r->fsize, (unsigned long long)eof);
    return 0;
}

static void rd_close(rd_t *r)
{
    if (r->f) fclose(r->f);
    r->f = NULL;
}

typedef struct {
    uint16_t type;
    uint32_t size;
    const uint8_t *data;
} msg_t;

typedef struct {
    msg_t *m;
    int n, cap;
    uint8_t **bufs;
    int nbufs, capbufs;
} ohdr_t;

static void oh_free(ohdr_t *o)
{
    for (int i = 0; i < o->nbufs; ++i) free(o->bufs[i]);
    free(o->bufs);
    free(o->m);
    memset(o, 0, sizeof *o);
}

static int oh_addmsg(ohdr_t *o, uint16_t type, uint32_t size, const uint8_t *data)
{
    if (o->n == o->cap) {
        o->cap = o->cap ? 2 * o->cap : 16;
        msg_t *m = (msg_t *)realloc(o->m, (size_t)o->cap * sizeof(msg_t));
        if (!m) return fail(PPF_H5_ENOMEM, "h5: out of memory");
        o->m = m;
    }
    o->m[o->n].type = type;
    o->m[o->n].size = size;
    o->m[o->n].data = data;
    o->n++;
    return 0;
}

static uint8_t *oh_readbuf(rd_t *r, ohdr_t *o, uint64_t addr, uint64_t len, int *rc)
{
    if (len > (1ULL << 30)) { *rc = fail(PPF_H5_EFORMAT, "h5: object header chunk too large"); return NULL; }
    uint8_t *b = (uint8_t *)malloc(len ? len : 1);
    if (!b) { *rc = fail(PPF_H5_ENOMEM, "h5: out of memory"); return NULL; }
    if ((*rc = rd_at(r, addr, b, len)) != 0) { free(b); return NULL; }
    if (o->nbufs == o->capbufs) {
        o->capbufs = o->capbufs ? 2 * o->capbufs : 4;
        o->bufs = (uint8_t **)realloc(o->bufs, (size_t)o->capbufs * sizeof(uint8_t *));
    }
    o->bufs[o->nbufs++] = b;
    return b;
}

#define MAX_CHUNKS 64

static int oh_read(rd_t *r, uint64_t addr, ohdr_t *o)
{
    memset(o, 0, sizeof *o);
    uint8_t pre[32];
    int rc = rd_at(r, addr, pre, 16);
    if (rc) return rc;
    uint64_t caddr[MAX_CHUNKS], clen[MAX_CHUNKS];
    int nch = 0, ich = 0;
    if (memcmp(pre, "OHDR", 4) == 0) {
        /* version 2 object header */
        if (pre[4] != 2) return fail(PPF_H5_EFORMAT, "h5: object header version %d", pre[4]);
        int flags = pre[5];
        int p = 6;
        if (flags & 0x20) p += 16;
        if (flags & 0x10) p += 4;
        if ((rc = rd_at(r, addr, pre, (size_t)p + 8)) != 0) return rc;
        int w = 1 << (flags & 3);
        uint64_t len0 = get_le(pre + p, w);
        p += w;
        int mhdr = 4 + ((flags & 0x04) ? 2 : 0);
        caddr[0] = addr + (uint64_t)p;
        clen[0] = len0;
        nch = 1;
        while (ich < nch) {
            uint8_t *b = oh_readbuf(r, o, caddr[ich], clen[ich], &rc);
            if (!b) return rc;
            uint64_t q = 0, end = clen[ich];
            if (ich > 0) {
                if (end < 8 || memcmp(b, "OCHK", 4) != 0)
                    return fail(PPF_H5_EFORMAT, "h5: bad continuation block");
                q = 4;
                end -= 4;            /* checksum */
            }
            while (q + (uint64_t)mhdr <= end) {
                uint16_t type = b[q];
                uint32_t sz = (uint32_t)get_le(b + q + 1, 2);
                q += (uint64_t)mhdr;
                if (q + sz > end) return fail(PPF_H5_EFORMAT, "h5: truncated header message");
                if ((rc = oh_addmsg(o, type, sz, b + q)) != 0) return rc;
                if (type == 0x10) {
                    if (nch == MAX_CHUNKS) return fail(PPF_H5_EFORMAT, "h5: too many header chunks");
                    caddr[nch] = get_le(b + q, r->so);
                    clen[nch] = get_le(b + q + r->so, r->sl);
                    nch++;
                }
                q += sz;
            }
            ich++;
        }
        return 0;
    }
    if (pre[0] != 1) return fail(PPF_H5_EFORMAT, "h5: object header version %d", pre[0]);
    uint64_t hsize = get_le(pre + 8, 4);
    caddr[0] = addr + 16;
    clen[0] = hsize;
    nch = 1;
    while (ich < nch) {
        uint8_t *b = oh_readbuf(r, o, caddr[ich], clen[ich], &rc);
        if (!b) return rc;
        uint64_t q = 0, end = clen[ich];
        while (q + 8 <= end) {
            uint16_t type = (uint16_t)get_le(b + q, 2);
            uint32_t sz = (uint32_t)get_le(b + q + 2, 2);
            q += 8;
            if (q + sz > end) return fail(PPF_H5_EFORMAT, "h5: truncated header message");
            if ((rc = oh_addmsg(o, type, sz, b + q)) != 0) return rc;
            if (type == 0x10) {
                if (nch == MAX_CHUNKS) return fail(PPF_H5_EFORMAT, "h5: too many header chunks");
                caddr[nch] = get_le(b + q, r->so);
                clen[nch] = get_le(b + q + r->so, r->sl);
                nch++;
            }
            q += sz;
        }
        ich++;
    }
    return 0;
}

static const msg_t *oh_find(const ohdr_t *o, uint16_t type)
{
    for (int i = 0; i < o->n; ++i)
        if (o->m[i].type == type) return &o->m[i];
    return NULL;
}

/* Search a v1 group B-tree (type 0) for `name`; *found = object header. */
static int symtab_lookup(rd_t *r, uint64_t node, const uint8_t *heap, uint64_t heapsz,
                         const char *name, uint64_t *found, int depth)
{
    if (depth > 32) return fail(PPF_H5_EFORMAT, "h5: group B-tree too deep");
    uint8_t hdr[64];
    int rc = rd_at(r, node, hdr, 8 + 2 * (size_t)r->so);
    if (rc) return rc;
    if (memcmp(hdr, "TREE", 4) != 0 || hdr[4] != 0)
        return fail(PPF_H5_EFORMAT, "h5: bad group B-tree node");
    int level = hdr[5];
    int nused = (int)get_le(hdr + 6, 2);
    size_t es = (size_t)r->sl + (size_t)r->so;
    size_t bytes = (size_t)nused * es + (size_t)r->sl;
    uint8_t *b = (uint8_t *)malloc(bytes);
    if (!b) return fail(PPF_H5_ENOMEM, "h5: out of memory");
    if ((rc = rd_at(r, node + 8 + 2 * (uint64_t)r->so, b, bytes)) != 0) { free(b); return rc; }
    for (int i = 0; i < nused && !*found; ++i) {
        uint64_t child = get_le(b + (size_t)i * es + r->sl, r->so);
        if (level > 0) {
            if ((rc = symtab_lookup(r, child, heap, heapsz, name, found, depth + 1)) != 0) break;
            continue;
        }
        uint8_t sh[8];
        if ((rc = rd_at(r, child, sh, 8)) != 0) break;
        if (memcmp(sh, "SNOD", 4) != 0) { rc = fail(PPF_H5_EFORMAT, "h5: bad symbol table node"); break; }
        int nsym = (int)get_le(sh + 6, 2);
        size_t ent = 2 * (size_t)r->so + 24;
        uint8_t *e = (uint8_t *)malloc((size_t)nsym * ent + 1);
        if (!e) { rc = fail(PPF_H5_ENOMEM, "h5: out of memory"); break; }
        if ((rc = rd_at(r, child + 8, e, (size_t)nsym * ent)) != 0) { free(e); break; }
        for (int s = 0; s < nsym; ++s) {
            uint64_t off = get_le(e + (size_t)s * ent, r->so);
            if (off >= heapsz) continue;
            const char *nm = (const char *)heap + off;
            if ((uint64_t)strnlen(nm, heapsz - off) < heapsz - off && strcmp(nm, name) == 0) {
                *found = get_le(e + (size_t)s * ent + r->so, r->so);
                break;
            }
        }
        free(e);
    }
    free(b);
    return rc;
}

static int group_lookup(rd_t *r, uint64_t group, const char *name, uint64_t *out)
{
    ohdr_t o;
    int rc = oh_read(r, group, &o);
    if (rc) { oh_free(&o); return rc; }
    uint64_t found = 0;
    const msg_t *st = oh_find(&o, 0x11);
    if (st) {
        uint64_t bt = get_le(st->data, r->so);
        uint64_t hp = get_le(st->data + r->so, r->so);
        uint8_t hh[64];
        if ((rc = rd_at(r, hp, hh, 8 + 2 * (size_t)r->sl + r->so)) != 0) { oh_free(&o); return rc; }
        if (memcmp(hh, "HEAP", 4) != 0) { oh_free(&o); return fail(PPF_H5_EFORMAT, "h5: bad local heap"); }
        uint64_t hsz = get_le(hh + 8, r->sl);
        uint64_t hda = get_le(hh + 8 + 2 * r->sl, r->so);
        if (hsz > (1ULL << 30)) { oh_free(&o); return fail(PPF_H5_EFORMAT, "h5: local heap too large"); }
        uint8_t *heap = (uint8_t *)malloc(hsz + 1);
        if (!heap) { oh_free(&o); return fail(PPF_H5_ENOMEM, "h5: out of memory"); }
        if ((rc = rd_at(r, hda, heap, hsz)) == 0)
            rc = symtab_lookup(r, bt, heap, hsz, name, &found, 0);
        free(heap);
        if (rc) { oh_free(&o); return rc; }
    }
    int dense = 0;
    for (int i = 0; i < o.n && !found; ++i) {
        const msg_t *m = &o.m[i];
        if (m->type == 0x02) {          /* link info: dense storage address */
            int fl = m->data[1];
            const uint8_t *p = m->data + 2 + ((fl & 1) ? 8 : 0);
            if (get_le(p, r->so) != (r->so == 8 ? UNDEF_ADDR : 0xffffffffULL)) dense = 1;
            continue;
        }
        if (m->type != 0x06) continue;  /* link message */
        const uint8_t *p = m->data;
        int fl = p[1];
        p += 2;
        int ltype = 0;
        if (fl & 0x08) ltype = *p++;
        if (fl & 0x04) p += 8;
        if (fl & 0x10) p += 1;
        int w = 1 << (fl & 3);
        uint64_t nlen = get_le(p, w);
        p += w;
        if (nlen == strlen(name) && memcmp(p, name, nlen) == 0) {
            if (ltype != 0) { oh_free(&o); return fail(PPF_H5_EFORMAT, "h5: '%s' is not a hard link", name); }
            found = get_le(p + nlen, r->so);
        }
    }
    oh_free(&o);
    if (!found) {
        if (dense) return fail(PPF_H5_EFORMAT, "h5: group uses dense link storage (unsupported)");
        return fail(PPF_H5_ENOTFOUND, "h5: no dataset '%s'", name);
    }
    *out = found;
    return 0;
}

typedef struct {
    int64_t dims[3];
    int esize;        /* 4 or 8 */
    int big_endian;
    int lclass;       /* 0 compact, 1 contiguous, 2 chunked */
    uint64_t addr;    /* contiguous data / chunk index / single chunk */
    const uint8_t *compact;
    uint64_t compact_size;
    int chunk_index;  /* 0: v1 B-tree, 1: single chunk, 2: implicit */
    int64_t cdims[3];
} dset_t;

static int dset_info(rd_t *r, const char *path_name, ohdr_t *o, dset_t *d)
{
    memset(o, 0, sizeof *o);
    memset(d, 0, sizeof *d);
    const char *name = path_name;
    while (*name == '/') ++name;
    if (!*name || strchr(name, '/')) return fail(PPF_H5_EARG, "h5: dataset name '%s' must be a root-level name", path_name);
    uint64_t addr = 0;
    int rc = group_lookup(r, r->root, name, &addr);
    if (rc) return rc;
    if ((rc = oh_read(r, addr, o)) != 0) return rc;
    const msg_t *sp = oh_find(o, 0x01), *ty = oh_find(o, 0x03), *ly = oh_find(o, 0x08);
    if (!sp || !ty || !ly) return fail(PPF_H5_EFORMAT, "h5: '%s' is not a dataset", name);
    const msg_t *fp = oh_find(o, 0x0B);
    if (fp && fp->size >= 2 && fp->data[1] > 0)
        return fail(PPF_H5_EFORMAT, "h5: dataset '%s' is filtered/compressed (unsupported)", name);
    /* dataspace */
    int sver = sp->data[0], rank = sp->data[1];
    if (rank != 3) return fail(PPF_H5_EDIMS, "h5: dataset '%s' has rank %d, expected 3", name, rank);
    const uint8_t *dp = sp->data + (sver == 1 ? 8 : 4);
    for (int i = 0; i < 3; ++i) d->dims[i] = (int64_t)get_le(dp + (size_t)i * r->sl, r->sl);
    /* datatype */
    int tclass = ty->data[0] & 0x0f;
    if (tclass != 1) return fail(PPF_H5_ETYPE, "h5: dataset '%s' is not floating point (class %d)", name, tclass);
    if (ty->data[1] & 0x40) return fail(PPF_H5_ETYPE, "h5: VAX float order unsupported");
    d->big_endian = ty->data[1] & 1;
    d->esize = (int)get_le(ty->data + 4, 4);
    if (d->esize != 4 && d->esize != 8) return fail(PPF_H5_ETYPE, "h5: float size %d unsupported", d->esize);
    int prec = (int)get_le(ty->data + 10, 2);
    if (prec != 8 * d->esize) return fail(PPF_H5_ETYPE, "h5: float precision %d unsupported", prec);
    /* layout */
    const uint8_t *l = ly->data;
    int lver = l[0];
    if (lver == 1 || lver == 2) {
        int nd = l[1];
        d->lclass = l[2];
        const uint8_t *p = l + 8;
        if (d->lclass != 0) { d->addr = get_le(p, r->so); p += r->so; }
        if (d->lclass == 2) {
            if (nd != 4) return fail(PPF_H5_EDIMS, "h5: chunk rank mismatch");
            for (int i = 0; i < 3; ++i) d->cdims[i] = (int64_t)get_le(p + 4 * i, 4);
        }
        p += 4 * nd;
        if (d->lclass == 0) { d->compact_size = get_le(p, 4); d->compact = p + 4; }
    } else if (lver == 3 || lver == 4) {
        d->lclass = l[1];
        const uint8_t *p = l + 2;
        if (d->lclass == 0) {
            d->compact_size = get_le(p, 2);
            d->compact = p + 2;
        } else if (d->lclass == 1) {
            d->addr = get_le(p, r->so);
        } else if (d->lclass == 2 && lver == 3) {
            int nd = p[0];
            if (nd != 4) return fail(PPF_H5_EDIMS, "h5: chunk rank mismatch");
            d->addr = get_le(p + 1, r->so);
            for (int i = 0; i < 3; ++i) d->cdims[i] = (int64_t)get_le(p + 1 + r->so + 4 * i, 4);
        } else if (d->lclass == 2) {
            int flags = p[0], nd = p[1], enc = p[2];
            if (nd != 4) return fail(PPF_H5_EDIMS, "h5: chunk rank mismatch");
            p += 3;
            for (int i = 0; i < 3; ++i) d->cdims[i] = (int64_t)get_le(p + (size_t)enc * i, enc);
            p += (size_t)enc * nd;
            int idx = *p++;
            if (idx == 1) {
                if (flags & 2) return fail(PPF_H5_EFORMAT, "h5: filtered single chunk unsupported");
                d->chunk_index = 1;
            } else if (idx == 2) {
                d->chunk_index = 2;
            } else {
                return fail(PPF_H5_EFORMAT, "h5: chunk index type %d unsupported", idx);
            }
            d->addr = get_le(p, r->so);
        } else {
            return fail(PPF_H5_EFORMAT, "h5: layout class %d unsupported", d->lclass);
        }
    } else {
        return fail(PPF_H5_EFORMAT, "h5: layout version %d unsupported", lver);
    }
    for (int i = 0; i < 3; ++i)
        if (d->dims[i] <= 0 || d->dims[i] > (1 << 20) || (d->lclass == 2 && d->cdims[i] <= 0))
            return fail(PPF_H5_EDIMS, "h5: bad dimensions in '%s'", name);
    return 0;
}

static void convert(const uint8_t *src, double *dst, int64_t n, int esize, int be)
{
    for (int64_t i = 0; i < n; ++i) {
        uint8_t b[8];
        const uint8_t *s = src + i * esize;
        for (int k = 0; k < esize; ++k) b[k] = be ? s[esize - 1 - k] : s[k];
        if (esize == 8) { double v; memcpy(&v, b, 8); dst[i] = v; }
        else { float v; memcpy(&v, b, 4); dst[i] = (double)v; }
    }
}

/* copy one chunk (offset off[], full chunk dims cd[]) into out[] */
static int put_chunk(rd_t *r, const dset_t *d, uint64_t addr, const int64_t off[3], double *out)
{
    const int64_t *cd = d->cdims;
    int64_t n = cd[0] * cd[1] * cd[2];
    uint8_t *raw = (uint8_t *)malloc((size_t)(n * d->esize));
    if (!raw) return fail(PPF_H5_ENOMEM, "h5: out of memory");
    int rc = rd_at(r, addr, raw, (size_t)(n * d->esize));
    if (rc) { free(raw); return rc; }
    double *row = (double *)malloc((size_t)cd[2] * sizeof(double));
    if (!row) { free(raw); return fail(PPF_H5_ENOMEM, "h5: out of memory"); }
    for (int64_t i = 0; i < cd[0] && off[0] + i < d->dims[0]; ++i)
        for (int64_t j = 0; j < cd[1] && off[1] + j < d->dims[1]; ++j) {
            int64_t nk = cd[2];
            if (off[2] + nk > d->dims[2]) nk = d->dims[2] - off[2];
            if (nk <= 0) continue;
            convert(raw + ((i * cd[1] + j) * cd[2]) * d->esize, row, nk, d->esize, d->big_endian);
            memcpy(out + ((off[0] + i) * d->dims[1] + off[1] + j) * d->dims[2] + off[2], row,
                   (size_t)nk * sizeof(double));
        }
    free(row);
    free(raw);
    return 0;
}

static int chunk_btree(rd_t *r, const dset_t *d, uint64_t node, double *out, int depth)
{
    if (depth > 32) return fail(PPF_H5_EFORMAT, "h5: chunk B-tree too deep");
    uint8_t hdr[64];
    int rc = rd_at(r, node, hdr, 8 + 2 * (size_t)r->so);
    if (rc) return rc;
    if (memcmp(hdr, "TREE", 4) != 0 || hdr[4] != 1) return fail(PPF_H5_EFORMAT, "h5: bad chunk B-tree node");
    int level = hdr[5], nused = (int)get_le(hdr + 6, 2);
    size_t ks = 8 + 4 * 8, es = ks + (size_t)r->so;
    size_t bytes = (size_t)nused * es + ks;
    uint8_t *b = (uint8_t *)malloc(bytes);
    if (!b) return fail(PPF_H5_ENOMEM, "h5: out of memory");
    if ((rc = rd_at(r, node + 8 + 2 * (uint64_t)r->so, b, bytes)) != 0) { free(b); return rc; }
    for (int i = 0; i < nused && !rc; ++i) {
        const uint8_t *k = b + (size_t)i * es;
        uint64_t child = get_le(k + ks, r->so);
        if (level > 0) { rc = chunk_btree(r, d, child, out, depth + 1); continue; }
        if (get_le(k + 4, 4) != 0) { rc = fail(PPF_H5_EFORMAT, "h5: filtered chunk unsupported"); break; }
        int64_t off[3];
        int bad = 0;
        for (int q = 0; q < 3; ++q) {
            const uint64_t u = get_le(k + 8 + 8 * q, 8);
            /* a chunk origin is a multiple of the chunk size inside the
             * dataset; anything else would place the copy outside `out` */
            if (u >= (uint64_t)d->dims[q] || u % (uint64_t)d->cdims[q] != 0) bad = 1;
            off[q] = (int64_t)u;
        }
        if (bad) { rc = fail(PPF_H5_EFORMAT, "h5: chunk offset outside the dataset or off the chunk grid"); break; }
        rc = put_chunk(r, d, child, off, out);
    }
    free(b);
    return rc;
}

int ppf_h5_dims(const char *path, const char *name, int64_t dims[3])
{
    if (!path || !name || !dims) return fail(PPF_H5_EARG, "h5: null argument");
    rd_t r;
    int rc = rd_open(&r, path);
    if (!rc) {
        ohdr_t o;
        dset_t d;
        rc = dset_info(&r, name, &o, &d);
        if (!rc) memcpy(dims, d.dims, sizeof d.dims);
        oh_free(&o);
    }
    rd_close(&r);
    return rc;
}

int ppf_h5_read3d(const char *path, const char *name, int64_t dims[3], double *out, int64_t capacity)
{
    if (!path || !name || !dims || !out) return fail(PPF_H5_EARG, "h5: null argument");
    rd_t r;
    int rc = rd_open(&r, path);
    ohdr_t o;
    memset(&o, 0, sizeof o);
    dset_t d;
    if (!rc) rc = dset_info(&r, name, &o, &d);
    if (!rc) {
        memcpy(dims, d.dims, sizeof d.dims);
        int64_t n = d.dims[0] * d.dims[1] * d.dims[2];
        if (n > capacity) {
            rc = fail(PPF_H5_EDIMS, "h5: dataset '%s' has %lld elements, buffer holds %lld", name,
                      (long long)n, (long long)capacity);
        } else if (d.lclass == 0) {
            if (d.compact_size < (uint64_t)(n * d.esize)) rc = fail(PPF_H5_EFORMAT, "h5: short compact data");
            else convert(d.compact, out, n, d.esize, d.big_endian);
        } else if (d.lclass == 1) {
            if (d.addr == UNDEF_ADDR) {
                memset(out, 0, (size_t)n * sizeof(double));   /* never written: fill value 0 */
            } else if (d.esize == 8 && !d.big_endian) {
                rc = rd_at(&r, d.addr, out, (size_t)n * 8);
            } else {
                const int64_t blk = 1 << 20;
                uint8_t *raw = (uint8_t *)malloc((size_t)(blk * d.esize));
                for (int64_t s = 0; s < n && !rc; s += blk) {
                    int64_t m = n - s < blk ? n - s : blk;
                    rc = rd_at(&r, d.addr + (uint64_t)(s * d.esize), raw, (size_t)(m * d.esize));
                    if (!rc) convert(raw, out + s, m, d.esize, d.big_endian);
                }
                free(raw);
            }
        } else {
            memset(out, 0, (size_t)n * sizeof(double));       /* missing chunks read as 0 */
            if (d.chunk_index == 0) {
                if (d.addr != UNDEF_ADDR) rc = chunk_btree(&r, &d, d.addr, out, 0);
            } else if (d.chunk_index == 1) {
                int64_t off[3] = {0, 0, 0};
                if (d.addr != UNDEF_ADDR) rc = put_chunk(&r, &d, d.addr, off, out);
            } else {
                int64_t nc[3];
                for (int q = 0; q < 3; ++q) nc[q] = (d.dims[q] + d.cdims[q] - 1) / d.cdims[q];
                uint64_t csz = (uint64_t)(d.cdims[0] * d.cdims[1] * d.cdims[2] * d.esize);
                uint64_t a = d.addr;
                for (int64_t i = 0; i < nc[0] && !rc; ++i)
                    for (int64_t j = 0; j < nc[1] && !rc; ++j)
                        for (int64_t k = 0; k < nc[2] && !rc; ++k, a += csz) {
                            int64_t off[3] = {i * d.cdims[0], j * d.cdims[1], k * d.cdims[2]};
                            rc = put_chunk(&r, &d, a, off, out);
                        }
            }
        }
    }
    oh_free(&o);
    rd_close(&r);
    return rc;
}

/* ------------------------------------------------------------------ */
/* writer: superblock v0, symbol-table root group, v1 object headers  */
/* ------------------------------------------------------------------ */

#define LEAF_K 4        /* group leaf node K: a symbol node holds 2K = 8 entries */
#define GROUP_K 16      /* group internal node K */
#define CHUNK_K 32      /* indexed-storage K (fixed for superblock v0) */

static uint64_t round8(uint64_t v) { return (v + 7) & ~7ULL; }

static int wr_bytes(FILE *f, uint64_t *pos, const void *b, uint64_t n)
{
    if (n && fwrite(b, 1, (size_t)n, f) != n) return fail(PPF_H5_EIO, "h5: write failed");
    *pos += n;
    return 0;
}

/* one v1 object-header message: 8-byte header, data padded to 8 */
static size_t put_msg(uint8_t *p, uint16_t type, uint8_t flags, const uint8_t *data, size_t n)
{
    size_t padded = (size_t)round8(n);
    put_le(p, type, 2);
    put_le(p + 2, padded, 2);
    p[4] = flags;
    p[5] = p[6] = p[7] = 0;
    memset(p + 8, 0, padded);
    memcpy(p + 8, data, n);
    return 8 + padded;
}

static size_t chunk_node_size(void)
{
    /* header + (2K+1) keys of (4 + 4 + 4*8) bytes + 2K child addresses */
    return 24 + (2 * CHUNK_K + 1) * 40 + 2 * CHUNK_K * 8;
}

typedef struct {
    int64_t off[3];
    uint64_t addr;
} chunk_ent;

/* object header of one rank-3 float dataset: dataspace, datatype, fill
 * value, layout (contiguous at `addr` with `bytes`, or chunked with its
 * B-tree at `addr`); returns the header size */
static uint64_t ds_header_size(int chunked) { return 16 + (8 + 32) + (8 + 24) + (8 + 8) + (8 + (chunked ? 32 : 24)); }

static void ds_header(uint8_t *buf, const int64_t d[3], int es, const int64_t *chunk, uint64_t addr, uint64_t bytes)
{
    const uint64_t sz = ds_header_size(chunk != NULL);
    memset(buf, 0, sz);
    buf[0] = 1;
    put_le(buf + 2, 4, 2);
    put_le(buf + 4, 1, 4);
    put_le(buf + 8, sz - 16, 4);
    size_t p = 16;
    uint8_t m[64];
    memset(m, 0, sizeof m);                    /* dataspace v1, rank 3 */
    m[0] = 1; m[1] = 3;
    for (int q = 0; q < 3; ++q) put_le(m + 8 + 8 * q, (uint64_t)d[q], 8);
    p += put_msg(buf + p, 0x0001, 0, m, 32);
    memset(m, 0, sizeof m);                    /* datatype v1, IEEE float LE */
    m[0] = 0x11;
    m[1] = 0x20;                               /* mantissa normalisation: implied MSB */
    m[2] = (uint8_t)(es * 8 - 1);              /* sign bit position */
    put_le(m + 4, (uint64_t)es, 4);
    put_le(m + 8, 0, 2);
    put_le(m + 10, (uint64_t)es * 8, 2);
    m[12] = es == 8 ? 52 : 23;                 /* exponent location */
    m[13] = es == 8 ? 11 : 8;                  /* exponent size */
    m[14] = 0;                                 /* mantissa location */
    m[15] = es == 8 ? 52 : 23;                 /* mantissa size */
    put_le(m + 16, es == 8 ? 1023 : 127, 4);
    p += put_msg(buf + p, 0x0003, 1, m, 20);
    memset(m, 0, sizeof m);                    /* fill value v2: early, never, undefined */
    m[0] = 2; m[1] = 1; m[2] = 2; m[3] = 0;
    p += put_msg(buf + p, 0x0005, 1, m, 4);
    memset(m, 0, sizeof m);                    /* layout v3 */
    m[0] = 3;
    if (!chunk) {
        m[1] = 1;
        put_le(m + 2, addr, 8);
        put_le(m + 10, bytes, 8);
        put_msg(buf + p, 0x0008, 0, m, 18);
    } else {
        m[1] = 2;
        m[2] = 4;
        put_le(m + 3, addr, 8);
        for (int q = 0; q < 3; ++q) put_le(m + 11 + 4 * q, (uint64_t)chunk[q], 4);
        put_le(m + 23, (uint64_t)es, 4);
        put_msg(buf + p, 0x0008, 0, m, 27);
    }
}

int ppf_h5_write3d(const char *path, int n, const char *const *names, const double *const *data,
                   const int64_t dims[3], int dtype, const int64_t *chunk)
{
    return ppf_h5_write3d_meta(path, n, names, data, dims, dtype, chunk, NULL, NULL, 0);
}

int ppf_h5_write3d_meta(const char *path, int n, const char *const *names, const double *const *data,
                        const int64_t dims[3], int dtype, const int64_t *chunk, const char *meta_name,
                        const double *meta, int nmeta)
{
    if (!path || !names || !data || !dims || n < 1) return fail(PPF_H5_EARG, "h5: bad argument");
    const int has_meta = meta_name != NULL;
    if (has_meta && (!meta || nmeta < 1 || nmeta > 4096)) return fail(PPF_H5_EARG, "h5: bad metadata");
    const int nt = n + has_meta;                   /* datasets in the file: fields, then the metadata */
    const char *all[2 * LEAF_K + 1];
    if (nt > 2 * LEAF_K) return fail(PPF_H5_EARG, "h5: at most %d datasets per file", 2 * LEAF_K);
    for (int i = 0; i < n; ++i) all[i] = names[i];
    if (has_meta) all[n] = meta_name;
    if (dtype != PPF_H5_F64 && dtype != PPF_H5_F32) return fail(PPF_H5_EARG, "h5: bad dtype");
    for (int i = 0; i < 3; ++i) {
        if (dims[i] <= 0) return fail(PPF_H5_EDIMS, "h5: bad dims");
        if (chunk && (chunk[i] <= 0 || chunk[i] > dims[i])) return fail(PPF_H5_EDIMS, "h5: bad chunk dims");
    }
    for (int i = 0; i < nt; ++i) {
        if (!all[i] || !all[i][0] || strlen(all[i]) > 255 || strchr(all[i], '/'))
            return fail(PPF_H5_EARG, "h5: bad dataset name");
        for (int j = 0; j < i; ++j)
            if (strcmp(all[i], all[j]) == 0) return fail(PPF_H5_EARG, "h5: duplicate dataset name");
    }
    const int es = dtype == PPF_H5_F64 ? 8 : 4;
    const int64_t nel = dims[0] * dims[1] * dims[2];

    /* sorted order of names (symbol nodes must be sorted by name) */
    int order[2 * LEAF_K];
    for (int i = 0; i < nt; ++i) order[i] = i;
    for (int i = 1; i < nt; ++i)
        for (int j = i; j > 0 && strcmp(all[order[j - 1]], all[order[j]]) > 0; --j) {
            int t = order[j]; order[j] = order[j - 1]; order[j - 1] = t;
        }

    /* ---- plan addresses ---- */
    const uint64_t A_ROOT = 96;                         /* superblock v0 is 96 bytes */
    const uint64_t ROOT_SZ = 16 + 8 + 16;
    const uint64_t A_HEAP = A_ROOT + ROOT_SZ;
    const uint64_t A_HEAPDATA = A_HEAP + 32;
    uint64_t name_off[2 * LEAF_K];
    uint64_t hs = 8;                                    /* offset 0: the empty name */
    for (int s = 0; s < nt; ++s) { name_off[order[s]] = hs; hs += round8(strlen(all[order[s]]) + 1); }
    const uint64_t A_BTREE = A_HEAPDATA + hs;
    const uint64_t BTREE_SZ = 24 + (2 * GROUP_K + 1) * 8 + 2 * GROUP_K * 8;
    const uint64_t A_SNOD = A_BTREE + BTREE_SZ;
    const uint64_t SNOD_SZ = 8 + 2 * LEAF_K * 40;

    /* dataset object header: dataspace 32, datatype 24, fill 8, layout 24|32 (+8 each header) */
    const uint64_t DS_SZ = ds_header_size(chunk != NULL);
    uint64_t a_ds[2 * LEAF_K];
    uint64_t pos = A_SNOD + SNOD_SZ;
    for (int i = 0; i < n; ++i) { a_ds[i] = pos; pos += DS_SZ; }
    if (has_meta) { a_ds[n] = pos; pos += ds_header_size(0); }

    /* chunk index plan */
    int64_t ncd[3] = {1, 1, 1}, nchunks = 1, csz = 0;
    int nlevels = 0;
    int64_t nodes_per_level[8] = {0};
    uint64_t idx_bytes = 0;
    if (chunk) {
        for (int q = 0; q < 3; ++q) { ncd[q] = (dims[q] + chunk[q] - 1) / chunk[q]; nchunks *= ncd[q]; }
        csz = chunk[0] * chunk[1] * chunk[2] * es;
        int64_t cnt = nchunks;
        do {
            int64_t nodes = (cnt + 2 * CHUNK_K - 1) / (2 * CHUNK_K);
            if (nlevels == 8) return fail(PPF_H5_EDIMS, "h5: too many chunks");
            nodes_per_level[nlevels++] = nodes;
            idx_bytes += (uint64_t)nodes * chunk_node_size();
            cnt = nodes;
        } while (cnt > 1);
    }
    uint64_t a_idx[2 * LEAF_K], a_data[2 * LEAF_K];
    for (int i = 0; i < n; ++i) {
        a_idx[i] = chunk ? pos : UNDEF_ADDR;
        pos += idx_bytes;
    }
    for (int i = 0; i < n; ++i) {
        a_data[i] = pos;
        pos += chunk ? (uint64_t)(nchunks * csz) : (uint64_t)(nel * es);
    }
    uint64_t a_meta = 0;
    if (has_meta) { a_meta = pos; pos += (uint64_t)nmeta * 8; }
    const uint64_t eof = pos;

    FILE *f = fopen(path, "wb");
    if (!f) return fail(PPF_H5_EIO, "h5: cannot create '%s'", path);
    uint64_t w = 0;
    int rc = 0;
    uint8_t buf[4096];

    /* ---- superblock v0 ---- */
    memset(buf, 0, 96);
    memcpy(buf, H5SIG, 8);
    buf[13] = 8;                                      /* size of offsets */
    buf[14] = 8;                                      /* size of lengths */
    put_le(buf + 16, LEAF_K, 2);
    put_le(buf + 18, GROUP_K, 2);
    put_le(buf + 24, 0, 8);                           /* base address */
    put_le(buf + 32, UNDEF_ADDR, 8);                  /* free-space info */
    put_le(buf + 40, eof, 8);                         /* end of file */
    put_le(buf + 48, UNDEF_ADDR, 8);                  /* driver info */
    put_le(buf + 56, 0, 8);                           /* root entry: name offset */
    put_le(buf + 64, A_ROOT, 8);                      /*   object header */
    put_le(buf + 72, 1, 4);                           /*   cache type 1 */
    put_le(buf + 80, A_BTREE, 8);                     /*   scratch: B-tree */
    put_le(buf + 88, A_HEAP, 8);                      /*   scratch: heap */
    rc = wr_bytes(f, &w, buf, 96);

    /* ---- root group object header: one symbol-table message ---- */
    if (!rc) {
        memset(buf, 0, ROOT_SZ);
        buf[0] = 1;
        put_le(buf + 2, 1, 2);
        put_le(buf + 4, 1, 4);
        put_le(buf + 8, 8 + 16, 4);
        uint8_t st[16];
        put_le(st, A_BTREE, 8);
        put_le(st + 8, A_HEAP, 8);
        put_msg(buf + 16, 0x11, 1, st, 16);
        rc = wr_bytes(f, &w, buf, ROOT_SZ);
    }
    /* ---- local heap + names ---- */
    if (!rc) {
        memset(buf, 0, 32);
        memcpy(buf, "HEAP", 4);
        put_le(buf + 8, hs, 8);
        put_le(buf + 16, HEAP_FREE_NULL, 8);
        put_le(buf + 24, A_HEAPDATA, 8);
        rc = wr_bytes(f, &w, buf, 32);
    }
    if (!rc) {
        memset(buf, 0, hs);
        for (int i = 0; i < nt; ++i) memcpy(buf + name_off[i], all[i], strlen(all[i]));
        rc = wr_bytes(f, &w, buf, hs);
    }
    /* ---- group B-tree: one leaf pointing at one symbol node ---- */
    if (!rc) {
        memset(buf, 0, BTREE_SZ);
        memcpy(buf, "TREE", 4);
        buf[4] = 0;
        buf[5] = 0;
        put_le(buf + 6, 1, 2);
        put_le(buf + 8, UNDEF_ADDR, 8);
        put_le(buf + 16, UNDEF_ADDR, 8);
        put_le(buf + 24, 0, 8);                        /* key 0: "" */
        put_le(buf + 32, A_SNOD, 8);                   /* child 0 */
        put_le(buf + 40, name_off[order[nt - 1]], 8);  /* key 1: largest name */
        rc = wr_bytes(f, &w, buf, BTREE_SZ);
    }
    /* ---- symbol table node ---- */
    if (!rc) {
        memset(buf, 0, SNOD_SZ);
        memcpy(buf, "SNOD", 4);
        buf[4] = 1;
        put_le(buf + 6, (uint64_t)nt, 2);
        for (int s = 0; s < nt; ++s) {
            uint8_t *e = buf + 8 + 40 * s;
            put_le(e, name_off[order[s]], 8);
            put_le(e + 8, a_ds[order[s]], 8);
        }
        rc = wr_bytes(f, &w, buf, SNOD_SZ);
    }
    /* ---- dataset object headers ---- */
    for (int i = 0; i < n && !rc; ++i) {
        ds_header(buf, dims, es, chunk, chunk ? a_idx[i] : a_data[i], (uint64_t)(nel * es));
        rc = wr_bytes(f, &w, buf, DS_SZ);
    }
    if (has_meta && !rc) {
        const int64_t md[3] = {1, 1, nmeta};
        ds_header(buf, md, 8, NULL, a_meta, (uint64_t)nmeta * 8);
        rc = wr_bytes(f, &w, buf, ds_header_size(0));
    }
    /* ---- chunk B-trees (one per dataset, levels bottom-up) ---- */
    if (chunk && !rc) {
        chunk_ent *cur = (chunk_ent *)malloc((size_t)nchunks * sizeof(chunk_ent));
        chunk_ent *nxt = (chunk_ent *)malloc((size_t)nchunks * sizeof(chunk_ent));
        uint8_t *node = (uint8_t *)malloc(chunk_node_size());
        if (!cur || !nxt || !node) rc = fail(PPF_H5_ENOMEM, "h5: out of memory");
        for (int i = 0; i < n && !rc; ++i) {
            int64_t c = 0;
            for (int64_t a = 0; a < ncd[0]; ++a)
                for (int64_t b = 0; b < ncd[1]; ++b)
                    for (int64_t d = 0; d < ncd[2]; ++d, ++c) {
                        cur[c].off[0] = a * chunk[0];
                        cur[c].off[1] = b * chunk[1];
                        cur[c].off[2] = d * chunk[2];
                        cur[c].addr = a_data[i] + (uint64_t)(c * csz);
                    }
            int64_t cnt = nchunks;
            /* the right bound of the whole tree: one past the last chunk */
            int64_t endkey[3] = {cur[cnt - 1].off[0] + chunk[0], cur[cnt - 1].off[1] + chunk[1],
                                 cur[cnt - 1].off[2] + chunk[2]};
            /* the root (top level) must sit at a_idx[i], where the layout message
             * points: lay the levels out root first, build them leaf first */
            uint64_t lvl_addr[8];
            uint64_t acc = a_idx[i];
            for (int L = nlevels - 1; L >= 0; --L) { lvl_addr[L] = acc; acc += (uint64_t)nodes_per_level[L] * chunk_node_size(); }
            /* buffer the whole index in memory, then write it in address order */
            uint8_t *idx = (uint8_t *)calloc(1, idx_bytes);
            if (!idx) { rc = fail(PPF_H5_ENOMEM, "h5: out of memory"); break; }
            for (int L = 0; L < nlevels; ++L) {
                int64_t nodes = nodes_per_level[L];
                for (int64_t nd = 0; nd < nodes; ++nd) {
                    int64_t first = nd * 2 * CHUNK_K;
                    int64_t cntn = cnt - first < 2 * CHUNK_K ? cnt - first : 2 * CHUNK_K;
                    uint64_t naddr = lvl_addr[L] + (uint64_t)nd * chunk_node_size();
                    memset(node, 0, chunk_node_size());
                    memcpy(node, "TREE", 4);
                    node[4] = 1;
                    node[5] = (uint8_t)L;
                    put_le(node + 6, (uint64_t)cntn, 2);
                    put_le(node + 8, nd > 0 ? naddr - chunk_node_size() : UNDEF_ADDR, 8);
                    put_le(node + 16, nd + 1 < nodes ? naddr + chunk_node_size() : UNDEF_ADDR, 8);
                    uint8_t *k = node + 24;
                    for (int64_t e = 0; e < cntn; ++e) {
                        const chunk_ent *ce = &cur[first + e];
                        put_le(k, L == 0 ? (uint64_t)csz : 0, 4);
                        put_le(k + 4, 0, 4);
                        for (int q = 0; q < 3; ++q) put_le(k + 8 + 8 * q, (uint64_t)ce->off[q], 8);
                        put_le(k + 32, 0, 8);
                        put_le(k + 40, ce->addr, 8);
                        k += 48;
                    }
                    /* right key: next sibling's first key, or the tree's end */
                    const int64_t *rk = first + cntn < cnt ? cur[first + cntn].off : endkey;
                    put_le(k, 0, 4);
                    put_le(k + 4, 0, 4);
                    for (int q = 0; q < 3; ++q) put_le(k + 8 + 8 * q, (uint64_t)rk[q], 8);
                    put_le(k + 32, first + cntn < cnt ? 0 : (uint64_t)es, 8);
                    memcpy(idx + (naddr - a_idx[i]), node, chunk_node_size());
                    nxt[nd].off[0] = cur[first].off[0];
                    nxt[nd].off[1] = cur[first].off[1];
                    nxt[nd].off[2] = cur[first].off[2];
                    nxt[nd].addr = naddr;
                }
                chunk_ent *t = cur; cur = nxt; nxt = t;
                cnt = nodes;
            }
            rc = wr_bytes(f, &w, idx, idx_bytes);
            free(idx);
        }
        free(cur);
        free(nxt);
        free(node);
    }
    /* ---- raw data ---- */
    const int64_t blk = 1 << 16;
    const int64_t tmpn = chunk && chunk[2] > blk ? chunk[2] : blk;
    uint8_t *tmp = (uint8_t *)malloc((size_t)(tmpn * 8));
    if (!tmp && !rc) rc = fail(PPF_H5_ENOMEM, "h5: out of memory");
    for (int i = 0; i < n && !rc; ++i) {
        if (w != a_data[i]) { rc = fail(PPF_H5_EIO, "h5: internal layout error"); break; }
        if (!chunk) {
            for (int64_t s = 0; s < nel && !rc; s += blk) {
                int64_t m = nel - s < blk ? nel - s : blk;
                for (int64_t e = 0; e < m; ++e) {
                    if (es == 8) memcpy(tmp + e * 8, &data[i][s + e], 8);
                    else { float v = (float)data[i][s + e]; memcpy(tmp + e * 4, &v, 4); }
                }
                rc = wr_bytes(f, &w, tmp, (uint64_t)(m * es));
            }
        } else {
            for (int64_t a = 0; a < ncd[0] && !rc; ++a)
                for (int64_t b = 0; b < ncd[1] && !rc; ++b)
                    for (int64_t d = 0; d < ncd[2] && !rc; ++d)
                        for (int64_t ci = 0; ci < chunk[0] && !rc; ++ci)
                            for (int64_t cj = 0; cj < chunk[1] && !rc; ++cj) {
                                int64_t z = a * chunk[0] + ci, y = b * chunk[1] + cj;
                                for (int64_t ck = 0; ck < chunk[2]; ++ck) {
                                    int64_t x = d * chunk[2] + ck;
                                    double v = (z < dims[0] && y < dims[1] && x < dims[2])
                                                   ? data[i][(z * dims[1] + y) * dims[2] + x] : 0.0;
                                    if (es == 8) memcpy(tmp + ck * 8, &v, 8);
                                    else { float fv = (float)v; memcpy(tmp + ck * 4, &fv, 4); }
                                }
                                rc = wr_bytes(f, &w, tmp, (uint64_t)(chunk[2] * es));
                            }
        }
    }
    free(tmp);
    if (has_meta && !rc) {
        if (w != a_meta) rc = fail(PPF_H5_EIO, "h5: internal layout error");
        else rc = wr_bytes(f, &w, meta, (uint64_t)nmeta * 8);
    }
    if (!rc && w != eof) rc = fail(PPF_H5_EIO, "h5: internal size error");
    if (fclose(f) != 0 && !rc) rc = fail(PPF_H5_EIO, "h5: close failed");
    if (rc) remove(path);
    return rc;
}
