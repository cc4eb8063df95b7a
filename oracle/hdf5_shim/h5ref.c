/*
 * ORACLE -- test infrastructure.  See h5ref.h: the oracle side's own HDF5
 * subset, written from the file-format specification (superblock v0,
 * symbol-table groups, v1 object headers, v1 B-trees).  Independent of the
 * product's HDF5 code, so that the reference build and the golden-vector
 * scripts never run product code, and so that two separate implementations
 * of the format can be checked against each other.
 */
#include "h5ref.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static char g_msg[256];

static int fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof g_msg, fmt, ap);
    va_end(ap);
    return code;
}

const char *h5ref_error(void) { return g_msg; }

#define UNDEF 0xffffffffffffffffULL

/* ------------------------------------------------------------ writing ---- */

typedef struct {
    unsigned char *p;
    size_t n, cap;
} buf_t;

static int grow(buf_t *b, size_t need)
{
    if (need <= b->cap) return 0;
    size_t c = b->cap ? b->cap : 4096;
    while (c < need) c *= 2;
    unsigned char *q = (unsigned char *)realloc(b->p, c);
    if (!q) return -1;
    memset(q + b->cap, 0, c - b->cap);
    b->p = q;
    b->cap = c;
    return 0;
}

/* reserve `len` zeroed bytes at the end (8-byte aligned start); returns offset */
static size_t reserve(buf_t *b, size_t len)
{
    size_t at = (b->n + 7) & ~(size_t)7;
    if (grow(b, at + len)) return (size_t)-1;
    b->n = at + len;
    return at;
}

static void put_le(buf_t *b, size_t at, uint64_t v, int bytes)
{
    for (int i = 0; i < bytes; ++i) b->p[at + (size_t)i] = (unsigned char)(v >> (8 * i));
}

/* one object-header message of a v1 header: type, padded size, flags */
static size_t put_msg(buf_t *b, size_t at, int type, size_t dsize, int flags)
{
    const size_t padded = (dsize + 7) & ~(size_t)7;
    put_le(b, at, (uint64_t)type, 2);
    put_le(b, at + 2, (uint64_t)padded, 2);
    b->p[at + 4] = (unsigned char)flags;
    return at + 8;   /* start of the message data */
}

static void put_f64(buf_t *b, size_t at, double v)
{
    uint64_t u;
    memcpy(&u, &v, 8);
    put_le(b, at, u, 8);
}

static void put_f32(buf_t *b, size_t at, float v)
{
    uint32_t u;
    memcpy(&u, &v, 4);
    put_le(b, at, u, 4);
}

/* the IEEE float datatype message body (20 bytes) */
static void put_dtype(buf_t *b, size_t at, int f32)
{
    b->p[at] = 0x11;                         /* version 1, class 1 (floating point) */
    b->p[at + 1] = 0x20;                     /* little endian, implied mantissa msb */
    b->p[at + 2] = (unsigned char)(f32 ? 31 : 63);   /* sign bit position */
    b->p[at + 3] = 0;
    put_le(b, at + 4, f32 ? 4 : 8, 4);       /* size in bytes */
    put_le(b, at + 8, 0, 2);                 /* bit offset */
    put_le(b, at + 10, f32 ? 32 : 64, 2);    /* precision */
    b->p[at + 12] = (unsigned char)(f32 ? 23 : 52);   /* exponent location */
    b->p[at + 13] = (unsigned char)(f32 ? 8 : 11);    /* exponent size */
    b->p[at + 14] = 0;                                /* mantissa location */
    b->p[at + 15] = (unsigned char)(f32 ? 23 : 52);   /* mantissa size */
    put_le(b, at + 16, f32 ? 127 : 1023, 4);          /* exponent bias */
}

#define CHUNK_K 32           /* raw-data B-tree: up to 2K entries per node */
#define KEY_BYTES 40         /* chunk key of a rank-3 dataset: 4 + 4 + 4 x 8 */

typedef struct {
    uint64_t off[3];         /* chunk origin, elements */
    uint64_t addr;           /* child address (chunk or node) */
} ckey_t;

/* one raw-data B-tree node of level `level` over keys[0..n-1]; `last` is the
 * node's upper bound key; returns the node's address */
static size_t put_chunk_node(buf_t *b, int level, const ckey_t *keys, int n, const uint64_t last_off[3],
                             uint32_t chunk_bytes)
{
    const size_t sz = 24 + (size_t)(2 * CHUNK_K + 1) * KEY_BYTES + (size_t)(2 * CHUNK_K) * 8;
    size_t at = reserve(b, sz);
    if (at == (size_t)-1) return at;
    memcpy(b->p + at, "TREE", 4);
    b->p[at + 4] = 1;                        /* raw data chunks */
    b->p[at + 5] = (unsigned char)level;
    put_le(b, at + 6, (uint64_t)n, 2);
    put_le(b, at + 8, UNDEF, 8);
    put_le(b, at + 16, UNDEF, 8);
    size_t q = at + 24;
    for (int i = 0; i <= n; ++i) {
        const uint64_t *o = i < n ? keys[i].off : last_off;
        put_le(b, q, i < n ? chunk_bytes : 0, 4);
        put_le(b, q + 4, 0, 4);              /* filter mask */
        for (int d = 0; d < 3; ++d) put_le(b, q + 8 + 8 * (size_t)d, o[d], 8);
        put_le(b, q + 32, 0, 8);             /* the element dimension */
        q += KEY_BYTES;
        if (i < n) {
            put_le(b, q, keys[i].addr, 8);
            q += 8;
        }
    }
    return at;
}

int h5ref_write(const char *path, int n, const char *const *names, const double *const *data,
                const int64_t dims[3], int as_float32, const int64_t *chunk)
{
    if (!path || n < 1 || n > 8 || !names || !data || !dims) return fail(-6, "h5ref_write: bad arguments");
    for (int d = 0; d < 3; ++d)
        if (dims[d] < 1 || (chunk && (chunk[d] < 1))) return fail(-6, "h5ref_write: bad dims");
    const size_t es = as_float32 ? 4 : 8;
    const uint64_t count = (uint64_t)dims[0] * (uint64_t)dims[1] * (uint64_t)dims[2];
    buf_t b = {0, 0, 0};
    int rc = 0;

    /* names sorted as libhdf5 keeps a group's symbol table */
    int order[8];
    for (int i = 0; i < n; ++i) order[i] = i;
    for (int i = 1; i < n; ++i)
        for (int j = i; j > 0 && strcmp(names[order[j - 1]], names[order[j]]) > 0; --j) {
            int t = order[j];
            order[j] = order[j - 1];
            order[j - 1] = t;
        }

    const size_t sb = reserve(&b, 96);
    /* root object header: one symbol-table message */
    const size_t root = reserve(&b, 16 + 8 + 16);
    /* local heap with the names */
    size_t heap_len = 8, name_off[8];
    for (int i = 0; i < n; ++i) {
        const char *nm = names[order[i]];
        if (*nm == '/') ++nm;
        name_off[i] = heap_len;
        heap_len += (strlen(nm) + 1 + 7) & ~(size_t)7;
    }
    const size_t heap = reserve(&b, 32);
    const size_t heap_data = reserve(&b, heap_len);
    if (sb == (size_t)-1 || root == (size_t)-1 || heap == (size_t)-1 || heap_data == (size_t)-1) {
        rc = fail(-7, "h5ref_write: out of memory");
        goto done;
    }
    for (int i = 0; i < n; ++i) {
        const char *nm = names[order[i]];
        if (*nm == '/') ++nm;
        memcpy(b.p + heap_data + name_off[i], nm, strlen(nm));
    }
    memcpy(b.p + heap, "HEAP", 4);
    put_le(&b, heap + 8, heap_len, 8);
    put_le(&b, heap + 16, UNDEF, 8);         /* no free block */
    put_le(&b, heap + 24, heap_data, 8);
    /* group B-tree (one leaf child: the symbol table node), K = 16 */
    const size_t gtree = reserve(&b, 24 + 33 * 8 + 32 * 8);
    const size_t snod = reserve(&b, 8 + 8 * 40);
    memcpy(b.p + gtree, "TREE", 4);
    b.p[gtree + 4] = 0;
    b.p[gtree + 5] = 0;
    put_le(&b, gtree + 6, 1, 2);
    put_le(&b, gtree + 8, UNDEF, 8);
    put_le(&b, gtree + 16, UNDEF, 8);
    put_le(&b, gtree + 24, 0, 8);                        /* key 0: "" */
    put_le(&b, gtree + 32, snod, 8);                     /* child 0 */
    put_le(&b, gtree + 40, name_off[n - 1], 8);          /* key 1: the last name */
    memcpy(b.p + snod, "SNOD", 4);
    b.p[snod + 4] = 1;
    put_le(&b, snod + 6, (uint64_t)n, 2);
    /* root object header */
    b.p[root] = 1;
    put_le(&b, root + 2, 1, 2);
    put_le(&b, root + 4, 1, 4);
    put_le(&b, root + 8, 24, 4);
    {
        size_t m = put_msg(&b, root + 16, 0x11, 16, 0);
        put_le(&b, m, gtree, 8);
        put_le(&b, m + 8, heap, 8);
    }

    for (int i = 0; i < n; ++i) {
        const double *src = data[order[i]];
        /* object header: dataspace, datatype, fill value, layout */
        const size_t lay_len = chunk ? 27 : 18;
        const size_t hdr_data = (8 + 32) + (8 + 24) + (8 + 8) + (8 + ((lay_len + 7) & ~(size_t)7));
        const size_t oh = reserve(&b, 16 + hdr_data);
        if (oh == (size_t)-1) {
            rc = fail(-7, "h5ref_write: out of memory");
            goto done;
        }
        b.p[oh] = 1;
        put_le(&b, oh + 2, 4, 2);
        put_le(&b, oh + 4, 1, 4);
        put_le(&b, oh + 8, hdr_data, 4);
        size_t m = put_msg(&b, oh + 16, 0x01, 32, 0);          /* dataspace v1 */
        b.p[m] = 1;
        b.p[m + 1] = 3;
        for (int d = 0; d < 3; ++d) put_le(&b, m + 8 + 8 * (size_t)d, (uint64_t)dims[d], 8);
        m = put_msg(&b, m + 32, 0x03, 20, 1);                  /* datatype */
        put_dtype(&b, m, as_float32);
        m = put_msg(&b, m + 24, 0x05, 4, 1);                   /* fill value v2 */
        b.p[m] = 2;
        b.p[m + 1] = chunk ? 3 : 1;                            /* allocation: incremental / early */
        b.p[m + 2] = 2;                                        /* write fill value: if set */
        b.p[m + 3] = 0;                                        /* no fill value defined */
        m = put_msg(&b, m + 8, 0x08, lay_len, 0);              /* layout v3 */
        b.p[m] = 3;
        const size_t lay = m;
        /* symbol table entry */
        const size_t ent = snod + 8 + 40 * (size_t)i;
        put_le(&b, ent, name_off[i], 8);
        put_le(&b, ent + 8, oh, 8);
        if (!chunk) {
            const size_t bytes = (size_t)count * es;
            const size_t at = reserve(&b, bytes);
            if (at == (size_t)-1) {
                rc = fail(-7, "h5ref_write: out of memory");
                goto done;
            }
            for (uint64_t k = 0; k < count; ++k) {
                if (as_float32) put_f32(&b, at + (size_t)k * 4, (float)src[k]);
                else put_f64(&b, at + (size_t)k * 8, src[k]);
            }
            b.p[lay + 1] = 1;
            put_le(&b, lay + 2, at, 8);
            put_le(&b, lay + 10, bytes, 8);
            continue;
        }
        /* chunked: every chunk full size (edge chunks padded with zeros), in C order */
        uint64_t nc[3];
        for (int d = 0; d < 3; ++d) nc[d] = ((uint64_t)dims[d] + (uint64_t)chunk[d] - 1) / (uint64_t)chunk[d];
        const uint64_t nchunks = nc[0] * nc[1] * nc[2];
        const size_t cbytes = (size_t)(chunk[0] * chunk[1] * chunk[2]) * es;
        ckey_t *keys = (ckey_t *)calloc((size_t)nchunks, sizeof(ckey_t));
        if (!keys) {
            rc = fail(-7, "h5ref_write: out of memory");
            goto done;
        }
        uint64_t k = 0;
        for (uint64_t a = 0; a < nc[0]; ++a)
            for (uint64_t bb = 0; bb < nc[1]; ++bb)
                for (uint64_t c = 0; c < nc[2]; ++c, ++k) {
                    const uint64_t o[3] = {a * (uint64_t)chunk[0], bb * (uint64_t)chunk[1], c * (uint64_t)chunk[2]};
                    const size_t at = reserve(&b, cbytes);
                    if (at == (size_t)-1) break;
                    for (int64_t z = 0; z < chunk[0]; ++z)
                        for (int64_t y = 0; y < chunk[1]; ++y)
                            for (int64_t x = 0; x < chunk[2]; ++x) {
                                const uint64_t gz = o[0] + (uint64_t)z, gy = o[1] + (uint64_t)y, gx = o[2] + (uint64_t)x;
                                if (gz >= (uint64_t)dims[0] || gy >= (uint64_t)dims[1] || gx >= (uint64_t)dims[2]) continue;
                                const double v = src[(gz * (uint64_t)dims[1] + gy) * (uint64_t)dims[2] + gx];
                                const size_t e = (size_t)((z * chunk[1] + y) * chunk[2] + x);
                                if (as_float32) put_f32(&b, at + e * 4, (float)v);
                                else put_f64(&b, at + e * 8, v);
                            }
                    memcpy(keys[k].off, o, sizeof o);
                    keys[k].addr = at;
                }
        if (k != nchunks) {
            free(keys);
            rc = fail(-7, "h5ref_write: out of memory");
            goto done;
        }
        /* B-tree levels: leaves of up to 2K chunks, then nodes of up to 2K children */
        const uint64_t end_off[3] = {nc[0] * (uint64_t)chunk[0], 0, 0};
        int level = 0;
        uint64_t cnt = nchunks;
        while (1) {
            const uint64_t nodes = (cnt + 2 * CHUNK_K - 1) / (2 * CHUNK_K);
            ckey_t *up = (ckey_t *)calloc((size_t)nodes, sizeof(ckey_t));
            if (!up) {
                free(keys);
                rc = fail(-7, "h5ref_write: out of memory");
                goto done;
            }
            for (uint64_t j = 0; j < nodes; ++j) {
                const uint64_t lo = j * 2 * CHUNK_K, hi = lo + 2 * CHUNK_K < cnt ? lo + 2 * CHUNK_K : cnt;
                const uint64_t *last = hi < cnt ? keys[hi].off : end_off;
                const size_t at = put_chunk_node(&b, level, keys + lo, (int)(hi - lo), last, (uint32_t)cbytes);
                memcpy(up[j].off, keys[lo].off, sizeof up[j].off);
                up[j].addr = at;
            }
            free(keys);
            keys = up;
            cnt = nodes;
            if (cnt == 1) break;
            ++level;
        }
        b.p[lay + 1] = 2;
        b.p[lay + 2] = 4;                    /* rank + 1 */
        put_le(&b, lay + 3, keys[0].addr, 8);
        for (int d = 0; d < 3; ++d) put_le(&b, lay + 11 + 4 * (size_t)d, (uint64_t)chunk[d], 4);
        put_le(&b, lay + 23, es, 4);
        free(keys);
    }
    /* superblock */
    memcpy(b.p + sb, "\x89HDF\r\n\x1a\n", 8);
    b.p[sb + 13] = 8;                        /* size of offsets */
    b.p[sb + 14] = 8;                        /* size of lengths */
    put_le(&b, sb + 16, 4, 2);               /* group leaf node K */
    put_le(&b, sb + 18, 16, 2);              /* group internal node K */
    put_le(&b, sb + 24, 0, 8);               /* base address */
    put_le(&b, sb + 32, UNDEF, 8);           /* free-space info */
    put_le(&b, sb + 40, b.n, 8);             /* end of file */
    put_le(&b, sb + 48, UNDEF, 8);           /* driver info */
    put_le(&b, sb + 56, 0, 8);               /* root entry: link name offset */
    put_le(&b, sb + 64, root, 8);            /*             object header */
    put_le(&b, sb + 72, 1, 4);               /*             cache type 1 */
    put_le(&b, sb + 80, gtree, 8);           /*             B-tree */
    put_le(&b, sb + 88, heap, 8);            /*             heap */
    {
        FILE *f = fopen(path, "wb");
        if (!f) {
            rc = fail(-1, "h5ref_write: cannot create %s", path);
            goto done;
        }
        const size_t w = fwrite(b.p, 1, b.n, f);
        if (fclose(f) != 0 || w != b.n) rc = fail(-1, "h5ref_write: write failed for %s", path);
    }
done:
    free(b.p);
    return rc;
}

/* ------------------------------------------------------------ reading ---- */

typedef struct {
    unsigned char *p;
    uint64_t n;
    uint64_t base;
    uint64_t root_oh, root_tree, root_heap;
} file_t;

static uint64_t get_le(const unsigned char *p, int bytes)
{
    uint64_t v = 0;
    for (int i = bytes - 1; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}

/* the bytes [addr, addr+len) of the file, or NULL when out of range */
static const unsigned char *at_(const file_t *f, uint64_t addr, uint64_t len)
{
    if (addr == UNDEF) return NULL;
    const uint64_t a = f->base + addr;
    if (a < f->base || a > f->n || len > f->n - a) return NULL;
    return f->p + a;
}

static void close_file(file_t *f) { free(f->p); }

static int open_file(const char *path, file_t *f)
{
    memset(f, 0, sizeof *f);
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail(-1, "cannot open %s", path);
    fseek(fp, 0, SEEK_END);
    long sz = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    if (sz <= 0) {
        fclose(fp);
        return fail(-1, "empty file %s", path);
    }
    f->p = (unsigned char *)malloc((size_t)sz);
    if (!f->p) {
        fclose(fp);
        return fail(-7, "out of memory");
    }
    f->n = (uint64_t)fread(f->p, 1, (size_t)sz, fp);
    fclose(fp);
    /* the superblock sits at 0, 512, 1024, 2048, ... (after a user block) */
    uint64_t sbo = UNDEF;
    for (uint64_t o = 0; o + 8 <= f->n; o = o ? 2 * o : 512)
        if (!memcmp(f->p + o, "\x89HDF\r\n\x1a\n", 8)) {
            sbo = o;
            break;
        }
    if (sbo == UNDEF) {
        close_file(f);
        return fail(-2, "%s: no HDF5 superblock", path);
    }
    const unsigned char *s = f->p + sbo;
    if (f->n - sbo < 100 || (s[8] != 0 && s[8] != 1) || s[13] != 8 || s[14] != 8) {
        close_file(f);
        return fail(-2, "%s: superblock version %d / offset size %d outside the oracle's subset", path, s[8], s[13]);
    }
    const int extra = s[8] == 1 ? 4 : 0;     /* v1 adds indexed-storage K + reserved */
    const unsigned char *e = s + 24 + extra + 32;   /* root group symbol table entry */
    const uint64_t stored_base = get_le(s + 24 + extra, 8);
    /* addresses are relative to the base address, which is the superblock's
     * own position when a user block precedes it */
    f->base = stored_base ? stored_base : sbo;
    f->root_oh = get_le(e + 8, 8);
    if (get_le(e + 16, 4) == 1) {
        f->root_tree = get_le(e + 24, 8);
        f->root_heap = get_le(e + 32, 8);
    } else {
        f->root_tree = f->root_heap = UNDEF;
    }
    return 0;
}

/* visit the messages of a v1 object header (following continuations);
 * cb returns nonzero to stop */
typedef int (*msg_cb)(const file_t *f, int type, const unsigned char *d, uint64_t len, int flags, void *u);

static int walk_header(const file_t *f, uint64_t addr, msg_cb cb, void *u)
{
    const unsigned char *h = at_(f, addr, 16);
    if (!h) return fail(-2, "object header out of range");
    if (h[0] != 1) return fail(-2, "object header version %d outside the oracle's subset", h[0]);
    uint64_t blocks[16][2];
    int nb = 1, nmsg = (int)get_le(h + 2, 2), seen = 0;
    blocks[0][0] = addr + 16;
    blocks[0][1] = get_le(h + 8, 4);
    for (int bi = 0; bi < nb; ++bi) {
        const unsigned char *p = at_(f, blocks[bi][0], blocks[bi][1]);
        if (!p) return fail(-2, "object header block out of range");
        uint64_t o = 0;
        while (o + 8 <= blocks[bi][1] && seen < nmsg) {
            const int type = (int)get_le(p + o, 2);
            const uint64_t len = get_le(p + o + 2, 2);
            const int flags = p[o + 4];
            if (o + 8 + len > blocks[bi][1]) return fail(-2, "object header message out of range");
            ++seen;
            if (type == 0x10) {                      /* continuation */
                if (nb == 16) return fail(-2, "too many header continuation blocks");
                blocks[nb][0] = get_le(p + o + 8, 8);
                blocks[nb][1] = get_le(p + o + 16, 8);
                ++nb;
            } else if (type != 0) {
                const int r = cb(f, type, p + o + 8, len, flags, u);
                if (r) return r > 0 ? 0 : r;
            }
            o += 8 + len;
        }
    }
    return 0;
}

typedef struct {
    int rank;
    uint64_t dims[8];
    int cls, size, big;                      /* datatype class, bytes, big endian */
    int layout;                              /* 0 compact, 1 contiguous, 2 chunked, -1 none */
    uint64_t addr, bytes;                    /* contiguous data / chunk B-tree address */
    const unsigned char *compact;
    uint32_t cdims[8];
    int filtered, shared;
    uint64_t tree, heap;                     /* a group's symbol table */
} dset_t;

static int dset_msg(const file_t *f, int type, const unsigned char *d, uint64_t len, int flags, void *u)
{
    (void)f;
    dset_t *s = (dset_t *)u;
    if (flags & 2) s->shared = 1;
    if (type == 0x01 && !(flags & 2)) {
        const int ver = d[0];
        s->rank = d[1];
        if (s->rank > 8) return fail(-4, "rank %d", s->rank);
        const unsigned char *q = d + (ver == 1 ? 8 : 4);
        if ((uint64_t)(q - d) + 8 * (uint64_t)s->rank > len) return fail(-2, "dataspace message truncated");
        for (int i = 0; i < s->rank; ++i) s->dims[i] = get_le(q + 8 * i, 8);
    } else if (type == 0x03 && !(flags & 2)) {
        s->cls = d[0] & 15;
        s->big = d[1] & 1;
        s->size = (int)get_le(d + 4, 4);
    } else if (type == 0x0b) {
        s->filtered = 1;
    } else if (type == 0x08 && (d[0] == 1 || d[0] == 2)) {
        /* versions 1-2 (libhdf5 1.6 and older): version, dimensionality
         * (including the element size), class, 5 reserved bytes */
        const int nd = d[1];
        const unsigned char *q = d + 8;
        if (nd < 1 || nd > 8) return fail(-2, "layout rank %d", nd);
        s->layout = d[2];
        if (s->layout == 1 || s->layout == 2) {
            s->addr = get_le(q, 8);
            q += 8;
        }
        for (int i = 0; i < nd; ++i) s->cdims[i] = (uint32_t)get_le(q + 4 * i, 4);
        if (s->layout == 1) {
            uint64_t b = 1;
            for (int i = 0; i < nd; ++i) b *= s->cdims[i];
            s->bytes = b;                    /* the dims times the element size */
        } else if (s->layout == 0) {
            s->bytes = get_le(q + 4 * nd, 4);
            s->compact = q + 4 * nd + 4;
        }
    } else if (type == 0x08) {
        if (d[0] != 3) return fail(-2, "layout message version %d outside the oracle's subset", d[0]);
        s->layout = d[1];
        if (s->layout == 0) {
            s->bytes = get_le(d + 2, 2);
            s->compact = d + 4;
        } else if (s->layout == 1) {
            s->addr = get_le(d + 2, 8);
            s->bytes = get_le(d + 10, 8);
        } else if (s->layout == 2) {
            const int nd = d[2];
            if (nd < 1 || nd > 8) return fail(-2, "chunk rank %d", nd);
            s->addr = get_le(d + 3, 8);
            for (int i = 0; i < nd; ++i) s->cdims[i] = (uint32_t)get_le(d + 11 + 4 * i, 4);
        }
    } else if (type == 0x11) {
        s->tree = get_le(d, 8);
        s->heap = get_le(d + 8, 8);
    }
    return 0;
}

static int describe(const file_t *f, uint64_t oh, dset_t *s)
{
    memset(s, 0, sizeof *s);
    s->layout = -1;
    s->rank = -1;
    s->tree = s->heap = UNDEF;
    return walk_header(f, oh, dset_msg, s);
}

/* visit the entries of a symbol-table group: (name, object header) */
typedef int (*ent_cb)(const char *name, uint64_t oh, void *u);

static int walk_group_tree(const file_t *f, uint64_t node, const unsigned char *names, uint64_t nlen, ent_cb cb,
                           void *u, int depth)
{
    if (depth > 32) return fail(-2, "group B-tree too deep");
    const unsigned char *t = at_(f, node, 24);
    if (!t || memcmp(t, "TREE", 4) || t[4] != 0) return fail(-2, "bad group B-tree node");
    const int level = t[5], n = (int)get_le(t + 6, 2);
    const unsigned char *kc = at_(f, node + 24, (uint64_t)(2 * n + 1) * 8);
    if (!kc) return fail(-2, "group B-tree node out of range");
    for (int i = 0; i < n; ++i) {
        const uint64_t child = get_le(kc + 8 + 16 * (uint64_t)i, 8);
        if (level > 0) {
            int r = walk_group_tree(f, child, names, nlen, cb, u, depth + 1);
            if (r) return r;
            continue;
        }
        const unsigned char *sn = at_(f, child, 8);
        if (!sn || memcmp(sn, "SNOD", 4)) return fail(-2, "bad symbol table node");
        const int ns = (int)get_le(sn + 6, 2);
        const unsigned char *ents = at_(f, child + 8, (uint64_t)ns * 40);
        if (!ents) return fail(-2, "symbol table node out of range");
        for (int j = 0; j < ns; ++j) {
            const uint64_t no = get_le(ents + 40 * (uint64_t)j, 8);
            if (no >= nlen || !memchr(names + no, 0, (size_t)(nlen - no))) return fail(-2, "bad name offset");
            int r = cb((const char *)names + no, get_le(ents + 40 * (uint64_t)j + 8, 8), u);
            if (r) return r;
        }
    }
    return 0;
}

static int walk_root(const file_t *f, ent_cb cb, void *u)
{
    uint64_t tree = f->root_tree, heap = f->root_heap;
    if (tree == UNDEF) {
        dset_t g;
        int rc = describe(f, f->root_oh, &g);
        if (rc) return rc;
        tree = g.tree;
        heap = g.heap;
    }
    const unsigned char *h = at_(f, heap, 32);
    if (!h || memcmp(h, "HEAP", 4)) return fail(-2, "root group has no local heap");
    const uint64_t nlen = get_le(h + 8, 8), naddr = get_le(h + 24, 8);
    const unsigned char *names = at_(f, naddr, nlen);
    if (!names) return fail(-2, "heap data out of range");
    return walk_group_tree(f, tree, names, nlen, cb, u, 0);
}

typedef struct {
    const char *want;
    uint64_t oh;
    int found;
} find_t;

static int find_cb(const char *name, uint64_t oh, void *u)
{
    find_t *q = (find_t *)u;
    if (!strcmp(name, q->want)) {
        q->oh = oh;
        q->found = 1;
        return 1;
    }
    return 0;
}

static int open_dataset(const char *path, const char *name, file_t *f, dset_t *s)
{
    int rc = open_file(path, f);
    if (rc) return rc;
    find_t q = {name && *name == '/' ? name + 1 : name, 0, 0};
    rc = walk_root(f, find_cb, &q);
    if (rc < 0) {
        close_file(f);
        return rc;
    }
    if (!q.found) {
        close_file(f);
        return fail(-3, "%s: no dataset %s", path, name);
    }
    rc = describe(f, q.oh, s);
    if (rc) {
        close_file(f);
        return rc;
    }
    if (s->rank != 3) {
        close_file(f);
        return fail(-4, "%s: %s has rank %d, not 3", path, name, s->rank);
    }
    if (s->shared || s->cls != 1 || (s->size != 4 && s->size != 8)) {
        close_file(f);
        return fail(-5, "%s: %s is not an IEEE float32/float64 dataset", path, name);
    }
    if (s->filtered) {
        close_file(f);
        return fail(-2, "%s: %s is filtered (compressed)", path, name);
    }
    return 0;
}

int h5ref_dims(const char *path, const char *name, int64_t dims[3])
{
    file_t f;
    dset_t s;
    int rc = open_dataset(path, name, &f, &s);
    if (rc) return rc;
    for (int i = 0; i < 3; ++i) dims[i] = (int64_t)s.dims[i];
    close_file(&f);
    return 0;
}

static double load_elem(const unsigned char *p, int size, int big)
{
    unsigned char t[8];
    for (int i = 0; i < size; ++i) t[i] = big ? p[size - 1 - i] : p[i];
    if (size == 4) {
        uint32_t u = (uint32_t)get_le(t, 4);
        float v;
        memcpy(&v, &u, 4);
        return (double)v;
    }
    uint64_t u = get_le(t, 8);
    double v;
    memcpy(&v, &u, 8);
    return v;
}

static int read_chunks(const file_t *f, const dset_t *s, uint64_t node, double *out, int depth)
{
    if (depth > 32) return fail(-2, "chunk B-tree too deep");
    const unsigned char *t = at_(f, node, 24);
    if (!t || memcmp(t, "TREE", 4) || t[4] != 1) return fail(-2, "bad chunk B-tree node");
    const int level = t[5], n = (int)get_le(t + 6, 2);
    const uint64_t ks = 8 + 8 * 4;           /* chunk key of a rank-3 dataset */
    const unsigned char *kc = at_(f, node + 24, (uint64_t)n * (ks + 8) + ks);
    if (!kc) return fail(-2, "chunk B-tree node out of range");
    for (int i = 0; i < n; ++i) {
        const unsigned char *k = kc + (uint64_t)i * (ks + 8);
        const uint64_t child = get_le(k + ks, 8);
        if (level > 0) {
            int r = read_chunks(f, s, child, out, depth + 1);
            if (r) return r;
            continue;
        }
        const uint64_t bytes = get_le(k, 4);
        if (get_le(k + 4, 4) != 0) return fail(-2, "filtered chunk");
        uint64_t o[3];
        for (int d = 0; d < 3; ++d) {
            o[d] = get_le(k + 8 + 8 * d, 8);
            if (o[d] >= s->dims[d] || o[d] % s->cdims[d]) return fail(-2, "bad chunk offset");
        }
        const uint64_t need = (uint64_t)s->cdims[0] * s->cdims[1] * s->cdims[2] * (uint64_t)s->size;
        if (bytes < need) return fail(-2, "short chunk");
        const unsigned char *src = at_(f, child, need);
        if (!src) return fail(-1, "chunk out of range (truncated file?)");
        for (uint64_t z = 0; z < s->cdims[0] && o[0] + z < s->dims[0]; ++z)
            for (uint64_t y = 0; y < s->cdims[1] && o[1] + y < s->dims[1]; ++y)
                for (uint64_t x = 0; x < s->cdims[2] && o[2] + x < s->dims[2]; ++x) {
                    const uint64_t e = (z * s->cdims[1] + y) * s->cdims[2] + x;
                    out[((o[0] + z) * s->dims[1] + o[1] + y) * s->dims[2] + o[2] + x] =
                        load_elem(src + e * (uint64_t)s->size, s->size, s->big);
                }
    }
    return 0;
}

int h5ref_read(const char *path, const char *name, double *out, int64_t capacity)
{
    file_t f;
    dset_t s;
    int rc = open_dataset(path, name, &f, &s);
    if (rc) return rc;
    const uint64_t count = s.dims[0] * s.dims[1] * s.dims[2];
    if (!out || (uint64_t)capacity < count) {
        close_file(&f);
        return fail(-6, "output holds %lld of %llu values", (long long)capacity, (unsigned long long)count);
    }
    if (s.layout == 0 || s.layout == 1) {
        const unsigned char *src = s.layout == 0 ? s.compact : at_(&f, s.addr, count * (uint64_t)s.size);
        if (!src || s.bytes < count * (uint64_t)s.size) {
            close_file(&f);
            return fail(-1, "%s: %s data out of range (truncated file?)", path, name);
        }
        for (uint64_t k = 0; k < count; ++k) out[k] = load_elem(src + k * (uint64_t)s.size, s.size, s.big);
    } else if (s.layout == 2) {
        for (uint64_t k = 0; k < count; ++k) out[k] = 0.0;   /* unallocated chunks read as the fill value */
        if (s.cdims[3] != (uint32_t)s.size) {
            close_file(&f);
            return fail(-2, "chunk element size %u", s.cdims[3]);
        }
        for (int d = 0; d < 3; ++d)
            if (!s.cdims[d]) {
                close_file(&f);
                return fail(-2, "zero chunk dimension");
            }
        if (s.addr != UNDEF) rc = read_chunks(&f, &s, s.addr, out, 0);
    } else {
        rc = fail(-2, "%s: %s has no supported layout", path, name);
    }
    close_file(&f);
    return rc;
}

int h5ref_read_any(const char *path, const char *name, double *out, int64_t capacity, int *rank, int64_t dims[3])
{
    file_t f;
    int rc = open_file(path, &f);
    if (rc) return rc;
    find_t q = {name && *name == '/' ? name + 1 : name, 0, 0};
    rc = walk_root(&f, find_cb, &q);
    dset_t s;
    if (rc >= 0 && !q.found) rc = fail(-3, "%s: no dataset %s", path, name);
    if (rc >= 0) rc = describe(&f, q.oh, &s);
    if (rc >= 0 && (s.rank < 1 || s.rank > 3)) rc = fail(-4, "rank %d", s.rank);
    if (rc >= 0 && (s.shared || s.cls != 1 || (s.size != 4 && s.size != 8) || s.filtered || s.layout == 2))
        rc = fail(-5, "%s: %s is not a contiguous/compact IEEE float dataset", path, name);
    if (rc < 0) {
        close_file(&f);
        return rc;
    }
    uint64_t count = 1;
    for (int i = 0; i < s.rank; ++i) count *= s.dims[i];
    *rank = s.rank;
    for (int i = 0; i < 3; ++i) dims[i] = i < s.rank ? (int64_t)s.dims[i] : 0;
    const unsigned char *src = s.layout == 0 ? s.compact : at_(&f, s.addr, count * (uint64_t)s.size);
    if (!src || (uint64_t)capacity < count || s.bytes < count * (uint64_t)s.size) {
        close_file(&f);
        return fail(-1, "%s: %s data out of range or output too small", path, name);
    }
    for (uint64_t k = 0; k < count; ++k) out[k] = load_elem(src + k * (uint64_t)s.size, s.size, s.big);
    close_file(&f);
    return 0;
}

typedef struct {
    int want, at;
    char *name;
    int cap;
    uint64_t oh;
    int found;
} nth_t;

static int nth_cb(const char *name, uint64_t oh, void *u)
{
    nth_t *q = (nth_t *)u;
    if (q->at++ == q->want) {
        snprintf(q->name, (size_t)q->cap, "%s", name);
        q->oh = oh;
        q->found = 1;
        return 1;
    }
    return 0;
}

int h5ref_list(const char *path, int i, char *name, int name_cap, int *rank, int64_t dims[3])
{
    file_t f;
    int rc = open_file(path, &f);
    if (rc) return rc;
    char tmp[8];
    nth_t q = {i, 0, name ? name : tmp, name ? name_cap : (int)sizeof tmp, 0, 0};
    rc = walk_root(&f, nth_cb, &q);
    if (rc < 0 || !q.found) {
        close_file(&f);
        return rc < 0 ? rc : fail(-3, "no object %d", i);
    }
    dset_t s;
    rc = describe(&f, q.oh, &s);
    if (rank) *rank = rc ? -1 : s.rank;
    for (int d = 0; d < 3 && dims; ++d) dims[d] = (!rc && d < s.rank) ? (int64_t)s.dims[d] : 0;
    close_file(&f);
    return 0;
}
