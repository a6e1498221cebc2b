/* HDF5 datasets of the reference's stage files, read and written without libhdf5.
 *
 * What is read and written, and why that subset, is stated in include/kevd_h5.h.  The
 * structures follow the public HDF5 file format specification:
 *   superblock (versions 0-3), object header prefix (versions 1 and 2) and its messages
 *   (dataspace 0x0001, link info 0x0002, datatype 0x0003, fill value 0x0005, link 0x0006,
 *   external files 0x0007, layout 0x0008, filter pipeline 0x000B, continuation 0x0010,
 *   symbol table 0x0011), version 1 B-tree nodes of type 0 ("TREE"), group symbol
 *   nodes ("SNOD") and local heaps ("HEAP").
 * Addresses in a file are relative to the superblock's position (a user block may come
 * before it); the end-of-file address in the superblock is absolute.
 *
 * A written file is laid out as
 *   superblock (96 B) | root group object header (48 B) | per dataset: its elements,
 *   then its object header (128 B for floats, 120 B for integers) | root group index:
 *   local heap (32 B header + names), symbol nodes (328 B each, 8 entries), one level-0
 *   B-tree node (544 B).
 * Appending writes the new elements and object header after the last byte, a new index
 * after them, and repoints the root group's symbol-table message and the superblock at
 * the new index: nothing already written moves, and the old index becomes unused space.
 */
#define _FILE_OFFSET_BITS 64
#define _POSIX_C_SOURCE 200809L

#include "kevd_h5.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/types.h>

static _Thread_local char g_err[512];

static int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

const char* kevd_h5_last_error(void) { return g_err; }

static const uint8_t kSignature[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
static const uint64_t kUndef = UINT64_MAX;

/* Bounds on what one file may ask the reader to hold or walk. */
enum {
    kMaxHeaderBytes = 1 << 24,   /* one object header chunk or continuation block */
    kMaxHeapBytes = 1 << 26,     /* one local heap data segment                   */
    kMaxChunks = 1024,           /* object header chunks per object               */
    kMaxMessages = 1 << 16,      /* messages per object                           */
    kMaxDepth = 32,              /* B-tree levels and group nesting               */
    kMaxRank = 32
};

/* Message types. */
enum {
    kMsgNil = 0x0000,
    kMsgDataspace = 0x0001,
    kMsgLinkInfo = 0x0002,
    kMsgDatatype = 0x0003,
    kMsgFill = 0x0005,
    kMsgLink = 0x0006,
    kMsgExternal = 0x0007,
    kMsgLayout = 0x0008,
    kMsgFilters = 0x000B,
    kMsgContinuation = 0x0010,
    kMsgSymbolTable = 0x0011
};

/* Group node K values of files this library creates (libhdf5's defaults). */
enum { kLeafK = 4, kNodeK = 16 };

static uint64_t getle(const uint8_t* p, int n) {
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}

static void putle(uint8_t* p, uint64_t v, int n) {
    for (int i = 0; i < n; ++i) {
        p[i] = (uint8_t)(v & 0xff);
        v >>= 8;
    }
}

static int undefined(uint64_t a, int n) { return n >= 8 ? a == kUndef : a == ((1ull << (8 * n)) - 1); }

static uint64_t align8(uint64_t v) { return (v + 7) & ~(uint64_t)7; }

static int host_is_little_endian(void) {
    const uint16_t one = 1;
    uint8_t b;
    memcpy(&b, &one, 1);
    return b == 1;
}

/* ------------------------------------------------------------------ file access */

typedef struct {
    FILE* f;
    const char* path;
    uint64_t fsize;      /* bytes in the file                                   */
    uint64_t base;       /* absolute position of the superblock                 */
    int version;         /* superblock version                                  */
    int so, sl;          /* sizes of offsets and of lengths                     */
    int leaf_k, node_k;  /* group node K (versions 0 and 1)                     */
    uint64_t eof;        /* end-of-file address stored in the superblock (abs)  */
    uint64_t root;       /* root group object header (relative)                 */
    uint64_t eof_field;  /* absolute position of the superblock's EOF field     */
    uint64_t root_entry; /* absolute position of the root symbol table entry    */
} h5file;

static int rd(h5file* h, uint64_t addr, void* buf, uint64_t n) {
    if (undefined(addr, h->so) || addr > h->fsize - h->base || n > h->fsize - h->base - addr)
        return fail(KEVD_H5_ERR_FORMAT, "%s: address %llu + %llu bytes is outside the file", h->path,
                    (unsigned long long)addr, (unsigned long long)n);
    if (n == 0) return KEVD_H5_OK;
    if (fseeko(h->f, (off_t)(h->base + addr), SEEK_SET) != 0 || fread(buf, 1, (size_t)n, h->f) != n)
        return fail(KEVD_H5_ERR_IO, "%s: read failed", h->path);
    return KEVD_H5_OK;
}

static int wr_abs(h5file* h, uint64_t pos, const void* buf, uint64_t n) {
    if (n == 0) return KEVD_H5_OK;
    if (fseeko(h->f, (off_t)pos, SEEK_SET) != 0 || fwrite(buf, 1, (size_t)n, h->f) != n)
        return fail(KEVD_H5_ERR_IO, "%s: write failed", h->path);
    return KEVD_H5_OK;
}

static void h5_close(h5file* h) {
    if (h->f) fclose(h->f);
    h->f = NULL;
}

/* Opens `path` and decodes its superblock. */
static int h5_open(h5file* h, const char* path, const char* mode) {
    memset(h, 0, sizeof(*h));
    h->path = path;
    if (!path) return fail(KEVD_H5_ERR_ARG, "null path");
    h->f = fopen(path, mode);
    if (!h->f) return fail(KEVD_H5_ERR_IO, "%s: cannot open", path);
    if (fseeko(h->f, 0, SEEK_END) != 0) {
        h5_close(h);
        return fail(KEVD_H5_ERR_IO, "%s: cannot seek", path);
    }
    h->fsize = (uint64_t)ftello(h->f);
    /* The superblock sits at 0, 512, 1024, 2048, ... */
    uint64_t at = 0;
    int found = 0;
    for (;;) {
        uint8_t sig[8];
        if (at + 8 > h->fsize) break;
        if (fseeko(h->f, (off_t)at, SEEK_SET) != 0 || fread(sig, 1, 8, h->f) != 8) break;
        if (memcmp(sig, kSignature, 8) == 0) {
            found = 1;
            break;
        }
        at = at ? 2 * at : 512;
    }
    if (!found) {
        h5_close(h);
        return fail(KEVD_H5_ERR_FORMAT, "%s: no HDF5 superblock", path);
    }
    h->base = at;
    uint8_t sb[160];
    memset(sb, 0, sizeof(sb));
    const uint64_t avail = h->fsize - at < sizeof(sb) ? h->fsize - at : sizeof(sb);
    if (fseeko(h->f, (off_t)at, SEEK_SET) != 0 || fread(sb, 1, (size_t)avail, h->f) != avail) {
        h5_close(h);
        return fail(KEVD_H5_ERR_IO, "%s: read failed", path);
    }
    h->version = sb[8];
    uint64_t need = 0;
    if (h->version == 0 || h->version == 1) {
        h->so = sb[13];
        h->sl = sb[14];
        h->leaf_k = (int)getle(sb + 16, 2);
        h->node_k = (int)getle(sb + 18, 2);
        int p = 24 + (h->version == 1 ? 4 : 0);
        if ((h->so != 2 && h->so != 4 && h->so != 8) || (h->sl != 2 && h->sl != 4 && h->sl != 8)) goto bad;
        need = (uint64_t)p + 4 * h->so + 2 * h->so + 24;
        if (need > avail) goto bad;
        p += h->so;                       /* base address (the superblock's own position) */
        p += h->so;                       /* free-space info address                      */
        h->eof_field = at + (uint64_t)p;
        h->eof = getle(sb + p, h->so);
        p += h->so;
        p += h->so;                       /* driver information block                     */
        h->root_entry = at + (uint64_t)p; /* root group symbol table entry                */
        h->root = getle(sb + p + h->so, h->so);
    } else if (h->version == 2 || h->version == 3) {
        h->so = sb[9];
        h->sl = sb[10];
        if ((h->so != 2 && h->so != 4 && h->so != 8) || (h->sl != 2 && h->sl != 4 && h->sl != 8)) goto bad;
        int p = 12;
        need = (uint64_t)p + 4 * h->so + 4;
        if (need > avail) goto bad;
        p += h->so;                       /* base address       */
        p += h->so;                       /* extension address  */
        h->eof_field = at + (uint64_t)p;
        h->eof = getle(sb + p, h->so);
        p += h->so;
        h->root = getle(sb + p, h->so);
    } else {
        h5_close(h);
        return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: superblock version %d", path, h->version);
    }
    return KEVD_H5_OK;
bad:
    h5_close(h);
    return fail(KEVD_H5_ERR_FORMAT, "%s: corrupt superblock", path);
}

/* ------------------------------------------------------------------ object headers */

typedef struct {
    uint16_t type;
    uint8_t flags;
    uint32_t len;
    uint64_t addr;   /* relative address of the message data */
    uint8_t* data;
} h5msg;

typedef struct {
    h5msg* m;
    int n, cap;
} h5obj;

static void obj_free(h5obj* o) {
    for (int i = 0; i < o->n; ++i) free(o->m[i].data);
    free(o->m);
    memset(o, 0, sizeof(*o));
}

static int obj_push(h5obj* o, uint16_t type, uint8_t flags, const uint8_t* data, uint32_t len, uint64_t addr) {
    if (o->n >= kMaxMessages) return fail(KEVD_H5_ERR_FORMAT, "too many object header messages");
    if (o->n == o->cap) {
        const int cap = o->cap ? 2 * o->cap : 16;
        h5msg* m = (h5msg*)realloc(o->m, (size_t)cap * sizeof(h5msg));
        if (!m) return fail(KEVD_H5_ERR_IO, "out of host memory");
        o->m = m;
        o->cap = cap;
    }
    uint8_t* copy = (uint8_t*)malloc(len ? len : 1);
    if (!copy) return fail(KEVD_H5_ERR_IO, "out of host memory");
    memcpy(copy, data, len);
    h5msg* e = &o->m[o->n++];
    e->type = type;
    e->flags = flags;
    e->len = len;
    e->addr = addr;
    e->data = copy;
    return KEVD_H5_OK;
}

typedef struct {
    uint64_t addr, len;
} h5span;

/* Messages of one chunk: version 1 headers use an 8-byte message header (type 2,
 * size 2, flags 1, reserved 3), version 2 a 4- or 6-byte one (type 1, size 2, flags 1,
 * creation order 2 when the object tracks it). */
static int parse_chunk(h5file* h, h5obj* o, const uint8_t* b, uint64_t n, uint64_t addr, int v2, int track_order,
                       h5span* conts, int* nconts) {
    const uint64_t hdr = v2 ? (track_order ? 6u : 4u) : 8u;
    uint64_t p = 0;
    while (p + hdr <= n) {
        uint16_t type;
        uint32_t len;
        uint8_t flags;
        if (v2) {
            type = b[p];
            len = (uint32_t)getle(b + p + 1, 2);
            flags = b[p + 3];
        } else {
            type = (uint16_t)getle(b + p, 2);
            len = (uint32_t)getle(b + p + 2, 2);
            flags = b[p + 4];
        }
        if (p + hdr + len > n) return fail(KEVD_H5_ERR_FORMAT, "%s: object header message overruns its chunk", h->path);
        const uint8_t* d = b + p + hdr;
        if (type == kMsgContinuation) {
            if (len < (uint32_t)(h->so + h->sl)) return fail(KEVD_H5_ERR_FORMAT, "%s: short continuation message", h->path);
            if (*nconts >= kMaxChunks) return fail(KEVD_H5_ERR_FORMAT, "%s: too many object header chunks", h->path);
            conts[*nconts].addr = getle(d, h->so);
            conts[*nconts].len = getle(d + h->so, h->sl);
            ++*nconts;
        }
        int s = obj_push(o, type, flags, d, len, addr + p + hdr);
        if (s) return s;
        p += hdr + len;
    }
    return KEVD_H5_OK;
}

static int read_block(h5file* h, uint64_t addr, uint64_t n, uint8_t** out) {
    if (n > kMaxHeaderBytes) return fail(KEVD_H5_ERR_FORMAT, "%s: object header chunk of %llu bytes", h->path,
                                         (unsigned long long)n);
    uint8_t* b = (uint8_t*)malloc(n ? n : 1);
    if (!b) return fail(KEVD_H5_ERR_IO, "out of host memory");
    int s = rd(h, addr, b, n);
    if (s) {
        free(b);
        return s;
    }
    *out = b;
    return KEVD_H5_OK;
}

/* All messages of the object whose header is at `addr`, continuation blocks included. */
static int obj_read(h5file* h, uint64_t addr, h5obj* o) {
    memset(o, 0, sizeof(*o));
    h5span* conts = (h5span*)malloc(kMaxChunks * sizeof(h5span));
    if (!conts) return fail(KEVD_H5_ERR_IO, "out of host memory");
    int nconts = 0, s = KEVD_H5_OK, v2 = 0, track = 0;
    uint8_t pre[40] = {0};
    uint8_t* chunk = NULL;
    s = rd(h, addr, pre, 16);
    if (s) goto done;
    if (memcmp(pre, "OHDR", 4) == 0) {
        v2 = 1;
        s = rd(h, addr, pre, sizeof(pre) < h->fsize - h->base - addr ? sizeof(pre) : h->fsize - h->base - addr);
        if (s) goto done;
        if (pre[4] != 2) {
            s = fail(KEVD_H5_ERR_UNSUPPORTED, "%s: object header version %d", h->path, pre[4]);
            goto done;
        }
        const uint8_t fl = pre[5];
        track = (fl & 0x04) != 0;
        uint64_t p = 6;
        if (fl & 0x20) p += 16;   /* access, modification, change, birth times */
        if (fl & 0x10) p += 4;    /* attribute phase change values             */
        const int w = 1 << (fl & 3);
        const uint64_t size = getle(pre + p, w);
        p += (uint64_t)w;
        s = read_block(h, addr + p, size, &chunk);
        if (s) goto done;
        s = parse_chunk(h, o, chunk, size, addr + p, 1, track, conts, &nconts);
        free(chunk);
        chunk = NULL;
    } else if (pre[0] == 1) {
        const uint64_t size = getle(pre + 8, 4);
        s = read_block(h, addr + 16, size, &chunk);
        if (s) goto done;
        s = parse_chunk(h, o, chunk, size, addr + 16, 0, 0, conts, &nconts);
        free(chunk);
        chunk = NULL;
    } else {
        s = fail(KEVD_H5_ERR_UNSUPPORTED, "%s: object header version %d", h->path, pre[0]);
    }
    for (int c = 0; s == KEVD_H5_OK && c < nconts; ++c) {
        s = read_block(h, conts[c].addr, conts[c].len, &chunk);
        if (s) break;
        if (v2) {
            if (conts[c].len < 8 || memcmp(chunk, "OCHK", 4) != 0) {
                s = fail(KEVD_H5_ERR_FORMAT, "%s: bad continuation block", h->path);
            } else {
                s = parse_chunk(h, o, chunk + 4, conts[c].len - 8, conts[c].addr + 4, 1, track, conts, &nconts);
            }
        } else {
            s = parse_chunk(h, o, chunk, conts[c].len, conts[c].addr, 0, 0, conts, &nconts);
        }
        free(chunk);
        chunk = NULL;
    }
done:
    free(conts);
    if (s) obj_free(o);
    return s;
}

static const h5msg* obj_find(const h5obj* o, uint16_t type) {
    for (int i = 0; i < o->n; ++i)
        if (o->m[i].type == type) return &o->m[i];
    return NULL;
}

/* ------------------------------------------------------------------ groups */

/* Called for each link: name (not NUL-terminated), its object header and, for
 * symbol-table groups, the 40-byte (8-byte address) entry it came from.  Returns 0 to
 * go on, 1 to stop, or an error code above 1 (offset by 100). */
typedef int (*link_fn)(void* ctx, const char* name, size_t nlen, uint64_t obj, const uint8_t* entry);

typedef struct {
    uint8_t* data;
    uint64_t size;
} h5heap;

static int heap_load(h5file* h, uint64_t addr, h5heap* out) {
    uint8_t b[32];
    const uint64_t hs = 8 + 2 * (uint64_t)h->sl + h->so;
    int s = rd(h, addr, b, hs);
    if (s) return s;
    if (memcmp(b, "HEAP", 4) != 0 || b[4] != 0) return fail(KEVD_H5_ERR_FORMAT, "%s: bad local heap", h->path);
    const uint64_t size = getle(b + 8, h->sl);
    const uint64_t data = getle(b + 8 + 2 * h->sl, h->so);
    if (size > kMaxHeapBytes) return fail(KEVD_H5_ERR_FORMAT, "%s: local heap of %llu bytes", h->path,
                                          (unsigned long long)size);
    out->data = (uint8_t*)malloc(size + 1);
    if (!out->data) return fail(KEVD_H5_ERR_IO, "out of host memory");
    out->size = size;
    s = rd(h, data, out->data, size);
    if (s) {
        free(out->data);
        out->data = NULL;
        return s;
    }
    out->data[size] = 0;
    return KEVD_H5_OK;
}

static int heap_name(h5file* h, const h5heap* hp, uint64_t off, const char** name, size_t* nlen) {
    if (off >= hp->size) return fail(KEVD_H5_ERR_FORMAT, "%s: link name outside the local heap", h->path);
    const char* s = (const char*)hp->data + off;
    const size_t n = strnlen(s, (size_t)(hp->size - off));
    if (n == hp->size - off) return fail(KEVD_H5_ERR_FORMAT, "%s: unterminated link name", h->path);
    *name = s;
    *nlen = n;
    return KEVD_H5_OK;
}

static int snod_walk(h5file* h, uint64_t addr, const h5heap* hp, link_fn fn, void* ctx) {
    uint8_t b[8];
    int s = rd(h, addr, b, 8);
    if (s) return s;
    if (memcmp(b, "SNOD", 4) != 0 || b[4] != 1) return fail(KEVD_H5_ERR_FORMAT, "%s: bad symbol table node", h->path);
    const uint64_t nsym = getle(b + 6, 2), esz = 2 * (uint64_t)h->so + 24;
    uint8_t* e = (uint8_t*)malloc(nsym * esz + 1);
    if (!e) return fail(KEVD_H5_ERR_IO, "out of host memory");
    s = rd(h, addr + 8, e, nsym * esz);
    for (uint64_t i = 0; s == KEVD_H5_OK && i < nsym; ++i) {
        const uint8_t* en = e + i * esz;
        const char* name = NULL;
        size_t nlen = 0;
        s = heap_name(h, hp, getle(en, h->so), &name, &nlen);
        if (s) break;
        const int r = fn(ctx, name, nlen, getle(en + h->so, h->so), en);
        if (r == 1) s = 1;
        else if (r > 1) s = r;
    }
    free(e);
    return s;
}

static int btree_walk(h5file* h, uint64_t addr, int expect_level, int depth, const h5heap* hp, link_fn fn,
                      void* ctx) {
    if (depth > kMaxDepth) return fail(KEVD_H5_ERR_FORMAT, "%s: B-tree too deep", h->path);
    uint8_t b[8];
    int s = rd(h, addr, b, 8);
    if (s) return s;
    if (memcmp(b, "TREE", 4) != 0 || b[4] != 0) return fail(KEVD_H5_ERR_FORMAT, "%s: bad group B-tree node", h->path);
    const int level = b[5];
    if (expect_level >= 0 && level != expect_level) return fail(KEVD_H5_ERR_FORMAT, "%s: B-tree levels out of order", h->path);
    const uint64_t n = getle(b + 6, 2);
    const uint64_t kv = 8 + 2 * (uint64_t)h->so;        /* keys and children start here */
    const uint64_t bytes = (n + 1) * h->sl + n * h->so;
    uint8_t* kc = (uint8_t*)malloc(bytes + 1);
    if (!kc) return fail(KEVD_H5_ERR_IO, "out of host memory");
    s = rd(h, addr + kv, kc, bytes);
    for (uint64_t i = 0; s == KEVD_H5_OK && i < n; ++i) {
        const uint64_t child = getle(kc + h->sl + i * (h->sl + h->so), h->so);
        s = level > 0 ? btree_walk(h, child, level - 1, depth + 1, hp, fn, ctx) : snod_walk(h, child, hp, fn, ctx);
    }
    free(kc);
    return s;
}

/* Every link of the group whose object header is at `grp`. */
static int group_walk(h5file* h, uint64_t grp, link_fn fn, void* ctx) {
    h5obj o;
    int s = obj_read(h, grp, &o);
    if (s) return s;
    const h5msg* st = obj_find(&o, kMsgSymbolTable);
    if (st) {
        if (st->len < (uint32_t)(2 * h->so)) {
            obj_free(&o);
            return fail(KEVD_H5_ERR_FORMAT, "%s: short symbol table message", h->path);
        }
        const uint64_t bt = getle(st->data, h->so), heap = getle(st->data + h->so, h->so);
        obj_free(&o);
        h5heap hp = {NULL, 0};
        s = heap_load(h, heap, &hp);
        if (s) return s;
        s = btree_walk(h, bt, -1, 0, &hp, fn, ctx);
        free(hp.data);
        return s;
    }
    const h5msg* li = obj_find(&o, kMsgLinkInfo);
    if (li && li->len >= 2 + (uint32_t)h->so) {
        const uint64_t fheap = getle(li->data + 2 + ((li->data[1] & 1) ? 8 : 0), h->so);
        if (!undefined(fheap, h->so)) {
            obj_free(&o);
            return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: group with dense link storage", h->path);
        }
    }
    for (int i = 0; s == KEVD_H5_OK && i < o.n; ++i) {
        const h5msg* m = &o.m[i];
        if (m->type != kMsgLink) continue;
        const uint8_t* d = m->data;
        const uint64_t L = m->len;
        if (L < 2 || d[0] != 1) {
            s = fail(KEVD_H5_ERR_FORMAT, "%s: bad link message", h->path);
            break;
        }
        const uint8_t fl = d[1];
        uint64_t p = 2;
        int ltype = 0;
        if (fl & 0x08) ltype = d[p++];
        if (fl & 0x04) p += 8;
        if (fl & 0x10) p += 1;
        const int w = 1 << (fl & 3);
        if (p + (uint64_t)w > L) {
            s = fail(KEVD_H5_ERR_FORMAT, "%s: bad link message", h->path);
            break;
        }
        const uint64_t nlen = getle(d + p, w);
        p += (uint64_t)w;
        if (p + nlen > L) {
            s = fail(KEVD_H5_ERR_FORMAT, "%s: bad link message", h->path);
            break;
        }
        const char* name = (const char*)d + p;
        p += nlen;
        if (ltype != 0) continue;       /* soft and external links name no object here */
        if (p + (uint64_t)h->so > L) {
            s = fail(KEVD_H5_ERR_FORMAT, "%s: bad link message", h->path);
            break;
        }
        const int r = fn(ctx, name, (size_t)nlen, getle(d + p, h->so), NULL);
        if (r == 1) s = 1;
        else if (r > 1) s = r;
    }
    obj_free(&o);
    return s;
}

typedef struct {
    const char* name;
    size_t nlen;
    uint64_t obj;
    int found;
} find_ctx;

static int find_fn(void* c, const char* name, size_t nlen, uint64_t obj, const uint8_t* entry) {
    (void)entry;
    find_ctx* f = (find_ctx*)c;
    if (nlen == f->nlen && memcmp(name, f->name, nlen) == 0) {
        f->obj = obj;
        f->found = 1;
        return 1;
    }
    return 0;
}

/* Object header of the object at `path` ("/a/b", "a/b"). */
static int resolve(h5file* h, const char* path, uint64_t* obj) {
    uint64_t cur = h->root;
    const char* p = path;
    int depth = 0;
    while (*p) {
        while (*p == '/') ++p;
        if (!*p) break;
        const char* e = p;
        while (*e && *e != '/') ++e;
        if (++depth > kMaxDepth) return fail(KEVD_H5_ERR_ARG, "path too deep: %s", path);
        find_ctx f = {p, (size_t)(e - p), 0, 0};
        int s = group_walk(h, cur, find_fn, &f);
        if (s > 1) return s;
        if (!f.found) return fail(KEVD_H5_ERR_NOTFOUND, "%s: no object %.*s in %s", h->path, (int)(e - p), p, path);
        cur = f.obj;
        p = e;
    }
    *obj = cur;
    return KEVD_H5_OK;
}

/* ------------------------------------------------------------------ datasets */

typedef struct {
    int rank;
    uint64_t dims[kMaxRank];
    uint64_t count;
    int is_float;      /* IEEE binary32/binary64, else integer */
    int size;          /* bytes per element                     */
    int is_signed;
    int big_endian;
    int compact;
    uint64_t addr;     /* contiguous storage (relative)         */
    uint8_t* inline_data;
    uint64_t inline_len;
} h5dset;

static int parse_dataspace(h5file* h, const h5msg* m, h5dset* d) {
    const uint8_t* b = m->data;
    if (m->len < 4) return fail(KEVD_H5_ERR_FORMAT, "%s: short dataspace message", h->path);
    const int ver = b[0];
    d->rank = b[1];
    uint64_t p;
    int type = 1;
    if (ver == 1) {
        p = 8;
    } else if (ver == 2) {
        type = b[3];
        p = 4;
    } else {
        return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: dataspace version %d", h->path, ver);
    }
    if (d->rank > kMaxRank) return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: rank %d", h->path, d->rank);
    if (p + (uint64_t)d->rank * h->sl > m->len) return fail(KEVD_H5_ERR_FORMAT, "%s: short dataspace message", h->path);
    d->count = 1;
    for (int i = 0; i < d->rank; ++i) {
        d->dims[i] = getle(b + p + (uint64_t)i * h->sl, h->sl);
        if (d->dims[i] && d->count > (UINT64_C(1) << 62) / d->dims[i])
            return fail(KEVD_H5_ERR_FORMAT, "%s: dataspace too large", h->path);
        d->count *= d->dims[i];
    }
    if (type == 2) {        /* null dataspace */
        d->rank = 0;
        d->count = 0;
    } else if (type == 0) { /* scalar */
        d->rank = 0;
        d->count = 1;
    }
    return KEVD_H5_OK;
}

static int parse_datatype(h5file* h, const h5msg* m, h5dset* d) {
    const uint8_t* b = m->data;
    if (m->flags & 0x02) return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: committed (shared) datatype", h->path);
    if (m->len < 8) return fail(KEVD_H5_ERR_FORMAT, "%s: short datatype message", h->path);
    const int cls = b[0] & 0x0f;
    d->size = (int)getle(b + 4, 4);
    if (cls == 0) {
        if (m->len < 12) return fail(KEVD_H5_ERR_FORMAT, "%s: short datatype message", h->path);
        d->is_float = 0;
        d->big_endian = b[1] & 1;
        d->is_signed = (b[1] >> 3) & 1;
        const int off = (int)getle(b + 8, 2), prec = (int)getle(b + 10, 2);
        if ((d->size != 1 && d->size != 2 && d->size != 4 && d->size != 8) || off != 0 || prec != 8 * d->size)
            return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: integer of %d bytes, precision %d at bit %d", h->path,
                        d->size, prec, off);
        return KEVD_H5_OK;
    }
    if (cls == 1) {
        if (m->len < 20) return fail(KEVD_H5_ERR_FORMAT, "%s: short datatype message", h->path);
        if (b[1] & 0x40) return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: VAX float order", h->path);
        d->is_float = 1;
        d->big_endian = b[1] & 1;
        d->is_signed = 1;
        const int sign = b[2], off = (int)getle(b + 8, 2), prec = (int)getle(b + 10, 2);
        const int eloc = b[12], esz = b[13], mloc = b[14], msz = b[15];
        const uint32_t bias = (uint32_t)getle(b + 16, 4);
        const int f32 = d->size == 4 && sign == 31 && off == 0 && prec == 32 && eloc == 23 && esz == 8 && mloc == 0 &&
                        msz == 23 && bias == 127;
        const int f64 = d->size == 8 && sign == 63 && off == 0 && prec == 64 && eloc == 52 && esz == 11 && mloc == 0 &&
                        msz == 52 && bias == 1023;
        if (!f32 && !f64) return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: non-IEEE floating-point layout", h->path);
        return KEVD_H5_OK;
    }
    return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: datatype class %d", h->path, cls);
}

static int parse_layout(h5file* h, const h5msg* m, h5dset* d) {
    const uint8_t* b = m->data;
    const uint64_t L = m->len;
    if (L < 2) return fail(KEVD_H5_ERR_FORMAT, "%s: short layout message", h->path);
    const int ver = b[0];
    int cls;
    if (ver == 1 || ver == 2) {
        if (L < 8) return fail(KEVD_H5_ERR_FORMAT, "%s: short layout message", h->path);
        const int nd = b[1];
        cls = b[2];
        uint64_t p = 8;
        if (cls == 2) return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: chunked dataset", h->path);
        if (cls == 1) {
            if (p + (uint64_t)h->so > L) return fail(KEVD_H5_ERR_FORMAT, "%s: short layout message", h->path);
            d->addr = getle(b + p, h->so);
            return KEVD_H5_OK;
        }
        if (cls != 0) return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: layout class %d", h->path, cls);
        p += 4 * (uint64_t)nd;
        if (p + 4 > L) return fail(KEVD_H5_ERR_FORMAT, "%s: short layout message", h->path);
        d->compact = 1;
        d->inline_len = getle(b + p, 4);
        d->inline_data = (uint8_t*)b + p + 4;
        if (p + 4 + d->inline_len > L) return fail(KEVD_H5_ERR_FORMAT, "%s: short layout message", h->path);
        return KEVD_H5_OK;
    }
    if (ver == 3 || ver == 4) {
        cls = b[1];
        if (cls == 0) {
            if (L < 4) return fail(KEVD_H5_ERR_FORMAT, "%s: short layout message", h->path);
            d->compact = 1;
            d->inline_len = getle(b + 2, 2);
            d->inline_data = (uint8_t*)b + 4;
            if (4 + d->inline_len > L) return fail(KEVD_H5_ERR_FORMAT, "%s: short layout message", h->path);
            return KEVD_H5_OK;
        }
        if (cls == 1) {
            if (2 + (uint64_t)h->so + h->sl > L) return fail(KEVD_H5_ERR_FORMAT, "%s: short layout message", h->path);
            d->addr = getle(b + 2, h->so);
            return KEVD_H5_OK;
        }
        if (cls == 2) return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: chunked dataset", h->path);
        return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: layout class %d", h->path, cls);
    }
    return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: layout version %d", h->path, ver);
}

/* Describes the dataset at `name`; the object's messages stay in `o` (compact data
 * points into them). */
static int dset_open(h5file* h, const char* name, h5dset* d, h5obj* o) {
    memset(d, 0, sizeof(*d));
    uint64_t obj = 0;
    int s = resolve(h, name, &obj);
    if (s) return s;
    s = obj_read(h, obj, o);
    if (s) return s;
    const h5msg *sp = obj_find(o, kMsgDataspace), *ty = obj_find(o, kMsgDatatype), *ly = obj_find(o, kMsgLayout);
    if (!sp || !ty || !ly) {
        const int group = obj_find(o, kMsgSymbolTable) || obj_find(o, kMsgLink) || obj_find(o, kMsgLinkInfo);
        obj_free(o);
        return group ? fail(KEVD_H5_ERR_ARG, "%s: %s is a group", h->path, name)
                     : fail(KEVD_H5_ERR_FORMAT, "%s: %s is not a dataset", h->path, name);
    }
    if (obj_find(o, kMsgFilters)) s = fail(KEVD_H5_ERR_UNSUPPORTED, "%s: %s is filtered (compressed)", h->path, name);
    else if (obj_find(o, kMsgExternal)) s = fail(KEVD_H5_ERR_UNSUPPORTED, "%s: %s has external storage", h->path, name);
    if (!s) s = parse_dataspace(h, sp, d);
    if (!s) s = parse_datatype(h, ty, d);
    if (!s) s = parse_layout(h, ly, d);
    if (!s && d->compact && d->inline_len < d->count * (uint64_t)d->size)
        s = fail(KEVD_H5_ERR_FORMAT, "%s: compact data shorter than its dataspace", h->path);
    if (s) obj_free(o);
    return s;
}

static int type_size(int32_t t) {
    switch (t) {
        case KEVD_H5_F32: case KEVD_H5_I32: case KEVD_H5_U32: return 4;
        case KEVD_H5_F64: case KEVD_H5_I64: case KEVD_H5_U64: return 8;
        default: return 0;
    }
}

/* One stored element, decoded: a double for floats, a signed or unsigned 64-bit integer. */
typedef struct {
    int kind;   /* 0 double, 1 int64, 2 uint64 */
    double f;
    int64_t i;
    uint64_t u;
} h5val;

static h5val decode(const uint8_t* p, const h5dset* d) {
    uint8_t b[8];
    for (int k = 0; k < d->size; ++k) b[k] = d->big_endian ? p[d->size - 1 - k] : p[k];
    const uint64_t bits = getle(b, d->size);
    h5val v = {0, 0.0, 0, 0};
    if (d->is_float) {
        if (d->size == 4) {
            const uint32_t w = (uint32_t)bits;
            float x;
            memcpy(&x, &w, 4);
            v.f = x;
        } else {
            memcpy(&v.f, &bits, 8);
        }
    } else if (d->is_signed) {
        v.kind = 1;
        const int sh = 64 - 8 * d->size;
        v.i = (int64_t)(bits << sh) >> sh;
    } else {
        v.kind = 2;
        v.u = bits;
    }
    return v;
}

static void encode(h5val v, int32_t t, uint8_t* out) {
    if (t == KEVD_H5_F32 || t == KEVD_H5_F64) {
        const double x = v.kind == 0 ? v.f : v.kind == 1 ? (double)v.i : (double)v.u;
        if (t == KEVD_H5_F32) {
            const float y = v.kind == 0 ? (float)v.f : v.kind == 1 ? (float)v.i : (float)v.u;
            memcpy(out, &y, 4);
        } else {
            memcpy(out, &x, 8);
        }
        return;
    }
    /* Integer targets: truncate toward zero, clamp to the range, NaN to 0. */
    const int is_signed = t == KEVD_H5_I32 || t == KEVD_H5_I64;
    const int bytes = type_size(t);
    const int64_t smin = bytes == 4 ? INT32_MIN : INT64_MIN, smax = bytes == 4 ? INT32_MAX : INT64_MAX;
    const uint64_t umax = bytes == 4 ? UINT32_MAX : UINT64_MAX;
    uint64_t r = 0;
    if (is_signed) {
        int64_t y;
        if (v.kind == 0) {
            if (isnan(v.f)) y = 0;
            else if (v.f <= (double)smin) y = smin;
            else if (v.f >= (double)smax) y = smax;
            else y = (int64_t)v.f;
        } else if (v.kind == 1) {
            y = v.i < smin ? smin : v.i > smax ? smax : v.i;
        } else {
            y = v.u > (uint64_t)smax ? smax : (int64_t)v.u;
        }
        r = (uint64_t)y;
    } else {
        uint64_t y;
        if (v.kind == 0) {
            if (isnan(v.f) || v.f <= 0.0) y = 0;
            else if (v.f >= (double)umax) y = umax;
            else y = (uint64_t)v.f;
        } else if (v.kind == 1) {
            y = v.i < 0 ? 0 : (uint64_t)v.i > umax ? umax : (uint64_t)v.i;
        } else {
            y = v.u > umax ? umax : v.u;
        }
        r = y;
    }
    if (bytes == 4) {
        const uint32_t w = (uint32_t)r;
        memcpy(out, &w, 4);
    } else {
        memcpy(out, &r, 8);
    }
}

static int same_type(const h5dset* d, int32_t t) {
    if (d->big_endian || !host_is_little_endian()) return 0;
    switch (t) {
        case KEVD_H5_F32: return d->is_float && d->size == 4;
        case KEVD_H5_F64: return d->is_float && d->size == 8;
        case KEVD_H5_I32: return !d->is_float && d->size == 4 && d->is_signed;
        case KEVD_H5_U32: return !d->is_float && d->size == 4 && !d->is_signed;
        case KEVD_H5_I64: return !d->is_float && d->size == 8 && d->is_signed;
        case KEVD_H5_U64: return !d->is_float && d->size == 8 && !d->is_signed;
        default: return 0;
    }
}

static int32_t nearest_type(const h5dset* d) {
    if (d->is_float) return d->size == 4 ? KEVD_H5_F32 : KEVD_H5_F64;
    if (d->size <= 4) return d->is_signed ? KEVD_H5_I32 : KEVD_H5_U32;
    return d->is_signed ? KEVD_H5_I64 : KEVD_H5_U64;
}

int kevd_h5_dataset_info(const char* path, const char* name, int64_t* count, int32_t* type, int32_t* rank,
                         int64_t* dims) {
    if (!name) return fail(KEVD_H5_ERR_ARG, "null dataset name");
    h5file h;
    int s = h5_open(&h, path, "rb");
    if (s) return s;
    h5dset d;
    h5obj o;
    s = dset_open(&h, name, &d, &o);
    if (!s) {
        if (count) *count = (int64_t)d.count;
        if (type) *type = nearest_type(&d);
        if (rank) *rank = d.rank;
        if (dims)
            for (int i = 0; i < d.rank; ++i) dims[i] = (int64_t)d.dims[i];
        obj_free(&o);
    }
    h5_close(&h);
    return s;
}

int kevd_h5_read(const char* path, const char* name, int32_t type, void* out, int64_t count) {
    const int osz = type_size(type);
    if (!name || osz == 0 || count < 0 || (count > 0 && !out))
        return fail(KEVD_H5_ERR_ARG, "kevd_h5_read: bad argument");
    h5file h;
    int s = h5_open(&h, path, "rb");
    if (s) return s;
    h5dset d;
    h5obj o;
    s = dset_open(&h, name, &d, &o);
    if (s) {
        h5_close(&h);
        return s;
    }
    if ((uint64_t)count != d.count) {
        s = fail(KEVD_H5_ERR_ARG, "%s: %s holds %llu elements, %lld expected", path, name,
                 (unsigned long long)d.count, (long long)count);
    } else if (count > 0) {
        const uint64_t bytes = d.count * (uint64_t)d.size;
        uint8_t* dst = (uint8_t*)out;
        if (!d.compact && undefined(d.addr, h.so)) {
            memset(out, 0, (size_t)count * (size_t)osz);       /* never written: the default fill */
        } else if (same_type(&d, type)) {
            if (d.compact) memcpy(out, d.inline_data, (size_t)bytes);
            else s = rd(&h, d.addr, out, bytes);
        } else {
            const uint64_t blk = 1 << 16;
            uint8_t* tmp = d.compact ? NULL : (uint8_t*)malloc(blk * (uint64_t)d.size);
            if (!d.compact && !tmp) s = fail(KEVD_H5_ERR_IO, "out of host memory");
            for (uint64_t i0 = 0; s == KEVD_H5_OK && i0 < d.count; i0 += blk) {
                const uint64_t n = d.count - i0 < blk ? d.count - i0 : blk;
                const uint8_t* src;
                if (d.compact) {
                    src = d.inline_data + i0 * (uint64_t)d.size;
                } else {
                    s = rd(&h, d.addr + i0 * (uint64_t)d.size, tmp, n * (uint64_t)d.size);
                    src = tmp;
                }
                for (uint64_t i = 0; s == KEVD_H5_OK && i < n; ++i)
                    encode(decode(src + i * (uint64_t)d.size, &d), type, dst + (i0 + i) * (uint64_t)osz);
            }
            free(tmp);
        }
    }
    obj_free(&o);
    h5_close(&h);
    return s;
}

typedef struct {
    char* buf;
    uint64_t cap, used;
    int32_t n;
    int overflow;
} list_ctx;

static int list_fn(void* c, const char* name, size_t nlen, uint64_t obj, const uint8_t* entry) {
    (void)obj;
    (void)entry;
    list_ctx* l = (list_ctx*)c;
    if (l->used + nlen + 1 > l->cap) {
        l->overflow = 1;
        return 1;
    }
    memcpy(l->buf + l->used, name, nlen);
    l->buf[l->used + nlen] = 0;
    l->used += nlen + 1;
    ++l->n;
    return 0;
}

int kevd_h5_list(const char* path, char* buf, int64_t cap, int32_t* n) {
    if (!buf || cap < 0 || !n) return fail(KEVD_H5_ERR_ARG, "kevd_h5_list: bad argument");
    h5file h;
    int s = h5_open(&h, path, "rb");
    if (s) return s;
    list_ctx l = {buf, (uint64_t)cap, 0, 0, 0};
    s = group_walk(&h, h.root, list_fn, &l);
    h5_close(&h);
    if (s > 1) return s;
    if (l.overflow) return fail(KEVD_H5_ERR_ARG, "%s: the names need more than %lld bytes", path, (long long)cap);
    *n = l.n;
    return KEVD_H5_OK;
}

/* ------------------------------------------------------------------ writing */

/* One link of the root group being written: its name and the 40-byte symbol table
 * entry (name offset, object header, cache type, reserved, scratch pad). */
typedef struct {
    char* name;
    uint8_t entry[40];
} h5link;

static int link_cmp(const void* a, const void* b) {
    return strcmp(((const h5link*)a)->name, ((const h5link*)b)->name);
}

typedef struct {
    h5link* v;
    int n, cap;
} link_list;

static void links_free(link_list* l) {
    for (int i = 0; i < l->n; ++i) free(l->v[i].name);
    free(l->v);
    memset(l, 0, sizeof(*l));
}

static int links_push(link_list* l, const char* name, size_t nlen, const uint8_t* entry40) {
    if (l->n == l->cap) {
        const int cap = l->cap ? 2 * l->cap : 16;
        h5link* v = (h5link*)realloc(l->v, (size_t)cap * sizeof(h5link));
        if (!v) return fail(KEVD_H5_ERR_IO, "out of host memory");
        l->v = v;
        l->cap = cap;
    }
    char* s = (char*)malloc(nlen + 1);
    if (!s) return fail(KEVD_H5_ERR_IO, "out of host memory");
    memcpy(s, name, nlen);
    s[nlen] = 0;
    l->v[l->n].name = s;
    memcpy(l->v[l->n].entry, entry40, 40);
    ++l->n;
    return KEVD_H5_OK;
}

static int collect_fn(void* c, const char* name, size_t nlen, uint64_t obj, const uint8_t* entry) {
    (void)obj;
    if (!entry) return 100 + fail(KEVD_H5_ERR_UNSUPPORTED, "root group is not a symbol table");
    const int s = links_push((link_list*)c, name, nlen, entry);
    return s ? 100 + s : 0;
}

/* Writes the root group's index (local heap, symbol nodes, one B-tree node) at the
 * relative address `at`; returns the B-tree and heap addresses and the end. */
static int write_index(h5file* h, uint64_t at, link_list* links, uint64_t* btree, uint64_t* heap, uint64_t* end) {
    qsort(links->v, (size_t)links->n, sizeof(h5link), link_cmp);
    const int per_node = 2 * h->leaf_k;
    const int nsnod = (links->n + per_node - 1) / per_node;
    if (nsnod > 2 * h->node_k)
        return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: more than %d links in the root group", h->path,
                    2 * h->node_k * per_node);
    /* Local heap: "" at offset 0, then each name NUL-terminated and padded to 8 bytes. */
    uint64_t hsize = 8;
    for (int i = 0; i < links->n; ++i) hsize += align8(strlen(links->v[i].name) + 1);
    const uint64_t heap_hdr = 32, snod_size = 8 + (uint64_t)per_node * 40;
    const uint64_t bt_size = 24 + (uint64_t)(2 * h->node_k + 1) * 8 + (uint64_t)(2 * h->node_k) * 8;
    const uint64_t total = heap_hdr + hsize + (uint64_t)nsnod * snod_size + bt_size;
    uint8_t* b = (uint8_t*)calloc(1, total);
    if (!b) return fail(KEVD_H5_ERR_IO, "out of host memory");
    *heap = at;
    memcpy(b, "HEAP", 4);
    putle(b + 8, hsize, 8);
    putle(b + 16, 1, 8);                       /* no free block: the free-list terminator */
    putle(b + 24, at + heap_hdr, 8);
    uint64_t* name_off = (uint64_t*)malloc((size_t)(links->n ? links->n : 1) * sizeof(uint64_t));
    if (!name_off) {
        free(b);
        return fail(KEVD_H5_ERR_IO, "out of host memory");
    }
    uint64_t off = 8;
    for (int i = 0; i < links->n; ++i) {
        const size_t len = strlen(links->v[i].name);
        memcpy(b + heap_hdr + off, links->v[i].name, len);
        name_off[i] = off;
        off += align8(len + 1);
    }
    const uint64_t snod0 = heap_hdr + hsize;
    for (int s = 0; s < nsnod; ++s) {
        uint8_t* p = b + snod0 + (uint64_t)s * snod_size;
        const int first = s * per_node, cnt = links->n - first < per_node ? links->n - first : per_node;
        memcpy(p, "SNOD", 4);
        p[4] = 1;
        putle(p + 6, (uint64_t)cnt, 2);
        for (int j = 0; j < cnt; ++j) {
            uint8_t* e = p + 8 + (uint64_t)j * 40;
            memcpy(e, links->v[first + j].entry, 40);
            putle(e, name_off[first + j], 8);
        }
    }
    const uint64_t bt0 = snod0 + (uint64_t)nsnod * snod_size;
    uint8_t* t = b + bt0;
    memcpy(t, "TREE", 4);
    t[4] = 0;                                  /* group node   */
    t[5] = 0;                                  /* leaf level   */
    putle(t + 6, (uint64_t)nsnod, 2);
    putle(t + 8, kUndef, 8);                   /* left sibling */
    putle(t + 16, kUndef, 8);                  /* right sibling */
    uint8_t* kc = t + 24;
    putle(kc, 0, 8);                           /* key 0: the empty name */
    for (int s = 0; s < nsnod; ++s) {
        const int last = (s + 1) * per_node < links->n ? (s + 1) * per_node - 1 : links->n - 1;
        putle(kc + 8 + (uint64_t)s * 16, at + snod0 + (uint64_t)s * snod_size, 8);   /* child s          */
        putle(kc + 16 + (uint64_t)s * 16, name_off[last], 8);                        /* key s+1: its last */
    }
    free(name_off);
    *btree = at + bt0;
    *end = at + total;
    const int r = wr_abs(h, h->base + at, b, total);
    free(b);
    return r;
}

/* Points the root group's symbol-table message and the superblock at a new index. */
static int patch_root(h5file* h, uint64_t stab_msg, uint64_t btree, uint64_t heap, uint64_t end) {
    uint8_t v[16];
    putle(v, btree, 8);
    putle(v + 8, heap, 8);
    int s = wr_abs(h, h->base + stab_msg, v, 16);
    if (s) return s;
    uint8_t entry[24];
    memset(entry, 0, sizeof(entry));
    putle(entry, 1, 4);                        /* cache type 1: B-tree and heap in the scratch pad */
    putle(entry + 8, btree, 8);
    putle(entry + 16, heap, 8);
    s = wr_abs(h, h->root_entry + 16, entry, 24);
    if (s) return s;
    uint8_t e[8];
    putle(e, h->base + end, 8);
    return wr_abs(h, h->eof_field, e, 8);
}

static int dtype_message(int32_t type, uint8_t* m) {
    memset(m, 0, 24);
    switch (type) {
        case KEVD_H5_F32:
        case KEVD_H5_F64: {
            const int f32 = type == KEVD_H5_F32;
            m[0] = 0x11;                       /* version 1, floating point          */
            m[1] = 0x20;                       /* little-endian, implied msb          */
            m[2] = f32 ? 31 : 63;              /* sign bit                            */
            putle(m + 4, f32 ? 4 : 8, 4);
            putle(m + 8, 0, 2);                /* bit offset                          */
            putle(m + 10, f32 ? 32 : 64, 2);   /* precision                           */
            m[12] = f32 ? 23 : 52;             /* exponent location                   */
            m[13] = f32 ? 8 : 11;              /* exponent size                       */
            m[14] = 0;                         /* mantissa location                   */
            m[15] = f32 ? 23 : 52;             /* mantissa size                       */
            putle(m + 16, f32 ? 127 : 1023, 4);
            return 24;
        }
        default: {
            const int bytes = type_size(type), sgn = type == KEVD_H5_I32 || type == KEVD_H5_I64;
            m[0] = 0x10;                       /* version 1, fixed point              */
            m[1] = sgn ? 0x08 : 0x00;          /* little-endian, signed flag          */
            putle(m + 4, (uint64_t)bytes, 4);
            putle(m + 8, 0, 2);
            putle(m + 10, (uint64_t)(8 * bytes), 2);
            return 16;
        }
    }
}

/* Version 1 object header of a one-dimensional contiguous dataset. */
static uint64_t dataset_header(uint8_t* b, int32_t type, uint64_t count, uint64_t data_addr) {
    uint8_t dt[24];
    const int dtlen = dtype_message(type, dt);
    const uint64_t body = (8 + 24) + (8 + (uint64_t)dtlen) + (8 + 8) + (8 + 24);
    memset(b, 0, 16 + body);
    b[0] = 1;
    putle(b + 2, 4, 2);                        /* messages        */
    putle(b + 4, 1, 4);                        /* reference count */
    putle(b + 8, body, 4);
    uint8_t* p = b + 16;
    /* dataspace: version 1, rank 1, maximum dimensions present */
    putle(p, kMsgDataspace, 2);
    putle(p + 2, 24, 2);
    p[8] = 1;
    p[9] = 1;
    p[10] = 1;
    putle(p + 16, count, 8);
    putle(p + 24, count, 8);
    p += 32;
    putle(p, kMsgDatatype, 2);
    putle(p + 2, (uint64_t)dtlen, 2);
    p[4] = 1;                                  /* constant */
    memcpy(p + 8, dt, (size_t)dtlen);
    p += 8 + dtlen;
    /* fill value: version 2, allocation late, fill if set, default value (size 0) */
    putle(p, kMsgFill, 2);
    putle(p + 2, 8, 2);
    p[4] = 1;
    p[8] = 2;
    p[9] = 2;
    p[10] = 2;
    p[11] = 1;
    putle(p + 12, 0, 4);
    p += 16;
    /* layout: version 3, contiguous, address and size */
    putle(p, kMsgLayout, 2);
    putle(p + 2, 24, 2);
    p[8] = 3;
    p[9] = 1;
    putle(p + 10, data_addr, 8);
    putle(p + 18, count * (uint64_t)type_size(type), 8);
    return 16 + body;
}

static int check_name(const char* name, const char** stripped) {
    if (!name) return fail(KEVD_H5_ERR_ARG, "null dataset name");
    while (*name == '/') ++name;
    if (!*name || strchr(name, '/') || strlen(name) > 4096)
        return fail(KEVD_H5_ERR_ARG, "dataset name must be one non-empty component of the root group");
    *stripped = name;
    return KEVD_H5_OK;
}

int kevd_h5_create(const char* path) {
    if (!path) return fail(KEVD_H5_ERR_ARG, "null path");
    if (!host_is_little_endian()) return fail(KEVD_H5_ERR_UNSUPPORTED, "big-endian host");
    FILE* f = fopen(path, "wb");
    if (!f) return fail(KEVD_H5_ERR_IO, "%s: cannot create", path);
    /* superblock version 0 (96 bytes) and the root group's object header (48 bytes) */
    uint8_t b[144];
    memset(b, 0, sizeof(b));
    memcpy(b, kSignature, 8);
    b[13] = 8;                                 /* size of offsets */
    b[14] = 8;                                 /* size of lengths */
    putle(b + 16, kLeafK, 2);
    putle(b + 18, kNodeK, 2);
    putle(b + 24, 0, 8);                       /* base address    */
    putle(b + 32, kUndef, 8);                  /* free space      */
    putle(b + 40, 144, 8);                     /* end of file     */
    putle(b + 48, kUndef, 8);                  /* driver info     */
    putle(b + 56, 0, 8);                       /* root entry: name offset    */
    putle(b + 64, 96, 8);                      /*             object header  */
    putle(b + 72, 1, 4);                       /*             cache type 1   */
    uint8_t* o = b + 96;
    o[0] = 1;
    putle(o + 2, 2, 2);                        /* symbol table + null message */
    putle(o + 4, 1, 4);
    putle(o + 8, 32, 4);
    putle(o + 16, kMsgSymbolTable, 2);
    putle(o + 18, 16, 2);
    o[20] = 1;
    /* o + 24 .. 39: B-tree and heap addresses, written by patch_root; o + 40: null message */
    const int ok = fwrite(b, 1, sizeof(b), f) == sizeof(b);
    if (fclose(f) != 0 || !ok) return fail(KEVD_H5_ERR_IO, "%s: write failed", path);
    h5file h;
    int s = h5_open(&h, path, "r+b");
    if (s) return s;
    link_list links = {NULL, 0, 0};
    uint64_t bt, hp, end;
    s = write_index(&h, 144, &links, &bt, &hp, &end);
    if (!s) s = patch_root(&h, 96 + 24, bt, hp, end);
    if (fclose(h.f) != 0 && !s) s = fail(KEVD_H5_ERR_IO, "%s: write failed", path);
    h.f = NULL;
    return s;
}

int kevd_h5_append(const char* path, const char* name, int32_t type, const void* data, int64_t count) {
    const char* nm;
    int s = check_name(name, &nm);
    if (s) return s;
    if (type_size(type) == 0 || count < 0 || (count > 0 && !data))
        return fail(KEVD_H5_ERR_ARG, "kevd_h5_append: bad argument");
    if (!host_is_little_endian()) return fail(KEVD_H5_ERR_UNSUPPORTED, "big-endian host");
    h5file h;
    s = h5_open(&h, path, "r+b");
    if (s) return s;
    if ((h.version != 0 && h.version != 1) || h.so != 8 || h.sl != 8 || h.leaf_k < 1 || h.node_k < 1) {
        h5_close(&h);
        return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: appending needs a version 0/1 superblock with 8-byte addresses",
                    path);
    }
    h5obj root;
    s = obj_read(&h, h.root, &root);
    if (s) {
        h5_close(&h);
        return s;
    }
    const h5msg* st = obj_find(&root, kMsgSymbolTable);
    const uint64_t stab_msg = st ? st->addr : 0;
    obj_free(&root);
    if (!st) {
        h5_close(&h);
        return fail(KEVD_H5_ERR_UNSUPPORTED, "%s: root group is not a symbol table", path);
    }
    link_list links = {NULL, 0, 0};
    s = group_walk(&h, h.root, collect_fn, &links);
    if (s > 100) s -= 100;
    for (int i = 0; s == KEVD_H5_OK && i < links.n; ++i)
        if (strcmp(links.v[i].name, nm) == 0) s = fail(KEVD_H5_ERR_ARG, "%s: %s exists", path, nm);
    if (!s) {
        uint64_t end = h.fsize - h.base;
        if (h.eof > h.base && h.eof - h.base > end) end = h.eof - h.base;
        const uint64_t bytes = (uint64_t)count * (uint64_t)type_size(type);
        const uint64_t daddr = (end + 15) & ~(uint64_t)15;
        const uint64_t oaddr = align8(daddr + bytes);
        s = wr_abs(&h, h.base + daddr, data, bytes);
        uint8_t ohb[16 + 136];
        const uint64_t olen = dataset_header(ohb, type, (uint64_t)count, bytes ? daddr : kUndef);
        if (!s) s = wr_abs(&h, h.base + oaddr, ohb, olen);
        uint8_t entry[40];
        memset(entry, 0, sizeof(entry));
        putle(entry + 8, oaddr, 8);
        if (!s) s = links_push(&links, nm, strlen(nm), entry);
        uint64_t bt, hp, iend;
        if (!s) s = write_index(&h, align8(oaddr + olen), &links, &bt, &hp, &iend);
        if (!s) s = patch_root(&h, stab_msg, bt, hp, iend);
    }
    links_free(&links);
    if (fclose(h.f) != 0 && !s) s = fail(KEVD_H5_ERR_IO, "%s: write failed", path);
    h.f = NULL;
    return s;
}

int kevd_h5_write(const char* path, int32_t n, const char* const* names, const int32_t* types,
                  const void* const* data, const int64_t* counts) {
    if (n < 0 || (n > 0 && (!names || !types || !data || !counts)))
        return fail(KEVD_H5_ERR_ARG, "kevd_h5_write: bad argument");
    for (int32_t i = 0; i < n; ++i) {
        const char* nm;
        int s = check_name(names[i], &nm);
        if (s) return s;
        if (type_size(types[i]) == 0 || counts[i] < 0 || (counts[i] > 0 && !data[i]))
            return fail(KEVD_H5_ERR_ARG, "kevd_h5_write: bad dataset %d", i);
    }
    int s = kevd_h5_create(path);
    for (int32_t i = 0; s == KEVD_H5_OK && i < n; ++i) s = kevd_h5_append(path, names[i], types[i], data[i], counts[i]);
    return s;
}
