/*
 * matio.c -- Level-5 MAT-file reading and writing for the standalone harness
 * (readFiles / SaveResults of GENFIRE_Reconstructor.m:82-112, :205-207).
 *
 * The layout follows MathWorks' published "MAT-File Format" description:
 * a 128-byte header (text, subsystem offset, version 0x0100, endian mark
 * "IM"), then data elements, each an 8-byte tag (type, byte count) or a
 * 4-byte "small" tag with up to 4 bytes of data, padded to 8 bytes.
 * miMATRIX elements hold array flags, dimensions, the name and the real
 * (and imaginary) data, stored in any numeric type; miCOMPRESSED elements
 * hold one zlib stream (RFC 1950) of such an element.  The DEFLATE decoder
 * (RFC 1951: stored, fixed-Huffman and dynamic-Huffman blocks, canonical
 * codes decoded one bit at a time) is written here so the harness needs no
 * library beyond libgenfire and libc.  Its canonical-code decoder is the
 * published bit-at-a-time method of RFC 1951 section 3.2.2 (codes of each length
 * counted, symbols listed in code order, a running first code and index per
 * length), the same method as Mark Adler's reference decoder puff.c in the
 * zlib distribution.  Hosts are little-endian (x86-64 and
 * AArch64 Linux); big-endian files are rejected.
 */
#include "matio.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ DEFLATE */

typedef struct {
    const uint8_t *in;
    size_t len, pos;
    uint64_t buf;   /* bits not yet consumed, least significant first */
    int cnt;
    int bad;
    uint8_t *out;   /* output window (the whole output) */
    size_t olen, ocap;
    int grow;       /* realloc out when full (else overflow is an error) */
} inflater;

static uint32_t take(inflater *s, int n)
{
    while (s->cnt < n) {
        if (s->pos >= s->len) {
            s->bad = 1;
            return 0;
        }
        s->buf |= (uint64_t)s->in[s->pos++] << s->cnt;
        s->cnt += 8;
    }
    const uint32_t v = (uint32_t)(s->buf & ((1ull << n) - 1ull));
    s->buf >>= n;
    s->cnt -= n;
    return v;
}

static int put(inflater *s, uint8_t b)
{
    if (s->olen == s->ocap) {
        if (!s->grow) return -1;
        size_t nc = s->ocap ? 2 * s->ocap : 65536;
        uint8_t *p = (uint8_t *)realloc(s->out, nc);
        if (!p) return -1;
        s->out = p;
        s->ocap = nc;
    }
    s->out[s->olen++] = b;
    return 0;
}

/* canonical Huffman code: number of codes of each length and the symbols in
 * code order */
typedef struct {
    uint16_t count[16];
    uint16_t sym[320];
} huff;

static int huff_build(huff *h, const uint8_t *lens, int n)
{
    uint16_t start[16];
    memset(h->count, 0, sizeof h->count);
    for (int i = 0; i < n; ++i) h->count[lens[i]]++;
    h->count[0] = 0;
    /* over-subscribed sets are malformed; incomplete ones are allowed (a
     * single distance code, for example) */
    int left = 1;
    for (int l = 1; l < 16; ++l) {
        left = 2 * left - h->count[l];
        if (left < 0) return -1;
    }
    start[1] = 0;
    for (int l = 1; l < 15; ++l) start[l + 1] = (uint16_t)(start[l] + h->count[l]);
    for (int i = 0; i < n; ++i)
        if (lens[i]) h->sym[start[lens[i]]++] = (uint16_t)i;
    return 0;
}

/* codes of length l are the consecutive integers after those of length l-1
 * (shifted left by one), so a code is found by comparing the bits read so far
 * with the first code of each length */
static int huff_decode(inflater *s, const huff *h)
{
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
        code |= (int)take(s, 1);
        if (s->bad) return -1;
        const int c = h->count[l];
        if (code - first < c) return h->sym[index + code - first];
        index += c;
        first = (first + c) << 1;
        code <<= 1;
    }
    return -1;
}

/* RFC 1951 section 3.2.5 */
static const uint16_t len_base[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27,
                                      31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
static const uint8_t len_extra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
static const uint16_t dist_base[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                       193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
static const uint8_t dist_extra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
/* order of the code-length code lengths in a dynamic block header (section 3.2.7) */
static const uint8_t clen_order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

static int inflate_codes(inflater *s, const huff *lit, const huff *dist)
{
    for (;;) {
        const int sym = huff_decode(s, lit);
        if (sym < 0) return -1;
        if (sym < 256) {
            if (put(s, (uint8_t)sym)) return -1;
        } else if (sym == 256) {
            return 0;
        } else {
            const int li = sym - 257;
            if (li >= 29) return -1;
            const int length = len_base[li] + (int)take(s, len_extra[li]);
            const int di = huff_decode(s, dist);
            if (di < 0 || di >= 30 || s->bad) return -1;
            const size_t d = dist_base[di] + take(s, dist_extra[di]);
            if (s->bad || d > s->olen) return -1;
            for (int k = 0; k < length; ++k)
                if (put(s, s->out[s->olen - d])) return -1;
        }
    }
}

static int inflate_stored(inflater *s)
{
    s->buf = 0;  /* skip to the byte boundary */
    s->cnt = 0;
    if (s->pos + 4 > s->len) return -1;
    const unsigned n = s->in[s->pos] | (s->in[s->pos + 1] << 8);
    const unsigned nn = s->in[s->pos + 2] | (s->in[s->pos + 3] << 8);
    s->pos += 4;
    if ((n ^ 0xFFFFu) != nn || s->pos + n > s->len) return -1;
    for (unsigned k = 0; k < n; ++k)
        if (put(s, s->in[s->pos + k])) return -1;
    s->pos += n;
    return 0;
}

static int inflate_fixed(inflater *s)
{
    uint8_t l[320];
    huff lit, dist;
    int i = 0;
    for (; i < 144; ++i) l[i] = 8;
    for (; i < 256; ++i) l[i] = 9;
    for (; i < 280; ++i) l[i] = 7;
    for (; i < 288; ++i) l[i] = 8;
    huff_build(&lit, l, 288);
    for (i = 0; i < 30; ++i) l[i] = 5;
    huff_build(&dist, l, 30);
    return inflate_codes(s, &lit, &dist);
}

static int inflate_dynamic(inflater *s)
{
    const int nlit = (int)take(s, 5) + 257, ndist = (int)take(s, 5) + 1, nclen = (int)take(s, 4) + 4;
    if (s->bad || nlit > 286 || ndist > 30) return -1;
    uint8_t l[320];
    memset(l, 0, sizeof l);
    for (int i = 0; i < nclen; ++i) l[clen_order[i]] = (uint8_t)take(s, 3);
    huff clen;
    if (s->bad || huff_build(&clen, l, 19)) return -1;
    uint8_t lens[320];
    int n = 0;
    while (n < nlit + ndist) {
        const int sym = huff_decode(s, &clen);
        if (sym < 0) return -1;
        if (sym < 16) {
            lens[n++] = (uint8_t)sym;
            continue;
        }
        int rep;
        uint8_t v = 0;
        if (sym == 16) {
            if (n == 0) return -1;
            v = lens[n - 1];
            rep = 3 + (int)take(s, 2);
        } else if (sym == 17) {
            rep = 3 + (int)take(s, 3);
        } else {
            rep = 11 + (int)take(s, 7);
        }
        if (s->bad || n + rep > nlit + ndist) return -1;
        while (rep--) lens[n++] = v;
    }
    if (lens[256] == 0) return -1;  /* no end-of-block code */
    huff lit, dist;
    if (huff_build(&lit, lens, nlit) || huff_build(&dist, lens + nlit, ndist)) return -1;
    return inflate_codes(s, &lit, &dist);
}

static int inflate_run(inflater *s)
{
    if (s->len < 2) return -1;
    const uint8_t cmf = s->in[0], flg = s->in[1];
    if ((cmf & 15) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20)) return -1;  /* deflate, no dictionary */
    s->pos = 2;
    int last;
    do {
        last = (int)take(s, 1);
        const int type = (int)take(s, 2);
        if (s->bad) return -1;
        int r;
        if (type == 0) r = inflate_stored(s);
        else if (type == 1) r = inflate_fixed(s);
        else if (type == 2) r = inflate_dynamic(s);
        else r = -1;
        if (r || s->bad) return -1;
    } while (!last);
    /* Adler-32 of the output, big-endian, after the byte boundary */
    s->buf = 0;
    s->cnt = 0;
    if (s->pos + 4 <= s->len) {
        uint32_t a = 1, b = 0;
        for (size_t i = 0; i < s->olen; ++i) {
            a = (a + s->out[i]) % 65521u;
            b = (b + a) % 65521u;
        }
        const uint32_t want = ((uint32_t)s->in[s->pos] << 24) | ((uint32_t)s->in[s->pos + 1] << 16) |
                              ((uint32_t)s->in[s->pos + 2] << 8) | s->in[s->pos + 3];
        if (want != ((b << 16) | a)) return -1;
    }
    return 0;
}

int64_t mat_inflate(const uint8_t *in, size_t in_len, uint8_t *out, size_t out_cap)
{
    inflater s;
    memset(&s, 0, sizeof s);
    s.in = in;
    s.len = in_len;
    s.out = out;
    s.ocap = out_cap;
    return inflate_run(&s) ? -1 : (int64_t)s.olen;
}

/* ------------------------------------------------------------------ reading */

enum {
    miINT8 = 1, miUINT8 = 2, miINT16 = 3, miUINT16 = 4, miINT32 = 5, miUINT32 = 6, miSINGLE = 7,
    miDOUBLE = 9, miINT64 = 12, miUINT64 = 13, miMATRIX = 14, miCOMPRESSED = 15
};

static void say(char *err, size_t n, const char *fmt, ...)
{
    if (!err || !n) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, n, fmt, ap);
    va_end(ap);
}

static uint32_t rd32(const uint8_t *p)
{
    uint32_t v;
    memcpy(&v, p, 4);
    return v;
}

/* one data element at *pos of buf[0..len): its type, byte count and data;
 * advances *pos past it (with the 8-byte padding of the format) */
static int element(const uint8_t *buf, size_t len, size_t *pos, uint32_t *type, uint32_t *nbytes, const uint8_t **data)
{
    if (*pos + 8 > len) return -1;
    const uint32_t w = rd32(buf + *pos);
    if (w >> 16) {  /* small element: 4-byte tag, data in the next 4 bytes */
        *type = w & 0xFFFFu;
        *nbytes = w >> 16;
        if (*nbytes > 4) return -1;
        *data = buf + *pos + 4;
        *pos += 8;
        return 0;
    }
    *type = w;
    *nbytes = rd32(buf + *pos + 4);
    if (*pos + 8 + (size_t)*nbytes > len) return -1;
    *data = buf + *pos + 8;
    size_t adv = 8 + (size_t)*nbytes;
    if (*type != miCOMPRESSED) adv = (adv + 7) & ~(size_t)7;
    *pos += adv;
    if (*pos > len) *pos = len;
    return 0;
}

static int type_size(uint32_t t)
{
    switch (t) {
    case miINT8: case miUINT8: return 1;
    case miINT16: case miUINT16: return 2;
    case miINT32: case miUINT32: case miSINGLE: return 4;
    case miDOUBLE: case miINT64: case miUINT64: return 8;
    default: return 0;
    }
}

static double value(uint32_t t, const uint8_t *p)
{
    switch (t) {
    case miINT8: { int8_t v; memcpy(&v, p, 1); return v; }
    case miUINT8: return *p;
    case miINT16: { int16_t v; memcpy(&v, p, 2); return v; }
    case miUINT16: { uint16_t v; memcpy(&v, p, 2); return v; }
    case miINT32: { int32_t v; memcpy(&v, p, 4); return v; }
    case miUINT32: { uint32_t v; memcpy(&v, p, 4); return v; }
    case miSINGLE: { float v; memcpy(&v, p, 4); return v; }
    case miDOUBLE: { double v; memcpy(&v, p, 8); return v; }
    case miINT64: { int64_t v; memcpy(&v, p, 8); return (double)v; }
    default: { uint64_t v; memcpy(&v, p, 8); return (double)v; }
    }
}

static int numeric_part(uint32_t t, uint32_t nbytes, const uint8_t *d, int64_t numel, double **out)
{
    const int es = type_size(t);
    if (!es || (int64_t)nbytes != numel * es) return -1;
    double *v = (double *)malloc(sizeof(double) * (size_t)(numel > 0 ? numel : 1));
    if (!v) return -1;
    for (int64_t i = 0; i < numel; ++i) v[i] = value(t, d + (size_t)i * es);
    *out = v;
    return 0;
}

/* an miMATRIX element's contents; returns 1 if it is a numeric or logical
 * array (filled in), 0 if another class, -1 if malformed */
static int matrix(const uint8_t *b, size_t len, mat_array *a)
{
    size_t pos = 0;
    uint32_t t, n;
    const uint8_t *d;
    memset(a, 0, sizeof *a);
    if (element(b, len, &pos, &t, &n, &d) || t != miUINT32 || n < 8) return -1;
    const uint32_t flags = rd32(d);
    a->mx_class = (int)(flags & 0xFFu);
    a->is_complex = (flags >> 8) & 0x08 ? 1 : 0;
    a->is_logical = (flags >> 8) & 0x02 ? 1 : 0;
    if (element(b, len, &pos, &t, &n, &d) || t != miINT32 || n < 8 || n % 4) return -1;
    a->ndims = (int)(n / 4);
    if (a->ndims > 8) return -1;
    a->numel = 1;
    for (int k = 0; k < a->ndims; ++k) {
        int32_t v;
        memcpy(&v, d + 4 * k, 4);
        if (v < 0) return -1;
        a->dims[k] = v;
        a->numel *= v;
    }
    if (element(b, len, &pos, &t, &n, &d) || t != miINT8) return -1;
    const size_t nl = n < sizeof a->name - 1 ? n : sizeof a->name - 1;
    memcpy(a->name, d, nl);
    a->name[nl] = 0;
    if (a->mx_class < 6 || a->mx_class > 15) return 0;  /* cell, struct, object, char, sparse */
    if (element(b, len, &pos, &t, &n, &d) || numeric_part(t, n, d, a->numel, &a->re)) return -1;
    if (a->is_complex) {
        if (element(b, len, &pos, &t, &n, &d) || numeric_part(t, n, d, a->numel, &a->im)) {
            free(a->re);
            a->re = NULL;
            return -1;
        }
    }
    return 1;
}

int mat_read(const char *path, const char *name, mat_array *out, char *err, size_t err_len)
{
    memset(out, 0, sizeof *out);
    FILE *f = fopen(path, "rb");
    if (!f) {
        say(err, err_len, "cannot open %s", path);
        return -1;
    }
    fseek(f, 0, SEEK_END);
    const long fl = ftell(f);
    fseek(f, 0, SEEK_SET);
    uint8_t *buf = (uint8_t *)malloc(fl > 0 ? (size_t)fl : 1);
    if (!buf || fl < 128 || fread(buf, 1, (size_t)fl, f) != (size_t)fl) {
        fclose(f);
        free(buf);
        say(err, err_len, "%s: not a MAT file (too short)", path);
        return -1;
    }
    fclose(f);
    const size_t len = (size_t)fl;
    if (!memcmp(buf, "MATLAB 7.3", 10)) {
        free(buf);
        say(err, err_len, "%s: Level 7.3 (HDF5) MAT files are not supported; save with -v7 or -v6", path);
        return -1;
    }
    if (buf[126] != 'I' || buf[127] != 'M') {
        free(buf);
        say(err, err_len, "%s: not a little-endian Level-5 MAT file", path);
        return -1;
    }
    size_t pos = 128;
    int rc = -1;
    while (pos + 8 <= len) {
        uint32_t t, n;
        const uint8_t *d;
        if (element(buf, len, &pos, &t, &n, &d)) break;
        const uint8_t *m = NULL;
        size_t ml = 0;
        inflater s;
        memset(&s, 0, sizeof s);
        if (t == miCOMPRESSED) {
            s.in = d;
            s.len = n;
            s.grow = 1;
            if (inflate_run(&s)) {
                free(s.out);
                say(err, err_len, "%s: corrupt compressed element", path);
                rc = -1;
                break;
            }
            size_t ip = 0;
            uint32_t it, inb;
            const uint8_t *id;
            if (element(s.out, s.olen, &ip, &it, &inb, &id) == 0 && it == miMATRIX) {
                m = id;
                ml = inb;
            }
        } else if (t == miMATRIX) {
            m = d;
            ml = n;
        }
        if (m) {
            mat_array a;
            const int r = matrix(m, ml, &a);
            if (r < 0) {
                free(s.out);
                say(err, err_len, "%s: malformed array element", path);
                rc = -1;
                break;
            }
            if (r == 1 && (!name || !strcmp(name, a.name))) {
                *out = a;
                free(s.out);
                rc = 0;
                break;
            }
            mat_free(&a);
        }
        free(s.out);
    }
    free(buf);
    if (rc && err && !err[0]) say(err, err_len, "%s: no numeric array%s%s", path, name ? " named " : "", name ? name : "");
    return rc;
}

void mat_free(mat_array *a)
{
    free(a->re);
    free(a->im);
    a->re = a->im = NULL;
}

/* ------------------------------------------------------------------ writing */

static int w32(FILE *f, uint32_t v) { return fwrite(&v, 4, 1, f) == 1 ? 0 : -1; }

static int pad8(FILE *f, size_t n)
{
    static const uint8_t z[8] = {0};
    const size_t p = (8 - n % 8) % 8;
    return p ? (fwrite(z, 1, p, f) == p ? 0 : -1) : 0;
}

int mat_write(const char *path, int count, const mat_var *vars, char *err, size_t err_len)
{
    FILE *f = fopen(path, "wb");
    if (!f) {
        say(err, err_len, "cannot create %s", path);
        return -1;
    }
    char hdr[128];
    memset(hdr, ' ', 116);
    const char *text = "MATLAB 5.0 MAT-file, written by genfire_run (libgenfire)";
    memcpy(hdr, text, strlen(text));
    memset(hdr + 116, 0, 8);            /* no subsystem data */
    hdr[124] = 0x00; hdr[125] = 0x01;  /* version 0x0100 */
    hdr[126] = 'I'; hdr[127] = 'M';
    int bad = fwrite(hdr, 1, 128, f) != 128;
    for (int v = 0; v < count && !bad; ++v) {
        const mat_var *x = &vars[v];
        int64_t numel = 1;
        for (int k = 0; k < x->ndims; ++k) numel *= x->dims[k];
        const int es = x->mx_class == MAT_DOUBLE ? 8 : x->mx_class == MAT_SINGLE ? 4 : 1;
        const uint32_t dtype = x->mx_class == MAT_DOUBLE ? miDOUBLE : x->mx_class == MAT_SINGLE ? miSINGLE : miUINT8;
        const size_t nlen = strlen(x->name);
        const size_t dbytes = (size_t)numel * es;
        const size_t sz = 16 + 8 + ((4 * (size_t)x->ndims + 7) & ~(size_t)7) + 8 + ((nlen + 7) & ~(size_t)7) + 8 +
                          ((dbytes + 7) & ~(size_t)7);
        bad |= w32(f, miMATRIX) | w32(f, (uint32_t)sz);
        /* array flags: class, logical flag */
        bad |= w32(f, miUINT32) | w32(f, 8) | w32(f, (uint32_t)x->mx_class | (x->mx_class == MAT_LOGICAL ? 0x0200u : 0u)) |
               w32(f, 0);
        bad |= w32(f, miINT32) | w32(f, (uint32_t)(4 * x->ndims));
        for (int k = 0; k < x->ndims; ++k) bad |= w32(f, (uint32_t)x->dims[k]);
        bad |= pad8(f, 4 * (size_t)x->ndims);
        bad |= w32(f, miINT8) | w32(f, (uint32_t)nlen);
        bad |= fwrite(x->name, 1, nlen, f) != nlen;
        bad |= pad8(f, nlen);
        bad |= w32(f, dtype) | w32(f, (uint32_t)dbytes);
        bad |= fwrite(x->data, 1, dbytes, f) != dbytes;
        bad |= pad8(f, dbytes);
    }
    bad |= fclose(f) != 0;
    if (bad) say(err, err_len, "write to %s failed", path);
    return bad ? -1 : 0;
}
