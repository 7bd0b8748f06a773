/*
 * io.c - slice files at the edges of a reconstruction graph: classic TIFF
 * (TIFF 6.0 baseline structure: header, chained IFDs, strips) with one
 * slice per page, and raw float32. Byte order is handled explicitly, so the
 * code behaves the same on every host.
 */
#include "ufoir.h"

#include <errno.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static __thread char g_io_err[512];

static int io_fail(int status, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_io_err, sizeof(g_io_err), fmt, ap);
    va_end(ap);
    return status;
}

const char *ufoir_io_last_error(void)
{
    return g_io_err;
}

/* ------------------------------------------------------------------ TIFF */

enum {
    TAG_WIDTH = 256, TAG_HEIGHT = 257, TAG_BITS = 258, TAG_COMPRESSION = 259, TAG_PHOTOMETRIC = 262,
    TAG_STRIP_OFFSETS = 273, TAG_SAMPLES = 277, TAG_ROWS_PER_STRIP = 278, TAG_STRIP_BYTES = 279,
    TAG_PLANAR = 284, TAG_TILE_WIDTH = 322, TAG_SAMPLE_FORMAT = 339
};
enum { T_BYTE = 1, T_SHORT = 3, T_LONG = 4 };

typedef struct {
    FILE *f;
    int big_endian;
    uint64_t size;
} tiff_reader;

typedef struct {
    uint32_t width, height, bits, compression, samples, rows_per_strip, planar, sample_format;
    int tiled;
    uint32_t n_strips;
    uint32_t strip_offsets_type, strip_bytes_type;
    uint32_t strip_offsets_at, strip_bytes_at;   /* file offset of the arrays (or the value itself, inline) */
    int strip_offsets_inline, strip_bytes_inline;
    uint32_t next;
} tiff_page;

static uint32_t rd16(const tiff_reader *r, const unsigned char *b)
{
    return r->big_endian ? (uint32_t) ((b[0] << 8) | b[1]) : (uint32_t) (b[0] | (b[1] << 8));
}

static uint32_t rd32(const tiff_reader *r, const unsigned char *b)
{
    return r->big_endian ? ((uint32_t) b[0] << 24) | ((uint32_t) b[1] << 16) | ((uint32_t) b[2] << 8) | b[3]
                         : (uint32_t) b[0] | ((uint32_t) b[1] << 8) | ((uint32_t) b[2] << 16) |
                               ((uint32_t) b[3] << 24);
}

static int read_at(tiff_reader *r, uint64_t off, void *buf, size_t n)
{
    if (off > r->size || n > r->size - off)
        return -1;
    if (fseek(r->f, (long) off, SEEK_SET) != 0)
        return -1;
    return fread(buf, 1, n, r->f) == n ? 0 : -1;
}

static int tiff_open(tiff_reader *r, const char *path, uint32_t *first_ifd)
{
    memset(r, 0, sizeof(*r));
    r->f = fopen(path, "rb");
    if (!r->f)
        return io_fail(UFOIR_ERR_IO, "%s: %s", path, strerror(errno));
    if (fseek(r->f, 0, SEEK_END) == 0) {
        const long sz = ftell(r->f);
        r->size = sz > 0 ? (uint64_t) sz : 0;
    }
    unsigned char h[8];
    if (read_at(r, 0, h, 8))
        return io_fail(UFOIR_ERR_IO, "%s: too short for a TIFF header", path);
    if (h[0] == 'I' && h[1] == 'I')
        r->big_endian = 0;
    else if (h[0] == 'M' && h[1] == 'M')
        r->big_endian = 1;
    else
        return io_fail(UFOIR_ERR_IO, "%s: not a TIFF file", path);
    const uint32_t magic = rd16(r, h + 2);
    if (magic == 43)
        return io_fail(UFOIR_ERR_IO, "%s: BigTIFF is not supported", path);
    if (magic != 42)
        return io_fail(UFOIR_ERR_IO, "%s: not a TIFF file", path);
    *first_ifd = rd32(r, h + 4);
    return UFOIR_OK;
}

static int type_size(uint32_t t)
{
    return t == T_BYTE ? 1 : t == T_SHORT ? 2 : t == T_LONG ? 4 : 0;
}

static int tiff_page_read(tiff_reader *r, const char *path, uint32_t ifd, tiff_page *pg)
{
    memset(pg, 0, sizeof(*pg));
    pg->bits = 1;
    pg->compression = 1;
    pg->samples = 1;
    pg->planar = 1;
    pg->sample_format = 1;
    pg->rows_per_strip = 0xFFFFFFFFu;
    unsigned char b2[2];
    if (ifd & 1u || read_at(r, ifd, b2, 2))
        return io_fail(UFOIR_ERR_IO, "%s: bad IFD offset %u", path, ifd);
    const uint32_t n = rd16(r, b2);
    unsigned char *e = (unsigned char *) malloc((size_t) n * 12 + 4);
    if (!e)
        return io_fail(UFOIR_ERR_NOMEM, "out of host memory");
    if (read_at(r, (uint64_t) ifd + 2, e, (size_t) n * 12 + 4)) {
        free(e);
        return io_fail(UFOIR_ERR_IO, "%s: truncated IFD", path);
    }
    for (uint32_t i = 0; i < n; i++) {
        const unsigned char *x = e + 12 * i;
        const uint32_t tag = rd16(r, x), type = rd16(r, x + 2), count = rd32(r, x + 4);
        const int ts = type_size(type);
        /* a single SHORT/LONG value sits left-justified in the value field */
        const uint32_t v = type == T_SHORT ? rd16(r, x + 8) : rd32(r, x + 8);
        const int inline_values = ts > 0 && (uint64_t) count * (uint64_t) ts <= 4;
        switch (tag) {
        case TAG_WIDTH: pg->width = v; break;
        case TAG_HEIGHT: pg->height = v; break;
        case TAG_BITS: pg->bits = v; break;
        case TAG_COMPRESSION: pg->compression = v; break;
        case TAG_SAMPLES: pg->samples = v; break;
        case TAG_ROWS_PER_STRIP: pg->rows_per_strip = v; break;
        case TAG_PLANAR: pg->planar = v; break;
        case TAG_SAMPLE_FORMAT: pg->sample_format = v; break;
        case TAG_TILE_WIDTH: pg->tiled = 1; break;
        case TAG_STRIP_OFFSETS:
        case TAG_STRIP_BYTES:
            if (type != T_SHORT && type != T_LONG) {
                free(e);
                return io_fail(UFOIR_ERR_IO, "%s: strip table of type %u", path, type);
            }
            if (tag == TAG_STRIP_OFFSETS) {
                pg->n_strips = count;
                pg->strip_offsets_type = type;
                pg->strip_offsets_inline = inline_values;
                pg->strip_offsets_at = inline_values ? (uint32_t) (ifd + 2 + 12 * i + 8) : v;
            } else {
                pg->strip_bytes_type = type;
                pg->strip_bytes_inline = inline_values;
                pg->strip_bytes_at = inline_values ? (uint32_t) (ifd + 2 + 12 * i + 8) : v;
            }
            break;
        default:
            break;
        }
    }
    pg->next = rd32(r, e + 12 * n);
    free(e);
    if (pg->tiled)
        return io_fail(UFOIR_ERR_IO, "%s: tiled TIFF is not supported", path);
    if (pg->compression != 1)
        return io_fail(UFOIR_ERR_IO, "%s: compression %u is not supported (uncompressed only)", path,
                       pg->compression);
    if (pg->samples != 1)
        return io_fail(UFOIR_ERR_IO, "%s: %u samples per pixel (one expected)", path, pg->samples);
    const int ok_format = (pg->sample_format == 3 && pg->bits == 32) ||
                          (pg->sample_format == 1 && (pg->bits == 8 || pg->bits == 16));
    if (!ok_format)
        return io_fail(UFOIR_ERR_IO, "%s: %u-bit samples of format %u (float32, uint16 or uint8 expected)", path,
                       pg->bits, pg->sample_format);
    if (pg->width == 0 || pg->height == 0 || pg->n_strips == 0)
        return io_fail(UFOIR_ERR_IO, "%s: page without image data", path);
    if (pg->rows_per_strip == 0)
        return io_fail(UFOIR_ERR_IO, "%s: RowsPerStrip is 0", path);
    return UFOIR_OK;
}

static int strip_value(tiff_reader *r, uint32_t at, uint32_t type, uint32_t idx, uint32_t *out)
{
    unsigned char b[4];
    const int ts = type_size(type);
    if (read_at(r, (uint64_t) at + (uint64_t) idx * (uint64_t) ts, b, (size_t) ts))
        return -1;
    *out = type == T_SHORT ? rd16(r, b) : rd32(r, b);
    return 0;
}

int ufoir_io_tiff_info(const char *path, unsigned int *width, unsigned int *height, unsigned int *pages)
{
    if (!path)
        return io_fail(UFOIR_ERR_INVALID, "no path");
    tiff_reader r;
    uint32_t ifd = 0;
    int rc = tiff_open(&r, path, &ifd);
    unsigned int count = 0;
    tiff_page pg, first;
    memset(&first, 0, sizeof(first));
    while (rc == UFOIR_OK && ifd != 0) {
        if (count >= 1000000) {
            rc = io_fail(UFOIR_ERR_IO, "%s: IFD chain does not end", path);
            break;
        }
        rc = tiff_page_read(&r, path, ifd, &pg);
        if (rc)
            break;
        if (count == 0)
            first = pg;
        else if (pg.width != first.width || pg.height != first.height)
            rc = io_fail(UFOIR_ERR_IO, "%s: page %u is %ux%u, page 0 is %ux%u", path, count, pg.width, pg.height,
                         first.width, first.height);
        count++;
        ifd = pg.next;
    }
    if (r.f)
        fclose(r.f);
    if (rc)
        return rc;
    if (count == 0)
        return io_fail(UFOIR_ERR_IO, "%s: no pages", path);
    if (width)
        *width = first.width;
    if (height)
        *height = first.height;
    if (pages)
        *pages = count;
    return UFOIR_OK;
}

int ufoir_io_read_tiff(const char *path, unsigned int page, float *out, size_t count)
{
    if (!path || !out)
        return io_fail(UFOIR_ERR_INVALID, "no path or output");
    tiff_reader r;
    uint32_t ifd = 0;
    int rc = tiff_open(&r, path, &ifd);
    tiff_page pg;
    unsigned int p = 0;
    unsigned char *buf = NULL;
    while (rc == UFOIR_OK) {
        if (ifd == 0) {
            rc = io_fail(UFOIR_ERR_IO, "%s: page %u beyond the last (%u pages)", path, page, p);
            break;
        }
        rc = tiff_page_read(&r, path, ifd, &pg);
        if (rc || p == page)
            break;
        ifd = pg.next;
        if (++p > 1000000)
            rc = io_fail(UFOIR_ERR_IO, "%s: IFD chain does not end", path);
    }
    if (rc == UFOIR_OK && (size_t) pg.width * pg.height != count)
        rc = io_fail(UFOIR_ERR_INVALID, "%s: page %u holds %ux%u samples, %zu requested", path, page, pg.width,
                     pg.height, count);
    const size_t bps = pg.bits / 8, row_bytes = (size_t) pg.width * bps;
    uint32_t row = 0;
    for (uint32_t s = 0; rc == UFOIR_OK && s < pg.n_strips && row < pg.height; s++) {
        uint32_t off, bytes;
        if (strip_value(&r, pg.strip_offsets_at, pg.strip_offsets_type, s, &off) ||
            strip_value(&r, pg.strip_bytes_at, pg.strip_bytes_type, s, &bytes)) {
            rc = io_fail(UFOIR_ERR_IO, "%s: truncated strip table", path);
            break;
        }
        uint32_t rows = pg.rows_per_strip;
        if (rows > pg.height - row)
            rows = pg.height - row;
        const size_t need = (size_t) rows * row_bytes;
        if (bytes < need) {
            rc = io_fail(UFOIR_ERR_IO, "%s: strip %u holds %u bytes, %zu needed", path, s, bytes, need);
            break;
        }
        unsigned char *nb = (unsigned char *) realloc(buf, need);
        if (!nb) {
            rc = io_fail(UFOIR_ERR_NOMEM, "out of host memory");
            break;
        }
        buf = nb;
        if (read_at(&r, off, buf, need)) {
            rc = io_fail(UFOIR_ERR_IO, "%s: strip %u outside the file", path, s);
            break;
        }
        float *o = out + (size_t) row * pg.width;
        const size_t n = (size_t) rows * pg.width;
        for (size_t i = 0; i < n; i++) {
            const unsigned char *x = buf + i * bps;
            if (pg.bits == 32) {
                const uint32_t u = rd32(&r, x);
                memcpy(&o[i], &u, 4);
            } else if (pg.bits == 16) {
                o[i] = (float) rd16(&r, x);
            } else {
                o[i] = (float) x[0];
            }
        }
        row += rows;
    }
    if (rc == UFOIR_OK && row < pg.height)
        rc = io_fail(UFOIR_ERR_IO, "%s: strips cover %u of %u rows", path, row, pg.height);
    free(buf);
    if (r.f)
        fclose(r.f);
    return rc;
}

static void put16(unsigned char *b, uint32_t v)
{
    b[0] = (unsigned char) (v & 0xFF);
    b[1] = (unsigned char) (v >> 8);
}

static void put32(unsigned char *b, uint32_t v)
{
    b[0] = (unsigned char) (v & 0xFF);
    b[1] = (unsigned char) ((v >> 8) & 0xFF);
    b[2] = (unsigned char) ((v >> 16) & 0xFF);
    b[3] = (unsigned char) (v >> 24);
}

int ufoir_io_write_tiff(const char *path, const float *data, unsigned int width, unsigned int height,
                        unsigned int pages)
{
    if (!path || !data || width == 0 || height == 0 || pages == 0)
        return io_fail(UFOIR_ERR_INVALID, "write_tiff: empty image or no path");
    const uint64_t page_bytes = (uint64_t) width * height * 4;
    enum { N_TAGS = 11 };
    const uint64_t ifd_bytes = 2 + 12 * N_TAGS + 4;
    if (8 + (page_bytes + ifd_bytes) * pages > 0xFFFFFFF0ull)
        return io_fail(UFOIR_ERR_INVALID, "write_tiff: %u pages of %ux%u exceed 4 GiB (classic TIFF)", pages,
                       width, height);
    FILE *f = fopen(path, "wb");
    if (!f)
        return io_fail(UFOIR_ERR_IO, "%s: %s", path, strerror(errno));
    unsigned char h[8] = {'I', 'I', 0, 0, 0, 0, 0, 0};
    put16(h + 2, 42);
    put32(h + 4, (uint32_t) (8 + page_bytes));      /* IFD of page 0 follows its pixels */
    int rc = fwrite(h, 1, 8, f) == 8 ? UFOIR_OK : io_fail(UFOIR_ERR_IO, "%s: write failed", path);
    unsigned char *row = (unsigned char *) malloc((size_t) width * 4);
    if (!row && rc == UFOIR_OK)
        rc = io_fail(UFOIR_ERR_NOMEM, "out of host memory");
    for (unsigned int p = 0; rc == UFOIR_OK && p < pages; p++) {
        const uint64_t data_at = 8 + (page_bytes + ifd_bytes) * p;
        for (unsigned int y = 0; rc == UFOIR_OK && y < height; y++) {
            const float *src = data + ((size_t) p * height + y) * width;
            for (unsigned int x = 0; x < width; x++) {
                uint32_t u;
                memcpy(&u, &src[x], 4);
                put32(row + 4 * (size_t) x, u);
            }
            if (fwrite(row, 4, width, f) != width)
                rc = io_fail(UFOIR_ERR_IO, "%s: write failed", path);
        }
        unsigned char ifd[2 + 12 * N_TAGS + 4];
        memset(ifd, 0, sizeof(ifd));
        put16(ifd, N_TAGS);
        const uint32_t tags[N_TAGS][3] = {
            {TAG_WIDTH, T_LONG, width},        {TAG_HEIGHT, T_LONG, height},
            {TAG_BITS, T_SHORT, 32},           {TAG_COMPRESSION, T_SHORT, 1},
            {TAG_PHOTOMETRIC, T_SHORT, 1},     {TAG_STRIP_OFFSETS, T_LONG, (uint32_t) data_at},
            {TAG_SAMPLES, T_SHORT, 1},         {TAG_ROWS_PER_STRIP, T_LONG, height},
            {TAG_STRIP_BYTES, T_LONG, (uint32_t) page_bytes}, {TAG_PLANAR, T_SHORT, 1},
            {TAG_SAMPLE_FORMAT, T_SHORT, 3}};
        for (int t = 0; t < N_TAGS; t++) {
            unsigned char *x = ifd + 2 + 12 * t;
            put16(x, tags[t][0]);
            put16(x + 2, tags[t][1]);
            put32(x + 4, 1);
            if (tags[t][1] == T_SHORT)
                put16(x + 8, tags[t][2]);
            else
                put32(x + 8, tags[t][2]);
        }
        const uint32_t next = p + 1 < pages ? (uint32_t) (8 + (page_bytes + ifd_bytes) * (p + 1) + page_bytes) : 0;
        put32(ifd + 2 + 12 * N_TAGS, next);
        if (rc == UFOIR_OK && fwrite(ifd, 1, sizeof(ifd), f) != sizeof(ifd))
            rc = io_fail(UFOIR_ERR_IO, "%s: write failed", path);
    }
    free(row);
    if (fclose(f) != 0 && rc == UFOIR_OK)
        rc = io_fail(UFOIR_ERR_IO, "%s: close failed", path);
    return rc;
}

/* ------------------------------------------------------------------- raw */

int ufoir_io_read_raw(const char *path, uint64_t offset, float *out, size_t count)
{
    if (!path || (!out && count))
        return io_fail(UFOIR_ERR_INVALID, "no path or output");
    FILE *f = fopen(path, "rb");
    if (!f)
        return io_fail(UFOIR_ERR_IO, "%s: %s", path, strerror(errno));
    int rc = UFOIR_OK;
    if (fseek(f, (long) offset, SEEK_SET) != 0 || fread(out, sizeof(float), count, f) != count)
        rc = io_fail(UFOIR_ERR_IO, "%s: fewer than %zu floats at offset %llu", path, count,
                     (unsigned long long) offset);
    fclose(f);
    return rc;
}

int ufoir_io_write_raw(const char *path, const float *data, size_t count)
{
    if (!path || (!data && count))
        return io_fail(UFOIR_ERR_INVALID, "no path or data");
    FILE *f = fopen(path, "wb");
    if (!f)
        return io_fail(UFOIR_ERR_IO, "%s: %s", path, strerror(errno));
    int rc = fwrite(data, sizeof(float), count, f) == count ? UFOIR_OK : io_fail(UFOIR_ERR_IO, "%s: write failed", path);
    if (fclose(f) != 0 && rc == UFOIR_OK)
        rc = io_fail(UFOIR_ERR_IO, "%s: close failed", path);
    return rc;
}
