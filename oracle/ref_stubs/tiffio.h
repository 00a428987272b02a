/* Stand-in for libtiff (not on this machine) with the three calls
 * ResidualProducer::readTile makes on a tile held in a memory file: TIFFClientOpen,
 * TIFFReadEncodedStrip of strip 0, TIFFClose.  TEST INFRASTRUCTURE ONLY
 * (oracle/ref_build.py compiles the reference's residual producer against it).
 *
 * The types are libtiff 3's (tsize_t a 32-bit int, toff_t a 32-bit unsigned), which
 * the function-pointer casts in readTile (mfs_read, mfs_lseek, ...) were written for.
 * TIFFReadEncodedStrip reads the first image directory of a little- or big-endian
 * TIFF -- StripOffsets (273), StripByteCounts (279), Compression (259), and the strip's
 * decoded size from ImageWidth (256), ImageLength (257), BitsPerSample (258),
 * SamplesPerPixel (277), RowsPerStrip (278) -- and returns strip 0 inflated by zlib
 * (Compression 8 or 32946, Deflate) or copied (1, none), at most that size, the forms
 * of the reference's pyramids (one strip per tile, no predictor). */
#ifndef TIFFIO_STUB_H
#define TIFFIO_STUB_H

#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include <zlib.h>

#include <vector>

typedef int32_t tsize_t;
typedef uint32_t toff_t;
typedef uint32_t tstrip_t;
typedef void *tdata_t;
typedef void *thandle_t;
typedef tsize_t (*TIFFReadWriteProc)(thandle_t, tdata_t, tsize_t);
typedef toff_t (*TIFFSeekProc)(thandle_t, toff_t, int);
typedef int (*TIFFCloseProc)(thandle_t);
typedef toff_t (*TIFFSizeProc)(thandle_t);
typedef int (*TIFFMapFileProc)(thandle_t, tdata_t *, toff_t *);
typedef void (*TIFFUnmapFileProc)(thandle_t, tdata_t, toff_t);

struct TIFF {
    std::vector<unsigned char> bytes;
    thandle_t handle;
    TIFFCloseProc close;
};

/* the whole file, read through the client's procedures */
inline TIFF *TIFFClientOpen(const char *, const char *, thandle_t h, TIFFReadWriteProc rd, TIFFReadWriteProc,
                            TIFFSeekProc sk, TIFFCloseProc cl, TIFFSizeProc sz, TIFFMapFileProc, TIFFUnmapFileProc)
{
    TIFF *t = new TIFF;
    t->handle = h;
    t->close = cl;
    const toff_t n = sz(h);
    t->bytes.resize(n);
    sk(h, 0, SEEK_SET);
    if (n && rd(h, t->bytes.data(), (tsize_t)n) != (tsize_t)n) t->bytes.clear();
    return t;
}

inline uint32_t tiff_stub_rd(const unsigned char *p, int size, bool le)
{
    uint32_t v = 0;
    for (int k = 0; k < size; ++k) v |= (uint32_t)p[le ? k : size - 1 - k] << (8 * k);
    return v;
}

/* strip 0 into buf; the decoded size, or -1 */
inline tsize_t TIFFReadEncodedStrip(TIFF *t, tstrip_t strip, tdata_t buf, tsize_t)
{
    const std::vector<unsigned char> &b = t->bytes;
    if (strip != 0 || b.size() < 8) return -1;
    const bool le = b[0] == 'I';
    const uint32_t ifd = tiff_stub_rd(&b[4], 4, le);
    if ((size_t)ifd + 2 > b.size()) return -1;
    const uint32_t count = tiff_stub_rd(&b[ifd], 2, le);
    uint32_t comp = 1, off = 0, cnt = 0, width = 0, length = 0, bits = 1, spp = 1, rows = 0xFFFFFFFFu;
    for (uint32_t k = 0; k < count && (size_t)ifd + 2 + 12 * (k + 1) <= b.size(); ++k) {
        const unsigned char *e = &b[ifd + 2 + 12 * k];
        const uint32_t tag = tiff_stub_rd(e, 2, le), type = tiff_stub_rd(e + 2, 2, le), num = tiff_stub_rd(e + 4, 4, le);
        const int size = type == 3 ? 2 : 4;
        const unsigned char *v = e + 8;
        if ((uint32_t)size * num > 4) {
            const uint32_t at = tiff_stub_rd(e + 8, 4, le);
            if ((size_t)at + size > b.size()) return -1;
            v = &b[at];
        }
        const uint32_t value = tiff_stub_rd(v, size, le);
        if (tag == 259) comp = value;
        if (tag == 273) off = value;
        if (tag == 279) cnt = value;
        if (tag == 256) width = value;
        if (tag == 257) length = value;
        if (tag == 258) bits = value;
        if (tag == 277) spp = value;
        if (tag == 278) rows = value;
    }
    if ((size_t)off + cnt > b.size()) return -1;
    const uint64_t strip_bytes = (uint64_t)width * (rows < length ? rows : length) * spp * bits / 8;
    if (strip_bytes == 0 || strip_bytes > (1u << 24)) return -1;
    if (comp == 1) {
        if (cnt > strip_bytes) return -1;
        memcpy(buf, &b[off], cnt);
        return (tsize_t)cnt;
    }
    if (comp != 8 && comp != 32946) return -1;
    z_stream z;
    memset(&z, 0, sizeof(z));
    if (inflateInit(&z) != Z_OK) return -1;
    z.next_in = (Bytef *)&b[off];
    z.avail_in = cnt;
    z.next_out = (Bytef *)buf;
    z.avail_out = (uInt)strip_bytes;
    const int rc = inflate(&z, Z_FINISH);
    const tsize_t n = (tsize_t)z.total_out;
    inflateEnd(&z);
    return rc == Z_STREAM_END ? n : -1;
}

inline void TIFFClose(TIFF *t)
{
    if (t->close) t->close(t->handle);
    delete t;
}

#endif
