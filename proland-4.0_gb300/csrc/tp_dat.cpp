// Residual pyramid files (.dat): header, tile offsets, and one single-strip
// deflate TIFF per tile (ResidualProducer.cpp:93-107, 253-340; written by
// HeightMipmap.cpp:561-655).  The TIFF strip parser and the inflate decoder
// (RFC 1950/1951) are this library's own, so the host side needs no zlib or
// libtiff.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "tp_internal.h"

namespace {

// ---------------------------------------------------------------- inflate
struct BitReader {
    const uint8_t *p;
    size_t n, pos = 0;
    uint32_t bitbuf = 0;
    int bitcnt = 0;
    bool bad = false;
    BitReader(const uint8_t *d, size_t len) : p(d), n(len) {}
    int bit()
    {
        if (bitcnt == 0) {
            if (pos >= n) {
                bad = true;
                return 0;
            }
            bitbuf = p[pos++];
            bitcnt = 8;
        }
        int b = bitbuf & 1;
        bitbuf >>= 1;
        --bitcnt;
        return b;
    }
    uint32_t bits(int k)
    {
        uint32_t v = 0;
        for (int i = 0; i < k; ++i) v |= (uint32_t)bit() << i;
        return v;
    }
    void align() { bitcnt = 0; }
};

// Canonical Huffman decoding table: counts per code length and symbols in
// code order (the construction of RFC 1951 section 3.2.2).
struct Huffman {
    uint16_t count[16];
    std::vector<uint16_t> symbol;
    bool build(const uint8_t *lengths, int n)
    {
        std::memset(count, 0, sizeof count);
        for (int i = 0; i < n; ++i) count[lengths[i]]++;
        count[0] = 0;
        int left = 1;
        for (int len = 1; len < 16; ++len) {
            left <<= 1;
            left -= count[len];
            if (left < 0) return false;  // over-subscribed
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int len = 1; len < 15; ++len) offs[len + 1] = offs[len] + count[len];
        symbol.assign(n, 0);
        for (int i = 0; i < n; ++i)
            if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
        return true;
    }
    int decode(BitReader &br) const
    {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= br.bit();
            const int c = count[len];
            if (code - c < first) return symbol[index + (code - first)];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
            if (br.bad) return -1;
        }
        return -1;
    }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_block(BitReader &br, const Huffman &lit, const Huffman &dist, std::vector<uint8_t> &out, size_t limit)
{
    for (;;) {
        int sym = lit.decode(br);
        if (sym < 0 || br.bad) return false;
        if (sym < 256) {
            if (out.size() >= limit) return false;
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return true;
        } else {
            sym -= 257;
            if (sym >= 29) return false;
            const int len = kLenBase[sym] + (int)br.bits(kLenExtra[sym]);
            const int ds = dist.decode(br);
            if (ds < 0 || ds >= 30) return false;
            const size_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
            if (d > out.size() || out.size() + len > limit || br.bad) return false;
            const size_t from = out.size() - d;
            for (int k = 0; k < len; ++k) out.push_back(out[from + k]);
        }
    }
}

// Raw deflate stream -> bytes (at most `limit`).  false on a corrupt stream.
bool inflate_raw(const uint8_t *data, size_t n, std::vector<uint8_t> &out, size_t limit)
{
    BitReader br(data, n);
    int last = 0;
    do {
        last = br.bit();
        const int type = (int)br.bits(2);
        if (br.bad) return false;
        if (type == 0) {
            br.align();
            if (br.pos + 4 > n) return false;
            const uint16_t len = (uint16_t)(data[br.pos] | (data[br.pos + 1] << 8));
            const uint16_t nlen = (uint16_t)(data[br.pos + 2] | (data[br.pos + 3] << 8));
            br.pos += 4;
            if ((uint16_t)~len != nlen || br.pos + len > n || out.size() + len > limit) return false;
            out.insert(out.end(), data + br.pos, data + br.pos + len);
            br.pos += len;
        } else if (type == 1) {
            // the fixed codes of RFC 1951 section 3.2.6 (built once, thread-safe static)
            struct Fixed {
                Huffman lit, dist;
                Fixed()
                {
                    uint8_t l[288];
                    int i = 0;
                    for (; i < 144; ++i) l[i] = 8;
                    for (; i < 256; ++i) l[i] = 9;
                    for (; i < 280; ++i) l[i] = 7;
                    for (; i < 288; ++i) l[i] = 8;
                    lit.build(l, 288);
                    uint8_t d[30];
                    for (int k = 0; k < 30; ++k) d[k] = 5;
                    dist.build(d, 30);
                }
            };
            static const Fixed fixed;
            if (!inflate_block(br, fixed.lit, fixed.dist, out, limit)) return false;
        } else if (type == 2) {
            const int hlit = (int)br.bits(5) + 257, hdist = (int)br.bits(5) + 1, hclen = (int)br.bits(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int k = 0; k < hclen; ++k) cl[order[k]] = (uint8_t)br.bits(3);
            Huffman clh;
            if (!clh.build(cl, 19)) return false;
            uint8_t lens[320] = {0};
            int k = 0;
            while (k < hlit + hdist) {
                int sym = clh.decode(br);
                if (sym < 0 || br.bad) return false;
                if (sym < 16) {
                    lens[k++] = (uint8_t)sym;
                } else {
                    int rep = 0;
                    uint8_t val = 0;
                    if (sym == 16) {
                        if (k == 0) return false;
                        val = lens[k - 1];
                        rep = 3 + (int)br.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)br.bits(3);
                    } else {
                        rep = 11 + (int)br.bits(7);
                    }
                    if (k + rep > hlit + hdist) return false;
                    while (rep--) lens[k++] = val;
                }
            }
            Huffman lh, dh;
            if (!lh.build(lens, hlit) || !dh.build(lens + hlit, hdist)) return false;
            if (!inflate_block(br, lh, dh, out, limit)) return false;
        } else {
            return false;
        }
    } while (!last);
    return true;
}

uint32_t adler32(const uint8_t *d, size_t n)
{
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < n; ++i) {
        a = (a + d[i]) % 65521u;
        b = (b + a) % 65521u;
    }
    return (b << 16) | a;
}

// zlib stream (RFC 1950): 2-byte header, deflate data, big-endian Adler-32.
bool inflate_zlib(const uint8_t *data, size_t n, std::vector<uint8_t> &out, size_t limit)
{
    if (n < 6) return false;
    if ((data[0] & 0x0F) != 8 || ((data[0] << 8) | data[1]) % 31 != 0 || (data[1] & 0x20)) return false;
    out.clear();
    if (!inflate_raw(data + 2, n - 6, out, limit)) return false;
    const uint32_t want = ((uint32_t)data[n - 4] << 24) | ((uint32_t)data[n - 3] << 16) | ((uint32_t)data[n - 2] << 8) | data[n - 1];
    return adler32(out.data(), out.size()) == want;
}

// ---------------------------------------------------------------- TIFF strip
uint32_t rd16(const uint8_t *p, bool le) { return le ? (p[0] | (p[1] << 8)) : ((p[0] << 8) | p[1]); }
uint32_t rd32(const uint8_t *p, bool le)
{
    return le ? (p[0] | (p[1] << 8) | (p[2] << 16) | ((uint32_t)p[3] << 24))
              : (((uint32_t)p[0] << 24) | (p[1] << 16) | (p[2] << 8) | p[3]);
}

}  // namespace

// Decodes strip 0 of a TIFF in memory into raw bytes.
bool tp::decode_tiff_strip(const uint8_t *t, size_t n, std::vector<uint8_t> &raw, size_t limit)
{
    if (n < 8) return false;
    bool le;
    if (t[0] == 'I' && t[1] == 'I') le = true;
    else if (t[0] == 'M' && t[1] == 'M') le = false;
    else return false;
    if (rd16(t + 2, le) != 42) return false;
    const uint32_t ifd = rd32(t + 4, le);
    if ((size_t)ifd + 2 > n) return false;
    const uint32_t count = rd16(t + ifd, le);
    if ((size_t)ifd + 2 + 12ull * count > n) return false;
    uint32_t comp = 1, off = 0, cnt = 0;
    bool have_off = false, have_cnt = false;
    for (uint32_t k = 0; k < count; ++k) {
        const uint8_t *e = t + ifd + 2 + 12 * k;
        const uint32_t tag = rd16(e, le), type = rd16(e + 2, le), num = rd32(e + 4, le);
        auto value = [&](uint32_t idx) -> uint32_t {
            const uint32_t sz = type == 3 ? 2 : 4;
            const uint8_t *v = e + 8;
            if (sz * num > 4) {
                const uint32_t p = rd32(e + 8, le);
                if ((size_t)p + sz * (idx + 1) > n) return 0xFFFFFFFFu;
                v = t + p;
            }
            return type == 3 ? rd16(v + 2 * idx, le) : rd32(v + 4 * idx, le);
        };
        if (type != 3 && type != 4) continue;
        if (tag == 259) comp = value(0);
        if (tag == 273) { off = value(0); have_off = true; }
        if (tag == 279) { cnt = value(0); have_cnt = true; }
    }
    if (!have_off || !have_cnt || off == 0xFFFFFFFFu || (size_t)off + cnt > n) return false;
    if (comp == 8 || comp == 32946) return inflate_zlib(t + off, cnt, raw, limit);
    if (comp == 1) {
        if (cnt > limit) return false;
        raw.assign(t + off, t + off + cnt);
        return true;
    }
    return false;
}

// ---------------------------------------------------------------- .dat file

namespace tp {

int dat_tile_width(const tp_dat *d, int level)
{
    const int ts = level < d->min_level ? d->tile_size >> (d->min_level - level) : d->tile_size;
    return ts + 5;
}

int dat_tile_id(const tp_dat *d, int level, int tx, int ty)
{
    if (level < d->min_level) return level;
    const int l = level - d->min_level;
    return d->min_level + tx + ty * (1 << l) + ((1 << (2 * l)) - 1) / 3;
}

// Decodes tile (level, tx, ty) of the pyramid into int16 samples (width^2).
int dat_tile_int16(const tp_dat *d, int level, int tx, int ty, std::vector<int16_t> &out, int *width)
{
    if (level < 0 || level > d->max_level || tx < 0 || ty < 0 || (tx >> level) != 0 || (ty >> level) != 0)
        return fail(TP_E_BAD_ARG, "dat: tile outside the pyramid");
    const int id = dat_tile_id(d, level, tx, ty);
    if (id < 0 || id >= d->ntiles) return fail(TP_E_BAD_ARG, "dat: tile id outside the pyramid");
    uint32_t a, b;
    std::memcpy(&a, d->bytes.data() + 28 + 8 * (size_t)id, 4);
    std::memcpy(&b, d->bytes.data() + 32 + 8 * (size_t)id, 4);
    if (b < a || d->header + b > d->bytes.size()) return fail(TP_E_IO, "dat: tile offsets outside the file");
    const int w = dat_tile_width(d, level);
    std::vector<uint8_t> raw;
    if (!decode_tiff_strip(d->bytes.data() + d->header + a, b - a, raw, (size_t)2 * w * w + 64))
        return fail(TP_E_IO, "dat: corrupt or truncated tile strip");
    if (raw.size() < (size_t)2 * w * w) return fail(TP_E_IO, "dat: short tile strip");
    out.resize((size_t)w * w);
    for (size_t k = 0; k < out.size(); ++k) out[k] = (int16_t)(uint16_t)(raw[2 * k] | (raw[2 * k + 1] << 8));
    *width = w;
    return TP_OK;
}

}  // namespace tp

extern "C" int tp_dat_open(const char *path, tp_dat **out)
{
    if (!path || !out) return tp::fail(TP_E_BAD_ARG, "tp_dat_open: bad arguments");
    *out = nullptr;
    FILE *f = std::fopen(path, "rb");
    if (!f) return tp::fail(TP_E_IO, std::string("cannot open residual file '") + path + "'");
    auto *d = new tp_dat;
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (size > 0) {
        d->bytes.resize((size_t)size);
        if (std::fread(d->bytes.data(), 1, (size_t)size, f) != (size_t)size) d->bytes.clear();
    }
    std::fclose(f);
    if (d->bytes.size() < 28) {
        delete d;
        return tp::fail(TP_E_IO, "residual file truncated (header)");
    }
    int32_t h[6];
    std::memcpy(h, d->bytes.data(), 24);
    std::memcpy(&d->scale, d->bytes.data() + 24, 4);
    d->min_level = h[0];
    d->max_level = h[1];
    d->tile_size = h[2];
    d->root_level = h[3];
    d->root_tx = h[4];
    d->root_ty = h[5];
    if (d->min_level < 0 || d->min_level > 24 || d->max_level < d->min_level || d->max_level > 24 || d->tile_size < 1 ||
        d->tile_size > 4096) {
        delete d;
        return tp::fail(TP_E_IO, "residual file header is corrupt");
    }
    const int l = d->max_level - d->min_level;
    d->ntiles = d->min_level + ((1 << (l * 2 + 2)) - 1) / 3;
    d->header = sizeof(float) + sizeof(int32_t) * (6 + (size_t)d->ntiles * 2);
    if (d->bytes.size() < d->header) {
        delete d;
        return tp::fail(TP_E_IO, "residual file truncated (offsets)");
    }
    *out = d;
    return TP_OK;
}

extern "C" int tp_dat_close(tp_dat *d)
{
    if (d && d->dev_bytes) cudaFree(d->dev_bytes);
    delete d;
    return TP_OK;
}

extern "C" int tp_dat_info(const tp_dat *d, int *info7, float *scale)
{
    if (!d || !info7) return tp::fail(TP_E_BAD_ARG, "tp_dat_info: bad arguments");
    info7[0] = d->min_level;
    info7[1] = d->max_level;
    info7[2] = d->tile_size;
    info7[3] = d->root_level;
    info7[4] = d->root_tx;
    info7[5] = d->root_ty;
    info7[6] = d->ntiles;
    if (scale) *scale = d->scale;
    return TP_OK;
}

extern "C" int tp_dat_read_tile(const tp_dat *d, int level, int tx, int ty, int16_t *out, int capacity, int *width)
{
    if (!d || !out || !width) return tp::fail(TP_E_BAD_ARG, "tp_dat_read_tile: bad arguments");
    std::vector<int16_t> v;
    int w = 0;
    int rc = tp::dat_tile_int16(d, level, tx, ty, v, &w);
    if (rc) return rc;
    if ((int)v.size() > capacity) return tp::fail(TP_E_BAD_ARG, "tp_dat_read_tile: output too small");
    std::memcpy(out, v.data(), sizeof(int16_t) * v.size());
    *width = w;
    return TP_OK;
}

extern "C" int tp_inflate_zlib(const uint8_t *data, size_t n, uint8_t *out, size_t capacity, size_t *written)
{
    if (!data || !out || !written) return tp::fail(TP_E_BAD_ARG, "tp_inflate_zlib: bad arguments");
    std::vector<uint8_t> v;
    if (!inflate_zlib(data, n, v, capacity)) return tp::fail(TP_E_IO, "corrupt zlib stream");
    std::memcpy(out, v.data(), v.size());
    *written = v.size();
    return TP_OK;
}
