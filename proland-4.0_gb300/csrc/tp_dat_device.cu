// Residual pyramid tiles decoded on the device (ResidualProducer::readTile,
// ResidualProducer.cpp:268-340): the .dat file's bytes live in device memory; one
// warp per tile finds the tile's strip (tile-id offsets, TIFF directory), lane 0
// inflates it (zlib wrapper, RFC 1951 blocks, Adler-32 check) into a scratch
// buffer, then the warp writes int16 x scale into the tile's residual slot (tiles
// below the file's minLevel are smaller and land in the slot's lower-left corner,
// the rest of the slot is zero).  Every read is checked against the file and the
// strip, every write against the tile: a corrupt strip marks the tile's status and
// leaves it zero.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "tp_internal.h"

namespace {

struct DatJob {
    int id;      // tile id in the file, -1 for a zero tile
    int width;   // width of the stored tile (<= the slot width)
    int slot;    // residual slot
    int pad;
};

struct Bits {
    const uint8_t *p;
    uint32_t n, pos;
    uint64_t buf;
    int cnt;
    bool bad;
};

__device__ __forceinline__ void refill(Bits &b)
{
    while (b.cnt <= 56) {
        if (b.pos < b.n) b.buf |= (uint64_t)b.p[b.pos] << b.cnt;
        else if (b.pos >= b.n + 8) b.bad = true;  // more than 8 bytes past the end: truncated
        ++b.pos;
        b.cnt += 8;
    }
}

__device__ __forceinline__ uint32_t getbits(Bits &b, int k)
{
    if (k == 0) return 0;
    if (b.cnt < k) refill(b);
    const uint32_t v = (uint32_t)(b.buf & ((1ull << k) - 1));
    b.buf >>= k;
    b.cnt -= k;
    return v;
}

// Canonical Huffman code (RFC 1951 3.2.2): counts per length, symbols in code order,
// and a 9-bit table of the short codes indexed by the next stream bits.
struct Huff {
    uint16_t count[16];
    uint16_t symbol[320];
    uint16_t fast[512];  // (symbol << 4) | length, 0 when the code is longer than 9 bits
};

__device__ bool huff_build(Huff &h, const uint8_t *len, int n)
{
    for (int i = 0; i < 16; ++i) h.count[i] = 0;
    for (int i = 0; i < n; ++i) h.count[len[i]]++;
    h.count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
        left <<= 1;
        left -= h.count[l];
        if (left < 0) return false;
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + h.count[l];
    for (int i = 0; i < n; ++i)
        if (len[i]) h.symbol[offs[len[i]]++] = (uint16_t)i;
    for (int i = 0; i < 512; ++i) h.fast[i] = 0;
    // canonical codes, bit-reversed into the table
    uint32_t code = 0;
    int idx = 0;
    for (int l = 1; l <= 9; ++l) {
        for (int k = 0; k < h.count[l]; ++k, ++idx, ++code) {
            uint32_t rev = 0;
            for (int b = 0; b < l; ++b) rev |= ((code >> b) & 1u) << (l - 1 - b);
            for (uint32_t fill = rev; fill < 512; fill += (1u << l)) h.fast[fill] = (uint16_t)((h.symbol[idx] << 4) | l);
        }
        code <<= 1;
    }
    return true;
}

__device__ int huff_decode(Bits &b, const Huff &h)
{
    if (b.cnt < 16) refill(b);
    const uint16_t e = h.fast[b.buf & 511];
    if (e) {
        const int l = e & 15;
        b.buf >>= l;
        b.cnt -= l;
        return e >> 4;
    }
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
        code |= (int)getbits(b, 1);
        const int c = h.count[l];
        if (code - c < first) return h.symbol[index + (code - first)];
        index += c;
        first += c;
        first <<= 1;
        code <<= 1;
    }
    return -1;
}

__constant__ uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
__constant__ uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
__constant__ uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
__constant__ uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

__device__ bool inflate_block(Bits &b, const Huff &lit, const Huff &dist, uint8_t *out, uint32_t &n, uint32_t limit)
{
    for (;;) {
        int sym = huff_decode(b, lit);
        if (sym < 0 || b.bad) return false;
        if (sym < 256) {
            if (n >= limit) return false;
            out[n++] = (uint8_t)sym;
        } else if (sym == 256) {
            return true;
        } else {
            sym -= 257;
            if (sym >= 29) return false;
            const uint32_t len = kLenBase[sym] + getbits(b, kLenExtra[sym]);
            const int ds = huff_decode(b, dist);
            if (ds < 0 || ds >= 30) return false;
            const uint32_t d = kDistBase[ds] + getbits(b, kDistExtra[ds]);
            if (d > n || n + len > limit || b.bad) return false;
            for (uint32_t k = 0; k < len; ++k, ++n) out[n] = out[n - d];
        }
    }
}

// Raw deflate data -> out (at most `limit` bytes); false on a corrupt stream.
__device__ bool inflate_raw(const uint8_t *data, uint32_t size, uint8_t *out, uint32_t &n, uint32_t limit, Huff &h1,
                            Huff &h2)
{
    Bits b{data, size, 0, 0, 0, false};
    int last = 0;
    n = 0;
    do {
        last = (int)getbits(b, 1);
        const int type = (int)getbits(b, 2);
        if (b.bad) return false;
        if (type == 0) {
            // stored block: drop to the byte boundary (the bytes buffered past it are unread)
            const uint32_t byte = b.pos - (uint32_t)(b.cnt / 8);
            b.buf = 0;
            b.cnt = 0;
            b.pos = byte;
            if (b.pos + 4 > size) return false;
            const uint32_t len = data[b.pos] | (data[b.pos + 1] << 8), nlen = data[b.pos + 2] | (data[b.pos + 3] << 8);
            b.pos += 4;
            if ((len ^ 0xFFFFu) != nlen || b.pos + len > size || n + len > limit) return false;
            for (uint32_t k = 0; k < len; ++k) out[n++] = data[b.pos + k];
            b.pos += len;
        } else if (type == 1) {
            uint8_t l[288];
            int i = 0;
            for (; i < 144; ++i) l[i] = 8;
            for (; i < 256; ++i) l[i] = 9;
            for (; i < 280; ++i) l[i] = 7;
            for (; i < 288; ++i) l[i] = 8;
            huff_build(h1, l, 288);
            for (i = 0; i < 30; ++i) l[i] = 5;
            huff_build(h2, l, 30);
            if (!inflate_block(b, h1, h2, out, n, limit)) return false;
        } else if (type == 2) {
            const int hlit = (int)getbits(b, 5) + 257, hdist = (int)getbits(b, 5) + 1, hclen = (int)getbits(b, 4) + 4;
            const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19];
            for (int k = 0; k < 19; ++k) cl[k] = 0;
            for (int k = 0; k < hclen; ++k) cl[order[k]] = (uint8_t)getbits(b, 3);
            if (!huff_build(h1, cl, 19)) return false;
            uint8_t lens[320];
            int k = 0;
            while (k < hlit + hdist) {
                const int sym = huff_decode(b, h1);
                if (sym < 0 || b.bad) return false;
                if (sym < 16) {
                    lens[k++] = (uint8_t)sym;
                } else {
                    int rep;
                    uint8_t val = 0;
                    if (sym == 16) {
                        if (k == 0) return false;
                        val = lens[k - 1];
                        rep = 3 + (int)getbits(b, 2);
                    } else if (sym == 17) {
                        rep = 3 + (int)getbits(b, 3);
                    } else {
                        rep = 11 + (int)getbits(b, 7);
                    }
                    if (k + rep > hlit + hdist) return false;
                    while (rep--) lens[k++] = val;
                }
            }
            if (!huff_build(h1, lens, hlit) || !huff_build(h2, lens + hlit, hdist)) return false;
            if (!inflate_block(b, h1, h2, out, n, limit)) return false;
        } else {
            return false;
        }
    } while (!last);
    return !b.bad;
}

__device__ uint32_t rd16(const uint8_t *p, bool le) { return le ? (p[0] | (p[1] << 8)) : ((p[0] << 8) | p[1]); }
__device__ uint32_t rd32(const uint8_t *p, bool le)
{
    return le ? (p[0] | (p[1] << 8) | (p[2] << 16) | ((uint32_t)p[3] << 24))
              : (((uint32_t)p[0] << 24) | (p[1] << 16) | (p[2] << 8) | p[3]);
}

// Strip 0 of the TIFF t[0, n) -> out; the same checks as the host decoder.
__device__ bool tiff_strip(const uint8_t *t, uint32_t n, uint8_t *out, uint32_t &got, uint32_t limit, Huff &h1, Huff &h2)
{
    if (n < 8) return false;
    bool le;
    if (t[0] == 'I' && t[1] == 'I') le = true;
    else if (t[0] == 'M' && t[1] == 'M') le = false;
    else return false;
    if (rd16(t + 2, le) != 42) return false;
    const uint32_t ifd = rd32(t + 4, le);
    if ((uint64_t)ifd + 2 > n) return false;
    const uint32_t count = rd16(t + ifd, le);
    if ((uint64_t)ifd + 2 + 12ull * count > n) return false;
    uint32_t comp = 1, off = 0xFFFFFFFFu, cnt = 0xFFFFFFFFu;
    for (uint32_t k = 0; k < count; ++k) {
        const uint8_t *e = t + ifd + 2 + 12 * k;
        const uint32_t tag = rd16(e, le), type = rd16(e + 2, le), num = rd32(e + 4, le);
        if (type != 3 && type != 4) continue;
        const uint32_t sz = type == 3 ? 2 : 4;
        const uint8_t *v = e + 8;
        if ((uint64_t)sz * num > 4) {
            const uint32_t p = rd32(e + 8, le);
            if ((uint64_t)p + sz > n) return false;
            v = t + p;
        }
        const uint32_t value = type == 3 ? rd16(v, le) : rd32(v, le);
        if (tag == 259) comp = value;
        if (tag == 273) off = value;
        if (tag == 279) cnt = value;
    }
    if (off == 0xFFFFFFFFu || cnt == 0xFFFFFFFFu || (uint64_t)off + cnt > n) return false;
    const uint8_t *s = t + off;
    if (comp == 1) {
        if (cnt > limit) return false;
        for (uint32_t k = 0; k < cnt; ++k) out[k] = s[k];
        got = cnt;
        return true;
    }
    if (comp != 8 && comp != 32946) return false;
    // zlib: header, deflate data, big-endian Adler-32
    if (cnt < 6 || (s[0] & 0x0F) != 8 || ((s[0] << 8) | s[1]) % 31 != 0 || (s[1] & 0x20)) return false;
    if (!inflate_raw(s + 2, cnt - 6, out, got, limit, h1, h2)) return false;
    uint32_t a = 1, b2 = 0;
    for (uint32_t k = 0; k < got; ++k) {
        a = (a + out[k]) % 65521u;
        b2 = (b2 + a) % 65521u;
    }
    const uint32_t want = ((uint32_t)s[cnt - 4] << 24) | ((uint32_t)s[cnt - 3] << 16) | ((uint32_t)s[cnt - 2] << 8) | s[cnt - 1];
    return ((b2 << 16) | a) == want;
}

constexpr int kWarps = 4;

__global__ void __launch_bounds__(32 * kWarps) dat_decode_kernel(const uint8_t *__restrict__ file, uint64_t file_size,
                                                                 uint64_t header, int ntiles,
                                                                 const DatJob *__restrict__ jobs, int njobs, float scale,
                                                                 float *__restrict__ res, int pitch, long long slot_stride,
                                                                 int W, uint8_t *__restrict__ scratch, uint64_t per_job,
                                                                 int *__restrict__ status)
{
    __shared__ Huff tables[kWarps][2];  // the decoding lane's code tables
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j = blockIdx.x * kWarps + warp;
    if (j >= njobs) return;
    const DatJob J = jobs[j];
    uint8_t *raw = scratch + (uint64_t)j * per_job;
    int ok = 0;
    if (lane == 0) {
        if (J.id < 0) {
            ok = 2;  // a tile outside the pyramid: zeros
        } else if (J.id < ntiles && J.width >= 1 && J.width <= W) {
            const uint32_t a = rd32(file + 28 + 8 * (uint64_t)J.id, true), b = rd32(file + 32 + 8 * (uint64_t)J.id, true);
            if (b >= a && header + b <= file_size) {
                Huff &h1 = tables[warp][0], &h2 = tables[warp][1];
                uint32_t got = 0;
                const uint32_t need = 2u * J.width * J.width;
                if (tiff_strip(file + header + a, b - a, raw, got, (uint32_t)per_job, h1, h2) && got >= need) ok = 1;
            }
        }
        if (!ok) status[j] = 1;
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    __syncwarp();
    float *dst = res + (long long)J.slot * slot_stride;
    const int w = J.width;
    for (int k = lane; k < W * W; k += 32) {
        const int y = k / W, x = k - y * W;
        float v = 0.0f;
        if (ok == 1 && x < w && y < w) {
            const int o = 2 * (y * w + x);
            v = (float)(int16_t)(uint16_t)(raw[o] | (raw[o + 1] << 8)) * scale;
        }
        dst[(long long)y * pitch + x] = v;
    }
}

}  // namespace

namespace tp {

// Device copy of a residual file's bytes (uploaded once, freed with the file).
int dat_device_bytes(tp_dat *d, const uint8_t **out)
{
    std::lock_guard<std::mutex> lk(d->dev_mu);
    if (!d->dev_bytes) {
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, d->bytes.size());
        if (e == cudaSuccess) e = cudaMemcpy(p, d->bytes.data(), d->bytes.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            if (p) cudaFree(p);
            return cuda_fail("residual file upload", e);
        }
        d->dev_bytes = static_cast<uint8_t *>(p);
    }
    *out = d->dev_bytes;
    return TP_OK;
}

}  // namespace tp

// Decodes n tiles (level, tx, ty in the file's pyramid; level < 0 for a zero tile)
// into residual slots on the device, values int16 x scale.
extern "C" int tp_dat_decode_device(tp_dat *d, const int *levels, const int *txs, const int *tys, int n, float scale,
                                    tp_storage *residuals, const int *slots, void *stream)
{
    if (!d || n < 0 || (n > 0 && (!levels || !txs || !tys || !slots)) || !residuals)
        return tp::fail(TP_E_BAD_ARG, "tp_dat_decode_device: bad arguments");
    if (residuals->on_device != 1 || residuals->channels != 1 || residuals->W != d->tile_size + 5)
        return tp::fail(TP_E_BAD_ARG, "tp_dat_decode_device: residual storage must be a 1-channel device storage of the file's tile width");
    if (n == 0) return TP_OK;
    std::vector<DatJob> h(n);
    for (int k = 0; k < n; ++k) {
        if (slots[k] < 0 || slots[k] >= residuals->capacity) return tp::fail(TP_E_BAD_ARG, "tp_dat_decode_device: bad slot");
        const int l = levels[k];
        if (l < 0) {
            h[k] = DatJob{-1, 0, slots[k], 0};
            continue;
        }
        if (l > d->max_level || txs[k] < 0 || tys[k] < 0 || (txs[k] >> l) != 0 || (tys[k] >> l) != 0)
            return tp::fail(TP_E_BAD_ARG, "tp_dat_decode_device: tile outside the pyramid");
        h[k] = DatJob{tp::dat_tile_id(d, l, txs[k], tys[k]), tp::dat_tile_width(d, l), slots[k], 0};
    }
    const uint8_t *bytes = nullptr;
    int rc = tp::dat_device_bytes(d, &bytes);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint64_t per_job = ((uint64_t)2 * residuals->W * residuals->W + 64 + 255) & ~255ull;
    void *buf = nullptr;
    const size_t bytes_jobs = (sizeof(DatJob) * n + 255) & ~(size_t)255, bytes_status = (sizeof(int) * n + 255) & ~(size_t)255;
    cudaError_t e = cudaMallocAsync(&buf, bytes_jobs + bytes_status + per_job * n, s);
    if (e != cudaSuccess) return tp::cuda_fail("tp_dat_decode_device: scratch", e);
    char *base = static_cast<char *>(buf);
    DatJob *jobs = reinterpret_cast<DatJob *>(base);
    int *status = reinterpret_cast<int *>(base + bytes_jobs);
    uint8_t *scratch = reinterpret_cast<uint8_t *>(base + bytes_jobs + bytes_status);
    e = cudaMemcpyAsync(jobs, h.data(), sizeof(DatJob) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, sizeof(int) * n, s);
    if (e == cudaSuccess) {
        dat_decode_kernel<<<(n + kWarps - 1) / kWarps, 32 * kWarps, 0, s>>>(
            bytes, d->bytes.size(), d->header, d->ntiles, jobs, n, scale, residuals->base, residuals->pitch,
            residuals->slot_stride, residuals->W, scratch, per_job, status);
        e = cudaGetLastError();
    }
    std::vector<int> st(n, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(st.data(), status, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(buf, s);
    if (e != cudaSuccess) return tp::cuda_fail("tp_dat_decode_device", e);
    for (int k = 0; k < n; ++k)
        if (st[k]) return tp::fail(TP_E_IO, "dat: corrupt or truncated tile strip (device decode)");
    return TP_OK;
}
