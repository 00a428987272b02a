// Ortho (colour) tiles, host side: the RGBA8 noise table, its device copy
// rotated for the four noise rotations, the batch entry points and the reader
// of OrthoCPUProducer's .dat pyramids.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "tp_internal.h"

// Launch state of the ortho batches of one storage: device job array and the
// [counter | done per job] words.
struct OrthoState {
    tp_ortho_job *jobs = nullptr;
    size_t jobs_cap = 0;
    int *flags = nullptr;
    size_t flags_cap = 0;
};

struct tp_ortho_dat {
    int max_level = -1, tile_size = 0, channels = 0, root = 0, root_tx = 0, root_ty = 0, flags = 0;
    int border = 2, ntiles = 0;
    size_t header = 0;
    std::vector<uint8_t> bytes;
};

namespace {

// createOrthoNoise (OrthoProducer.cpp:26-122): six layers (edge patterns 0, 1, 3,
// 5, 7, 15) of W x W RGBA8; 128 in the corners, mirrored random border bands
// whose sequence depends on the edge bit (seeds 7654321 / 5647381), random
// centres from one sequence (seed 1234567) running through all layers.
void build_ortho_noise(int W, uint8_t *out)
{
    static const int kEdges[6] = {0, 1, 3, 5, 7, 15};
    tp::Lcg centre(1234567);
    auto byte = [](tp::Lcg &g) { return (uint8_t)(int)(g.unit() * 255.0f); };
    for (int layer = 0; layer < 6; ++layer) {
        uint8_t *t = out + (size_t)layer * W * W * 4;
        const int e = kEdges[layer];
        std::memset(t, 128, (size_t)W * W * 4);
        auto at = [&](int x, int y, int c) -> uint8_t & { return t[4 * ((size_t)y * W + x) + c]; };
        {
            tp::Lcg g((e & 1) ? 5647381 : 7654321);  // bottom: rows 2, 3 and their mirror 1, 0
            for (int y = 2; y < 4; ++y)
                for (int x = 4; x < W - 4; ++x)
                    for (int c = 0; c < 4; ++c) at(x, y, c) = at(W - 1 - x, 3 - y, c) = byte(g);
        }
        {
            tp::Lcg g((e & 2) ? 5647381 : 7654321);  // right: columns W-3, W-4 and W-2, W-1
            for (int x = W - 3; x >= W - 4; --x)
                for (int y = 4; y < W - 4; ++y)
                    for (int c = 0; c < 4; ++c) at(x, y, c) = at(2 * W - 5 - x, W - 1 - y, c) = byte(g);
        }
        {
            tp::Lcg g((e & 4) ? 5647381 : 7654321);  // top: rows W-2, W-1 and W-3, W-4
            for (int y = W - 2; y < W; ++y)
                for (int x = 4; x < W - 4; ++x)
                    for (int c = 0; c < 4; ++c) at(x, y, c) = at(W - 1 - x, 2 * W - 5 - y, c) = byte(g);
        }
        {
            tp::Lcg g((e & 8) ? 5647381 : 7654321);  // left: columns 1, 0 and 2, 3
            for (int x = 1; x >= 0; --x)
                for (int y = 4; y < W - 4; ++y)
                    for (int c = 0; c < 4; ++c) at(x, y, c) = at(3 - x, W - 1 - y, c) = byte(g);
        }
        for (int y = 4; y < W - 4; ++y)
            for (int x = 4; x < W - 4; ++x)
                for (int c = 0; c < 4; ++c) at(x, y, c) = byte(centre);
    }
}

bool valid_width(int W) { return W >= 8 && W <= 1024 && W % 4 == 0; }

// Device table [rotation][layer][row][pitch] of RGBA8 words for tile width W:
// entry (i, j) of rotation R is the layer's texel at the shader's rotated
// coordinates (NEAREST at texel centres): R=0 (i, j), 1 (j, W-1-i),
// 2 (W-1-i, W-1-j), 3 (W-1-j, i).
const uint32_t *device_ortho_noise(int W, int pitch, int *err)
{
    static std::mutex mu;
    static std::map<std::tuple<int, int, int>, uint32_t *> tables;  // (device, W, pitch)
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    auto it = tables.find(std::make_tuple(dev, W, pitch));
    if (it != tables.end()) return it->second;
    std::vector<uint8_t> t((size_t)6 * W * W * 4);
    build_ortho_noise(W, t.data());
    std::vector<uint32_t> h((size_t)4 * 6 * W * pitch, 0u);
    for (int r = 0; r < 4; ++r)
        for (int l = 0; l < 6; ++l)
            for (int j = 0; j < W; ++j)
                for (int i = 0; i < W; ++i) {
                    int x, y;
                    switch (r) {
                    case 0: x = i; y = j; break;
                    case 1: x = j; y = W - 1 - i; break;
                    case 2: x = W - 1 - i; y = W - 1 - j; break;
                    default: x = W - 1 - j; y = i; break;
                    }
                    uint32_t w;
                    std::memcpy(&w, &t[((size_t)l * W * W + (size_t)y * W + x) * 4], 4);
                    h[(((size_t)r * 6 + l) * W + j) * pitch + i] = w;
                }
    uint32_t *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(uint32_t) * h.size());
    if (e == cudaSuccess) e = cudaMemcpy(d, h.data(), sizeof(uint32_t) * h.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        if (d) cudaFree(d);
        *err = tp::cuda_fail("ortho noise table", e);
        return nullptr;
    }
    tables[std::make_tuple(dev, W, pitch)] = d;
    return d;
}

int check_storages(tp_storage *o, tp_storage *r)
{
    if (!o || o->on_device != 1 || o->channels != 1)
        return tp::fail(TP_E_BAD_ARG, "ortho: a one-channel device storage of RGBA8 texels is required");
    if (!valid_width(o->W)) return tp::fail(TP_E_BAD_ARG, "ortho: tile width must be a multiple of 4 in [8, 1024]");
    if (r && (r->on_device != 1 || r->channels != 1 || r->W != o->W))
        return tp::fail(TP_E_BAD_ARG, "ortho: residual storage must be a one-channel device storage of the same width");
    int pitch = 0;
    if (tp::ortho_smem_bytes(o->W, &pitch) > 227 * 1024)
        return tp::fail(TP_E_BAD_ARG, "ortho: tile width too large for the parent window");
    return TP_OK;
}

int check_jobs(tp_storage *o, tp_storage *r, const tp_ortho_job *jobs, int n)
{
    char buf[200];
    for (int k = 0; k < n; ++k) {
        const tp_ortho_job &j = jobs[k];
        auto bad = [&](const char *what) {
            snprintf(buf, sizeof buf, "ortho: job %d (level %d, %d, %d): %s", k, j.level, j.tx, j.ty, what);
            return tp::fail(TP_E_BAD_ARG, buf);
        };
        if (j.level < 0 || j.level > 30 || j.tx < 0 || j.ty < 0 || (j.tx >> j.level) != 0 || (j.ty >> j.level) != 0)
            return bad("bad quadtree coordinates");
        if (j.out_slot < 0 || j.out_slot >= o->capacity) return bad("bad out_slot");
        if (j.level > 0) {
            if (j.parent_slot < 0 || j.parent_slot >= o->capacity || j.parent_slot == j.out_slot)
                return tp::fail(TP_E_MISSING_PARENT, "ortho: parent tile missing or equal to the output");
        }
        if (j.residual_slot >= 0 && (!r || j.residual_slot >= r->capacity)) return bad("bad residual_slot");
        if (j.noise_rot < 0 || j.noise_rot > 3 || j.noise_layer < 0 || j.noise_layer > 5)
            return bad("bad noise rotation / layer");
        if (j.parent_job < -1 || j.parent_job >= k) return bad("parent_job must precede the job");
        if (j.parent_job >= 0) {
            const tp_ortho_job &p = jobs[j.parent_job];
            if (p.out_slot != j.parent_slot || p.level != j.level - 1 || p.tx != j.tx / 2 || p.ty != j.ty / 2)
                return bad("parent_job does not produce the parent tile");
        }
    }
    return TP_OK;
}

int ortho_batch(tp_storage *o, tp_storage *r, const tp_ortho_params *p, const tp_ortho_job *jobs,
                const tp_ortho_job *jobs_dev, int n, void *stream)
{
    if (!p || n < 0) return tp::fail(TP_E_BAD_ARG, "ortho: bad arguments");
    int rc = check_storages(o, r);
    if (rc) return rc;
    if (n == 0) return TP_OK;
    if (jobs && (rc = check_jobs(o, r, jobs, n))) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::lock_guard<std::mutex> lk(o->copy_mu);
    if (!o->ortho) o->ortho = new OrthoState;
    OrthoState &st = *o->ortho;
    if (jobs && st.jobs_cap < (size_t)n) {
        cudaStreamSynchronize(s);  // a previous batch may still read the old array
        if (st.jobs) cudaFree(st.jobs);
        st.jobs = nullptr;
        st.jobs_cap = 0;
        cudaError_t e = cudaMalloc(&st.jobs, sizeof(tp_ortho_job) * n);
        if (e != cudaSuccess) return tp::cuda_fail("cudaMalloc (ortho jobs)", e);
        st.jobs_cap = n;
    }
    if (st.flags_cap < (size_t)n + 1) {
        cudaStreamSynchronize(s);
        if (st.flags) cudaFree(st.flags);
        st.flags = nullptr;
        st.flags_cap = 0;
        cudaError_t e = cudaMalloc(&st.flags, sizeof(int) * (n + 1));
        if (e != cudaSuccess) return tp::cuda_fail("cudaMalloc (ortho flags)", e);
        st.flags_cap = n + 1;
    }
    int err = TP_OK;
    const uint32_t *noise = device_ortho_noise(o->W, o->pitch, &err);
    if (!noise) return err;
    cudaError_t e = cudaSuccess;
    if (jobs) e = cudaMemcpyAsync(st.jobs, jobs, sizeof(tp_ortho_job) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(st.flags, 0, sizeof(int) * (n + 1), s);
    if (e != cudaSuccess) return tp::cuda_fail("ortho batch set-up", e);
    tp::OrthoLaunch L{};
    L.jobs = jobs ? st.jobs : jobs_dev;
    L.njobs = n;
    L.counter = st.flags;
    L.done = st.flags + 1;
    L.tiles = reinterpret_cast<uint32_t *>(o->base);
    L.slot_stride = o->slot_stride;
    L.pitch = o->pitch;
    if (r) {
        L.res = reinterpret_cast<const uint32_t *>(r->base);
        L.res_slot_stride = r->slot_stride;
        L.res_pitch = r->pitch;
    }
    L.noise = noise;
    L.W = o->W;
    tp::ortho_smem_bytes(o->W, &L.win_pitch);
    L.p = *p;
    L.cap = tp::checked_capacity(o);
    L.res_cap = tp::checked_capacity(r);
    rc = tp::status_device_ptr(&L.status);
    if (rc) return rc;
    return tp::launch_ortho(L, stream);
}

int read_ortho_tile(const tp_ortho_dat *d, int level, int tx, int ty, std::vector<uint8_t> &raw, int *width)
{
    if (level < 0 || level > d->max_level || tx < 0 || ty < 0 || (tx >> level) != 0 || (ty >> level) != 0)
        return tp::fail(TP_E_BAD_ARG, "ortho dat: tile outside the pyramid");
    if (d->flags & 1) return tp::fail(TP_E_BAD_ARG, "ortho dat: DXT-compressed tiles are not decoded");
    const int id = tx + ty * (1 << level) + ((1 << (2 * level)) - 1) / 3;
    if (id < 0 || id >= d->ntiles) return tp::fail(TP_E_BAD_ARG, "ortho dat: tile id outside the pyramid");
    int64_t a, b;
    std::memcpy(&a, d->bytes.data() + 28 + 16 * (size_t)id, 8);
    std::memcpy(&b, d->bytes.data() + 36 + 16 * (size_t)id, 8);
    if (a < 0 || b < a || d->header + (size_t)b > d->bytes.size())
        return tp::fail(TP_E_IO, "ortho dat: tile offsets outside the file");
    const int w = d->tile_size + 2 * d->border;
    const size_t need = (size_t)w * w * d->channels;
    if (!tp::decode_tiff_strip(d->bytes.data() + d->header + a, (size_t)(b - a), raw, need + 64))
        return tp::fail(TP_E_IO, "ortho dat: corrupt or truncated tile strip");
    if (raw.size() < need) return tp::fail(TP_E_IO, "ortho dat: short tile strip");
    raw.resize(need);
    *width = w;
    return TP_OK;
}

}  // namespace

void tp::ortho_release(tp_storage *s)
{
    if (!s || !s->ortho) return;
    if (s->ortho->jobs) cudaFree(s->ortho->jobs);
    if (s->ortho->flags) cudaFree(s->ortho->flags);
    delete s->ortho;
    s->ortho = nullptr;
}

extern "C" int tp_ortho_noise(int tile_width, uint8_t *out)
{
    if (!out || !valid_width(tile_width)) return tp::fail(TP_E_BAD_ARG, "tp_ortho_noise: bad arguments");
    build_ortho_noise(tile_width, out);
    return TP_OK;
}

extern "C" int tp_ortho_batch(tp_storage *ortho, tp_storage *residuals, const tp_ortho_params *params,
                              const tp_ortho_job *jobs, int n, void *stream)
{
    if (n > 0 && !jobs) return tp::fail(TP_E_BAD_ARG, "tp_ortho_batch: jobs is NULL");
    return ortho_batch(ortho, residuals, params, jobs, nullptr, n, stream);
}

extern "C" int tp_ortho_batch_device(tp_storage *ortho, tp_storage *residuals, const tp_ortho_params *params,
                                     const tp_ortho_job *jobs_dev, int n, void *stream)
{
    if (n > 0 && !jobs_dev) return tp::fail(TP_E_BAD_ARG, "tp_ortho_batch_device: jobs_dev is NULL");
    return ortho_batch(ortho, residuals, params, nullptr, jobs_dev, n, stream);
}

extern "C" int tp_ortho_dat_open(const char *path, tp_ortho_dat **out)
{
    if (!path || !out) return tp::fail(TP_E_BAD_ARG, "tp_ortho_dat_open: bad arguments");
    *out = nullptr;
    FILE *f = std::fopen(path, "rb");
    if (!f) return tp::fail(TP_E_IO, std::string("cannot open ortho file '") + path + "'");
    auto *d = new tp_ortho_dat;
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
        return tp::fail(TP_E_IO, "ortho file truncated (header)");
    }
    int32_t h[7];
    std::memcpy(h, d->bytes.data(), 28);
    d->max_level = h[0];
    d->tile_size = h[1];
    d->channels = h[2];
    d->root = h[3];
    d->root_tx = h[4];
    d->root_ty = h[5];
    d->flags = h[6];
    d->border = (d->flags & 2) ? 0 : 2;
    if (d->max_level < 0 || d->max_level > 14 || d->tile_size < 1 || d->tile_size > 4096 || d->channels < 1 ||
        d->channels > 4) {
        delete d;
        return tp::fail(TP_E_IO, "ortho file header is corrupt");
    }
    d->ntiles = (int)(((1ll << (d->max_level * 2 + 2)) - 1) / 3);
    d->header = 28 + 16 * (size_t)d->ntiles;
    if (d->bytes.size() < d->header) {
        delete d;
        return tp::fail(TP_E_IO, "ortho file truncated (offsets)");
    }
    *out = d;
    return TP_OK;
}

extern "C" int tp_ortho_dat_close(tp_ortho_dat *d)
{
    delete d;
    return TP_OK;
}

extern "C" int tp_ortho_dat_info(const tp_ortho_dat *d, int *info8)
{
    if (!d || !info8) return tp::fail(TP_E_BAD_ARG, "tp_ortho_dat_info: bad arguments");
    const int v[8] = {d->max_level, d->tile_size, d->channels, d->root, d->root_tx, d->root_ty, d->flags, d->ntiles};
    std::memcpy(info8, v, sizeof v);
    return TP_OK;
}

extern "C" int tp_ortho_dat_read_tile(const tp_ortho_dat *d, int level, int tx, int ty, uint8_t *out, int capacity,
                                      int *width)
{
    if (!d || !out || !width) return tp::fail(TP_E_BAD_ARG, "tp_ortho_dat_read_tile: bad arguments");
    std::vector<uint8_t> raw;
    int w = 0;
    int rc = read_ortho_tile(d, level, tx, ty, raw, &w);
    if (rc) return rc;
    if (raw.size() > (size_t)capacity) return tp::fail(TP_E_BAD_ARG, "tp_ortho_dat_read_tile: output too small");
    std::memcpy(out, raw.data(), raw.size());
    *width = w;
    return TP_OK;
}

extern "C" int tp_ortho_dat_read_rgba(const tp_ortho_dat *d, int level, int tx, int ty, uint32_t *out, int capacity,
                                      int *width)
{
    if (!d || !out || !width) return tp::fail(TP_E_BAD_ARG, "tp_ortho_dat_read_rgba: bad arguments");
    std::vector<uint8_t> raw;
    int w = 0;
    int rc = read_ortho_tile(d, level, tx, ty, raw, &w);
    if (rc) return rc;
    if ((size_t)w * w > (size_t)capacity) return tp::fail(TP_E_BAD_ARG, "tp_ortho_dat_read_rgba: output too small");
    const int c = d->channels;
    for (size_t k = 0; k < (size_t)w * w; ++k) {
        uint8_t v[4] = {0, 0, 0, 255};
        for (int ch = 0; ch < c; ++ch) v[ch] = raw[k * c + ch];
        out[k] = (uint32_t)v[0] | ((uint32_t)v[1] << 8) | ((uint32_t)v[2] << 16) | ((uint32_t)v[3] << 24);
    }
    *width = w;
    return TP_OK;
}
