// Error reporting, tile storage (slot pools) and the kernel-level batch entry.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>

#include "tp_internal.h"

namespace {
thread_local std::string g_last_error;
}

namespace tp {

int fail(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

int cuda_fail(const char *what, int err)
{
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(static_cast<cudaError_t>(err)));
    return fail(TP_E_CUDA, buf);
}

}  // namespace tp

extern "C" const char *tp_last_error(void) { return g_last_error.c_str(); }
extern "C" int tp_version(void) { return 1; }

extern "C" int tp_device_available(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n > 0 ? 1 : 0;
}

// ---------------------------------------------------------------- storage
extern "C" int tp_storage_create(int tile_width, int channels, int capacity, int on_device, tp_storage **out)
{
    if (!out) return tp::fail(TP_E_BAD_ARG, "tp_storage_create: out is NULL");
    *out = nullptr;
    if (tile_width < 5 || tile_width > 4096 || channels < 1 || channels > 8 || capacity < 1)
        return tp::fail(TP_E_BAD_ARG, "tp_storage_create: bad tile_width / channels / capacity");
    if (on_device && !tp_device_available()) return tp::fail(TP_E_NO_DEVICE, "no CUDA device");
    auto *s = new tp_storage;
    s->W = tile_width;
    s->channels = channels;
    s->capacity = capacity;
    s->pitch = tp::round_up(tile_width, 8);
    s->plane_stride = (long long)tile_width * s->pitch;
    s->slot_stride = s->plane_stride * channels;
    s->on_device = on_device != 0;
    size_t bytes = sizeof(float) * (size_t)s->slot_stride * capacity;
    cudaError_t e = s->on_device ? cudaMalloc(&s->base, bytes) : cudaMallocHost(&s->base, bytes);
    if (e != cudaSuccess) {
        delete s;
        return tp::cuda_fail("tp_storage_create: allocation", e);
    }
    e = s->on_device ? cudaMemset(s->base, 0, bytes) : (std::memset(s->base, 0, bytes), cudaSuccess);
    if (e != cudaSuccess) {
        cudaFree(s->base);
        delete s;
        return tp::cuda_fail("tp_storage_create: memset", e);
    }
    s->in_use.assign(capacity, 0);
    s->free_list.reserve(capacity);
    for (int k = capacity - 1; k >= 0; --k) s->free_list.push_back(k);
    *out = s;
    return TP_OK;
}

extern "C" int tp_storage_destroy(tp_storage *s)
{
    if (!s) return TP_OK;
    if (s->base) {
        if (s->on_device) cudaFree(s->base);
        else cudaFreeHost(s->base);
    }
    if (s->job_buf) cudaFree(s->job_buf);
    if (s->order_buf) cudaFree(s->order_buf);
    delete s;
    return TP_OK;
}

extern "C" int tp_storage_tile_size(const tp_storage *s) { return s ? s->W : TP_E_BAD_ARG; }
extern "C" int tp_storage_capacity(const tp_storage *s) { return s ? s->capacity : TP_E_BAD_ARG; }
extern "C" int tp_storage_channels(const tp_storage *s) { return s ? s->channels : TP_E_BAD_ARG; }
extern "C" int tp_storage_pitch(const tp_storage *s) { return s ? s->pitch : TP_E_BAD_ARG; }

extern "C" int tp_storage_free_slots(const tp_storage *s)
{
    if (!s) return TP_E_BAD_ARG;
    auto *m = const_cast<tp_storage *>(s);
    std::lock_guard<std::mutex> lk(m->mu);
    return (int)m->free_list.size();
}

extern "C" int tp_storage_new_slot(tp_storage *s)
{
    if (!s) return TP_E_BAD_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->free_list.empty()) return -1;
    int k = s->free_list.back();
    s->free_list.pop_back();
    s->in_use[k] = 1;
    return k;
}

extern "C" int tp_storage_delete_slot(tp_storage *s, int slot)
{
    if (!s || slot < 0 || slot >= s->capacity) return tp::fail(TP_E_BAD_ARG, "tp_storage_delete_slot: bad slot");
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->in_use[slot]) return tp::fail(TP_E_BAD_ARG, "tp_storage_delete_slot: slot is free");
    s->in_use[slot] = 0;
    s->free_list.push_back(slot);
    return TP_OK;
}

extern "C" float *tp_storage_plane(tp_storage *s, int slot, int channel)
{
    if (!s || slot < 0 || slot >= s->capacity || channel < 0 || channel >= s->channels) return nullptr;
    return s->base + (long long)slot * s->slot_stride + (long long)channel * s->plane_stride;
}

static int storage_copy(tp_storage *s, int first, int count, int channel, float *host, bool up, void *stream)
{
    if (!s || !host || first < 0 || count < 1 || first + count > s->capacity || channel < 0 || channel >= s->channels)
        return tp::fail(TP_E_BAD_ARG, "tp_storage copy: bad range");
    if (count == 0) return TP_OK;
    float *dev = s->base + (long long)first * s->slot_stride + (long long)channel * s->plane_stride;
    cudaMemcpy3DParms p;
    std::memset(&p, 0, sizeof p);
    cudaPitchedPtr hp = make_cudaPitchedPtr(host, sizeof(float) * s->W, s->W, s->W);
    cudaPitchedPtr dp = make_cudaPitchedPtr(dev, sizeof(float) * s->pitch, s->W, (size_t)s->W * s->channels);
    if (up) {
        p.srcPtr = hp;
        p.dstPtr = dp;
    } else {
        p.srcPtr = dp;
        p.dstPtr = hp;
    }
    p.extent = make_cudaExtent(sizeof(float) * s->W, s->W, count);
    p.kind = cudaMemcpyDefault;
    cudaError_t e = cudaMemcpy3DAsync(&p, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return tp::cuda_fail("cudaMemcpy3DAsync", e);
    return TP_OK;
}

extern "C" int tp_storage_upload(tp_storage *s, int first_slot, int count, int channel, const float *host, void *stream)
{
    return storage_copy(s, first_slot, count, channel, const_cast<float *>(host), true, stream);
}

extern "C" int tp_storage_download(tp_storage *s, int first_slot, int count, int channel, float *host, void *stream)
{
    return storage_copy(s, first_slot, count, channel, host, false, stream);
}

// ---------------------------------------------------------------- batch
static int ensure_buffer(void **buf, size_t *have, size_t need)
{
    if (*have >= need) return TP_OK;
    if (*buf) cudaFree(*buf);
    *buf = nullptr;
    *have = 0;
    size_t sz = std::max(need, (size_t)4096);
    cudaError_t e = cudaMalloc(buf, sz);
    if (e != cudaSuccess) return tp::cuda_fail("cudaMalloc (job buffer)", e);
    *have = sz;
    return TP_OK;
}

static int check_params(tp_storage *elev, tp_storage *res, tp_storage *nrm, const tp_elev_params *p,
                        tp::ElevLaunch *L)
{
    if (!elev || !p) return tp::fail(TP_E_BAD_ARG, "batch: elevation storage and params are required");
    if (!elev->on_device || elev->channels != 3)
        return tp::fail(TP_E_BAD_ARG, "batch: elevation storage must be a device storage with 3 channels");
    const int W = elev->W, n = W - 5;
    if (n < 8 || n % 8 != 0) return tp::fail(TP_E_BAD_ARG, "batch: tile width must be 8k + 5");
    if (W > 253) return tp::fail(TP_E_BAD_ARG, "batch: tile width above 253 is not supported");
    if (p->grid_size < 1 || n % p->grid_size != 0)
        return tp::fail(TP_E_BAD_ARG, "batch: grid_size must divide the tile size");
    if (p->noise_mode != 0 && p->noise_mode != 1) return tp::fail(TP_E_BAD_ARG, "batch: bad noise_mode");
    if (res) {
        if (!res->on_device || res->channels != 1) return tp::fail(TP_E_BAD_ARG, "batch: residual storage must be 1-channel device storage");
        if ((res->W - 5) % n != 0) return tp::fail(TP_E_BAD_ARG, "batch: residual tile size must be a multiple of the tile size");
    }
    if (nrm) {
        if (!nrm->on_device || nrm->channels != 2 || nrm->W != W - 4)
            return tp::fail(TP_E_BAD_ARG, "batch: normal storage must be 2-channel device storage of width W - 4");
        if (p->normal_format != 2) return tp::fail(TP_E_BAD_ARG, "batch: only normal format 2 (signed fp32) is supported");
    }
    const int g = n / p->grid_size;
    std::memset(L, 0, sizeof *L);
    L->elev = elev->base;
    L->W = W;
    L->pitch = elev->pitch;
    L->plane_stride = elev->plane_stride;
    L->slot_stride = elev->slot_stride;
    if (res) L->res = res->base;
    if (nrm) {
        L->nrm = nrm->base;
        L->nrm_pitch = nrm->pitch;
        L->nrm_plane_stride = nrm->plane_stride;
        L->nrm_slot_stride = nrm->slot_stride;
    }
    int err = TP_OK;
    L->noise = tp::device_noise_table(W, &err);
    if (!L->noise) return err;
    L->g = g;
    L->flip = p->flip ? 1 : 0;
    L->no_clamp = p->no_clamp ? 1 : 0;
    L->noise_mode = p->noise_mode;
    // band height: whole 101-wide tiles, quarters of 197-wide ones, unless asked
    int br = p->band_rows > 0 ? p->band_rows : (W <= 128 ? W : (W + 3) / 4);
    br = std::min(std::max(br, 8), W);
    L->bands = (W + br - 1) / br;
    br = (W + L->bands - 1) / L->bands;          // the tallest band actually launched
    if (br + 2 > 256) return tp::fail(TP_E_BAD_ARG, "batch: band taller than a TMA box");
    const int PE = elev->pitch;
    L->buf_floats = tp::round_up((br + 2) * PE, 32);
    // parent zf window: columns [d, d + n/2 + 5] (stencil and modulated-noise taps),
    // rows from the first computed row's parent row, (br + 1)/2 + 5 of them
    L->par_pitch = tp::round_up(n / 2 + 6, 4);
    L->par_rows = (br + 1) / 2 + 5;
    if (L->par_pitch > 256 || L->par_rows > 256) return tp::fail(TP_E_BAD_ARG, "batch: parent window above a TMA box");
    L->par_floats = tp::round_up(L->par_pitch * L->par_rows, 32);
    const int kmax = (n + 2 + g) / (2 * g);     // largest coarse-mesh index of a sample
    L->ck = kmax + 2;
    L->res_box_bytes = (uint32_t)(sizeof(float) * PE * (br + 2));
    L->par_box_bytes = (uint32_t)(sizeof(float) * L->par_pitch * L->par_rows);
    L->smem_bytes = (int)(sizeof(float) * ((size_t)L->buf_floats + L->par_floats + tp::round_up(L->ck * L->ck, 32)));
    if (L->smem_bytes > 200 * 1024) return tp::fail(TP_E_BAD_ARG, "batch: band too tall for shared memory");
    int rc = tp::tensor_map(elev, L->par_pitch, L->par_rows, &L->parent_map);
    if (rc) return rc;
    if (res) {
        rc = tp::tensor_map(res, PE, br + 2, &L->res_map);
        if (rc) return rc;
    } else {
        L->res_map = L->parent_map;  // never dereferenced by the kernel without residuals
    }
    return TP_OK;
}

static int check_job(const tp_storage *elev, const tp_storage *res, const tp_storage *nrm, const tp_tile_job &j,
                     int index, int n)
{
    const int W = elev->W, ts = W - 5;
    char buf[160];
    auto bad = [&](const char *what) {
        snprintf(buf, sizeof buf, "batch: job %d (level %d, %d, %d): %s", index, j.level, j.tx, j.ty, what);
        return tp::fail(TP_E_BAD_ARG, buf);
    };
    if (j.level < 0 || j.level > 30 || j.tx < 0 || j.ty < 0 || (j.tx >> j.level) != 0 || (j.ty >> j.level) != 0)
        return bad("bad quadtree coordinates");
    if (j.out_slot < 0 || j.out_slot >= elev->capacity) return bad("bad out_slot");
    if (j.level > 0) {
        if (j.parent_slot < 0 || j.parent_slot >= elev->capacity) {
            snprintf(buf, sizeof buf, "batch: job %d (level %d, %d, %d): parent tile missing", index, j.level, j.tx, j.ty);
            return tp::fail(TP_E_MISSING_PARENT, buf);
        }
        if (j.parent_slot == j.out_slot) return bad("parent_slot == out_slot");
    }
    if (j.parent_job >= index || j.parent_job < -1 || j.parent_job >= n) return bad("parent_job must precede the job");
    if (j.residual_slot >= 0) {
        if (!res || j.residual_slot >= res->capacity) return bad("bad residual_slot");
        if (j.rx < 0 || j.ry < 0 || j.rx % ts != 0 || j.ry % ts != 0 || j.rx + W > res->W || j.ry + W > res->W)
            return bad("residual window outside the residual tile");
    }
    if (j.normal_slot >= 0 && (!nrm || j.normal_slot >= nrm->capacity)) return bad("bad normal_slot");
    if (j.noise_layer < 0 || j.noise_layer > 5 || j.noise_rot < 0 || j.noise_rot > 3) return bad("bad noise layer / rotation");
    if (!(j.tile_meters > 0.0f)) return bad("tile_meters must be positive");
    return TP_OK;
}

extern "C" int tp_elevation_batch(tp_storage *elev, tp_storage *res, tp_storage *nrm, const tp_elev_params *params,
                                  const tp_tile_job *jobs, int n, void *stream)
{
    tp::ElevLaunch L;
    int rc = check_params(elev, res, nrm, params, &L);
    if (rc) return rc;
    if (n < 0 || (n > 0 && !jobs)) return tp::fail(TP_E_BAD_ARG, "batch: bad job array");
    if (n == 0) return TP_OK;
    std::vector<int> depth(n, 0);
    int max_depth = 0;
    for (int k = 0; k < n; ++k) {
        rc = check_job(elev, res, nrm, jobs[k], k, n);
        if (rc) return rc;
        if (jobs[k].parent_job >= 0) {
            const tp_tile_job &pj = jobs[jobs[k].parent_job];
            if (pj.out_slot != jobs[k].parent_slot || pj.level != jobs[k].level - 1 || pj.tx != jobs[k].tx / 2 ||
                pj.ty != jobs[k].ty / 2)
                return tp::fail(TP_E_BAD_ARG, "batch: parent_job does not produce the parent tile");
            depth[k] = depth[jobs[k].parent_job] + 1;
            max_depth = std::max(max_depth, depth[k]);
        }
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::lock_guard<std::mutex> lk(elev->mu);
    rc = ensure_buffer(&elev->job_buf, &elev->job_buf_bytes, sizeof(tp_tile_job) * n);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(elev->job_buf, jobs, sizeof(tp_tile_job) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return tp::cuda_fail("cudaMemcpyAsync (jobs)", e);
    L.jobs = static_cast<const tp_tile_job *>(elev->job_buf);
    if (max_depth == 0) {
        L.order = nullptr;
        L.first = 0;
        L.count = n * L.bands;
        return tp::launch_elevation(L, stream);
    }
    // dependency waves: all jobs of depth d run in one launch, after depth d - 1
    std::vector<int> order(n), start(max_depth + 2, 0);
    for (int k = 0; k < n; ++k) start[depth[k] + 1]++;
    for (int d = 0; d <= max_depth; ++d) start[d + 1] += start[d];
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int k = 0; k < n; ++k) order[fill[depth[k]]++] = k;
    rc = ensure_buffer(&elev->order_buf, &elev->order_buf_bytes, sizeof(int) * n);
    if (rc) return rc;
    e = cudaMemcpyAsync(elev->order_buf, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return tp::cuda_fail("cudaMemcpyAsync (order)", e);
    // the host vector must outlive the asynchronous copy from pageable memory:
    // cudaMemcpyAsync from pageable memory has staged it before returning
    L.order = static_cast<const int *>(elev->order_buf);
    for (int d = 0; d <= max_depth; ++d) {
        L.first = start[d] * L.bands;
        L.count = (start[d + 1] - start[d]) * L.bands;
        rc = tp::launch_elevation(L, stream);
        if (rc) return rc;
    }
    return TP_OK;
}

extern "C" int tp_elevation_batch_device(tp_storage *elev, tp_storage *res, tp_storage *nrm,
                                         const tp_elev_params *params, const tp_tile_job *jobs_dev, int n,
                                         void *stream)
{
    tp::ElevLaunch L;
    int rc = check_params(elev, res, nrm, params, &L);
    if (rc) return rc;
    if (n < 0 || (n > 0 && !jobs_dev)) return tp::fail(TP_E_BAD_ARG, "batch: bad job array");
    L.jobs = jobs_dev;
    L.order = nullptr;
    L.first = 0;
    L.count = n * L.bands;
    return tp::launch_elevation(L, stream);
}

extern "C" int tp_status(int *status, int clear)
{
    if (!status) return tp::fail(TP_E_BAD_ARG, "tp_status: status is NULL");
    return tp::read_status(status, clear != 0);
}

extern "C" int tp_stream_check(void *stream)
{
    cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return tp::cuda_fail("cudaStreamSynchronize", e);
    int st = 0;
    int rc = tp::read_status(&st, true);
    if (rc) return rc;
    if (st == TP_E_TIMEOUT) return tp::fail(TP_E_TIMEOUT, "a device-side wait gave up (status word set)");
    if (st != 0) return tp::fail(st, "device status word set");
    return TP_OK;
}
