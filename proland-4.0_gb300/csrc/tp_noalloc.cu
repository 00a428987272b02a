// tp_elevation_batch_noalloc: a batch of elevation (+ normal) tiles produced
// without allocating any memory.  It runs the same persistent frame kernel as
// tp_elevation_batch; what differs is where the kernel's scratch lives.  The
// allocating path keeps a work counter, per-job completion counts and the job
// records in device buffers it allocates (and grows) on first use, and the
// fp16 noise table of each tile width in a buffer allocated once per width.
// Here all four live in one fixed array of device memory defined below.
//
// Who needs it: a caller that may not allocate while it produces tiles -- a
// renderer that hands all device memory to its own pools before the first
// frame and so has none left for a library's lazily grown buffers, or a frame
// loop that cannot take the implicit device-wide synchronisation of a free or
// an out-of-memory failure halfway through a frame.  Everything the call
// touches is the caller's (tile storages, job array, stream) or that array.
//
// Limits: at most kMaxJobs jobs per call and tile widths up to kMaxWidth (the
// widest tile the frame kernel supports).  Larger requests are rejected with
// TP_E_BAD_ARG before anything is enqueued.
//
// Set-up: the first call on a device resolves the array's device address with
// cudaGetSymbolAddress while that device is current (this also loads the
// module onto the device), and the first call for a tile width writes that
// width's noise table into the array (a call with another width writes its
// own, replacing it).  Those set-up calls should come before any stream
// capture.
//
// Sharing: every call on a device uses the same array.  The counter and the
// completion counts must start at zero and are cleared on the call's stream
// before each launch; the job records are rewritten by each call.  Calls issued
// one after another on one stream are ordered by the stream; calls that overlap
// on the device (other streams, other host threads) race on the array, and the
// caller must serialise them.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "tp_internal.h"

namespace {

constexpr int kMaxJobs = 4096;
constexpr int kMaxWidth = 253;
constexpr int kMaxNoisePitch = (kMaxWidth + 7) / 8 * 8;
constexpr int kMaxDevices = 64;

// byte layout of the array: [counter, padded to 256 | completion counts | jobs | noise]
constexpr size_t kDoneOffset = 256;
constexpr size_t kJobsOffset = kDoneOffset + sizeof(int) * kMaxJobs;
constexpr size_t kNoiseOffset = kJobsOffset + sizeof(tp_tile_job) * kMaxJobs;
constexpr size_t kNoiseBytes = sizeof(__half) * 4 * 6 * (size_t)kMaxWidth * kMaxNoisePitch;
constexpr size_t kScratchBytes = kNoiseOffset + kNoiseBytes;  // 3,387,648 bytes
static_assert(kJobsOffset % 256 == 0 && kNoiseOffset % 256 == 0, "scratch regions stay 256-byte aligned");
static_assert(kScratchBytes <= (4u << 20), "the static scratch stays below 4 MiB");

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceScratch {
    unsigned char *base = nullptr;  // device address of g_noalloc_scratch on this device
    int noise_width = 0;            // tile width whose noise table the array holds
};

std::mutex g_mu;
DeviceScratch g_devices[kMaxDevices];
// host images of a noise table, written under g_mu during set-up only
float g_host_base[6 * kMaxWidth * kMaxWidth];
__half g_host_rot[4 * 6 * kMaxWidth * kMaxNoisePitch];

// The pre-rotated fp16 layout the frame kernel reads ([rotation][layer][row][pitch],
// pitch = W rounded up to 8; entry (r, l, j, i) is the texel sample (i, j) reads
// under rotation r), the layout of the tables tp::device_noise_table caches.
void rotate_noise(int W, const float *base, __half *rot)
{
    const int P = tp::round_up(W, 8);
    std::memset(rot, 0, sizeof(__half) * 4 * 6 * (size_t)W * P);
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
                    rot[(((size_t)r * 6 + l) * W + j) * P + i] = __float2half_rn(base[(size_t)l * W * W + x + (size_t)y * W]);
                }
}

// Per-device set-up (address of the array; noise table of width W), with the
// device current.  Called under g_mu.
int setup(int W, cudaStream_t s, DeviceScratch **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return tp::cuda_fail("tp_elevation_batch_noalloc: cudaGetDevice", e);
    if (dev < 0 || dev >= kMaxDevices) return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: device ordinal above 63");
    DeviceScratch &d = g_devices[dev];
    if (!d.base) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return tp::cuda_fail("tp_elevation_batch_noalloc: cudaGetSymbolAddress", e);
        d.base = static_cast<unsigned char *>(p);
    }
    if (d.noise_width != W) {
        tp::build_dem_noise(W, g_host_base);
        rotate_noise(W, g_host_base, g_host_rot);
        // ordered on the caller's stream after earlier calls that read the old table
        e = cudaMemcpyAsync(d.base + kNoiseOffset, g_host_rot, sizeof(__half) * 4 * 6 * (size_t)W * tp::round_up(W, 8),
                            cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return tp::cuda_fail("tp_elevation_batch_noalloc: noise table copy", e);
        e = cudaStreamSynchronize(s);  // the host image is rewritten by the next set-up
        if (e != cudaSuccess) return tp::cuda_fail("tp_elevation_batch_noalloc: noise table copy", e);
        d.noise_width = W;
    }
    *out = &d;
    return TP_OK;
}

// The launch layout of one tile width, by the rules the frame's class set-up
// applies (band height, shared-memory windows, coarse-mesh lattice), with the
// noise table taken from the array and tensor maps encoded on the caller's stack.
int layout(tp_storage *elev, tp_storage *res, tp_storage *nrm, const tp_elev_params *p, const __half *noise,
           tp::ClassLaunch *out, CUtensorMap *pmap, CUtensorMap *rmap)
{
    if (!elev || !p) return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: elevation storage and params are required");
    if (elev->on_device != 1 || elev->channels != 3)
        return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: elevation storage must be a device storage with 3 channels");
    const int W = elev->W, n = W - 5;
    if (n < 8 || n % 8 != 0) return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: tile width must be 8k + 5");
    if (W > kMaxWidth) return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: tile width above 253");
    if (p->grid_size < 1 || n % p->grid_size != 0)
        return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: grid_size must divide the tile size");
    if (p->noise_mode != 0 && p->noise_mode != 1) return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: bad noise_mode");
    if (res && (res->on_device != 1 || res->channels != 1 || (res->W - 5) % n != 0))
        return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: residual storage must be 1-channel device storage "
                                      "whose tile size is a multiple of the tile size");
    if (nrm && (nrm->on_device != 1 || nrm->channels != 2 || nrm->W != W - 4 || p->normal_format != 2))
        return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: normal storage must be 2-channel device storage "
                                      "of width W - 4, normal format 2");
    tp::ClassLaunch L;
    std::memset(&L, 0, sizeof L);
    L.elev = elev->base;
    L.W = W;
    L.pitch = elev->pitch;
    L.plane_stride = elev->plane_stride;
    L.slot_stride = elev->slot_stride;
    if (nrm) {
        L.nrm = nrm->base;
        L.nrm_pitch = nrm->pitch;
        L.nrm_plane_stride = nrm->plane_stride;
        L.nrm_slot_stride = nrm->slot_stride;
    }
    L.noise = noise;
    const int g = n / p->grid_size;
    L.g = g;
    L.gshift = -1;
    if ((g & (g - 1)) == 0) {
        int sh = 0;
        while ((1 << sh) < 2 * g) ++sh;
        L.gshift = sh;
    }
    L.flip = p->flip ? 1 : 0;
    L.no_clamp = p->no_clamp ? 1 : 0;
    L.noise_mode = p->noise_mode;
    int br = p->band_rows > 0 ? p->band_rows : (W <= 128 ? W : (W + 3) / 4);
    br = std::min(std::max(br, 8), W);
    L.bands = (W + br - 1) / br;
    br = (W + L.bands - 1) / L.bands;
    if (br + 2 > 256) return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: band taller than a TMA box");
    const int PE = elev->pitch;
    L.buf_floats = tp::round_up((br + 2) * PE, 32);
    L.par_pitch = tp::round_up(n / 2 + 6, 4);
    L.par_rows = (br + 1) / 2 + 5;
    L.par_floats = tp::round_up(L.par_pitch * L.par_rows, 32);
    L.ck = (n + 2 + g) / (2 * g) + 2;
    L.res_box_bytes = (uint32_t)(sizeof(float) * PE * (br + 2));
    L.par_box_bytes = (uint32_t)(sizeof(float) * L.par_pitch * L.par_rows);
    int rc = tp::encode_tensor_map(elev, L.par_pitch, L.par_rows, pmap);
    if (rc) return rc;
    if (res) {
        rc = tp::encode_tensor_map(res, PE, br + 2, rmap);
        if (rc) return rc;
    } else {
        *rmap = *pmap;  // never read: jobs without a residual storage have no residual slot
    }
    *out = L;
    return TP_OK;
}

}  // namespace

extern "C" int tp_elevation_batch_noalloc(tp_storage *elev, tp_storage *residuals, tp_storage *normals,
                                          const tp_elev_params *params, const tp_tile_job *jobs, int n,
                                          void *stream)
{
    if (!params || n < 0 || (n > 0 && !jobs))
        return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: bad params or job array");
    if (n > kMaxJobs) {
        char buf[160];
        snprintf(buf, sizeof buf, "tp_elevation_batch_noalloc: %d jobs exceed the static scratch's limit of %d per call",
                 n, kMaxJobs);
        return tp::fail(TP_E_BAD_ARG, buf);
    }
    if (!elev) return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: elevation storage is required");
    if (elev->W > kMaxWidth) return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: tile width above 253");
    int rc = tp::check_batch_jobs(elev, residuals, normals, jobs, n);
    if (rc) return rc;
    if (n == 0) return TP_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceScratch *d = nullptr;
    rc = setup(elev->W, s, &d);
    if (rc) return rc;
    tp::FrameLaunch F;
    std::memset(&F, 0, sizeof F);
    CUtensorMap pmap, rmap;
    rc = layout(elev, residuals, normals, params, reinterpret_cast<const __half *>(d->base + kNoiseOffset), &F.c, &pmap,
                &rmap);
    if (rc) return rc;
    tp_tile_job *jobs_dev = reinterpret_cast<tp_tile_job *>(d->base + kJobsOffset);
    cudaError_t e = cudaMemcpyAsync(jobs_dev, jobs, sizeof(tp_tile_job) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return tp::cuda_fail("tp_elevation_batch_noalloc: job copy", e);
    // the counter and the completion counts start at zero
    e = cudaMemsetAsync(d->base, 0, kDoneOffset + sizeof(int) * n, s);
    if (e != cudaSuccess) return tp::cuda_fail("tp_elevation_batch_noalloc: clearing the counters", e);
    F.c.jobs = jobs_dev;
    F.c.njobs = n;
    F.c.done = reinterpret_cast<int *>(d->base + kDoneOffset);
    F.counter = reinterpret_cast<int *>(d->base);
    F.stage_floats = F.c.buf_floats + F.c.par_floats + tp::round_up(F.c.ck * F.c.ck, 32);
    F.any_deps = 0;
    for (int i = 0; i < n; ++i)
        if (jobs[i].parent_job >= 0) F.any_deps = 1;
    F.stages = params->stages == 2 ? 2 : 1;
    const size_t per_cta = sizeof(float) * (size_t)F.stage_floats * F.stages + 128 + 1024;
    F.minb = 3 * per_cta <= 227 * 1024 ? 3 : 2;
    int per_sm = 0;
    rc = tp::frame_occupancy(F.stage_floats, F.stages, F.minb, F.c.noise_mode == 1, &per_sm);
    if (rc) return rc;
    if (per_sm < 1) return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: the kernel's stage does not fit in shared memory");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = std::min(n * F.c.bands, per_sm * std::max(sms, 1));
    return tp::launch_frame(F, &pmap, &rmap, grid, stream);
}
