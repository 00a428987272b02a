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
// widest tile the frame kernel supports).  The array also holds the noise table
// of every tile width used so far on the device, each written once, by the first
// call with that width, and never rewritten; widths 101, 197 and 253 together
// fill the space for tables.  Larger requests, and a width whose table no longer
// fits, are rejected with TP_E_BAD_ARG before anything is enqueued.
//
// Set-up: the first call on a device resolves the array's device address with
// cudaGetSymbolAddress while that device is current (this also loads the
// module onto the device), and the first call for a tile width writes that
// width's noise table into the array.  Those set-up calls should come before
// any stream capture.
//
// Job records: the call copies them into a file-scope host array (pageable
// memory, under a mutex) and from there to the device array, so the copy has
// left the caller's buffer when the call returns: the caller may refill or free
// its job array at once, pinned or not.
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
constexpr int kMaxTables = 8;

// bytes of one width's pre-rotated fp16 noise table, rounded to 256
constexpr size_t noise_table_bytes(int W)
{
    return (sizeof(__half) * 4 * 6 * (size_t)W * ((W + 7) / 8 * 8) + 255) / 256 * 256;
}

// byte layout of the array: [counter, padded to 256 | completion counts | jobs | noise tables]
constexpr size_t kDoneOffset = 256;
constexpr size_t kJobsOffset = kDoneOffset + sizeof(int) * kMaxJobs;
constexpr size_t kNoiseOffset = kJobsOffset + sizeof(tp_tile_job) * kMaxJobs;
constexpr size_t kNoiseBytes = noise_table_bytes(101) + noise_table_bytes(197) + noise_table_bytes(253);
constexpr size_t kScratchBytes = kNoiseOffset + kNoiseBytes;  // 5,783,296 bytes
static_assert(kJobsOffset % 256 == 0 && kNoiseOffset % 256 == 0, "scratch regions stay 256-byte aligned");
static_assert(kScratchBytes <= (6u << 20), "the static scratch stays below 6 MiB");

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceScratch {
    unsigned char *base = nullptr;  // device address of g_noalloc_scratch on this device
    int ntables = 0;                // noise tables written so far, in order of first use
    int table_width[kMaxTables] = {};
    size_t table_offset[kMaxTables] = {};
    size_t noise_used = 0;          // bytes of the noise region taken
};

std::mutex g_mu;
DeviceScratch g_devices[kMaxDevices];
// host images written under g_mu: a noise table during set-up, the job records of a call
float g_host_base[6 * kMaxWidth * kMaxWidth];
__half g_host_rot[4 * 6 * kMaxWidth * kMaxNoisePitch];
tp_tile_job g_host_jobs[kMaxJobs];

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

// Per-device set-up (address of the array; noise table of width W, written once),
// with the device current.  Called under g_mu.  `noise` receives the table.
int setup(int W, cudaStream_t s, DeviceScratch **out, const __half **noise)
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
    for (int t = 0; t < d.ntables; ++t)
        if (d.table_width[t] == W) {
            *out = &d;
            *noise = reinterpret_cast<const __half *>(d.base + kNoiseOffset + d.table_offset[t]);
            return TP_OK;
        }
    const size_t bytes = noise_table_bytes(W);
    if (d.ntables == kMaxTables || d.noise_used + bytes > kNoiseBytes) {
        char buf[200];
        snprintf(buf, sizeof buf,
                 "tp_elevation_batch_noalloc: no room left in the static scratch for the noise table of width %d "
                 "(%zu of %zu bytes taken by %d earlier widths)", W, d.noise_used, kNoiseBytes, d.ntables);
        return tp::fail(TP_E_BAD_ARG, buf);
    }
    tp::build_dem_noise(W, g_host_base);
    rotate_noise(W, g_host_base, g_host_rot);
    const size_t off = d.noise_used;
    e = cudaMemcpyAsync(d.base + kNoiseOffset + off, g_host_rot, sizeof(__half) * 4 * 6 * (size_t)W * tp::round_up(W, 8),
                        cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return tp::cuda_fail("tp_elevation_batch_noalloc: noise table copy", e);
    e = cudaStreamSynchronize(s);  // the host image is rewritten by the next set-up
    if (e != cudaSuccess) return tp::cuda_fail("tp_elevation_batch_noalloc: noise table copy", e);
    d.table_width[d.ntables] = W;
    d.table_offset[d.ntables] = off;
    ++d.ntables;
    d.noise_used += bytes;
    *out = &d;
    *noise = reinterpret_cast<const __half *>(d.base + kNoiseOffset + off);
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
    tp::FrameLaunch F;
    std::memset(&F, 0, sizeof F);
    int br = 0;
    rc = tp::class_layout(elev, residuals, normals, params, "tp_elevation_batch_noalloc", &F.c, &br);
    if (rc) return rc;
    CUtensorMap pmap, rmap;
    rc = tp::encode_tensor_map(elev, F.c.par_pitch, F.c.par_rows, &pmap);
    if (rc) return rc;
    if (residuals) {
        rc = tp::encode_tensor_map(residuals, elev->pitch, br + 2, &rmap);
        if (rc) return rc;
    } else {
        rmap = pmap;  // never read: jobs without a residual storage have no residual slot
    }
    F.stage_floats = F.c.buf_floats + F.c.par_floats + tp::round_up(F.c.ck * F.c.ck, 32);
    F.stages = params->stages == 2 ? 2 : 1;
    const size_t per_cta = sizeof(float) * (size_t)F.stage_floats * F.stages + 128 + 1024;
    F.minb = 3 * per_cta <= 227 * 1024 ? 3 : 2;
    int per_sm = 0;
    rc = tp::frame_occupancy(F.stage_floats, F.stages, F.minb, F.c.noise_mode == 1, &per_sm);
    if (rc) return rc;
    if (per_sm < 1) return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_noalloc: the kernel's stage does not fit in shared memory");
    F.any_deps = 0;
    for (int i = 0; i < n; ++i)
        if (jobs[i].parent_job >= 0) F.any_deps = 1;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::lock_guard<std::mutex> lk(g_mu);
    DeviceScratch *d = nullptr;
    rc = setup(elev->W, s, &d, &F.c.noise);
    if (rc) return rc;
    // through pageable host memory: the copy has taken the records when it returns
    std::memcpy(g_host_jobs, jobs, sizeof(tp_tile_job) * n);
    tp_tile_job *jobs_dev = reinterpret_cast<tp_tile_job *>(d->base + kJobsOffset);
    cudaError_t e = cudaMemcpyAsync(jobs_dev, g_host_jobs, sizeof(tp_tile_job) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return tp::cuda_fail("tp_elevation_batch_noalloc: job copy", e);
    // the counter and the completion counts start at zero
    e = cudaMemsetAsync(d->base, 0, kDoneOffset + sizeof(int) * n, s);
    if (e != cudaSuccess) return tp::cuda_fail("tp_elevation_batch_noalloc: clearing the counters", e);
    F.c.jobs = jobs_dev;
    F.c.njobs = n;
    F.c.done = reinterpret_cast<int *>(d->base + kDoneOffset);
    F.counter = reinterpret_cast<int *>(d->base);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = std::min(n * F.c.bands, per_sm * std::max(sms, 1));
    return tp::launch_frame(F, &pmap, &rmap, grid, stream);
}
