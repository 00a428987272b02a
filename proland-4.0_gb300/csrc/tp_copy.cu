// Host <-> slot copies.  A host tile array is dense ([count][W][W], rows of W
// floats) while slots have a padded pitch; a strided DMA of 400-byte rows runs
// far below the host link's rate, so one linear copy moves the whole array into
// a device staging buffer and a kernel (re)packs rows between the staging buffer
// and the slot planes at HBM speed.
#include <cuda_runtime.h>

#include <algorithm>

#include "tp_internal.h"

namespace {

// One warp per row: dense row (count * W rows in all) <-> slot plane row.
// slot_map (device, optional): slot of each dense tile; consecutive slots otherwise.
__global__ void __launch_bounds__(256) repack_rows(const float *__restrict__ src, float *__restrict__ dst, int W,
                                                   int pitch, long long slot_stride, long long rows, bool to_slots,
                                                   const int *__restrict__ slot_map)
{
    const long long row = (long long)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (row >= rows) return;
    const int lane = threadIdx.x & 31;
    const long long tile = row / W;
    const int r = (int)(row - tile * W);
    const long long dense = row * W;
    const long long slot = (slot_map ? (long long)slot_map[tile] : tile) * slot_stride + (long long)r * pitch;
    if (to_slots) {
        for (int i = lane; i < W; i += 32) dst[slot + i] = __ldg(src + dense + i);
    } else {
        for (int i = lane; i < W; i += 32) dst[dense + i] = __ldg(src + slot + i);
    }
}

// Several plane copies in one launch (blockIdx.y picks the copy), one warp per
// row; rows of a copy are [count][rows] with independent tile and row strides on
// each side, so dense arrays and pitched slot planes can be either end.
__global__ void __launch_bounds__(256) repack_planes(tp::PlaneXfers x)
{
    const tp::PlaneXfer &p = x.p[blockIdx.y];
    const long long row = (long long)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (row >= (long long)p.count * p.rows) return;
    const int lane = threadIdx.x & 31;
    const long long tile = row / p.rows;
    const int r = (int)(row - tile * p.rows);
    const float *src = p.src + tile * p.src_tile + (long long)r * p.src_pitch;
    float *dst = p.dst + tile * p.dst_tile + (long long)r * p.dst_pitch;
    if (p.clamp0) {
        for (int i = lane; i < p.width; i += 32) dst[i] = fmaxf(__ldg(src + i), 0.0f);
    } else {
        for (int i = lane; i < p.width; i += 32) dst[i] = __ldg(src + i);
    }
}

int ensure_staging(tp_storage *s, size_t bytes)
{
    if (s->staging_bytes >= bytes) return TP_OK;
    if (s->staging) cudaFree(s->staging);
    s->staging = nullptr;
    s->staging_bytes = 0;
    cudaError_t e = cudaMalloc(&s->staging, bytes);
    if (e != cudaSuccess) return tp::cuda_fail("cudaMalloc (staging)", e);
    s->staging_bytes = bytes;
    return TP_OK;
}

}  // namespace

namespace tp {

int staged_copy(tp_storage *s, int first, int count, int channel, float *host, bool up, void *stream)
{
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t bytes = sizeof(float) * (size_t)count * s->W * s->W;
    std::lock_guard<std::mutex> lk(s->copy_mu);
    int rc = ensure_staging(s, bytes);
    if (rc) return rc;
    float *plane = s->base + (long long)first * s->slot_stride + (long long)channel * s->plane_stride;
    const long long rows = (long long)count * s->W;
    const unsigned blocks = (unsigned)((rows + 7) / 8);
    cudaError_t e;
    if (up) {
        e = cudaMemcpyAsync(s->staging, host, bytes, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return cuda_fail("cudaMemcpyAsync (upload)", e);
        repack_rows<<<blocks, 256, 0, st>>>(static_cast<const float *>(s->staging), plane, s->W, s->pitch,
                                            s->slot_stride, rows, true, nullptr);
    } else {
        repack_rows<<<blocks, 256, 0, st>>>(plane, static_cast<float *>(s->staging), s->W, s->pitch, s->slot_stride,
                                            rows, false, nullptr);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("repack kernel launch", e);
    if (!up) {
        e = cudaMemcpyAsync(host, s->staging, bytes, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return cuda_fail("cudaMemcpyAsync (download)", e);
    }
    return TP_OK;
}

int staged_copy_slots(tp_storage *s, const int *slots, int count, int channel, const float *host, void *stream)
{
    if (count <= 0) return TP_OK;
    for (int k = 0; k < count; ++k)
        if (slots[k] < 0 || slots[k] >= s->capacity) return fail(TP_E_BAD_ARG, "upload: slot out of range");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t bytes = sizeof(float) * (size_t)count * s->W * s->W;
    std::lock_guard<std::mutex> lk(s->copy_mu);
    int rc = ensure_staging(s, bytes + sizeof(int) * (size_t)count + 256);
    if (rc) return rc;
    int *dmap = reinterpret_cast<int *>(static_cast<char *>(s->staging) + ((bytes + 255) & ~(size_t)255));
    cudaError_t e = cudaMemcpyAsync(s->staging, host, bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dmap, slots, sizeof(int) * count, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail("cudaMemcpyAsync (slot upload)", e);
    float *plane = s->base + (long long)channel * s->plane_stride;
    const long long rows = (long long)count * s->W;
    repack_rows<<<(unsigned)((rows + 7) / 8), 256, 0, st>>>(static_cast<const float *>(s->staging), plane, s->W,
                                                            s->pitch, s->slot_stride, rows, true, dmap);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("repack kernel launch", e);
    return TP_OK;
}

int launch_repack_planes(const PlaneXfers &x, void *stream)
{
    if (x.n < 1 || x.n > kMaxPlaneXfers) return fail(TP_E_BAD_ARG, "repack: bad plane count");
    long long rows = 0;
    for (int i = 0; i < x.n; ++i) rows = std::max(rows, (long long)x.p[i].count * x.p[i].rows);
    if (rows == 0) return TP_OK;
    const dim3 grid((unsigned)((rows + 7) / 8), (unsigned)x.n);
    repack_planes<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(x);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("repack kernel launch", e);
    return TP_OK;
}

}  // namespace tp
