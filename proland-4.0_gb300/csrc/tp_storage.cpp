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
namespace {
// Debug builds put a guard region of a fixed byte before and after every storage's
// slots; release builds none.
#ifdef TP_DEBUG
constexpr size_t kGuardBytes = 65536;
#else
constexpr size_t kGuardBytes = 0;
#endif
constexpr int kGuardByte = 0xA5;
}  // namespace

extern "C" int tp_build_is_debug(void)
{
#ifdef TP_DEBUG
    return 1;
#else
    return 0;
#endif
}

extern "C" int tp_storage_check_guards(const tp_storage *s)
{
    if (!s) return tp::fail(TP_E_BAD_ARG, "tp_storage_check_guards: storage is NULL");
    if (!kGuardBytes || !s->alloc) return TP_OK;
    const size_t bytes = sizeof(float) * (size_t)s->slot_stride * s->capacity;
    std::string g(2 * kGuardBytes, '\0');
    cudaError_t e = cudaMemcpy(&g[0], s->alloc, kGuardBytes, cudaMemcpyDefault);
    if (e == cudaSuccess)
        e = cudaMemcpy(&g[kGuardBytes], reinterpret_cast<const char *>(s->base) + bytes, kGuardBytes, cudaMemcpyDefault);
    if (e != cudaSuccess) return tp::cuda_fail("tp_storage_check_guards", e);
    for (size_t i = 0; i < g.size(); ++i)
        if ((unsigned char)g[i] != kGuardByte) {
            char buf[160];
            snprintf(buf, sizeof buf, "tp_storage_check_guards: guard byte %zu %s the slots was overwritten",
                     i < kGuardBytes ? kGuardBytes - i : i - kGuardBytes + 1, i < kGuardBytes ? "before" : "after");
            return tp::fail(TP_E_BOUNDS, buf);
        }
    return TP_OK;
}

extern "C" int tp_debug_check_capacity(tp_storage *s, int capacity)
{
#ifdef TP_DEBUG
    if (!s || capacity < 0 || capacity > s->capacity) return tp::fail(TP_E_BAD_ARG, "tp_debug_check_capacity: bad arguments");
    s->check_cap = capacity;
    return TP_OK;
#else
    (void)s;
    (void)capacity;
    return tp::fail(TP_E_BAD_ARG, "tp_debug_check_capacity: debug builds only");
#endif
}
extern "C" int tp_storage_create(int tile_width, int channels, int capacity, int on_device, tp_storage **out)
{
    if (!out) return tp::fail(TP_E_BAD_ARG, "tp_storage_create: out is NULL");
    *out = nullptr;
    if (tile_width < 5 || tile_width > 4096 || channels < 1 || channels > 8 || capacity < 1 || on_device < 0 ||
        on_device > 2)
        return tp::fail(TP_E_BAD_ARG, "tp_storage_create: bad tile_width / channels / capacity / memory kind");
    if (on_device != 2 && !tp_device_available()) return tp::fail(TP_E_NO_DEVICE, "no CUDA device");
    auto *s = new tp_storage;
    s->W = tile_width;
    s->channels = channels;
    s->capacity = capacity;
    s->pitch = tp::round_up(tile_width, 8);
    s->plane_stride = (long long)tile_width * s->pitch;
    s->slot_stride = s->plane_stride * channels;
    s->on_device = on_device;
    size_t bytes = sizeof(float) * (size_t)s->slot_stride * capacity;
    if (on_device != 2) {
        const size_t total = bytes + 2 * kGuardBytes;
        void *p = nullptr;
        cudaError_t e = on_device == 1 ? cudaMalloc(&p, total) : cudaMallocHost(&p, total);
        if (e != cudaSuccess) {
            delete s;
            return tp::cuda_fail("tp_storage_create: allocation", e);
        }
        s->alloc = static_cast<float *>(p);
        s->base = s->alloc + kGuardBytes / sizeof(float);
        if (on_device == 1) {
            e = cudaMemset(s->base, 0, bytes);
            if (e == cudaSuccess && kGuardBytes) e = cudaMemset(s->alloc, kGuardByte, kGuardBytes);
            if (e == cudaSuccess && kGuardBytes)
                e = cudaMemset(reinterpret_cast<char *>(s->base) + bytes, kGuardByte, kGuardBytes);
        } else {
            std::memset(s->base, 0, bytes);
            std::memset(s->alloc, kGuardByte, kGuardBytes);
            std::memset(reinterpret_cast<char *>(s->base) + bytes, kGuardByte, kGuardBytes);
        }
        if (e != cudaSuccess) {
            if (on_device == 1) cudaFree(s->alloc);
            else cudaFreeHost(s->alloc);
            delete s;
            return tp::cuda_fail("tp_storage_create: memset", e);
        }
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
    if (s->alloc) {
        if (s->on_device == 1) cudaFree(s->alloc);
        else if (s->on_device == 0) cudaFreeHost(s->alloc);
    }
    if (s->batch_frame) tp_frame_destroy(s->batch_frame);
    if (s->staging) cudaFree(s->staging);
    tp::ortho_release(s);
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
    if (s->on_device == 2) return tp::fail(TP_E_BAD_ARG, "tp_storage copy: storage has no memory");
    if (s->on_device == 1) return tp::staged_copy(s, first, count, channel, host, up, stream);
    // host storage: plain pitched copy on the calling thread
    for (int t = 0; t < count; ++t) {
        float *plane = s->base + (long long)(first + t) * s->slot_stride + (long long)channel * s->plane_stride;
        for (int r = 0; r < s->W; ++r) {
            float *dense = host + ((size_t)t * s->W + r) * s->W;
            if (up) std::memcpy(plane + (size_t)r * s->pitch, dense, sizeof(float) * s->W);
            else std::memcpy(dense, plane + (size_t)r * s->pitch, sizeof(float) * s->W);
        }
    }
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
