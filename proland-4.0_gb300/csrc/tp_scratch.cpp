// Per-device state of the host side: growable device buffers for calls that stage
// their host arrays (job lists, meshes) on the device before a launch -- one buffer
// per (device, purpose), so that a process that switches devices never hands one
// device's memory to another's kernels -- and the devices' SM counts.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <utility>

#include "tp_internal.h"

namespace tp {

int device_scratch(int id, size_t bytes, void *stream, char **out)
{
    static std::mutex mu;
    static std::map<std::pair<int, int>, std::pair<char *, size_t>> bufs;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail("cudaGetDevice (scratch)", e);
    std::lock_guard<std::mutex> lk(mu);
    auto &b = bufs[std::make_pair(dev, id)];
    if (b.second < bytes) {
        if (b.first) {
            // the previous user's launch may still read it
            cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
            cudaFree(b.first);
        }
        b = std::make_pair(nullptr, (size_t)0);
        char *p = nullptr;
        e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) return cuda_fail("cudaMalloc (scratch)", e);
        b = std::make_pair(p, bytes);
    }
    *out = b.first;
    return TP_OK;
}

int device_sm_count()
{
    static std::mutex mu;
    static std::map<int, int> counts;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    int &n = counts[dev];
    if (n <= 0) {
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

}  // namespace tp
