// Internal declarations shared by the host C++ and the CUDA translation units.
#pragma once

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/proland_gb300.h"

namespace tp {

// Records `msg` as the calling thread's last error and returns `code`.
int fail(int code, const std::string &msg);
int cuda_fail(const char *what, int err);

// Rounds up to a multiple of m.
inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

}  // namespace tp

// A pool of equally sized tile slots (device or pinned host memory).
struct tp_storage {
    int W = 0;            // tile width
    int channels = 0;     // planes per slot
    int capacity = 0;
    int pitch = 0;        // floats per row (W rounded up to 8: rows start on 32-byte sectors)
    long long plane_stride = 0;  // W * pitch floats
    long long slot_stride = 0;   // channels * plane_stride floats
    bool on_device = true;
    float *base = nullptr;
    std::vector<int> free_list;  // stack of free slot indices
    std::vector<uint8_t> in_use;
    std::mutex mu;
    // device scratch for job arrays of batches produced into this storage
    void *job_buf = nullptr;
    size_t job_buf_bytes = 0;
    void *order_buf = nullptr;
    size_t order_buf_bytes = 0;
};

namespace tp {

// Device noise table (6 layers of W x W fp16-rounded floats) for tile width W,
// created on first use and kept for the life of the process.
const float *device_noise_table(int W, int *err);

// Host noise table (the product's own restatement of createDemNoise).
void build_dem_noise(int W, float *out);

struct ElevLaunch {
    const tp_tile_job *jobs;  // device
    const int *order;         // device, or nullptr for identity
    int first, count;
    float *elev;
    int W, pitch;
    long long plane_stride, slot_stride;
    const float *res;
    int res_pitch;
    long long res_slot_stride;
    float *nrm;
    int nrm_pitch;
    long long nrm_plane_stride, nrm_slot_stride;
    const float *noise;
    int g, flip, no_clamp, noise_mode;
    int wlo, ww, wh;  // parent window: origin offset (<= 0), smem row pitch, rows
};

int launch_elevation(const ElevLaunch &a, void *stream);

}  // namespace tp
