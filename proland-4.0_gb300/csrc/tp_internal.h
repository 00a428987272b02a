// Internal declarations shared by the host C++ and the CUDA translation units.
#pragma once

#include <cuda.h>
#include <cuda_fp16.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <utility>
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
    // TMA descriptors over this pool, by box (width, height)
    std::map<std::pair<int, int>, CUtensorMap> maps;
};

namespace tp {

// Device noise table for tile width W: the six DEM noise layers (fp16, as the
// reference's R16F texture), pre-rotated for the four rotations, laid out
// [rotation][layer][row][pitch] with pitch = W rounded up to 8.
const __half *device_noise_table(int W, int *err);

// Host noise table (the product's own restatement of createDemNoise): 6 * W * W floats.
void build_dem_noise(int W, float *out);

// TMA descriptor of a float pool seen as a 3D tensor (x: W samples, y: W rows,
// z: slot * channels + channel), cached on the storage.
int tensor_map(tp_storage *s, int box_x, int box_y, const CUtensorMap **out);

struct ElevLaunch {
    const tp_tile_job *jobs;  // device
    const int *order;         // device, or nullptr for identity
    int first, count;         // units (job slot * bands + band)
    int bands;                // row bands per tile
    float *elev;
    int W, pitch;
    long long plane_stride, slot_stride;
    const float *res;
    float *nrm;
    int nrm_pitch;
    long long nrm_plane_stride, nrm_slot_stride;
    const __half *noise;
    int g, flip, no_clamp, noise_mode;
    // shared-memory layout of a unit
    int buf_floats;           // (band rows + 2) * pitch, rounded to 128 bytes
    int par_pitch, par_rows;  // parent zf window
    int par_floats;
    int ck;                   // coarse-mesh lattice side
    uint32_t res_box_bytes, par_box_bytes;
    int smem_bytes;
    const CUtensorMap *parent_map, *res_map;
};

int launch_elevation(const ElevLaunch &a, void *stream);
int read_status(int *status, bool clear);

}  // namespace tp
