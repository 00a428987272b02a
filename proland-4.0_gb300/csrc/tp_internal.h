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

// Linear congruential generator of Proland's math/noise.h:50-68: the next seed is
// (seed * 1103515245 + 12345) mod 2^31 (the reference's `long` arithmetic masked
// to 31 bits gives this on 32- and 64-bit longs alike).
struct Lcg {
    uint32_t state;
    explicit Lcg(uint32_t seed) : state(seed) {}
    uint32_t next()
    {
        state = (uint32_t)(((uint64_t)state * 1103515245ull + 12345ull) & 0x7FFFFFFFull);
        return state;
    }
    // uniform in [0, 1) with 24 bits: the top 24 of the 31-bit state
    float unit() { return (float)(next() >> 7) / 16777216.0f; }
    float signed_unit() { return unit() * 2.0f - 1.0f; }
};

}  // namespace tp

// A pool of equally sized tile slots (device or pinned host memory).
struct tp_storage {
    int W = 0;            // tile width
    int channels = 0;     // planes per slot
    int capacity = 0;
    int pitch = 0;        // floats per row (W rounded up to 8: rows start on 32-byte sectors)
    long long plane_stride = 0;  // W * pitch floats
    long long slot_stride = 0;   // channels * plane_stride floats
    int on_device = 1;            // 1 device memory, 0 pinned host memory, 2 none (bookkeeping only)
    float *base = nullptr;
    float *alloc = nullptr;      // the allocation: base, preceded (debug builds) by a guard region
    int check_cap = 0;           // debug builds: the capacity the device-side checks use (0: capacity)
    std::vector<int> free_list;  // stack of free slot indices
    std::vector<uint8_t> in_use;
    std::mutex mu;
    // frame reused by the batch calls that produce into this storage
    struct tp_frame *batch_frame = nullptr;
    // TMA descriptors over this pool, by box (width, height)
    std::map<std::pair<int, int>, CUtensorMap> maps;
    // device staging buffer of host <-> slot copies
    void *staging = nullptr;
    size_t staging_bytes = 0;
    std::mutex copy_mu;
    // launch state of the ortho batches that write into this storage
    struct OrthoState *ortho = nullptr;
};

// A residual pyramid file held in memory (header fields and all its bytes).
struct tp_dat {
    int min_level = 0, max_level = -1, tile_size = 0, root_level = 0, root_tx = 0, root_ty = 0;
    float scale = 1.0f;
    int ntiles = 0;
    std::vector<uint8_t> bytes;  // whole file
    size_t header = 0;
    uint8_t *dev_bytes = nullptr;  // device copy, made on the first device decode
    std::mutex dev_mu;
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
// The same descriptor written into `out` (no cache).
int encode_tensor_map(const tp_storage *s, int box_x, int box_y, CUtensorMap *out);
// Validates a host job array against the storages as a one-class frame does.
int check_batch_jobs(tp_storage *elev, tp_storage *res, tp_storage *nrm, const tp_tile_job *jobs, int n);

constexpr int kFrameThreads = 256;

// One tile width of a frame, as the persistent kernel sees it.
struct ClassLaunch {
    const tp_tile_job *jobs;  // device
    int njobs;
    int bands;                // row bands per tile
    int band_rows;            // rows of every band but the last, which takes the rest
    int *done;                // per-job count of completed bands (device)
    float *elev;
    int W, pitch;
    long long plane_stride, slot_stride;
    float *nrm;
    int nrm_pitch;
    long long nrm_plane_stride, nrm_slot_stride;
    const __half *noise;
    int g, gshift, flip, no_clamp, noise_mode;
    int elev_cap, res_cap, nrm_cap;  // slots the device-side checks of debug builds accept
    // shared-memory layout of a unit within a stage
    int buf_floats;           // (band rows + 2) * pitch, rounded to 128 bytes
    int par_pitch, par_rows;  // parent zf window
    int par_floats;
    int ck;                   // coarse-mesh lattice side
    uint32_t res_box_bytes, par_box_bytes;
};

// One persistent launch: the jobs of one tile width.
struct FrameLaunch {
    ClassLaunch c;
    int *counter;             // next unit to take (device)
    int stage_floats;         // shared-memory stage of one unit
    int any_deps;             // some job waits on a parent produced in this launch
    int minb;                 // kernel variant: CTAs per SM the register budget targets (2 or 3)
    int stages;               // 1: one stage per CTA; 2: double-buffered (next unit's copies in flight)
};

int launch_frame(const FrameLaunch &f, const CUtensorMap *pmap, const CUtensorMap *rmap, int grid, void *stream);
// Validates one tile width's storages and parameters and fills its launch layout
// (band rows, shared-memory windows, coarse-mesh lattice); `noise`, `jobs`, `done`
// and the tensor maps are left to the caller.  `band_rows` receives the tallest
// band (the residual box is band_rows + 2 rows of the elevation pitch).  Error
// messages start with `who`.
int class_layout(tp_storage *elev, tp_storage *res, tp_storage *nrm, const tp_elev_params *p, const char *who,
                 ClassLaunch *out, int *band_rows);
int frame_occupancy(int stage_floats, int stages, int minb, bool mod, int *blocks_per_sm);

// Copies `count` slots' plane `channel` between a dense host array and the slots
// through the storage's staging buffer (one linear copy + a repack kernel).
int staged_copy(tp_storage *s, int first, int count, int channel, float *host, bool up, void *stream);
int read_status(int *status, bool clear);
// The device address of the status word (kernels of other files report through it).
int status_device_ptr(int **out);
// The capacity a storage's device-side checks use (debug builds).
// A layer mesh's fragment program, pass state and fill depth (tp_layer_mesh), checked
// by tp_elevation_layers and tp_layer_builder_set_pass: TP_OK or TP_E_BAD_ARG.
int check_layer_pass(int program, int state, float fill_depth, const char *who);
inline int checked_capacity(const tp_storage *s) { return s ? (s->check_cap > 0 ? s->check_cap : s->capacity) : 0; }
// One plane copy of repack_planes: `count` tiles of `rows` rows of `width` floats.
struct PlaneXfer {
    const float *src;
    float *dst;
    long long src_tile, dst_tile;  // floats between tiles
    int src_pitch, dst_pitch;      // floats between rows
    int rows, width, count;
    int clamp0;                    // 1: dst = max(src, 0)
};
constexpr int kMaxPlaneXfers = 8;
struct PlaneXfers {
    PlaneXfer p[kMaxPlaneXfers];
    int n;
};
// A growable device buffer per (current device, id) for calls that stage host arrays on
// the device; callers serialise their own uses (and synchronise their stream before
// the buffer is handed out again).  Grows by a free and a new allocation after a
// synchronisation of `stream`.
enum ScratchId { kScratchNormals = 0, kScratchNormalFormats = 1, kScratchLayers = 2, kScratchSynth = 3, kScratchPairs = 4 };
int device_scratch(int id, size_t bytes, void *stream, char **out);
// Synthetic residual tiles (generator in tp_synth.h): into residual slots on the
// device, or one tile into host memory (row pitch `pitch` floats); same bits.
int synthetic_residuals_device(tp_storage *s, uint32_t seed, const int *slots, const int *levels, const int *txs,
                               const int *tys, const float *sigmas, int n, void *stream);
void synthetic_residual_host(uint32_t seed, int level, int tx, int ty, float sigma, int W, float *out, int pitch);
// Multiprocessors of the current device (cached per device).
int device_sm_count();
// Runs the x.n plane copies in one launch on `stream`.
int launch_repack_planes(const PlaneXfers &x, void *stream);

// Uploads `count` dense host tiles into the given (not necessarily consecutive) slots.
int staged_copy_slots(tp_storage *s, const int *slots, int count, int channel, const float *host, void *stream);
// Spherical-deformation frame of one tile (NormalProducer.cpp:215-273), computed in
// FP64 on the host and cast to float: patch corners relative to their mean (C,
// row-major 4x4 with a row of ones), corner verticals (N), corner distances (L),
// world-to-tangent rotation (W2T, row-major 3x3), radius and tile size.
struct SphereFrame {
    float C[16];
    float N[16];
    float L[4];
    float W2T[9];
    float R;
    float size;
};
void sphere_frame(double root_quad_size, int level, int tx, int ty, SphereFrame *f);

// Normal tiles from produced elevation tiles (flat, or spherical with one frame per tile).
int launch_normals(tp_storage *elev, tp_storage *nrm, const int *eslots, const int *nslots, const float *meters,
                   int count, void *stream, const SphereFrame *frames = nullptr);
// Normal tiles in format 0-3 (4 channels for 0/1), coarse normals from parent normal
// slots (pslots, -1 for none), spherical frames and parent-to-tangent rotations (9
// floats per job, row-major) when given.  No job may be another's parent.
int launch_normals_format(tp_storage *elev, tp_storage *nrm, const int *eslots, const int *nslots, const float *meters,
                          const int *pslots, const int *txs, const int *tys, int count, int format, int grid_mesh,
                          void *stream, const SphereFrame *frames, const float *p2t);
void parent_to_tangent(double root_quad_size, int level, int tx, int ty, float *p2t);
// Residual pyramid files.
int dat_tile_width(const tp_dat *d, int level);
int dat_tile_id(const tp_dat *d, int level, int tx, int ty);
int dat_tile_int16(const tp_dat *d, int level, int tx, int ty, std::vector<int16_t> &out, int *width);
int dat_device_bytes(tp_dat *d, const uint8_t **out);
// Strip 0 of a TIFF held in memory, decoded (deflate or none) into raw bytes, at
// most `limit` of them; false for a corrupt or unsupported strip.
bool decode_tiff_strip(const uint8_t *t, size_t n, std::vector<uint8_t> &raw, size_t limit);

// One persistent ortho launch (tp_ortho.cu): tiles are RGBA8 texels packed in
// 32-bit words; the noise table is [rotation][layer][row][pitch] words.
struct OrthoLaunch {
    const tp_ortho_job *jobs;  // device
    int njobs;
    int *counter;              // next job to take
    int *done;                 // per-job completion (device)
    uint32_t *tiles;
    long long slot_stride;     // words
    int pitch;                 // words per row
    const uint32_t *res;
    long long res_slot_stride;
    int res_pitch;
    const uint32_t *noise;
    int W, win_pitch;
    tp_ortho_params p;
    int *status;               // the device status word
    int cap, res_cap;          // slots the device-side checks of debug builds accept
};
int ortho_smem_bytes(int W, int *win_pitch);
int launch_ortho(const OrthoLaunch &L, void *stream);
void ortho_release(tp_storage *s);

}  // namespace tp
