/*
 * proland_gb300 -- GB300-native terrain tile production (elevation upsample +
 * residual + noise + normals) behind Proland's TileStorage / TileCache /
 * TileProducer protocol.
 *
 * C ABI only: plain pointers, ints and floats; cudaStream_t is passed as void*.
 * Every function returns TP_OK (0) or a negative TP_E_* code and never aborts;
 * tp_last_error() gives a message for the last failure on the calling thread.
 *
 * Reference interfaces each entry point replaces are cited as file:line,
 * relative to the Proland 4.0 source root (src/...).
 *
 * Tile layout.  A tile of width W (W = n + 5 for elevation/residual tiles with a
 * 2-sample border, n + 1 for normal tiles) is stored as `channels` planes of W
 * rows x `pitch` floats (pitch = W rounded up to 8), row-major, x fastest, row 0
 * the bottom (GL) row.  A slot is channels * W * pitch floats; the slots of a
 * storage are one contiguous device allocation.  Elevation slots have three
 * planes (zf, zc, zm) -- the reference's RGB32F texel split into planes;
 * normal slots (format 2) have two (nx, ny).
 */
#ifndef PROLAND_GB300_H
#define PROLAND_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TP_OK 0
#define TP_E_BAD_ARG (-1)        /* invalid argument, size or state */
#define TP_E_CACHE_FULL (-2)     /* no free and no evictable slot (TileCache.cpp:198-199) */
#define TP_E_MISSING_PARENT (-3) /* a child tile's parent is neither resident nor in the batch */
#define TP_E_TIMEOUT (-4)        /* a device-side dependency wait gave up; status word set */
#define TP_E_CUDA (-5)           /* a CUDA runtime call failed */
#define TP_E_IO (-6)             /* residual file missing, truncated or corrupt */
#define TP_E_NO_DEVICE (-7)      /* no CUDA device (the library has no CPU fallback) */
#define TP_E_BOUNDS (-8)         /* debug builds: a device-side index check failed (the access was skipped) */

const char *tp_last_error(void);
/* Library version, and whether the CUDA kernels can run here (1) or not (0). */
int tp_version(void);
int tp_device_available(void);

/* ------------------------------------------------------------------------
 * Storage: a pool of equally sized tile slots.
 * Replaces TileStorage (core/.../producer/TileStorage.h:140-182),
 * GPUTileStorage::init (core/.../producer/GPUTileStorage.cpp:151-205) and
 * CPUTileStorage<float> (core/.../producer/CPUTileStorage.h:43-151).
 * on_device = 1 allocates device memory, 0 pinned host memory, 2 no memory at
 * all (slot bookkeeping only, usable without a GPU). */
typedef struct tp_storage tp_storage;
int tp_storage_create(int tile_width, int channels, int capacity, int on_device, tp_storage **out);
int tp_storage_destroy(tp_storage *s);
/* Debug builds (libproland_gb300_debug.so, built with TP_DEBUG; see build.py): every
 * storage's slots sit between two guard regions of a fixed byte pattern, and the
 * kernels that take device job arrays check each job's slot and parent indexes
 * against the storages' capacities before using them (a bad job sets the status
 * word to TP_E_BOUNDS and is skipped).  tp_build_is_debug returns 1 in debug
 * builds; tp_storage_check_guards returns TP_OK while the guards are intact (always
 * in release builds) and TP_E_BOUNDS once a write crossed them;
 * tp_debug_check_capacity lowers the capacity the device-side checks use (debug
 * builds only; 0 restores it), so that a test can plant an out-of-range slot that
 * still lies inside the allocation. */
int tp_build_is_debug(void);
int tp_storage_check_guards(const tp_storage *s);
int tp_debug_check_capacity(tp_storage *s, int capacity);
int tp_storage_tile_size(const tp_storage *s);   /* getTileSize */
int tp_storage_capacity(const tp_storage *s);    /* getCapacity */
int tp_storage_free_slots(const tp_storage *s);  /* getFreeSlots */
int tp_storage_channels(const tp_storage *s);
int tp_storage_pitch(const tp_storage *s);       /* floats per row */
/* newSlot / deleteSlot (TileStorage.cpp:90-100): slot index or -1 when full */
int tp_storage_new_slot(tp_storage *s);
int tp_storage_delete_slot(tp_storage *s, int slot);
/* Address of plane `channel` of `slot` (device or pinned host memory). */
float *tp_storage_plane(tp_storage *s, int slot, int channel);
/* Copies `count` consecutive slots' plane `channel` from/to a dense host array
 * [count][W][W] (pitch W), asynchronously on `stream` (one linear host<->device
 * copy through a staging buffer owned by the storage, repacked on the device);
 * host memory should be pinned.  Copies of one storage must be issued on one
 * stream (they share the staging buffer).  Host storages copy synchronously. */
int tp_storage_upload(tp_storage *s, int first_slot, int count, int channel,
                      const float *host, void *stream);
int tp_storage_download(tp_storage *s, int first_slot, int count, int channel,
                        float *host, void *stream);

/* ------------------------------------------------------------------------
 * Kernel-level batch: produce elevation (+ normal) tiles whose inputs are
 * named by slot.  This is what ElevationProducer::doCreateTile
 * (terrain/.../dem/ElevationProducer.cpp:280-405) plus
 * NormalProducer::doCreateTile (terrain/.../dem/NormalProducer.cpp:164-289)
 * compute for one tile, for a whole frame of tiles in one launch. */
typedef struct {
    int32_t level, tx, ty;
    int32_t out_slot;       /* elevation slot written */
    int32_t parent_slot;    /* elevation slot of (level-1, tx/2, ty/2); -1 at level 0 */
    int32_t residual_slot;  /* residual slot, -1 when ResidualProducer::hasTile is false */
    int32_t rx, ry;         /* residual window: (tx % mod) * n, (ty % mod) * n */
    int32_t normal_slot;    /* normal slot written, -1: elevation only */
    int32_t noise_rot;      /* 0..3, from the tile's edge noise signs */
    int32_t noise_layer;    /* 0..5 */
    float noise_amp;        /* noiseAmp[level] (0 when level >= size) */
    float rscale;           /* residual value scale (residualOSH.w) */
    float tile_meters;      /* rootQuadSize / 2^level */
    int32_t parent_job;     /* index of the job in this batch writing the parent, -1 if resident */
    int32_t reserved;
} tp_tile_job;

/* Per-producer constants of a batch (one tile width). */
typedef struct {
    int32_t grid_size;      /* gridMeshSize (default 24): zc uses g = n / grid_size */
    int32_t flip;           /* flipDiagonals */
    int32_t no_clamp;       /* NO_CLAMP: zm = zf instead of max(zf, 0) */
    int32_t noise_mode;     /* 0: zf += |amp| N (terrain1 shader); 1: slope/curvature modulated (demo shader) */
    int32_t normal_format;  /* 2: two signed fp32 planes (the only one supported by the batch kernel) */
    int32_t band_rows;      /* rows per kernel work unit; 0 picks the tuned default */
    int32_t stages;         /* shared-memory stages per CTA: 1, or 2 to prefetch the next unit (0: 1) */
    int32_t reserved;
} tp_elev_params;

/* Produces n jobs on `stream` in one persistent launch (a one-class frame).
 * `jobs` is host memory; it is copied into a device buffer owned by the storage
 * `elev`.  A job whose parent is produced by an earlier job of the same batch
 * names it in parent_job: the launch orders it after its parent.
 * `residuals`/`normals` may be NULL when unused.  One batch per storage and
 * stream at a time. */
int tp_elevation_batch(tp_storage *elev, tp_storage *residuals, tp_storage *normals,
                       const tp_elev_params *params, const tp_tile_job *jobs, int n,
                       void *stream);
/* Same with the job array already in device memory (no host->device copy). */
int tp_elevation_batch_device(tp_storage *elev, tp_storage *residuals, tp_storage *normals,
                              const tp_elev_params *params, const tp_tile_job *jobs_dev, int n,
                              void *stream);
/* Normal tiles of already produced elevation tiles: job k reads elevation slot
 * jobs[k].out_slot and writes normal slot jobs[k].normal_slot (format 2), sample
 * spacing tile_meters / (W - 5).  root_quad_size > 0: the tiles lie on the sphere
 * of a cube-face planet of that root quad size (NormalProducer with deformation,
 * NormalProducer.cpp:215-273; terrain2/normalShader.glsl); 0: flat.  Returns once
 * the launch has completed (it synchronises `stream`: the job array goes through a
 * device buffer shared by all calls). */
int tp_normal_batch(tp_storage *elev, tp_storage *normals, const tp_tile_job *jobs, int n, double root_quad_size,
                    void *stream);
/* The same in any of the reference's normal formats (NormalProducer.cpp:195;
 * demo normalShader.glsl:93-124): 0 = (nf, nc) signed, 1 = (nf, nc) as 8-bit
 * unsigned (stored as k / 255), 2 = nf signed, 3 = nf as 8-bit unsigned; formats
 * 0 and 1 need 4-channel normal slots, their coarse normals nc average the parent
 * normal tile (parent_normal_slots[k], or nc = nf when NULL or -1) at the
 * coarse-mesh vertices of grid_mesh (gridMeshSize, 24 in the examples).  Jobs are
 * produced level by level, parents first; returns once they have completed. */
int tp_normal_batch_format(tp_storage *elev, tp_storage *normals, const tp_tile_job *jobs, int n,
                           double root_quad_size, int format, const int *parent_normal_slots, int grid_mesh,
                           void *stream);
/* Same as tp_elevation_batch, allocating nothing.  (No counterpart in the
 * reference: its producers draw on GL textures created up front.)  For callers
 * that may not allocate while producing tiles: the kernel's scratch (work
 * counter, completion counts, job records, fp16 noise tables) is one static
 * device array of 5,783,296 bytes, shared by all calls on a device.  At most
 * 4096 jobs per call and tile widths up to 253; the array keeps the noise table
 * of each width used so far (written once, by the first call with that width;
 * widths 101, 197 and 253 together fill the room for tables).  More is rejected
 * with TP_E_BAD_ARG.  The first call on a device, and the first call for each
 * tile width, do set-up and should come before any stream capture.  The job
 * records are taken from `jobs` before the call returns (the array may be
 * refilled or freed at once, pinned or not).  Calls issued one after another on
 * one stream are ordered; calls that overlap on the device race on the array. */
int tp_elevation_batch_noalloc(tp_storage *elev, tp_storage *residuals, tp_storage *normals,
                               const tp_elev_params *params, const tp_tile_job *jobs, int n,
                               void *stream);

/* ------------------------------------------------------------------------
 * Host-buffer batches: the tiles of a frame whose inputs and outputs live in host
 * memory, as CPUElevationProducer::doCreateTile's slots do
 * (terrain/.../dem/CPUElevationProducer.cpp:156-248: parent tile in, W x W
 * floats out), with the GPU path's zc, zm, noise and normals
 * (ElevationProducer.cpp:280-405, NormalProducer.cpp:164-289).  The pipeline
 * owns device slots for `nbuf` chunks of `chunk` tiles and three internal
 * streams; a call splits its jobs into chunks and overlaps, chunk by chunk, the
 * host->device copy of the next chunk, the persistent elevation launch of the
 * current one and the device->host copy of the previous one.  Host memory
 * should be pinned for the copies to be asynchronous. */
typedef struct tp_pipeline tp_pipeline;
int tp_pipeline_create(int tile_width, int chunk, int nbuf, tp_pipeline **out);
int tp_pipeline_destroy(tp_pipeline *p);
/* Dense host tile arrays of a call; tile k of each array belongs to job k. */
typedef struct {
    const float *parent_zf;  /* [n][W][W] parent zf planes (ignored for level-0 jobs) */
    const float *parent_zm;  /* [n][W][W] parent zm planes; NULL: derived from parent_zf
                                (max(zf, 0), or zf under no_clamp), as the parent's
                                own production wrote it */
    const float *residual;   /* [n][W][W] residual tiles; NULL when no job has one */
    float *zf, *zc, *zm;     /* [n][W][W] outputs; zc and zm may be NULL (not copied back:
                                CPUElevationProducer::doCreateTile, CPUElevationProducer.cpp:240-243,
                                fills zf only, and zm = max(zf, 0), or zf under no_clamp) */
    float *nx, *ny;          /* [n][W-4][W-4] normal outputs (format 2); NULL: none */
} tp_host_tiles;
/* Produces n independent jobs (parent_job must be -1) from host tiles into host
 * tiles.  The slot fields of the jobs are replaced by the pipeline's own; a job
 * with residual_slot < 0 adds no residual; residual windows must be (0, 0) (host
 * residual tiles are W x W).  Work is ordered after what `stream` holds at the
 * call, and `stream` waits for the last copy: synchronise `stream` before
 * reading the outputs.  Calls on one pipeline are ordered among themselves. */
int tp_elevation_batch_host(tp_pipeline *p, const tp_elev_params *params, const tp_tile_job *jobs, int n,
                            const tp_host_tiles *io, void *stream);

/* ------------------------------------------------------------------------
 * Frames: all tile requests of a frame -- for up to two tile widths (e.g. 101
 * and 197) -- produced by one persistent launch per tile width.  The CTAs take
 * work units (bands of tiles) from a device counter in list order; a job naming
 * its parent's job (parent_job, which must come earlier in the same class) waits
 * on that job's completion counter, so parents are produced before children
 * inside the launch.  This is the batched form of TileProducer's task graph
 * (core/.../producer/TileProducer.cpp:749-771, CreateTile::run :199-217).
 * tp_frame_graph_launch captures the frame (counter reset + launch) into a CUDA
 * graph on its first call and replays it afterwards; the job arrays are
 * uploaded once, before the capture.  One frame per stream at a time. */
typedef struct tp_frame tp_frame;
/* The storages named by tp_frame_add must outlive every launch of the frame (its
 * tensor maps and job arrays point into them); destroy or clear the frame first. */
int tp_frame_create(tp_frame **out);
int tp_frame_destroy(tp_frame *f);
int tp_frame_clear(tp_frame *f);
int tp_frame_add(tp_frame *f, tp_storage *elev, tp_storage *residuals, tp_storage *normals,
                 const tp_elev_params *params, const tp_tile_job *jobs, int n);
/* Same with a job array in device memory, owned by the caller (not validated);
 * has_dependencies = 0 promises that no job names a parent_job. */
int tp_frame_add_device(tp_frame *f, tp_storage *elev, tp_storage *residuals, tp_storage *normals,
                        const tp_elev_params *params, const tp_tile_job *jobs_dev, int n,
                        int has_dependencies);
int tp_frame_launch(tp_frame *f, void *stream);
int tp_frame_graph_launch(tp_frame *f, void *stream);
int tp_frame_units(const tp_frame *f);   /* work units of one launch */
/* A frame with two tile widths launches the second width's persistent kernel on a
 * stream forked from `stream` and joined back into it (in a graph: two parallel
 * kernel nodes), so that its CTAs start while the first kernel's last wave drains;
 * the widths share no data.  on = 0 launches them one after the other on `stream`.
 * Overlap is the default. */
int tp_frame_overlap_classes(tp_frame *f, int on);
/* Autotuner: times each tile width's launch under every candidate work-unit
 * shape -- band height (whole tile vs 2..6 bands), one or two shared-memory
 * stages per CTA, two or three CTAs per SM -- `repeats` times each, on the
 * frame's own inputs (its outputs are rewritten), and keeps the fastest. */
int tp_frame_autotune(tp_frame *f, void *stream, int repeats);
int tp_frame_config(const tp_frame *f, int klass, int *band_rows, int *stages, int *ctas_per_sm);

/* Device status word: TP_OK, or the first TP_E_* code a kernel reported (a
 * dependency or copy wait that gave up).  tp_status reads it (and clears it when
 * `clear`); tp_stream_check synchronises `stream`, then reads and clears it. */
int tp_status(int *status, int clear);
int tp_stream_check(void *stream);

/* ------------------------------------------------------------------------
 * Tile cache and producers: the TileCache / TileProducer protocol.
 *
 * tp_cache replaces TileCache (core/.../producer/TileCache.h:201-309,
 * TileCache.cpp:150-377): tiles keyed by (producer, level, tx, ty) with a users
 * count; tiles without users stay cached in an LRU list and their slots are
 * recycled oldest first; getTile returns NULL (TP_E_CACHE_FULL in
 * tp_last_error) when no slot is free or recyclable.
 * tp_producer replaces TileProducer (core/.../producer/TileProducer.h:147-378)
 * for the three producers of this path:
 *   residuals  ResidualProducer (terrain/.../dem/ResidualProducer.cpp:70-438):
 *              a .dat pyramid (file, delta, zscale), a host callback, or zero
 *              residuals for an empty file name;
 *   elevations ElevationProducer (ElevationProducer.cpp:178-579);
 *   normals    NormalProducer (NormalProducer.cpp:71-385), flat deformation.
 * getTile acquires the tile; a tile not produced yet is queued together with
 * the tiles it is made from (startCreateTile), which it holds until it is
 * produced.  tp_scheduler_run produces every queued tile of the producers
 * given (and of those they use) on `stream`: the batched doCreateTile of a
 * frame, parents before children, normals fused into the elevation launch.
 * The caches' storages must be used from one stream. */
typedef struct tp_cache tp_cache;
typedef struct tp_producer tp_producer;
typedef struct tp_tile tp_tile;
typedef struct tp_dat tp_dat;
/* Host residual source: fills `out` (width x width floats, row-major) with the
 * residual tile (level, tx, ty); returns 0 on success. */
typedef int (*tp_residual_source)(void *user, int level, int tx, int ty, float *out, int width);

/* A cache uses its storage, a producer its cache and the producers it reads (residuals,
 * elevations): each must outlive what uses it (destroy producers, then caches, then
 * storages). */
int tp_cache_create(tp_storage *storage, const char *name, tp_cache **out);
int tp_cache_destroy(tp_cache *c);
int tp_cache_used_tiles(tp_cache *c);     /* getUsedTiles */
int tp_cache_unused_tiles(tp_cache *c);   /* getUnusedTiles */
int tp_cache_stats(tp_cache *c, long long *queries, long long *misses);

int tp_residual_producer_create(tp_cache *cache, const char *file, int delta, float zscale, tp_producer **out);
int tp_residual_producer_set_source(tp_producer *p, tp_residual_source fn, void *user);
/* A residual producer whose tiles are synthetic: iid samples of zero mean and
 * standard deviation sigma0 * ratio^level per tile (sum of twelve uniforms, an
 * approximately normal law bounded by 6 sigma), a counter-based function of
 * (seed, level, tx, ty, sample), made on the device in the scheduler run (on the
 * host for host storages and tp_residual_tile).  The stand-in for a residual
 * pyramid that the streaming and quadtree workloads use (the reference's
 * ResidualProducer reads them from a .dat file, ResidualProducer.cpp:268-340). */
int tp_residual_producer_set_synthetic(tp_producer *p, double sigma0, double ratio, unsigned seed);
/* A residual producer over a .dat file decodes its tiles on the device (1) or on
 * the host (0, the default). */
int tp_residual_producer_set_device_decode(tp_producer *p, int on);
/* noise_amp: per-level amplitudes (ElevationProducer.cpp:488-499); face as in
 * ElevationProducer.cpp:509-515 (0 flat, 1..6 cube faces). */
int tp_elevation_producer_create(tp_cache *cache, tp_producer *residuals, const float *noise_amp, int n_noise,
                                 const tp_elev_params *params, int face, tp_producer **out);
int tp_normal_producer_create(tp_cache *cache, tp_producer *elevations, int deform, tp_producer **out);
/* A normal producer's output format (0-3 as tp_normal_batch_format; a 4-channel
 * storage starts at 0, a 2-channel one at 2) and the coarse mesh size. */
int tp_normal_producer_set_format(tp_producer *p, int format, int grid_mesh);
int tp_producer_destroy(tp_producer *p);
int tp_producer_id(const tp_producer *p);
int tp_producer_border(const tp_producer *p);                                  /* getBorder */
int tp_producer_set_root_quad_size(tp_producer *p, float size);              /* setRootQuadSize */
int tp_producer_has_tile(const tp_producer *p, int level, int tx, int ty);    /* hasTile */
tp_tile *tp_producer_get_tile(tp_producer *p, int level, int tx, int ty);    /* getTile */
tp_tile *tp_producer_find_tile(tp_producer *p, int level, int tx, int ty, int include_cache, int done); /* findTile */
int tp_producer_put_tile(tp_producer *p, tp_tile *t);                          /* putTile: users left */
int tp_producer_prefetch_tile(tp_producer *p, int level, int tx, int ty);    /* prefetchTile */
int tp_producer_invalidate_tiles(tp_producer *p);                             /* invalidateTiles */
int tp_producer_queued(const tp_producer *p);                                  /* tiles waiting for production */
/* A held tile's coordinates, slot, users and state, read without the cache's lock:
 * for inspection while no other thread acquires or releases that tile. */
int tp_tile_info(const tp_tile *t, int *level, int *tx, int *ty, int *slot, int *users, int *done);
/* Produces every queued tile of the producers and of the producers they use, on
 * `stream`: residual tiles first (host decode and one upload, or device decode),
 * then each elevation producer's queue in one persistent launch (with the flat
 * normals of the same tiles fused in; a producer with layers: one launch and one
 * layer pass per level, normals afterwards), then the remaining normals, then
 * ortho residuals and ortho tiles.  Residual uploads, layer passes and normal
 * launches synchronise `stream`; the elevation and ortho launches return at once. */
int tp_scheduler_run(tp_producer *const *producers, int n, void *stream);
/* Batched doCreateTile (TileProducer.h:331-378 in the frame form): acquires each
 * requested tile as tp_producer_get_tile does, then produces every queued tile of
 * `p` and its inputs in one scheduler run on `stream`.  tiles_out[i] holds one user
 * (release with tp_producer_put_tile).  On failure (e.g. TP_E_CACHE_FULL) no tile
 * of the call stays acquired. */
typedef struct {
    int32_t level, tx, ty;
} tp_tile_req;
int tp_create_tiles(tp_producer *p, const tp_tile_req *reqs, int n, tp_tile **tiles_out, void *stream);
int tp_create_tile(tp_producer *p, int level, int tx, int ty, tp_tile **tile_out, void *stream);
/* The TileSamplers of one terrain node (core/.../terrain/TileSampler.cpp:416-461,
 * TileSampler::getTiles walking the terrain quadtree, one sampler per producer):
 * a sampler holds one user on each of its producers' tiles (e.g. elevations and
 * normals) of every quad of the current quadtree.  tp_sampler_update takes the next
 * frame's quadtree (requests parents first, e.g. from tp_quadtree_requests): it
 * releases the tiles of quads that disappeared (putTile: they join the caches'
 * LRUs), acquires the new quads' tiles (getTile, producers in the order given) and
 * produces them in one scheduler run on `stream` (normal tiles of new elevation
 * tiles fused into the elevation launch); *new_count receives the number of new
 * quads.  Releases and acquisitions follow TileSampler::putTiles / getTiles's walk of
 * the quadtree (parents first, children in index order (tx & 1) + 2 (ty & 1)), so
 * that a full cache evicts the tiles the reference's would; the new quads are
 * reported in request order.  On failure (TP_E_CACHE_FULL) no tile of the update
 * stays acquired.
 * tp_sampler_new_tiles copies the last update's new quads (returns their count);
 * tp_sampler_find returns a held tile of producer number `producer`.  Destroying
 * the sampler releases every tile it holds. */
typedef struct tp_sampler tp_sampler;
int tp_sampler_create(tp_producer *const *producers, int n, tp_sampler **out);
int tp_sampler_destroy(tp_sampler *s);
int tp_sampler_update(tp_sampler *s, const tp_tile_req *reqs, int n, void *stream, int *new_count);
int tp_sampler_new_tiles(const tp_sampler *s, tp_tile_req *out, int capacity);
int tp_sampler_held(const tp_sampler *s);
tp_tile *tp_sampler_find(const tp_sampler *s, int producer, int level, int tx, int ty);

/* Tracing (the reference logs per-tile lines on its "DEM" topic, ElevationProducer.cpp:282-286,
 * and counts cache queries and misses; it has no timer): flags bit 0 wraps the library's
 * launches and host phases in NVTX ranges (seen by Nsight tools), bit 1 accumulates host
 * time per phase (sampler release / acquire, residuals, elevation jobs, frame set-up, frame
 * launch, finish, normals, layers, learned).  The TP_TRACE environment variable sets the
 * flags at load.  tp_trace_set returns the previous flags; tp_trace_host_times copies up to
 * n phases' seconds and call counts (optionally resetting them) and returns the number of
 * phases; tp_trace_phase_name names phase i. */
int tp_trace_set(int flags);
int tp_trace_host_times(double *seconds, long long *calls, int n, int reset);
const char *tp_trace_phase_name(int phase);
/* The tiles of a terrain quadtree for one camera position (the TileSampler's
 * requests): TerrainQuad::update's split rule (TerrainQuad.cpp:80-105) with
 * TerrainNode::getCameraDist (TerrainNode.cpp:92-97), root quad [-size/2, size/2]^2,
 * every quad visible; parents first.  *count receives the number of quads even
 * when it exceeds `capacity` (then TP_E_BAD_ARG). */
int tp_quadtree_requests(double root_size, int max_level, float split_dist, float dist_factor, double cam_x,
                         double cam_y, double cam_z, double ground, tp_tile_req *out, int capacity, int *count);
/* A residual producer's tile computed on the host (the reference keeps residual
 * tiles in CPU storage): `out` is width x width, width the cache's tile width. */
int tp_residual_tile(tp_producer *p, int level, int tx, int ty, float *out, int width);
/* Spherical-deformation frame of a tile (NormalProducer.cpp:215-273), 47 floats:
 * C[16], N[16], L[4], W2T[9], R, size (normal producers with deform = 1 use it). */
int tp_sphere_frame(double root_quad_size, int level, int tx, int ty, float *out47);

/* ------------------------------------------------------------------------
 * Elevation layers: the TileLayer draws over produced elevation tiles and the
 * blend pass that folds them into zm (ElevationProducer.cpp:383-399: layers drawn
 * into the tile's framebuffer, which holds (zf, zc, zm, w = 0) with depth 1 after
 * the upsample, then blendShader).  The blend sets zm to zf min(w, 1) + z (1 -
 * min(w, 1)) (blend_mode 0: graph1/edit3/river1 blendShader.glsl) or to the 3x3 box
 * filter of that value, clamped at the tile edge (blend_mode 1:
 * demo/shaders/elevation/blendShader.glsl).  zf and zc are not changed (the layers
 * mask them).
 *
 * Meshes are triangles whose vertices are (x, y, a, u) -- x, y in the tile's clip
 * coordinates ([-1, 1] spans the W x W texels), a and u the two interpolated
 * attributes -- drawn in order, each with a fragment program and a pass state:
 *  - TP_LAYER_ROAD, the road elevation layer (RoadElevationLayer.cpp:388-437 with
 *    graph1/roadLayerElevationShader.glsl): a = altitude, u = signed road-width
 *    coordinate, as ElevationGraphLayer::drawCurveAltitude builds them
 *    (ElevationGraphLayer.cpp:82-380).  At d = |u|: z = a + 0.03 (1 - smoothstep(0.98,
 *    1, d)), w = smoothstep(1, 2, d), depth 0.1 d + 0.3.
 *  - TP_LAYER_WATER, _WATER_RIVER, _WATER_LARGE, the water elevation layer
 *    (WaterElevationLayer.cpp:240-350 with river1/waterLayerElevationShader.glsl,
 *    uniform river = 0, 1, 2): a = st.x, u = st.y, d = |u|; z = a (river 0) or
 *    (a - 1) + max(d - 1, 0); w = smoothstep(1, 2, d); depth 0.1 d + 0.3 (river 0),
 *    0.1 d + 0.15 (river 1) or 1 (river 2).
 *  - TP_LAYER_FILL (river1/fillShader.glsl): z = a, w = u (the colour's blue and
 *    alpha: give every vertex the same two values), depth fill_depth.
 * Fragment depths are clamped to [0, 1].  The pass state (tp_layer_mesh.state) is a
 * depth test (TP_DEPTH_LESS, _ALWAYS, _NOTEQUAL against the stored depth) and write
 * masks (TP_NO_DEPTH_WRITE, TP_NO_Z_WRITE, TP_NO_W_WRITE), as the layers set them
 * with setDepthTest / setDepthMask / setColorMask; 0 is the road layer's (LESS,
 * depth, z and w written).  NOTEQUAL with depth writes is refused (TP_E_BAD_ARG).
 * clear_depth clears the depth buffer to 1 before its mesh (the layers' fb->clear of
 * depth).  Rasterisation: window coordinates snapped to 1/256 texel, a texel is
 * covered when its centre is inside the triangle (top-left rule for centres on an
 * edge, y up), attributes interpolated at the texel centre as a0 + (a1 - a0) l1 +
 * (a2 - a0) l2 from the barycentric weights l_k, fp32 depth, triangles drawn in
 * order; vertices beyond 32768 texels of the tile's origin drop their triangle. */
#define TP_TRIANGLES 0
#define TP_TRIANGLE_STRIP 1
#define TP_LAYER_ROAD 0
#define TP_LAYER_WATER 1
#define TP_LAYER_WATER_RIVER 2
#define TP_LAYER_WATER_LARGE 3
#define TP_LAYER_FILL 4
#define TP_DEPTH_LESS 0
#define TP_DEPTH_ALWAYS 1
#define TP_DEPTH_NOTEQUAL 2
#define TP_NO_DEPTH_WRITE 4
#define TP_NO_Z_WRITE 8
#define TP_NO_W_WRITE 16
typedef struct {
    int32_t first_vertex;  /* first vertex of the mesh in the call's vertex array */
    int32_t count;         /* vertices drawn (not indexed) or indices drawn (indexed) */
    int32_t first_index;   /* first index in the call's index array; -1: not indexed.
                              Indices count from first_vertex. */
    int32_t mode;          /* TP_TRIANGLES or TP_TRIANGLE_STRIP */
    int32_t clear_depth;   /* 1: the depth buffer is cleared to 1 before this mesh (a new layer) */
    int32_t program;       /* TP_LAYER_* fragment program */
    int32_t state;         /* TP_DEPTH_* test | TP_NO_* write masks */
    float fill_depth;      /* the depth TP_LAYER_FILL writes */
} tp_layer_mesh;
typedef struct {
    int32_t slot;          /* elevation slot (zf, zc, zm) whose zm the layers change */
    int32_t first_mesh;    /* the tile's meshes, drawn in order; a mesh belongs to one job */
    int32_t n_meshes;
    int32_t reserved;
} tp_layer_job;
/* Draws the meshes of n tiles (one CTA per tile) and blends them into zm.  The
 * framebuffer starts as (zf, zc, zm, w = 0) with depth 1, as after the upsample.
 * `vertices` holds n_vertices x 4 floats.  Returns once the tiles are written (it
 * synchronises `stream`: the meshes go through a device buffer shared by all calls). */
int tp_elevation_layers(tp_storage *elev, const tp_layer_job *jobs, int n, const tp_layer_mesh *meshes,
                        int n_meshes, const float *vertices, int n_vertices, const uint32_t *indices,
                        int n_indices, int blend_mode, void *stream);
/* The same with the vertex and index arrays in device memory (e.g. meshes built on
 * the device); jobs and meshes stay in host memory.  Index values are not checked on
 * the host: one past the vertex array drops its triangle. */
int tp_elevation_layers_device(tp_storage *elev, const tp_layer_job *jobs, int n, const tp_layer_mesh *meshes,
                               int n_meshes, const float *vertices_dev, int n_vertices, const uint32_t *indices_dev,
                               int n_indices, int blend_mode, void *stream);
/* Layers of an elevation producer (TileProducer::addLayer, TileProducer.h:281;
 * TileLayer::doCreateTile, TileLayer.h:199): for each tile the producer makes,
 * each layer's callback adds the meshes it draws for (level, tx, ty) to the
 * builder; the first mesh a callback adds clears the depth buffer (the road
 * layer's fb->clear of depth).  A producer with layers makes its tiles level by
 * level, each level's launch followed by its layer pass, so that children read
 * their parents' blended zm (coarse elevation zc), and computes normals after the
 * blend.  blend_mode as above (0 by default). */
typedef struct tp_layer_builder tp_layer_builder;
int tp_layer_builder_add_mesh(tp_layer_builder *b, const float *vertices, int n_vertices, const uint32_t *indices,
                              int n_indices, int mode);
/* The fragment program and pass state of the meshes a callback adds next (the
 * program choice and the setDepthTest / setDepthMask / setColorMask calls of a layer's
 * doCreateTile); each callback starts with the road layer's (TP_LAYER_ROAD, 0, 0). */
int tp_layer_builder_set_pass(tp_layer_builder *b, int program, int state, float fill_depth);
typedef int (*tp_layer_fn)(void *user, int level, int tx, int ty, tp_layer_builder *b);
int tp_elevation_producer_add_layer(tp_producer *p, tp_layer_fn fn, void *user);
int tp_elevation_producer_set_blend(tp_producer *p, int blend_mode);

/* Residual pyramid files (ResidualProducer.cpp:93-107, 253-340): header
 * {minLevel, maxLevel, tileSize, rootLevel, rootTx, rootTy, ntiles} and int16
 * tiles decoded from their deflate TIFF strips. */
int tp_dat_open(const char *path, tp_dat **out);
int tp_dat_close(tp_dat *d);
int tp_dat_info(const tp_dat *d, int *info7, float *scale);
int tp_dat_read_tile(const tp_dat *d, int level, int tx, int ty, int16_t *out, int capacity, int *width);
int tp_inflate_zlib(const uint8_t *data, size_t n, uint8_t *out, size_t capacity, size_t *written);
/* Tiles of the pyramid decoded on the device (the file's bytes are copied to the
 * device once): tile k = (levels[k], txs[k], tys[k]) in the file's pyramid, or a zero
 * tile when levels[k] < 0, written as int16 x scale into slots[k] of `residuals` (a
 * 1-channel device storage of width tileSize + 5; smaller tiles below minLevel fill
 * the slot's lower-left corner, the rest is zero).  TP_E_IO for a corrupt strip
 * (known when the call returns: it synchronises `stream`). */
int tp_dat_decode_device(tp_dat *d, const int *levels, const int *txs, const int *tys, int n, float scale,
                         tp_storage *residuals, const int *slots, void *stream);

/* ------------------------------------------------------------------------
 * Noise helpers (host).  createDemNoise (ElevationProducer.cpp:50-133) and the
 * per-tile layer choice (ElevationProducer.cpp:345-376). */
int tp_dem_noise(int tile_width, float *out /* 6 * W * W, fp16-rounded */);
float tp_cnoise(float x, float y);               /* noise.cpp:118-165, period 0 */
int tp_noise_select(int face, int level, int tx, int ty, int *rot, int *layer);

/* ------------------------------------------------------------------------
 * Ortho (colour) tiles: OrthoProducer::doCreateTile
 * (terrain/.../ortho/OrthoProducer.cpp:292-382) with the upsample shader
 * (terrain/examples/terrain3/upsampleOrthoShader.glsl): 2x upsample of the
 * parent with the (1,3,3,9)/16 masks floored to integers, the residual
 * ((r - 128) * scale) or, at level 0, the root colour, then the rotated RGBA8
 * noise layer added in RGB or HSV, written as 8-bit channels.  Tiles are W x W
 * texels, W = tileSize + 4 with W a multiple of 4 (e.g. 196); an ortho storage is
 * a one-channel storage (tp_storage_create(W, 1, ...)) whose 32-bit texels hold
 * RGBA8, red in the low byte, so tp_storage_upload/download move them as they
 * are.  Residual storages hold the same texels (OrthoCPUProducer tiles of fewer
 * channels are read as GL does: missing green / blue 0, alpha 255). */
typedef struct {
    int32_t level, tx, ty;
    int32_t out_slot;       /* ortho slot written */
    int32_t parent_slot;    /* ortho slot of (level-1, tx/2, ty/2); -1 at level 0 */
    int32_t residual_slot;  /* residual slot, -1 when the residual producer has no tile */
    int32_t noise_rot;      /* 0..3 and 0..5: the tile's edge noise signs (tp_noise_select) */
    int32_t noise_layer;
    float noise_amp;        /* noiseAmp[level] (rs; 0 beyond the list) */
    int32_t parent_job;     /* index of the job in this batch writing the parent, -1 if resident */
    int32_t reserved[2];
} tp_ortho_job;

typedef struct {
    float root_color[4];    /* rnoise / 255 (default 0.5) */
    float noise_color[4];   /* cnoise / 255 (default 1) */
    float scale;            /* residual scale (default 2) */
    int32_t hsv;            /* noise added in HSV space */
    int32_t reserved[2];
} tp_ortho_params;

/* createOrthoNoise (OrthoProducer.cpp:26-122): 6 layers of W x W RGBA8 bytes. */
int tp_ortho_noise(int tile_width, uint8_t *out /* 6 * W * W * 4 */);
/* Produces n ortho jobs in one persistent launch on `stream`; a job naming its
 * parent's job (earlier in the list) is ordered after it.  `residuals` may be NULL
 * when no job has a residual.  One batch per storage and stream at a time. */
int tp_ortho_batch(tp_storage *ortho, tp_storage *residuals, const tp_ortho_params *params,
                   const tp_ortho_job *jobs, int n, void *stream);
/* Same with the job array in device memory (not validated on the host). */
int tp_ortho_batch_device(tp_storage *ortho, tp_storage *residuals, const tp_ortho_params *params,
                          const tp_ortho_job *jobs_dev, int n, void *stream);
/* Self-check of the known-divisor division the ortho kernel uses for its constant
 * divisors (6, 255, 0.4): compares it with the correctly rounded division for all
 * 2^32 dividends on the device; *mismatches receives the number of differing
 * results (0 expected) and *first_mismatch the bits of the first one (or ~0). */
int tp_division_self_test(float divisor, unsigned long long *mismatches, uint32_t *first_mismatch);
/* The sphere-normal kernel's quotients with a shared denominator (the correctly
 * rounded reciprocal of the denominator, then one exact-remainder correction per
 * numerator) against the correctly rounded division: n_random pseudo-random pairs
 * (all signs, exponents -64..63) and every positive dividend for each of the given
 * divisors; *mismatches receives the number of differing quotients. */
int tp_sphere_division_self_test(unsigned long long n_random, unsigned seed, const float *divisors, int n_divisors,
                                 unsigned long long *mismatches, unsigned long long *first_mismatch);

/* The ortho producers behind the TileCache / TileProducer protocol above
 * (tp_producer_get_tile / put_tile / has_tile / border, tp_scheduler_run,
 * tp_create_tiles).  tp_ortho_residual_producer_create is OrthoCPUProducer
 * (OrthoCPUProducer.cpp:70-254): tiles of an ortho .dat file decoded on the host
 * and uploaded as RGBA8 texels, or, with no file, zero tiles at levels 0 and 1;
 * its cache holds one-channel slots of width tileSize + 2 border.
 * tp_ortho_producer_create is OrthoProducer (OrthoProducer.cpp:145-382): a tile
 * needs its parent (level > 0) and, where the residual producer has one, the
 * residual tile of the same (level, tx, ty); noise_amp as its `noise` attribute,
 * face as its `face` (tp_noise_select), max_level -1 for no limit (hasTile).  A
 * scheduler run produces all queued ortho tiles in one launch, parents first. */
int tp_ortho_residual_producer_create(tp_cache *cache, const char *file, tp_producer **out);
int tp_ortho_producer_create(tp_cache *cache, tp_producer *residuals, const tp_ortho_params *params,
                             const float *noise_amp, int n_noise, int face, int max_level, tp_producer **out);

/* OrthoCPUProducer's pyramids (OrthoCPUProducer.cpp:70-236): a header of 7
 * int32 {maxLevel, tileSize, channels, root, tx, ty, flags} (flags bit 0: DXT
 * tiles, bit 1: tiles without border), 2 * ntiles int64 offsets, one
 * single-strip deflate TIFF of (tileSize + 2 border)^2 x channels bytes per tile;
 * tile id tx + ty 2^level + (4^level - 1) / 3 (:250-253). */
typedef struct tp_ortho_dat tp_ortho_dat;
int tp_ortho_dat_open(const char *path, tp_ortho_dat **out);
int tp_ortho_dat_close(tp_ortho_dat *d);
int tp_ortho_dat_info(const tp_ortho_dat *d, int *info8 /* the 7 header fields, ntiles */);
/* Tile bytes (width^2 x channels, interleaved); DXT tiles give TP_E_BAD_ARG. */
int tp_ortho_dat_read_tile(const tp_ortho_dat *d, int level, int tx, int ty, uint8_t *out, int capacity,
                           int *width);
/* The same tile as RGBA8 texels (width^2 words, missing channels as above). */
int tp_ortho_dat_read_rgba(const tp_ortho_dat *d, int level, int tx, int ty, uint32_t *out, int capacity,
                           int *width);

/* ------------------------------------------------------------------------
 * Preprocess on the device (HeightMipmap.cpp:199-323, 399-559): residual
 * pyramids from a height field, as the reference's preprocess tool builds them.
 * tp_fbm_heights: a procedural value-noise fBm (octaves of base_cells * 2^o
 * cells, gain 1/2, the octave sum normalised to `amplitude` metres) sampled on a
 * size x size grid spanning [0, 1]^2, in int16 units of `quantum` metres.
 * tp_preprocess_level: all 4^level tiles (width tile_size + 5, row-major by
 * (ty, tx)) of one level of the pyramid over a base grid of
 * tile_size * 2^max_level + 1 samples: the approximate tiles (input of the
 * next level), and for level >= 1 the upsampled parents, the residuals (as
 * floats) and their int16 encoding; any of the last three may be NULL. */
int tp_fbm_heights(int size, int octaves, int base_cells, float amplitude, float quantum, uint32_t seed,
                   int16_t *out_dev, void *stream);
int tp_preprocess_level(const int16_t *base_dev, int tile_size, int max_level, int level, float scale,
                        const float *parent_approx_dev, float *approx_dev, float *upsampled_dev,
                        float *residual_dev, int16_t *encoded_dev, void *stream);
/* (upsampled parent, residual) tile pairs at any level of the same procedural fBm,
 * sampled in double precision on the tiles' own windows (no base grid, no
 * quantisation): sample (i, j) of tile (level, tx, ty) is the field at
 * ((i + ts tx - 2), (j + ts ty - 2)) / (ts 2^level); up = the interpolating stencil
 * of the parent tile's fp32 samples (CPUElevationProducer.cpp:194-245 order), res =
 * the child's sample in double - up, rounded once; fine = the child's samples (may be
 * NULL).  Deep levels (below the finest octave's cells, where a base grid would not
 * fit in memory) have truth this way.  Outputs are [n][ts + 5][ts + 5] device
 * arrays; levels >= 1. */
int tp_fbm_pairs(int octaves, int base_cells, float amplitude, uint32_t seed, int tile_size, const int *levels,
                 const int *txs, const int *tys, int n, float *up_dev, float *res_dev, float *fine_dev, void *stream);

/* ------------------------------------------------------------------------
 * Learned residual predictor (no counterpart in the reference: it stands in for
 * stored residuals below a terrain's finest stored level).  A 5-layer 3x3
 * convolutional net, 32 features, GELU, bf16 weights and activations with fp32
 * accumulation on the tensor cores.  Input: the upsampled parent tile (minus its
 * mean, over the level's input sigma), the sample parities and a constant
 * channel, plus a learned per-level embedding; output: the residual tile over
 * the level's output sigma.  Parameters are one flat fp32 array (per layer
 * W[cout][9][cin] then b[cout]; then the embedding [24][32]).  Device arrays are
 * dense n x W x W fp32 tiles; `levels` are host arrays of n ints in [0, 24). */
typedef struct tp_learned tp_learned;
int tp_learned_create(int tile_width, int max_batch, tp_learned **out);
int tp_learned_destroy(tp_learned *net);
int tp_learned_param_count(const tp_learned *net);
int tp_learned_init(tp_learned *net, uint32_t seed);
int tp_learned_get_params(tp_learned *net, float *host, int count);
int tp_learned_set_params(tp_learned *net, const float *host, int count);
int tp_learned_get_grads(tp_learned *net, float *host, int count);
int tp_learned_set_sigmas(tp_learned *net, const float *sigma_in, const float *sigma_out, int nlevels);
/* Checkpoints (training resumed where it stopped): Adam's first and second moments
 * (param_count floats each) and its step count, and the per-level sigmas (up to 24
 * levels).  With tp_learned_get_params / set_params they are the whole training state. */
/* Inference by fused layer pairs (1: layers 0 + 1 and 2 + 3 in one launch each, the
 * hidden activations between the two layers of a pair kept in shared memory) or one
 * launch per layer (0, the default: faster on GB300).  Both give the same bits. */
int tp_learned_set_fused(tp_learned *net, int on);
int tp_learned_get_state(tp_learned *net, float *m, float *v, int count, int *step);
int tp_learned_set_state(tp_learned *net, const float *m, const float *v, int count, int step);
int tp_learned_get_sigmas(tp_learned *net, float *sigma_in, float *sigma_out, int nlevels);
/* Predicted residuals (metres) into out_dev (may be NULL); training = 1 keeps
 * what tp_learned_backward needs.  An inference pass (training = 0) is enqueued on
 * `stream` and the call returns (the caller orders its reads of out_dev on the
 * stream); a kernel's failure in it is reported by the next call that synchronises:
 * tp_learned_check, a training pass, tp_learned_backward, tp_learned_predict_residuals.
 * A training pass returns once complete.  The net's buffers serve all its passes:
 * passes issued on different streams must be ordered by the caller. */
int tp_learned_forward(tp_learned *net, const float *up_dev, const int *levels, int n, int training,
                       float *out_dev, void *stream);
/* Synchronises `stream` and reports a kernel failure of the net's earlier passes. */
int tp_learned_check(tp_learned *net, void *stream);
/* Gradients of the mean squared error (in units of the level sigmas) against
 * target residuals (metres) of the last training forward pass; *loss = that error. */
int tp_learned_backward(tp_learned *net, const float *target_dev, float *loss, void *stream);
int tp_learned_adam(tp_learned *net, float lr, void *stream);
/* Training batch: tile src[k] (< n_src) of (up_src, res_src) under symmetry
 * dihedral[k] (bit 2 transposes, bit 0 mirrors x, bit 1 mirrors y). */
int tp_learned_gather(tp_learned *net, const float *up_src, const float *res_src, int n_src, const int *src,
                      const int *dihedral, int n, float *up_out, float *res_out, void *stream);
/* Learned residual tiles of n jobs (level >= 1, resident parent_slot, residual_slot
 * in `residuals`, a storage of the net's width): the jobs can then be produced by
 * tp_elevation_batch with those residual slots.  Returns once the tiles are written
 * (it synchronises `stream` and reports a kernel's failure). */
int tp_learned_predict_residuals(tp_learned *net, tp_storage *elev, const tp_tile_job *jobs, int n,
                                 tp_storage *residuals, void *stream);

#ifdef __cplusplus
}
#endif
#endif
