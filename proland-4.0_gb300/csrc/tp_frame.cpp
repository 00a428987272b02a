// Frames: the tile requests of one frame, for up to two tile widths, produced
// by one persistent launch (optionally replayed from a CUDA graph).  The batch
// entry points are one-class frames.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "tp_internal.h"
#include "tp_trace.h"

struct tp_frame {
    struct Class {
        tp_storage *elev = nullptr, *res = nullptr, *nrm = nullptr;
        tp_elev_params params{};
        std::vector<tp_tile_job> jobs;          // host copy (empty when jobs_dev is the caller's)
        const tp_tile_job *jobs_dev = nullptr;  // device job array used by the launch
        int njobs = 0;
        tp::ClassLaunch L{};
        const CUtensorMap *pmap = nullptr, *rmap = nullptr;
        bool device_deps = false;  // a device job list that names parent jobs
        int minb_override = 0;     // CTAs per SM the kernel variant targets (0: automatic)
    };
    Class cls[2];
    int nclasses = 0;
    // device buffers: [counter | done of class 0 | done of class 1], job arrays
    int *flags = nullptr;
    size_t flags_count = 0;
    tp_tile_job *jobs_buf = nullptr;
    size_t jobs_buf_count = 0;
    bool uploaded = false;
    // two tile widths: their launches on forked streams, so that the CTAs of one
    // start while the other's last wave drains
    bool overlap = true;
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    // CUDA graph of (reset + launch), built on first tp_frame_graph_launch
    cudaGraphExec_t graph = nullptr;
    cudaStream_t graph_stream = nullptr;
};

namespace {

int sm_count() { return tp::device_sm_count(); }

// Validates a class's storages and parameters and fills its launch layout.
int setup_class(tp_frame::Class &k)
{
    int br = 0;
    int rc = tp::class_layout(k.elev, k.res, k.nrm, &k.params, "frame", &k.L, &br);
    if (rc) return rc;
    int err = TP_OK;
    k.L.noise = tp::device_noise_table(k.elev->W, &err);
    if (!k.L.noise) return err;
    rc = tp::tensor_map(k.elev, k.L.par_pitch, k.L.par_rows, &k.pmap);
    if (rc) return rc;
    if (k.res) {
        rc = tp::tensor_map(k.res, k.elev->pitch, br + 2, &k.rmap);
        if (rc) return rc;
    } else {
        k.rmap = k.pmap;  // never used: jobs without a residual storage have no residual slot
    }
    return TP_OK;
}

int stage_floats_of(const tp::ClassLaunch &L)
{
    return L.buf_floats + L.par_floats + tp::round_up(L.ck * L.ck, 32);
}

int check_job(const tp_frame::Class &k, const tp_tile_job &j, int index, int n)
{
    const tp_storage *elev = k.elev, *res = k.res, *nrm = k.nrm;
    const int W = elev->W, ts = W - 5;
    char buf[200];
    auto bad = [&](int code, const char *what) {
        snprintf(buf, sizeof buf, "frame: job %d (level %d, %d, %d): %s", index, j.level, j.tx, j.ty, what);
        return tp::fail(code, buf);
    };
    if (j.level < 0 || j.level > 30 || j.tx < 0 || j.ty < 0 || (j.tx >> j.level) != 0 || (j.ty >> j.level) != 0)
        return bad(TP_E_BAD_ARG, "bad quadtree coordinates");
    if (j.out_slot < 0 || j.out_slot >= elev->capacity) return bad(TP_E_BAD_ARG, "bad out_slot");
    if (j.level > 0) {
        if (j.parent_slot < 0 || j.parent_slot >= elev->capacity) return bad(TP_E_MISSING_PARENT, "parent tile missing");
        if (j.parent_slot == j.out_slot) return bad(TP_E_BAD_ARG, "parent_slot == out_slot");
    }
    if (j.parent_job < -1 || j.parent_job >= index) return bad(TP_E_BAD_ARG, "parent_job must precede the job");
    if (j.residual_slot >= 0) {
        if (!res || j.residual_slot >= res->capacity) return bad(TP_E_BAD_ARG, "bad residual_slot");
        if (j.rx < 0 || j.ry < 0 || j.rx % ts != 0 || j.ry % ts != 0 || j.rx + W > res->W || j.ry + W > res->W)
            return bad(TP_E_BAD_ARG, "residual window outside the residual tile");
    }
    if (j.normal_slot >= 0 && (!nrm || j.normal_slot >= nrm->capacity)) return bad(TP_E_BAD_ARG, "bad normal_slot");
    if (j.noise_layer < 0 || j.noise_layer > 5 || j.noise_rot < 0 || j.noise_rot > 3)
        return bad(TP_E_BAD_ARG, "bad noise layer / rotation");
    if (!(j.tile_meters > 0.0f)) return bad(TP_E_BAD_ARG, "tile_meters must be positive");
    (void)n;
    return TP_OK;
}

int check_jobs(const tp_frame::Class &k, const tp_tile_job *jobs, int n)
{
    for (int i = 0; i < n; ++i) {
        int rc = check_job(k, jobs[i], i, n);
        if (rc) return rc;
        const tp_tile_job &j = jobs[i];
        if (j.parent_job >= 0) {
            const tp_tile_job &pj = jobs[j.parent_job];
            if (pj.out_slot != j.parent_slot || pj.level != j.level - 1 || pj.tx != j.tx / 2 || pj.ty != j.ty / 2)
                return tp::fail(TP_E_BAD_ARG, "frame: parent_job does not produce the parent tile");
        }
    }
    return TP_OK;
}

void drop_graph(tp_frame *f)
{
    if (f->graph) cudaGraphExecDestroy(f->graph);
    f->graph = nullptr;
}

// Uploads job arrays (first launch after a change) and assembles the launches
// (one persistent launch per tile width).
int prepare(tp_frame *f, tp::FrameLaunch *F, void *stream)
{
    if (f->nclasses == 0) return tp::fail(TP_E_BAD_ARG, "frame: no classes");
    size_t host_jobs = 0, ndone = 0;
    for (int c = 0; c < f->nclasses; ++c) {
        host_jobs += f->cls[c].jobs.size();
        ndone += f->cls[c].njobs;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t nflags = 2 + ndone;  // [counter 0 | counter 1 | done of class 0 | done of class 1]
    if (f->flags_count < nflags) {
        if (f->flags) cudaFree(f->flags);
        f->flags = nullptr;
        f->flags_count = 0;
        cudaError_t e = cudaMalloc(&f->flags, sizeof(int) * nflags);
        if (e != cudaSuccess) return tp::cuda_fail("cudaMalloc (frame flags)", e);
        f->flags_count = nflags;
        drop_graph(f);
    }
    if (!f->uploaded) {
        if (f->jobs_buf_count < host_jobs) {
            if (f->jobs_buf) cudaFree(f->jobs_buf);
            f->jobs_buf = nullptr;
            f->jobs_buf_count = 0;
            cudaError_t e = cudaMalloc(&f->jobs_buf, sizeof(tp_tile_job) * std::max<size_t>(host_jobs, 1));
            if (e != cudaSuccess) return tp::cuda_fail("cudaMalloc (frame jobs)", e);
            f->jobs_buf_count = host_jobs;
            drop_graph(f);
        }
        size_t off = 0;
        for (int c = 0; c < f->nclasses; ++c) {
            auto &k = f->cls[c];
            if (!k.jobs.empty()) {
                cudaError_t e = cudaMemcpyAsync(f->jobs_buf + off, k.jobs.data(), sizeof(tp_tile_job) * k.jobs.size(),
                                                cudaMemcpyHostToDevice, s);
                if (e != cudaSuccess) return tp::cuda_fail("cudaMemcpyAsync (frame jobs)", e);
                k.jobs_dev = f->jobs_buf + off;
                off += k.jobs.size();
            }
        }
        f->uploaded = true;
    }
    int done_off = 2;
    for (int c = 0; c < f->nclasses; ++c) {
        auto &k = f->cls[c];
        tp::FrameLaunch &L = F[c];
        std::memset(&L, 0, sizeof L);
        L.c = k.L;
        L.c.jobs = k.jobs_dev;
        L.c.njobs = k.njobs;
        L.c.done = f->flags + done_off;
        done_off += k.njobs;
        L.counter = f->flags + c;
        L.stage_floats = stage_floats_of(k.L);
        L.any_deps = 0;
        if (k.jobs.empty() && k.njobs > 0 && k.device_deps) L.any_deps = 1;  // as declared by the caller
        for (const auto &j : k.jobs)
            if (j.parent_job >= 0) L.any_deps = 1;
        // double-buffer when the class asks for it; three CTAs per SM when three
        // CTAs' stages fit in shared memory
        L.stages = k.params.stages == 2 ? 2 : 1;
        const size_t per_cta = sizeof(float) * (size_t)L.stage_floats * L.stages + 128 + 1024;
        L.minb = k.minb_override ? k.minb_override : (3 * per_cta <= 227 * 1024 ? 3 : 2);
    }
    return TP_OK;
}

int enqueue(tp_frame *f, const tp::FrameLaunch *F, void *stream)
{
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(f->flags, 0, sizeof(int) * f->flags_count, s);
    if (e != cudaSuccess) return tp::cuda_fail("cudaMemsetAsync (frame flags)", e);
    int active = 0;
    for (int c = 0; c < f->nclasses; ++c) active += F[c].c.njobs * F[c].c.bands > 0 ? 1 : 0;
    // the classes share no data: with two of them, the second goes on a side stream
    // forked from (and joined back into) `stream`; in a graph capture this makes
    // two parallel kernel nodes
    const bool fork = f->overlap && active == 2;
    if (fork) {
        if (!f->side) {
            e = cudaStreamCreateWithFlags(&f->side, cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f->fork_ev, cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&f->join_ev, cudaEventDisableTiming);
            if (e != cudaSuccess) return tp::cuda_fail("frame side stream", e);
        }
        e = cudaEventRecord(f->fork_ev, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(f->side, f->fork_ev, 0);
        if (e != cudaSuccess) return tp::cuda_fail("frame fork", e);
    }
    int launched = 0;
    for (int c = 0; c < f->nclasses; ++c) {
        const tp::FrameLaunch &L = F[c];
        const int units = L.c.njobs * L.c.bands;
        if (units == 0) continue;
        int per_sm = 0;
        int rc = tp::frame_occupancy(L.stage_floats, L.stages, L.minb, L.c.noise_mode == 1, &per_sm);
        if (rc) return rc;
        if (per_sm < 1) return tp::fail(TP_E_BAD_ARG, "frame: the kernel's stage does not fit in shared memory");
        const int grid = std::min(units, per_sm * sm_count());
        rc = tp::launch_frame(L, f->cls[c].pmap, f->cls[c].rmap, grid, fork && launched == 1 ? f->side : stream);
        if (rc) return rc;
        ++launched;
    }
    if (fork) {
        e = cudaEventRecord(f->join_ev, f->side);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, f->join_ev, 0);
        if (e != cudaSuccess) return tp::cuda_fail("frame join", e);
    }
    return TP_OK;
}

int add_class(tp_frame *f, tp_storage *elev, tp_storage *res, tp_storage *nrm, const tp_elev_params *p,
              const tp_tile_job *jobs, const tp_tile_job *jobs_dev, int n, bool device_deps = true)
{
    if (!f || !p) return tp::fail(TP_E_BAD_ARG, "tp_frame_add: frame and params are required");
    if (f->nclasses >= 2) return tp::fail(TP_E_BAD_ARG, "tp_frame_add: a frame holds at most two tile widths");
    if (n < 0 || (n > 0 && !jobs && !jobs_dev)) return tp::fail(TP_E_BAD_ARG, "tp_frame_add: bad job array");
    tp_frame::Class k;
    k.elev = elev;
    k.res = res;
    k.nrm = nrm;
    k.params = *p;
    int rc = setup_class(k);
    if (rc) return rc;
    if (jobs) {
        rc = check_jobs(k, jobs, n);
        if (rc) return rc;
        k.jobs.assign(jobs, jobs + n);
    } else {
        k.jobs_dev = jobs_dev;
        k.device_deps = device_deps;
    }
    k.njobs = n;
    f->cls[f->nclasses++] = std::move(k);
    f->uploaded = false;
    drop_graph(f);
    return TP_OK;
}

}  // namespace

int tp::class_layout(tp_storage *elev, tp_storage *res, tp_storage *nrm, const tp_elev_params *p, const char *who,
                     tp::ClassLaunch *out, int *band_rows)
{
    char buf[200];
    auto bad = [&](const char *what) {
        snprintf(buf, sizeof buf, "%s: %s", who, what);
        return tp::fail(TP_E_BAD_ARG, buf);
    };
    if (!elev || !p) return bad("an elevation storage and params are required");
    if (elev->on_device != 1 || elev->channels != 3) return bad("elevation storage must be a device storage with 3 channels");
    const int W = elev->W, n = W - 5;
    if (n < 8 || n % 8 != 0) return bad("tile width must be 8k + 5");
    if (W > 253) return bad("tile width above 253 is not supported");
    if (p->grid_size < 1 || n % p->grid_size != 0) return bad("grid_size must divide the tile size");
    if (p->noise_mode != 0 && p->noise_mode != 1) return bad("bad noise_mode");
    if (res) {
        if (res->on_device != 1 || res->channels != 1) return bad("residual storage must be 1-channel device storage");
        if ((res->W - 5) % n != 0) return bad("residual tile size must be a multiple of the tile size");
    }
    if (nrm) {
        if (nrm->on_device != 1 || nrm->channels != 2 || nrm->W != W - 4)
            return bad("normal storage must be 2-channel device storage of width W - 4");
        if (p->normal_format != 2) return bad("only normal format 2 (signed fp32) is supported");
    }
    tp::ClassLaunch L;
    std::memset(&L, 0, sizeof L);
    L.elev = elev->base;
    L.elev_cap = tp::checked_capacity(elev);
    L.res_cap = tp::checked_capacity(res);
    L.nrm_cap = tp::checked_capacity(nrm);
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
    // band height: whole 101-wide tiles, quarters of 197-wide ones, unless asked; the
    // bands are br rows each, the last one the rest
    int br = p->band_rows > 0 ? p->band_rows : (W <= 128 ? W : (W + 3) / 4);
    br = std::min(std::max(br, 8), W);
    L.bands = (W + br - 1) / br;
    L.band_rows = br;
    if (br + 2 > 256) return bad("band taller than a TMA box");
    const int PE = elev->pitch;
    L.buf_floats = tp::round_up((br + 2) * PE, 32);
    // parent zf window: columns [d, d + n/2 + 5] (stencil and modulated-noise taps),
    // rows from the first computed row's parent row, (br + 1)/2 + 5 of them
    L.par_pitch = tp::round_up(n / 2 + 6, 4);
    L.par_rows = (br + 1) / 2 + 5;
    if (L.par_pitch > 256 || L.par_rows > 256) return bad("parent window above a TMA box");
    L.par_floats = tp::round_up(L.par_pitch * L.par_rows, 32);
    const int kmax = (n + 2 + g) / (2 * g);  // largest coarse-mesh index of a sample
    L.ck = kmax + 2;
    L.res_box_bytes = (uint32_t)(sizeof(float) * PE * (br + 2));
    L.par_box_bytes = (uint32_t)(sizeof(float) * L.par_pitch * L.par_rows);
    *out = L;
    *band_rows = br;
    return TP_OK;
}

int tp::check_batch_jobs(tp_storage *elev, tp_storage *res, tp_storage *nrm, const tp_tile_job *jobs, int n)
{
    tp_frame::Class k;
    k.elev = elev;
    k.res = res;
    k.nrm = nrm;
    return check_jobs(k, jobs, n);
}

extern "C" int tp_frame_create(tp_frame **out)
{
    if (!out) return tp::fail(TP_E_BAD_ARG, "tp_frame_create: out is NULL");
    *out = new tp_frame;
    return TP_OK;
}

extern "C" int tp_frame_destroy(tp_frame *f)
{
    if (!f) return TP_OK;
    drop_graph(f);
    if (f->side) {
        cudaStreamSynchronize(f->side);
        cudaStreamDestroy(f->side);
        cudaEventDestroy(f->fork_ev);
        cudaEventDestroy(f->join_ev);
    }
    if (f->flags) cudaFree(f->flags);
    if (f->jobs_buf) cudaFree(f->jobs_buf);
    delete f;
    return TP_OK;
}

extern "C" int tp_frame_overlap_classes(tp_frame *f, int on)
{
    if (!f) return tp::fail(TP_E_BAD_ARG, "tp_frame_overlap_classes: frame is NULL");
    if (f->overlap != (on != 0)) drop_graph(f);
    f->overlap = on != 0;
    return TP_OK;
}

extern "C" int tp_frame_clear(tp_frame *f)
{
    if (!f) return tp::fail(TP_E_BAD_ARG, "tp_frame_clear: frame is NULL");
    for (auto &k : f->cls) k = tp_frame::Class();
    f->nclasses = 0;
    f->uploaded = false;
    drop_graph(f);
    return TP_OK;
}

extern "C" int tp_frame_add(tp_frame *f, tp_storage *elev, tp_storage *residuals, tp_storage *normals,
                            const tp_elev_params *params, const tp_tile_job *jobs, int n)
{
    return add_class(f, elev, residuals, normals, params, jobs, nullptr, n);
}

extern "C" int tp_frame_add_device(tp_frame *f, tp_storage *elev, tp_storage *residuals, tp_storage *normals,
                                   const tp_elev_params *params, const tp_tile_job *jobs_dev, int n,
                                   int has_dependencies)
{
    if (n > 0 && !jobs_dev) return tp::fail(TP_E_BAD_ARG, "tp_frame_add_device: jobs_dev is NULL");
    return add_class(f, elev, residuals, normals, params, nullptr, jobs_dev, n, has_dependencies != 0);
}

extern "C" int tp_frame_launch(tp_frame *f, void *stream)
{
    tp::TraceScope trace("frame launch", -1);
    if (!f) return tp::fail(TP_E_BAD_ARG, "tp_frame_launch: frame is NULL");
    tp::FrameLaunch F[2];
    int rc = prepare(f, F, stream);
    if (rc) return rc;
    return enqueue(f, F, stream);
}

extern "C" int tp_frame_graph_launch(tp_frame *f, void *stream)
{
    tp::TraceScope trace("frame graph launch", -1);
    if (!f) return tp::fail(TP_E_BAD_ARG, "tp_frame_graph_launch: frame is NULL");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!f->graph || f->graph_stream != s) {
        tp::FrameLaunch F[2];
        int rc = prepare(f, F, stream);  // uploads outside the graph
        if (rc) return rc;
        drop_graph(f);
        cudaStream_t cap = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
        if (e != cudaSuccess) return tp::cuda_fail("cudaStreamCreate", e);
        // set the kernels' attributes outside the capture
        for (int c = 0; c < f->nclasses; ++c) {
            int per_sm = 0;
            rc = tp::frame_occupancy(F[c].stage_floats, F[c].stages, F[c].minb, F[c].c.noise_mode == 1, &per_sm);
            if (rc) {
                cudaStreamDestroy(cap);
                return rc;
            }
        }
        e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaStreamDestroy(cap);
            return tp::cuda_fail("cudaStreamBeginCapture", e);
        }
        rc = enqueue(f, F, cap);
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(cap, &graph);
        cudaStreamDestroy(cap);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return tp::cuda_fail("cudaStreamEndCapture", e);
        e = cudaGraphInstantiate(&f->graph, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            f->graph = nullptr;
            return tp::cuda_fail("cudaGraphInstantiate", e);
        }
        f->graph_stream = s;
    }
    cudaError_t e = cudaGraphLaunch(f->graph, s);
    if (e != cudaSuccess) return tp::cuda_fail("cudaGraphLaunch", e);
    return TP_OK;
}

extern "C" int tp_frame_units(const tp_frame *f)
{
    if (!f) return tp::fail(TP_E_BAD_ARG, "tp_frame_units: frame is NULL");
    int u = 0;
    for (int c = 0; c < f->nclasses; ++c) u += f->cls[c].njobs * f->cls[c].L.bands;
    return u;
}

// ---------------------------------------------------------------- autotuner
namespace {

// Launch time (ms, mean of `repeats`) of class c alone under its current shape.
int time_class(tp_frame *f, int c, cudaStream_t s, int repeats, float *ms)
{
    tp::FrameLaunch F[2];
    int rc = prepare(f, F, s);
    if (rc) return rc;
    const tp::FrameLaunch &L = F[c];
    const int units = L.c.njobs * L.c.bands;
    int per_sm = 0;
    rc = tp::frame_occupancy(L.stage_floats, L.stages, L.minb, L.c.noise_mode == 1, &per_sm);
    if (rc) return rc;
    if (per_sm < 1) return tp::fail(TP_E_BAD_ARG, "autotune: shape does not fit");
    const int grid = std::min(units, per_sm * sm_count());
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float total = 0.0f;
    for (int r = -1; r < repeats; ++r) {  // r = -1: warm-up
        cudaMemsetAsync(f->flags, 0, sizeof(int) * f->flags_count, s);
        cudaEventRecord(e0, s);
        rc = tp::launch_frame(L, f->cls[c].pmap, f->cls[c].rmap, grid, s);
        cudaEventRecord(e1, s);
        if (rc) break;
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            rc = tp::cuda_fail("autotune", e);
            break;
        }
        float t = 0.0f;
        cudaEventElapsedTime(&t, e0, e1);
        if (r >= 0) total += t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    *ms = total / repeats;
    return TP_OK;
}

}  // namespace

extern "C" int tp_frame_autotune(tp_frame *f, void *stream, int repeats)
{
    if (!f || f->nclasses == 0) return tp::fail(TP_E_BAD_ARG, "tp_frame_autotune: empty frame");
    if (repeats < 1) repeats = 3;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    for (int c = 0; c < f->nclasses; ++c) {
        auto &k = f->cls[c];
        if (k.njobs == 0) continue;
        const int W = k.elev->W;
        std::vector<int> bands = W <= 128 ? std::vector<int>{W, (W + 1) / 2, (W + 2) / 3, (W + 3) / 4}
                                          : std::vector<int>{(W + 1) / 2, (W + 2) / 3, (W + 3) / 4, (W + 4) / 5, (W + 5) / 6};
        // heights whose rows with the two halo rows fill the elevation phase's strips
        // exactly: strips = 256 threads / column quads, each an even number of rows
        {
            const int strips = std::max(1, tp::kFrameThreads / (k.elev->pitch / 4));
            for (int r = 2 * strips - 2; r <= W / 2; r += 2 * strips)
                if (r >= 16 && std::find(bands.begin(), bands.end(), r) == bands.end()) bands.push_back(r);
        }
        const tp_elev_params orig = k.params;
        const int orig_minb = k.minb_override;
        float best = 1e30f;
        tp_elev_params best_p = orig;
        int best_minb = orig_minb;
        for (int br : bands)
            for (int stages = 1; stages <= 2; ++stages)
                for (int minb = 2; minb <= 3; ++minb) {
                    k.params = orig;
                    k.params.band_rows = br;
                    k.params.stages = stages;
                    k.minb_override = minb;
                    if (setup_class(k)) continue;
                    const size_t per_cta = sizeof(float) * (size_t)stage_floats_of(k.L) * stages + 128 + 1024;
                    if (per_cta * minb > 227 * 1024) continue;
                    f->uploaded = f->uploaded;  // job lists are unchanged
                    float ms = 0.0f;
                    if (time_class(f, c, s, repeats, &ms)) continue;
                    if (ms < best) {
                        best = ms;
                        best_p = k.params;
                        best_minb = minb;
                    }
                }
        k.params = best_p;
        k.minb_override = best_minb;
        int rc = setup_class(k);
        if (rc) return rc;
    }
    drop_graph(f);
    int st = 0;
    tp::read_status(&st, true);
    if (st != 0) return tp::fail(st, "autotune: a kernel reported a failure");
    return TP_OK;
}

extern "C" int tp_frame_config(const tp_frame *f, int klass, int *band_rows, int *stages, int *ctas_per_sm)
{
    if (!f || klass < 0 || klass >= f->nclasses) return tp::fail(TP_E_BAD_ARG, "tp_frame_config: bad class");
    const auto &k = f->cls[klass];
    if (band_rows) *band_rows = k.L.band_rows;
    if (stages) *stages = k.params.stages == 2 ? 2 : 1;
    if (ctas_per_sm) {
        const size_t per_cta = sizeof(float) * (size_t)stage_floats_of(k.L) * (k.params.stages == 2 ? 2 : 1) + 128 + 1024;
        *ctas_per_sm = k.minb_override ? k.minb_override : (3 * per_cta <= 227 * 1024 ? 3 : 2);
    }
    return TP_OK;
}

// ---------------------------------------------------------------- batch calls
static int batch(tp_storage *elev, tp_storage *res, tp_storage *nrm, const tp_elev_params *params,
                 const tp_tile_job *jobs, const tp_tile_job *jobs_dev, int n, void *stream)
{
    if (!elev) return tp::fail(TP_E_BAD_ARG, "batch: elevation storage is required");
    if (n == 0) return TP_OK;
    std::lock_guard<std::mutex> lk(elev->copy_mu);
    if (!elev->batch_frame) elev->batch_frame = new tp_frame;
    tp_frame *f = elev->batch_frame;
    tp_frame_clear(f);
    int rc = add_class(f, elev, res, nrm, params, jobs, jobs_dev, n, true);
    if (rc) return rc;
    return tp_frame_launch(f, stream);
}

extern "C" int tp_elevation_batch(tp_storage *elev, tp_storage *res, tp_storage *nrm, const tp_elev_params *params,
                                  const tp_tile_job *jobs, int n, void *stream)
{
    if (n < 0 || (n > 0 && !jobs)) return tp::fail(TP_E_BAD_ARG, "batch: bad job array");
    return batch(elev, res, nrm, params, jobs, nullptr, n, stream);
}

extern "C" int tp_elevation_batch_device(tp_storage *elev, tp_storage *res, tp_storage *nrm,
                                         const tp_elev_params *params, const tp_tile_job *jobs_dev, int n,
                                         void *stream)
{
    if (n < 0 || (n > 0 && !jobs_dev)) return tp::fail(TP_E_BAD_ARG, "batch: bad job array");
    return batch(elev, res, nrm, params, nullptr, jobs_dev, n, stream);
}
