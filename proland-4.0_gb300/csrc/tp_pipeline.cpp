// Host-buffer batches: a frame's tiles go host -> device -> host through a ring
// of device chunk buffers, with the copies of neighbouring chunks overlapping the
// persistent elevation launch of the current one (three streams: uploads, compute,
// downloads).  The per-tile arithmetic is the frame kernel's; only the data
// movement around it is organised here.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "tp_internal.h"

namespace {

constexpr int kMaxBuf = 4;

struct ChunkBuf {
    tp_storage *elev = nullptr;  // slots [0, chunk): outputs; [chunk, 2 chunk): parents
    tp_storage *res = nullptr;
    tp_storage *nrm = nullptr;
    float *in_stage = nullptr;   // dense [3][chunk][W][W]: parent zf, parent zm, residual
    float *out_stage = nullptr;  // dense [3][chunk][W][W] zf, zc, zm + [2][chunk][W-4][W-4] nx, ny
    tp_frame *frame = nullptr;
    cudaEvent_t in_ready = nullptr, in_consumed = nullptr, out_ready = nullptr, out_free = nullptr;
};

}  // namespace

struct tp_pipeline {
    int W = 0, chunk = 0, nbuf = 0;
    cudaStream_t up = nullptr, comp = nullptr, down = nullptr;
    ChunkBuf buf[kMaxBuf];
    tp_tile_job *jobs_host = nullptr;  // pinned: the call's jobs with the pipeline's slots
    tp_tile_job *jobs_dev = nullptr;
    size_t jobs_cap = 0;
    cudaEvent_t start = nullptr, jobs_up = nullptr, done = nullptr;
    std::mutex mu;
};

namespace {

int make_event(cudaEvent_t *e)
{
    cudaError_t r = cudaEventCreateWithFlags(e, cudaEventDisableTiming);
    return r == cudaSuccess ? TP_OK : tp::cuda_fail("cudaEventCreate", r);
}

void release(tp_pipeline *p)
{
    for (cudaStream_t s : {p->up, p->comp, p->down})
        if (s) cudaStreamSynchronize(s);
    for (int b = 0; b < kMaxBuf; ++b) {
        ChunkBuf &c = p->buf[b];
        if (c.frame) tp_frame_destroy(c.frame);
        if (c.elev) tp_storage_destroy(c.elev);
        if (c.res) tp_storage_destroy(c.res);
        if (c.nrm) tp_storage_destroy(c.nrm);
        if (c.in_stage) cudaFree(c.in_stage);
        if (c.out_stage) cudaFree(c.out_stage);
        for (cudaEvent_t e : {c.in_ready, c.in_consumed, c.out_ready, c.out_free})
            if (e) cudaEventDestroy(e);
    }
    if (p->jobs_host) cudaFreeHost(p->jobs_host);
    if (p->jobs_dev) cudaFree(p->jobs_dev);
    for (cudaEvent_t e : {p->start, p->jobs_up, p->done})
        if (e) cudaEventDestroy(e);
    for (cudaStream_t s : {p->up, p->comp, p->down})
        if (s) cudaStreamDestroy(s);
    delete p;
}

int ensure_jobs(tp_pipeline *p, size_t n)
{
    if (p->jobs_cap >= n) return TP_OK;
    // the old arrays may still be read by earlier calls' copies and launches
    for (cudaStream_t s : {p->up, p->comp, p->down}) cudaStreamSynchronize(s);
    if (p->jobs_host) cudaFreeHost(p->jobs_host);
    if (p->jobs_dev) cudaFree(p->jobs_dev);
    p->jobs_host = nullptr;
    p->jobs_dev = nullptr;
    p->jobs_cap = 0;
    const size_t cap = std::max<size_t>(n, 1024);
    cudaError_t e = cudaHostAlloc(reinterpret_cast<void **>(&p->jobs_host), sizeof(tp_tile_job) * cap,
                                  cudaHostAllocDefault);
    if (e != cudaSuccess) return tp::cuda_fail("cudaHostAlloc (pipeline jobs)", e);
    e = cudaMalloc(reinterpret_cast<void **>(&p->jobs_dev), sizeof(tp_tile_job) * cap);
    if (e != cudaSuccess) return tp::cuda_fail("cudaMalloc (pipeline jobs)", e);
    p->jobs_cap = cap;
    return TP_OK;
}

int copy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s)
{
    if (bytes == 0) return TP_OK;
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, s);
    return e == cudaSuccess ? TP_OK : tp::cuda_fail("cudaMemcpyAsync (pipeline)", e);
}

int wait(cudaStream_t s, cudaEvent_t e)
{
    cudaError_t r = cudaStreamWaitEvent(s, e, 0);
    return r == cudaSuccess ? TP_OK : tp::cuda_fail("cudaStreamWaitEvent", r);
}

int record(cudaEvent_t e, cudaStream_t s)
{
    cudaError_t r = cudaEventRecord(e, s);
    return r == cudaSuccess ? TP_OK : tp::cuda_fail("cudaEventRecord", r);
}

// Dense plane of `count` tiles <-> plane `channel` of consecutive slots from `first`.
tp::PlaneXfer slot_xfer(const float *dense, tp_storage *s, int first, int channel, int count, bool to_slots,
                        bool clamp0 = false)
{
    tp::PlaneXfer x{};
    float *plane = s->base + (long long)first * s->slot_stride + (long long)channel * s->plane_stride;
    const long long dense_tile = (long long)s->W * s->W;
    if (to_slots) {
        x.src = dense;
        x.dst = plane;
        x.src_tile = dense_tile;
        x.dst_tile = s->slot_stride;
        x.src_pitch = s->W;
        x.dst_pitch = s->pitch;
    } else {
        x.src = plane;
        x.dst = const_cast<float *>(dense);
        x.src_tile = s->slot_stride;
        x.dst_tile = dense_tile;
        x.src_pitch = s->pitch;
        x.dst_pitch = s->W;
    }
    x.rows = s->W;
    x.width = s->W;
    x.count = count;
    x.clamp0 = clamp0 ? 1 : 0;
    return x;
}

// Enqueues one chunk: jobs [off, off + m) through buffer b.
int run_chunk(tp_pipeline *p, ChunkBuf &c, const tp_elev_params *params, const tp_host_tiles *io, int off, int m,
              bool any_residual)
{
    const int W = p->W, Wn = W - 4, C = p->chunk;
    const size_t tile = (size_t)W * W, ntile = (size_t)Wn * Wn;
    const bool normals = io->nx != nullptr;
    int rc;
    // uploads
    if ((rc = wait(p->up, c.in_consumed))) return rc;
    const size_t in_bytes = sizeof(float) * tile * m;
    if (io->parent_zf && (rc = copy(c.in_stage, io->parent_zf + off * tile, in_bytes, cudaMemcpyHostToDevice, p->up)))
        return rc;
    if (io->parent_zf && io->parent_zm &&
        (rc = copy(c.in_stage + tile * C, io->parent_zm + off * tile, in_bytes, cudaMemcpyHostToDevice, p->up)))
        return rc;
    if (any_residual &&
        (rc = copy(c.in_stage + 2 * tile * C, io->residual + off * tile, in_bytes, cudaMemcpyHostToDevice, p->up)))
        return rc;
    if ((rc = record(c.in_ready, p->up))) return rc;
    // compute: dense inputs into slots, the persistent launch, slots into dense outputs
    if ((rc = wait(p->comp, c.in_ready))) return rc;
    tp::PlaneXfers in{};
    if (io->parent_zf) {
        in.p[in.n++] = slot_xfer(c.in_stage, c.elev, C, 0, m, true);
        in.p[in.n++] = io->parent_zm ? slot_xfer(c.in_stage + tile * C, c.elev, C, 2, m, true)
                                     : slot_xfer(c.in_stage, c.elev, C, 2, m, true, params->no_clamp == 0);
    }
    if (any_residual) in.p[in.n++] = slot_xfer(c.in_stage + 2 * tile * C, c.res, 0, 0, m, true);
    if (in.n && (rc = tp::launch_repack_planes(in, p->comp))) return rc;
    if ((rc = record(c.in_consumed, p->comp))) return rc;
    tp_frame_clear(c.frame);
    rc = tp_frame_add_device(c.frame, c.elev, any_residual ? c.res : nullptr, normals ? c.nrm : nullptr, params,
                             p->jobs_dev + off, m, 0);
    if (rc) return rc;
    if ((rc = tp_frame_launch(c.frame, p->comp))) return rc;
    if ((rc = wait(p->comp, c.out_free))) return rc;
    tp::PlaneXfers out{};
    float *outs[3] = {io->zf, io->zc, io->zm};  // zc and zm may be left out (NULL)
    for (int ch = 0; ch < 3; ++ch)
        if (outs[ch]) out.p[out.n++] = slot_xfer(c.out_stage + ch * tile * C, c.elev, 0, ch, m, false);
    float *nstage = c.out_stage + 3 * tile * C;
    if (normals)
        for (int ch = 0; ch < 2; ++ch) out.p[out.n++] = slot_xfer(nstage + ch * ntile * C, c.nrm, 0, ch, m, false);
    if ((rc = tp::launch_repack_planes(out, p->comp))) return rc;
    if ((rc = record(c.out_ready, p->comp))) return rc;
    // downloads
    if ((rc = wait(p->down, c.out_ready))) return rc;
    for (int ch = 0; ch < 3; ++ch)
        if (outs[ch] && (rc = copy(outs[ch] + off * tile, c.out_stage + ch * tile * C, sizeof(float) * tile * m,
                                   cudaMemcpyDeviceToHost, p->down)))
            return rc;
    if (normals) {
        float *nouts[2] = {io->nx, io->ny};
        for (int ch = 0; ch < 2; ++ch)
            if ((rc = copy(nouts[ch] + off * ntile, nstage + ch * ntile * C, sizeof(float) * ntile * m,
                           cudaMemcpyDeviceToHost, p->down)))
                return rc;
    }
    return record(c.out_free, p->down);
}

}  // namespace

extern "C" int tp_pipeline_create(int tile_width, int chunk, int nbuf, tp_pipeline **out)
{
    if (!out) return tp::fail(TP_E_BAD_ARG, "tp_pipeline_create: out is NULL");
    *out = nullptr;
    if (tile_width < 13 || (tile_width - 5) % 8 != 0 || tile_width > 253)
        return tp::fail(TP_E_BAD_ARG, "tp_pipeline_create: tile width must be 8k + 5, at most 253");
    if (nbuf == 0) nbuf = 3;
    if (chunk < 1 || chunk > 65536 || nbuf < 2 || nbuf > kMaxBuf)
        return tp::fail(TP_E_BAD_ARG, "tp_pipeline_create: chunk in [1, 65536], nbuf in [2, 4]");
    if (!tp_device_available()) return tp::fail(TP_E_NO_DEVICE, "tp_pipeline_create: no CUDA device");
    auto *p = new tp_pipeline;
    p->W = tile_width;
    p->chunk = chunk;
    p->nbuf = nbuf;
    int rc = TP_OK;
    for (cudaStream_t *s : {&p->up, &p->comp, &p->down}) {
        cudaError_t e = cudaStreamCreateWithFlags(s, cudaStreamNonBlocking);
        if (e != cudaSuccess && !rc) rc = tp::cuda_fail("cudaStreamCreate (pipeline)", e);
    }
    for (cudaEvent_t *e : {&p->start, &p->jobs_up, &p->done})
        if (!rc) rc = make_event(e);
    const size_t tile = (size_t)tile_width * tile_width, ntile = (size_t)(tile_width - 4) * (tile_width - 4);
    for (int b = 0; b < nbuf && !rc; ++b) {
        ChunkBuf &c = p->buf[b];
        if (!rc) rc = tp_storage_create(tile_width, 3, 2 * chunk, 1, &c.elev);
        if (!rc) rc = tp_storage_create(tile_width, 1, chunk, 1, &c.res);
        if (!rc) rc = tp_storage_create(tile_width - 4, 2, chunk, 1, &c.nrm);
        if (!rc) {
            cudaError_t e = cudaMalloc(&c.in_stage, sizeof(float) * 3 * tile * chunk);
            if (e == cudaSuccess) e = cudaMalloc(&c.out_stage, sizeof(float) * (3 * tile + 2 * ntile) * chunk);
            if (e != cudaSuccess) rc = tp::cuda_fail("cudaMalloc (pipeline stages)", e);
        }
        if (!rc) rc = tp_frame_create(&c.frame);
        for (cudaEvent_t *e : {&c.in_ready, &c.in_consumed, &c.out_ready, &c.out_free})
            if (!rc) rc = make_event(e);
    }
    if (rc) {
        release(p);
        return rc;
    }
    *out = p;
    return TP_OK;
}

extern "C" int tp_pipeline_destroy(tp_pipeline *p)
{
    if (!p) return TP_OK;
    release(p);
    return TP_OK;
}

extern "C" int tp_elevation_batch_host(tp_pipeline *p, const tp_elev_params *params, const tp_tile_job *jobs, int n,
                                       const tp_host_tiles *io, void *stream)
{
    if (!p || !params || !io || n < 0 || (n > 0 && !jobs))
        return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_host: bad arguments");
    if (n == 0) return TP_OK;
    if (!io->zf || (!io->nx) != (!io->ny))
        return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_host: the zf output (and nx with ny) is required");
    if (io->nx && params->normal_format != 2)
        return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_host: normals are produced in format 2 only");
    bool any_residual = false, any_parent = false;
    for (int k = 0; k < n; ++k) {
        const tp_tile_job &j = jobs[k];
        if (j.parent_job != -1) return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_host: jobs must be independent");
        if (j.residual_slot >= 0) {
            if (!io->residual) return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_host: residual tiles missing");
            if (j.rx != 0 || j.ry != 0)
                return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_host: residual windows must be (0, 0)");
            any_residual = true;
        }
        if (j.level > 0) any_parent = true;
    }
    if (any_parent && !io->parent_zf) return tp::fail(TP_E_BAD_ARG, "tp_elevation_batch_host: parent tiles missing");
    std::lock_guard<std::mutex> lk(p->mu);
    cudaStream_t caller = static_cast<cudaStream_t>(stream);
    // the pinned job array is rewritten below: the previous call's upload must be done
    cudaError_t e = cudaEventSynchronize(p->jobs_up);
    if (e != cudaSuccess) return tp::cuda_fail("cudaEventSynchronize (pipeline jobs)", e);
    int rc = ensure_jobs(p, (size_t)n);
    if (rc) return rc;
    const int C = p->chunk;
    for (int k = 0; k < n; ++k) {
        tp_tile_job j = jobs[k];
        const int local = k % C;
        j.out_slot = local;
        j.parent_slot = j.level > 0 ? C + local : -1;
        j.residual_slot = j.residual_slot >= 0 ? local : -1;
        j.normal_slot = io->nx ? local : -1;
        j.parent_job = -1;
        p->jobs_host[k] = j;
    }
    for (int off = 0; off < n; off += C) {
        const ChunkBuf &c = p->buf[(off / C) % p->nbuf];
        rc = tp::check_batch_jobs(c.elev, any_residual ? c.res : nullptr, io->nx ? c.nrm : nullptr,
                                  p->jobs_host + off, std::min(C, n - off));
        if (rc) return rc;
    }
    // order after the caller's stream, upload the jobs, run the chunks
    if ((rc = record(p->start, caller))) return rc;
    for (cudaStream_t s : {p->up, p->comp, p->down})
        if ((rc = wait(s, p->start))) return rc;
    rc = copy(p->jobs_dev, p->jobs_host, sizeof(tp_tile_job) * n, cudaMemcpyHostToDevice, p->up);
    if (!rc) rc = record(p->jobs_up, p->up);
    for (int off = 0; off < n && !rc; off += C)
        rc = run_chunk(p, p->buf[(off / C) % p->nbuf], params, io, off, std::min(C, n - off), any_residual);
    // the caller's stream waits for everything enqueued, also after a failure
    int rc2 = record(p->done, p->down);
    if (!rc2) rc2 = wait(caller, p->done);
    return rc ? rc : rc2;
}
