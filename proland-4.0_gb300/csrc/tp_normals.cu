// Normal tiles from elevation tiles already produced (NormalProducer::doCreateTile,
// NormalProducer.cpp:164-289): flat tiles requested after their elevation tile
// was produced and cached (same arithmetic as the fused kernel's normal phase,
// terrain/examples/terrain1/normalShader.glsl:57-74, point-sampled zm), and all
// tiles of a spherically deformed terrain (terrain/examples/terrain2/normalShader.glsl).
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "tp_internal.h"

namespace {

struct NormalJob {
    int eslot, nslot;
    float tile_meters;
    int frame;  // index of the job's spherical frame, -1 for flat deformation
};

// Each operation of the spherical path is rounded on its own (no fused
// multiply-add), in the order the shader writes it: the positions are ~R = 6.4e6
// and their neighbour differences cancel most of their digits, so a contraction
// that moves one rounding changes the normal by more than 1e-4.
__device__ __forceinline__ float m_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float a_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float s_(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float dot4(const float *r, const float *x)
{
    return a_(a_(a_(m_(r[0], x[0]), m_(r[1], x[1])), m_(r[2], x[2])), m_(r[3], x[3]));
}
__device__ __forceinline__ float dot3(const float *r, const float *x)
{
    return a_(a_(m_(r[0], x[0]), m_(r[1], x[1])), m_(r[2], x[2]));
}

// getWorldPosition of terrain2/normalShader.glsl:56-73 (the patch's projective
// mapping onto the sphere), for grid position (u, v) in samples and height h.
__device__ __forceinline__ void sphere_pos(const tp::SphereFrame &f, float n, float u, float v, float h, float *out)
{
    u = __fdiv_rn(u, n);
    v = __fdiv_rn(v, n);
    const float U = s_(1.0f, u), V = s_(1.0f, v);
    const float al[4] = {m_(U, V), m_(u, V), m_(U, v), m_(u, v)};
    const float d = dot4(al, f.L);
    float ap[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) ap[k] = __fdiv_rn(m_(al[k], f.L[k]), d);
    float up[3], cp[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        up[r] = dot4(f.N + r * 4, ap);
        cp[r] = dot4(f.C + r * 4, ap);
    }
    const float R = f.R;
    const float e0 = R / 32.0f, e1 = R / 64.0f;  // exact: powers of two
    float s = __fdiv_rn(s_(f.size, e0), s_(e1, e0));  // smoothstep(R/32, R/64, size)
    s = s < 0.0f ? 0.0f : (s > 1.0f ? 1.0f : s);
    s = m_(m_(s, s), s_(3.0f, m_(2.0f, s)));
    const float len = __fsqrt_rn(dot3(up, up));
    const float k = a_(m_(len, s_(1.0f, s)), s);
    const float hp = __fdiv_rn(a_(h, m_(R, s_(1.0f, k))), k);
#pragma unroll
    for (int r = 0; r < 3; ++r) out[r] = a_(cp[r], m_(hp, up[r]));
}

__global__ void __launch_bounds__(256) normals_kernel(const float *__restrict__ elev, int pitch, long long eplane,
                                                      long long eslot_stride, float *__restrict__ nrm, int npitch,
                                                      long long nplane, long long nslot_stride,
                                                      const NormalJob *__restrict__ jobs,
                                                      const tp::SphereFrame *__restrict__ frames, int W)
{
    const NormalJob J = jobs[blockIdx.x];
    if (J.frame >= 0) {
        // spherical deformation (terrain2/normalShader.glsl:75-88): world positions of
        // the four neighbours, their cross product rotated into the tile's tangent frame
        __shared__ tp::SphereFrame F;
        if (threadIdx.x == 0) F = frames[J.frame];
        __syncthreads();
        const float *zm = elev + (long long)J.eslot * eslot_stride + 2 * eplane;
        float *nx = nrm + (long long)J.nslot * nslot_stride;
        float *ny = nx + nplane;
        const int Wn = W - 4;
        const float n = (float)(W - 5);
        for (int idx = threadIdx.x; idx < Wn * npitch; idx += blockDim.x) {
            const int q = idx / npitch, p = idx - q * npitch;
            float vx = 0.0f, vy = 0.0f;
            if (p < Wn) {
                const float *c = zm + (long long)(q + 2) * pitch + (p + 2);
                float p0[3], p1[3], p2[3], p3[3];
                sphere_pos(F, n, (float)(p - 1), (float)q, __ldg(c - 1), p0);
                sphere_pos(F, n, (float)(p + 1), (float)q, __ldg(c + 1), p1);
                sphere_pos(F, n, (float)p, (float)(q - 1), __ldg(c - pitch), p2);
                sphere_pos(F, n, (float)p, (float)(q + 1), __ldg(c + pitch), p3);
                const float a[3] = {s_(p1[0], p0[0]), s_(p1[1], p0[1]), s_(p1[2], p0[2])};
                const float b[3] = {s_(p3[0], p2[0]), s_(p3[1], p2[1]), s_(p3[2], p2[2])};
                float cr[3] = {s_(m_(a[1], b[2]), m_(a[2], b[1])), s_(m_(a[2], b[0]), m_(a[0], b[2])),
                               s_(m_(a[0], b[1]), m_(a[1], b[0]))};
                const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot3(cr, cr)));
                cr[0] = m_(cr[0], inv);
                cr[1] = m_(cr[1], inv);
                cr[2] = m_(cr[2], inv);
                vx = dot3(F.W2T, cr);
                vy = dot3(F.W2T + 3, cr);
            }
            nx[(long long)q * npitch + p] = vx;
            ny[(long long)q * npitch + p] = vy;
        }
        return;
    }
    const float *zm = elev + (long long)J.eslot * eslot_stride + 2 * eplane;
    float *nx = nrm + (long long)J.nslot * nslot_stride;
    float *ny = nx + nplane;
    const int n = W - 5, Wn = W - 4, NQ = npitch / 4;
    const float h2 = __fmul_rn(2.0f, __fdiv_rn(J.tile_meters, (float)n));
    const float hh = h2 * h2;
    for (int idx = threadIdx.x; idx < Wn * NQ; idx += blockDim.x) {
        const int q = idx / NQ, m = idx - q * NQ;
        float vx[4], vy[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int p = 4 * m + k;
            vx[k] = vy[k] = 0.0f;
            if (p < Wn) {
                const float *c = zm + (long long)(q + 2) * pitch + (p + 2);
                const float ax = -__fsub_rn(__ldg(c + 1), __ldg(c - 1));
                const float ay = -__fsub_rn(__ldg(c + pitch), __ldg(c - pitch));
                const float inv = rsqrtf(ax * ax + ay * ay + hh);
                vx[k] = ax * inv;
                vy[k] = ay * inv;
            }
        }
        const long long o = (long long)q * npitch + 4 * m;
        *reinterpret_cast<float4 *>(nx + o) = make_float4(vx[0], vx[1], vx[2], vx[3]);
        *reinterpret_cast<float4 *>(ny + o) = make_float4(vy[0], vy[1], vy[2], vy[3]);
    }
}

}  // namespace

namespace tp {

int launch_normals(tp_storage *elev, tp_storage *nrm, const int *eslots, const int *nslots, const float *meters,
                   int count, void *stream, const SphereFrame *frames)
{
    if (count <= 0) return TP_OK;
    static std::mutex mu;
    static char *dbuf = nullptr;
    static size_t dcap = 0;
    std::lock_guard<std::mutex> lk(mu);
    std::vector<NormalJob> h(count);
    for (int k = 0; k < count; ++k) {
        if (eslots[k] < 0 || eslots[k] >= elev->capacity || nslots[k] < 0 || nslots[k] >= nrm->capacity)
            return fail(TP_E_BAD_ARG, "normals: slot out of range");
        h[k] = NormalJob{eslots[k], nslots[k], meters[k], frames ? k : -1};
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t jobs_bytes = (sizeof(NormalJob) * count + 255) & ~(size_t)255;
    const size_t need = jobs_bytes + (frames ? sizeof(SphereFrame) * count : 0);
    if (dcap < need) {
        if (dbuf) {
            cudaStreamSynchronize(s);
            cudaFree(dbuf);
        }
        dbuf = nullptr;
        dcap = 0;
        cudaError_t e = cudaMalloc(&dbuf, need);
        if (e != cudaSuccess) return cuda_fail("cudaMalloc (normal jobs)", e);
        dcap = need;
    }
    cudaError_t e = cudaMemcpyAsync(dbuf, h.data(), sizeof(NormalJob) * count, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && frames)
        e = cudaMemcpyAsync(dbuf + jobs_bytes, frames, sizeof(SphereFrame) * count, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail("cudaMemcpyAsync (normal jobs)", e);
    normals_kernel<<<count, 256, 0, s>>>(elev->base, elev->pitch, elev->plane_stride, elev->slot_stride, nrm->base,
                                         nrm->pitch, nrm->plane_stride, nrm->slot_stride,
                                         reinterpret_cast<const NormalJob *>(dbuf),
                                         reinterpret_cast<const SphereFrame *>(dbuf + jobs_bytes), elev->W);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("normals kernel launch", e);
    // the job buffer is reused by the next call: keep the host in step with it
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail("cudaStreamSynchronize (normals)", e);
    return TP_OK;
}

}  // namespace tp

// Kernel-level entry of the normal pass: job k reads elevation slot out_slot and
// writes normal slot normal_slot; with root_quad_size > 0 the tiles lie on the
// sphere of a cube-face terrain (NormalProducer's deform path), else on a plane.
extern "C" int tp_normal_batch(tp_storage *elev, tp_storage *normals, const tp_tile_job *jobs, int n,
                               double root_quad_size, void *stream)
{
    if (!elev || !normals || n < 0 || (n > 0 && !jobs)) return tp::fail(TP_E_BAD_ARG, "tp_normal_batch: bad arguments");
    if (elev->on_device != 1 || elev->channels != 3 || normals->on_device != 1 || normals->channels != 2 ||
        normals->W != elev->W - 4)
        return tp::fail(TP_E_BAD_ARG, "tp_normal_batch: device storages of W (3 channels) and W - 4 (2 channels) needed");
    if (n == 0) return TP_OK;
    std::vector<int> es(n), ns(n);
    std::vector<float> meters(n);
    std::vector<tp::SphereFrame> frames(root_quad_size > 0.0 ? n : 0);
    for (int k = 0; k < n; ++k) {
        const tp_tile_job &j = jobs[k];
        if (j.level < 0 || j.level > 30 || (j.tx >> j.level) != 0 || (j.ty >> j.level) != 0 || j.tx < 0 || j.ty < 0)
            return tp::fail(TP_E_BAD_ARG, "tp_normal_batch: bad quadtree coordinates");
        es[k] = j.out_slot;
        ns[k] = j.normal_slot;
        meters[k] = j.tile_meters;
        if (!(j.tile_meters > 0.0f)) return tp::fail(TP_E_BAD_ARG, "tp_normal_batch: tile_meters must be positive");
        if (root_quad_size > 0.0) tp::sphere_frame(root_quad_size, j.level, j.tx, j.ty, &frames[k]);
    }
    return tp::launch_normals(elev, normals, es.data(), ns.data(), meters.data(), n, stream,
                              root_quad_size > 0.0 ? frames.data() : nullptr);
}
