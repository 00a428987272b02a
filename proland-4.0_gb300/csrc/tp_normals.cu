// Normal tiles from elevation tiles already produced (NormalProducer::doCreateTile,
// NormalProducer.cpp:164-289): flat tiles requested after their elevation tile
// was produced and cached (same arithmetic as the fused kernel's normal phase,
// terrain/examples/terrain1/normalShader.glsl:57-74, point-sampled zm), and all
// tiles of a spherically deformed terrain (terrain/examples/terrain2/normalShader.glsl).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "tp_internal.h"
#include "tp_trace.h"
#include "tp_div.h"

namespace {

struct NormalJob {
    int eslot, nslot;
    float tile_meters;
    int frame;   // index of the job's spherical frame, -1 for flat deformation
    int pslot;   // parent normal slot for the coarse normals (formats 0/1), -1 for none
    int tx, ty;
    int pad;
};

// Normals in the reference's four formats (demo normalShader.glsl:116-124): 0 = nf, nc
// signed; 1 = the same as 8-bit unsigned (stored as k / 255); 2 = nf signed; 3 = nf
// as 8-bit unsigned.
__device__ __forceinline__ float unorm8(float v)
{
    v = fminf(fmaxf(v, 0.0f), 1.0f);
    return floorf(__fadd_rn(__fmul_rn(v, 255.0f), 0.5f)) / 255.0f;
}

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

// smoothstep(R/32, R/64, size) of getWorldPosition: one value per tile.
__device__ __forceinline__ float sphere_blend(const tp::SphereFrame &f)
{
    const float R = f.R;
    const float e0 = R / 32.0f, e1 = R / 64.0f;  // exact: powers of two
    float s = __fdiv_rn(s_(f.size, e0), s_(e1, e0));
    s = s < 0.0f ? 0.0f : (s > 1.0f ? 1.0f : s);
    return m_(m_(s, s), s_(3.0f, m_(2.0f, s)));
}

// getWorldPosition of terrain2/normalShader.glsl:56-73 (the patch's projective
// mapping onto the sphere), for grid position (u, v) = (un, vn) * n in samples
// (un = u / n and vn = v / n, correctly rounded) and height h; s = sphere_blend(f).
__device__ __forceinline__ void sphere_pos(const tp::SphereFrame &f, float s, float u, float v, float h, float *out)
{
    const float U = s_(1.0f, u), V = s_(1.0f, v);
    const float al[4] = {m_(U, V), m_(u, V), m_(U, v), m_(u, v)};
    const float d = dot4(al, f.L);
    const float rd = __frcp_rn(d);  // the four quotients share the denominator
    float ap[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) ap[k] = tp::div_rcp(m_(al[k], f.L[k]), d, rd);
    float up[3], cp[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        up[r] = dot4(f.N + r * 4, ap);
        cp[r] = dot4(f.C + r * 4, ap);
    }
    const float R = f.R;
    const float len = __fsqrt_rn(dot3(up, up));
    const float k = a_(m_(len, s_(1.0f, s)), s);
    const float hp = __fdiv_rn(a_(h, m_(R, s_(1.0f, k))), k);
#pragma unroll
    for (int r = 0; r < 3; ++r) out[r] = a_(cp[r], m_(hp, up[r]));
}

// m = ceil(2^32 / d) for 2 <= d <= 4096, so that floor(t / d) == umulhi(t, m): with
// m d = 2^32 + e, 0 < e <= d, t m / 2^32 = t / d + t e / (d 2^32), and the last term is
// below 1 / d when t e < 2^32, i.e. for every t below 2^20 (checked exhaustively for
// t < 80000); a band's flattened indices stay below 18 x 4094.
__device__ __forceinline__ uint32_t div_magic(int d) { return 0xFFFFFFFFu / (uint32_t)d + 1u; }

// Rows of world positions per band of normal rows (kSphereBand rows), kept in a
// shared-memory ring of kSphereBand + 2 rows: each grid position is evaluated once
// and read by the four normals around it.
constexpr int kSphereBand = 16;
constexpr int kSphereRing = kSphereBand + 2;

// The ring, then the quotients k / n of the grid coordinates k in [-1, W - 4].
__host__ __device__ constexpr int sphere_smem_floats(int W) { return 3 * kSphereRing * (W - 2) + (W - 2); }

// Positions of grid rows v in [v0, v1) (v in [-1, W - 4]), columns u in [-1, W - 4],
// heights from the zm plane (texel (u + 2, v + 2)), into the ring; qn[k + 1] = k / n.
__device__ __forceinline__ void sphere_rows(const tp::SphereFrame &F, float s, const float *qn,
                                            const float *__restrict__ zm, int pitch, int W, int v0, int v1,
                                            float *ring)
{
    const int PW = W - 2;
    float *X = ring, *Y = ring + kSphereRing * PW, *Z = ring + 2 * kSphereRing * PW;
    const int cnt = (v1 - v0) * PW;
    const uint32_t inv = div_magic(PW);
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const int r = (int)__umulhi((uint32_t)i, inv);  // i / PW
        const int c = i - r * PW, v = v0 + r;            // c = u + 1
        float o[3];
        sphere_pos(F, s, qn[c], qn[v + 1], __ldg(zm + (long long)(v + 2) * pitch + (c + 1)), o);
        const int k = ((v + 1) % kSphereRing) * PW + c;
        X[k] = o[0];
        Y[k] = o[1];
        Z[k] = o[2];
    }
}

// The normal at (p, q) from the ring (terrain2/normalShader.glsl:75-88): the cross
// product of the neighbour differences, normalised, rotated into the tangent frame.
__device__ __forceinline__ void sphere_normal(const tp::SphereFrame &F, const float *ring, int W, int p, int q,
                                              float &vx, float &vy)
{
    const int PW = W - 2;
    const float *X = ring, *Y = ring + kSphereRing * PW, *Z = ring + 2 * kSphereRing * PW;
    const int rq = ((q + 1) % kSphereRing) * PW, rm = (q % kSphereRing) * PW, rp = ((q + 2) % kSphereRing) * PW;
    const int i0 = rq + p, i1 = rq + p + 2, i2 = rm + p + 1, i3 = rp + p + 1;
    const float a[3] = {s_(X[i1], X[i0]), s_(Y[i1], Y[i0]), s_(Z[i1], Z[i0])};
    const float b[3] = {s_(X[i3], X[i2]), s_(Y[i3], Y[i2]), s_(Z[i3], Z[i2])};
    float cr[3] = {s_(m_(a[1], b[2]), m_(a[2], b[1])), s_(m_(a[2], b[0]), m_(a[0], b[2])),
                   s_(m_(a[0], b[1]), m_(a[1], b[0]))};
    const float inv = __frcp_rn(__fsqrt_rn(dot3(cr, cr)));  // RN(1 / s), as 1.0f / s is
    cr[0] = m_(cr[0], inv);
    cr[1] = m_(cr[1], inv);
    cr[2] = m_(cr[2], inv);
    vx = dot3(F.W2T, cr);
    vy = dot3(F.W2T + 3, cr);
}

// Runs the bands of one spherical tile: fills the ring, then calls
// epi(p, q, vx, vy) for every normal sample of the band.
template <class Epi>
__device__ __forceinline__ void sphere_tile(const tp::SphereFrame &F, const float *__restrict__ zm, int pitch, int W,
                                            float *ring, Epi epi)
{
    const int Wn = W - 4;
    const float nn = (float)(W - 5);
    const float s = sphere_blend(F);
    float *qn = ring + 3 * kSphereRing * (W - 2);
    for (int k = threadIdx.x; k < W - 2; k += blockDim.x) qn[k] = __fdiv_rn((float)(k - 1), nn);
    __syncthreads();
    sphere_rows(F, s, qn, zm, pitch, W, -1, min(kSphereBand, Wn) + 1, ring);
    for (int q0 = 0; q0 < Wn; q0 += kSphereBand) {
        const int q1 = min(q0 + kSphereBand, Wn);
        if (q0 > 0) sphere_rows(F, s, qn, zm, pitch, W, q0 + 1, q1 + 1, ring);
        __syncthreads();
        const int cnt = (q1 - q0) * Wn;
        const uint32_t inv = div_magic(Wn);
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
            const int r = (int)__umulhi((uint32_t)i, inv);  // i / Wn
            const int q = q0 + r, p = i - r * Wn;
            float vx, vy;
            sphere_normal(F, ring, W, p, q, vx, vy);
            epi(p, q, vx, vy);
        }
        __syncthreads();
    }
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
        extern __shared__ float ring[];
        __shared__ tp::SphereFrame F;
        if (threadIdx.x == 0) F = frames[J.frame];
        __syncthreads();
        const float *zm = elev + (long long)J.eslot * eslot_stride + 2 * eplane;
        float *nx = nrm + (long long)J.nslot * nslot_stride;
        float *ny = nx + nplane;
        const int Wn = W - 4;
        sphere_tile(F, zm, pitch, W, ring, [&](int p, int q, float vx, float vy) {
            nx[(long long)q * npitch + p] = vx;
            ny[(long long)q * npitch + p] = vy;
        });
        // the pitch padding of each row
        for (int idx = threadIdx.x; idx < Wn * (npitch - Wn); idx += blockDim.x) {
            const int q = idx / (npitch - Wn), p = Wn + idx % (npitch - Wn);
            nx[(long long)q * npitch + p] = 0.0f;
            ny[(long long)q * npitch + p] = 0.0f;
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

// All formats: nf as in the kernel above (flat finite differences or the sphere),
// then nc from the parent normal tile (formats 0/1 above level 0) and the format's
// encoding.  One CTA per tile.
__global__ void __launch_bounds__(256) normals_format_kernel(
    const float *__restrict__ elev, int pitch, long long eplane, long long eslot_stride, float *__restrict__ nrm,
    int npitch, long long nplane, long long nslot_stride, const NormalJob *__restrict__ jobs,
    const tp::SphereFrame *__restrict__ frames, const float *__restrict__ p2t, int W, int format, int g)
{
    const NormalJob J = jobs[blockIdx.x];
    __shared__ tp::SphereFrame F;
    __shared__ float R[9];
    if (threadIdx.x == 0 && J.frame >= 0) F = frames[J.frame];
    if (threadIdx.x < 9) R[threadIdx.x] = (J.frame >= 0 && p2t) ? p2t[9 * blockIdx.x + threadIdx.x] : 0.0f;
    __syncthreads();
    const float *zm = elev + (long long)J.eslot * eslot_stride + 2 * eplane;
    float *o = nrm + (long long)J.nslot * nslot_stride;
    const float *par = J.pslot >= 0 ? nrm + (long long)J.pslot * nslot_stride : nullptr;
    const int Wn = W - 4, n = W - 5;
    const int dxi = (J.tx & 1) * ((Wn - 1) / 2), dyi = (J.ty & 1) * ((Wn - 1) / 2);
    const bool coarse = (format == 0 || format == 1) && par;
    const float h2 = __fmul_rn(2.0f, __fdiv_rn(J.tile_meters, (float)n));
    const float hh = h2 * h2;
    auto emit = [&](int p, int q, float vx, float vy) {
        float cx = vx, cy = vy;
        if (coarse) {
            // the two coarse-mesh vertices g floor(ij / 2g + (1/2, 0)), g floor(ij / 2g + (0, 1/2))
            const int ax = g * ((p + g) / (2 * g)) + dxi, ay = g * (q / (2 * g)) + dyi;
            const int bx = g * (p / (2 * g)) + dxi, by = g * ((q + g) / (2 * g)) + dyi;
            cx = (__ldg(par + (long long)ay * npitch + ax) + __ldg(par + (long long)by * npitch + bx)) * 0.5f;
            cy = (__ldg(par + nplane + (long long)ay * npitch + ax) + __ldg(par + nplane + (long long)by * npitch + bx)) *
                 0.5f;
            if (format == 1) {
                cx = cx * 2.0f - 1.0f;
                cy = cy * 2.0f - 1.0f;
            }
            if (J.frame >= 0 && p2t) {
                const float cz = sqrtf(fmaxf(1.0f - (cx * cx + cy * cy), 0.0f));
                const float rx = R[0] * cx + R[1] * cy + R[2] * cz;
                const float ry = R[3] * cx + R[4] * cy + R[5] * cz;
                cx = rx;
                cy = ry;
            }
        }
        const long long k = (long long)q * npitch + p;
        if (format == 0) {
            o[k] = vx;
            o[nplane + k] = vy;
            o[2 * nplane + k] = cx;
            o[3 * nplane + k] = cy;
        } else if (format == 1) {
            o[k] = unorm8(vx * 0.5f + 0.5f);
            o[nplane + k] = unorm8(vy * 0.5f + 0.5f);
            o[2 * nplane + k] = unorm8(cx * 0.5f + 0.5f);
            o[3 * nplane + k] = unorm8(cy * 0.5f + 0.5f);
        } else if (format == 2) {
            o[k] = vx;
            o[nplane + k] = vy;
        } else {
            o[k] = unorm8(vx * 0.5f + 0.5f);
            o[nplane + k] = unorm8(vy * 0.5f + 0.5f);
        }
    };
    if (J.frame >= 0) {
        extern __shared__ float ring[];
        sphere_tile(F, zm, pitch, W, ring, emit);
        return;
    }
    for (int idx = threadIdx.x; idx < Wn * Wn; idx += blockDim.x) {
        const int q = idx / Wn, p = idx - q * Wn;
        const float *c = zm + (long long)(q + 2) * pitch + (p + 2);
        const float ax = -__fsub_rn(__ldg(c + 1), __ldg(c - 1));
        const float ay = -__fsub_rn(__ldg(c + pitch), __ldg(c - pitch));
        const float inv = rsqrtf(ax * ax + ay * ay + hh);
        emit(p, q, ax * inv, ay * inv);
    }
}

// Dynamic shared memory of a spherical launch (the position ring), with the
// kernel's limit raised when it exceeds the default 48 KB.
int sphere_smem_attr(const void *kernel, int W, size_t *bytes)
{
    *bytes = sizeof(float) * (size_t)sphere_smem_floats(W);
    if (*bytes > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*bytes);
        if (e != cudaSuccess) return tp::cuda_fail("cudaFuncSetAttribute (normals)", e);
    }
    return TP_OK;
}

}  // namespace

namespace tp {

// Normal tiles in any format, with coarse normals from parent normal slots
// (pslots[k] >= 0) and spherical frames / parent-to-tangent rotations when given.
// Jobs of one call must not be each other's parents (launch level by level).
int launch_normals_format(tp_storage *elev, tp_storage *nrm, const int *eslots, const int *nslots, const float *meters,
                          const int *pslots, const int *txs, const int *tys, int count, int format, int grid_mesh,
                          void *stream, const SphereFrame *frames, const float *p2t)
{
    if (count <= 0) return TP_OK;
    if (format < 0 || format > 3 || nrm->channels < ((format <= 1) ? 4 : 2))
        return fail(TP_E_BAD_ARG, "normals: format needs a normal storage of 4 (formats 0, 1) or 2 channels");
    const int Wn = elev->W - 4;
    if (grid_mesh < 1 || (Wn - 1) / grid_mesh < 1) return fail(TP_E_BAD_ARG, "normals: bad grid mesh size");
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    std::vector<NormalJob> h(count);
    for (int k = 0; k < count; ++k) {
        if (eslots[k] < 0 || eslots[k] >= elev->capacity || nslots[k] < 0 || nslots[k] >= nrm->capacity ||
            (pslots && (pslots[k] >= nrm->capacity || pslots[k] == nslots[k])))
            return fail(TP_E_BAD_ARG, "normals: slot out of range");
        h[k] = NormalJob{eslots[k], nslots[k], meters[k], frames ? k : -1, pslots ? pslots[k] : -1, txs[k], tys[k], 0};
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t jobs_bytes = (sizeof(NormalJob) * count + 255) & ~(size_t)255;
    const size_t frames_bytes = frames ? ((sizeof(SphereFrame) * count + 255) & ~(size_t)255) : 0;
    const size_t need = jobs_bytes + frames_bytes + (p2t ? sizeof(float) * 9 * count : 0);
    char *dbuf = nullptr;
    {
        int rc = device_scratch(kScratchNormalFormats, need, stream, &dbuf);
        if (rc) return rc;
    }
    cudaError_t e = cudaMemcpyAsync(dbuf, h.data(), sizeof(NormalJob) * count, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && frames)
        e = cudaMemcpyAsync(dbuf + jobs_bytes, frames, sizeof(SphereFrame) * count, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && p2t)
        e = cudaMemcpyAsync(dbuf + jobs_bytes + frames_bytes, p2t, sizeof(float) * 9 * count, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail("cudaMemcpyAsync (normal jobs)", e);
    size_t smem = 0;
    if (frames) {
        int rc = sphere_smem_attr(reinterpret_cast<const void *>(normals_format_kernel), elev->W, &smem);
        if (rc) return rc;
    }
    normals_format_kernel<<<count, 256, smem, s>>>(
        elev->base, elev->pitch, elev->plane_stride, elev->slot_stride, nrm->base, nrm->pitch, nrm->plane_stride,
        nrm->slot_stride, reinterpret_cast<const NormalJob *>(dbuf),
        reinterpret_cast<const SphereFrame *>(dbuf + jobs_bytes),
        p2t ? reinterpret_cast<const float *>(dbuf + jobs_bytes + frames_bytes) : nullptr, elev->W, format,
        (Wn - 1) / grid_mesh);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("normals kernel launch", e);
    e = cudaStreamSynchronize(s);  // the job buffer is reused by the next call
    if (e != cudaSuccess) return cuda_fail("cudaStreamSynchronize (normals)", e);
    return TP_OK;
}

int launch_normals(tp_storage *elev, tp_storage *nrm, const int *eslots, const int *nslots, const float *meters,
                   int count, void *stream, const SphereFrame *frames)
{
    if (count <= 0) return TP_OK;
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    std::vector<NormalJob> h(count);
    for (int k = 0; k < count; ++k) {
        if (eslots[k] < 0 || eslots[k] >= elev->capacity || nslots[k] < 0 || nslots[k] >= nrm->capacity)
            return fail(TP_E_BAD_ARG, "normals: slot out of range");
        h[k] = NormalJob{eslots[k], nslots[k], meters[k], frames ? k : -1, -1, 0, 0, 0};
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t jobs_bytes = (sizeof(NormalJob) * count + 255) & ~(size_t)255;
    const size_t need = jobs_bytes + (frames ? sizeof(SphereFrame) * count : 0);
    char *dbuf = nullptr;
    {
        int rc = device_scratch(kScratchNormals, need, stream, &dbuf);
        if (rc) return rc;
    }
    cudaError_t e = cudaMemcpyAsync(dbuf, h.data(), sizeof(NormalJob) * count, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && frames)
        e = cudaMemcpyAsync(dbuf + jobs_bytes, frames, sizeof(SphereFrame) * count, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail("cudaMemcpyAsync (normal jobs)", e);
    size_t smem = 0;
    if (frames) {
        int rc = sphere_smem_attr(reinterpret_cast<const void *>(normals_kernel), elev->W, &smem);
        if (rc) return rc;
    }
    normals_kernel<<<count, 256, smem, s>>>(elev->base, elev->pitch, elev->plane_stride, elev->slot_stride, nrm->base,
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
    tp::TraceScope trace("normal batch", -1);
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

// Kernel-level normals in any format: jobs as tp_normal_batch; parent_normal_slots[k]
// (or NULL) names the slot holding the parent normal tile for the coarse normals of
// formats 0 and 1.  Jobs run level by level, so a batch may hold parents and children.
extern "C" int tp_normal_batch_format(tp_storage *elev, tp_storage *normals, const tp_tile_job *jobs, int n,
                                      double root_quad_size, int format, const int *parent_normal_slots,
                                      int grid_mesh, void *stream)
{
    if (!elev || !normals || n < 0 || (n > 0 && !jobs) || format < 0 || format > 3)
        return tp::fail(TP_E_BAD_ARG, "tp_normal_batch_format: bad arguments");
    if (elev->on_device != 1 || elev->channels != 3 || normals->on_device != 1 || normals->W != elev->W - 4)
        return tp::fail(TP_E_BAD_ARG, "tp_normal_batch_format: device storages of widths W and W - 4 needed");
    std::vector<int> order(n);
    for (int k = 0; k < n; ++k) {
        const tp_tile_job &j = jobs[k];
        if (j.level < 0 || j.level > 30 || j.tx < 0 || j.ty < 0 || (j.tx >> j.level) != 0 || (j.ty >> j.level) != 0 ||
            !(j.tile_meters > 0.0f))
            return tp::fail(TP_E_BAD_ARG, "tp_normal_batch_format: bad job");
        order[k] = k;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return jobs[a].level < jobs[b].level; });
    size_t k = 0;
    while (k < order.size()) {
        const int level = jobs[order[k]].level;
        std::vector<int> es, ns, ps, txs, tys;
        std::vector<float> meters, p2t;
        std::vector<tp::SphereFrame> frames;
        for (; k < order.size() && jobs[order[k]].level == level; ++k) {
            const tp_tile_job &j = jobs[order[k]];
            es.push_back(j.out_slot);
            ns.push_back(j.normal_slot);
            ps.push_back(parent_normal_slots && j.level > 0 ? parent_normal_slots[order[k]] : -1);
            txs.push_back(j.tx);
            tys.push_back(j.ty);
            meters.push_back(j.tile_meters);
            if (root_quad_size > 0.0) {
                frames.emplace_back();
                tp::sphere_frame(root_quad_size, j.level, j.tx, j.ty, &frames.back());
                p2t.resize(p2t.size() + 9, 0.0f);
                if (j.level > 0) tp::parent_to_tangent(root_quad_size, j.level, j.tx, j.ty, &p2t[p2t.size() - 9]);
            }
        }
        int rc = tp::launch_normals_format(elev, normals, es.data(), ns.data(), meters.data(), ps.data(), txs.data(),
                                           tys.data(), (int)es.size(), format, grid_mesh, stream,
                                           root_quad_size > 0.0 ? frames.data() : nullptr,
                                           root_quad_size > 0.0 ? p2t.data() : nullptr);
        if (rc) return rc;
    }
    return TP_OK;
}

namespace {

// Random (x, y) pairs: sign, exponent in [-64, 63] and mantissa from a counter hash,
// and for every pair the quotient of div_rcp against __fdiv_rn.
__device__ __forceinline__ uint32_t st_hash(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ float st_float(uint32_t h, uint32_t m)
{
    return __uint_as_float((h & 0x80000000u) | ((uint32_t)(127 - 64 + (int)((h >> 24) & 127)) << 23) | (m & 0x7FFFFFu));
}

__global__ void sphere_division_check_kernel(uint64_t n, uint32_t seed, unsigned long long *mismatches,
                                             unsigned long long *first)
{
    unsigned long long bad = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t a = st_hash((uint32_t)i ^ seed), b = st_hash((uint32_t)(i >> 32) + 0x9E3779B9u * (uint32_t)i + seed);
        const float x = st_float(a, st_hash(a + 1u)), y = st_float(b, st_hash(b + 7u));
        const float f = tp::div_rcp(x, y, __frcp_rn(y)), e = __fdiv_rn(x, y);
        if (__float_as_uint(f) != __float_as_uint(e)) {
            ++bad;
            atomicMin(first, (unsigned long long)i);
        }
    }
    if (bad) atomicAdd(mismatches, bad);
}

// Every positive x (all 2^31 bit patterns below +inf) against one divisor y.
__global__ void sphere_division_sweep_kernel(float y, unsigned long long *mismatches, unsigned long long *first)
{
    unsigned long long bad = 0;
    const float z = __frcp_rn(y);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < 0x7F800000ull; b += stride) {
        const float x = __uint_as_float((uint32_t)b);
        const float f = tp::div_rcp(x, y, z), e = __fdiv_rn(x, y);
        if (__float_as_uint(f) != __float_as_uint(e)) {
            ++bad;
            atomicMin(first, (unsigned long long)b);
        }
    }
    if (bad) atomicAdd(mismatches, bad);
}

}  // namespace

extern "C" int tp_sphere_division_self_test(unsigned long long n_random, unsigned seed, const float *divisors,
                                            int n_divisors, unsigned long long *mismatches,
                                            unsigned long long *first_mismatch)
{
    if (!mismatches || n_divisors < 0 || (n_divisors > 0 && !divisors))
        return tp::fail(TP_E_BAD_ARG, "tp_sphere_division_self_test: bad arguments");
    unsigned long long *d = nullptr;
    cudaError_t e = cudaMalloc(&d, 2 * sizeof(unsigned long long));
    if (e != cudaSuccess) return tp::cuda_fail("cudaMalloc (division self-test)", e);
    const unsigned long long init[2] = {0ull, ~0ull};
    e = cudaMemcpy(d, init, sizeof init, cudaMemcpyHostToDevice);
    const int grid = tp::device_sm_count() * 8;
    if (e == cudaSuccess && n_random > 0) {
        sphere_division_check_kernel<<<grid, 256>>>(n_random, seed, d, d + 1);
        e = cudaGetLastError();
    }
    for (int k = 0; k < n_divisors && e == cudaSuccess; ++k) {
        sphere_division_sweep_kernel<<<grid, 256>>>(divisors[k], d, d + 1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    unsigned long long out[2] = {0ull, 0ull};
    if (e == cudaSuccess) e = cudaMemcpy(out, d, sizeof out, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return tp::cuda_fail("division self-test", e);
    *mismatches = out[0];
    if (first_mismatch) *first_mismatch = out[1];
    return TP_OK;
}
