// Normal tiles from elevation tiles already produced (NormalProducer::doCreateTile,
// NormalProducer.cpp:164-289, flat deformation): the normal tile requested after
// its elevation tile was produced and cached, so the fused frame launch cannot
// make it.  Same arithmetic as the fused kernel's normal phase
// (terrain/examples/terrain1/normalShader.glsl:57-74, point-sampled zm).
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "tp_internal.h"

namespace {

struct NormalJob {
    int eslot, nslot;
    float tile_meters;
};

__global__ void __launch_bounds__(256) normals_kernel(const float *__restrict__ elev, int pitch, long long eplane,
                                                      long long eslot_stride, float *__restrict__ nrm, int npitch,
                                                      long long nplane, long long nslot_stride,
                                                      const NormalJob *__restrict__ jobs, int W)
{
    const NormalJob J = jobs[blockIdx.x];
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
                   int count, void *stream)
{
    if (count <= 0) return TP_OK;
    static std::mutex mu;
    static NormalJob *dbuf = nullptr;
    static int dcap = 0;
    std::lock_guard<std::mutex> lk(mu);
    std::vector<NormalJob> h(count);
    for (int k = 0; k < count; ++k) {
        if (eslots[k] < 0 || eslots[k] >= elev->capacity || nslots[k] < 0 || nslots[k] >= nrm->capacity)
            return fail(TP_E_BAD_ARG, "normals: slot out of range");
        h[k] = NormalJob{eslots[k], nslots[k], meters[k]};
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (dcap < count) {
        if (dbuf) {
            cudaStreamSynchronize(s);
            cudaFree(dbuf);
        }
        dbuf = nullptr;
        dcap = 0;
        cudaError_t e = cudaMalloc(&dbuf, sizeof(NormalJob) * count);
        if (e != cudaSuccess) return cuda_fail("cudaMalloc (normal jobs)", e);
        dcap = count;
    }
    cudaError_t e = cudaMemcpyAsync(dbuf, h.data(), sizeof(NormalJob) * count, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail("cudaMemcpyAsync (normal jobs)", e);
    normals_kernel<<<count, 256, 0, s>>>(elev->base, elev->pitch, elev->plane_stride, elev->slot_stride, nrm->base,
                                         nrm->pitch, nrm->plane_stride, nrm->slot_stride, dbuf, elev->W);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("normals kernel launch", e);
    // the job buffer is reused by the next call: keep the host in step with it
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail("cudaStreamSynchronize (normals)", e);
    return TP_OK;
}

}  // namespace tp
