// Synthetic residual tiles written into residual slots on the device (the
// generator is in tp_synth.h; the host twin below gives the same bits).
#include <cuda_runtime.h>

#include <vector>

#include "tp_internal.h"
#include "tp_synth.h"

namespace {

struct SynthTile {
    int slot;
    uint32_t key;
    float sigma;
};

// one CTA per tile; thread t writes samples t, t + 256, ... of plane 0
__global__ void __launch_bounds__(256) synth_kernel(const SynthTile *tiles, float *base, int W, int pitch,
                                                    long long slot_stride)
{
    const SynthTile T = tiles[blockIdx.x];
    float *out = base + (long long)T.slot * slot_stride;
    const int n = W * W;
    for (int s = threadIdx.x; s < n; s += blockDim.x) {
        const int j = s / W, i = s - j * W;
        out[(long long)j * pitch + i] = __fmul_rn(tp::synth_unit(T.key, (uint32_t)s), T.sigma);
    }
}

}  // namespace

namespace tp {

void synthetic_residual_host(uint32_t seed, int level, int tx, int ty, float sigma, int W, float *out, int pitch)
{
    const uint32_t key = synth_key(seed, level, tx, ty);
    for (int j = 0; j < W; ++j)
        for (int i = 0; i < W; ++i)
            out[i + (size_t)j * pitch] = synth_unit(key, (uint32_t)(i + j * W)) * sigma;
}

int synthetic_residuals_device(tp_storage *s, uint32_t seed, const int *slots, const int *levels, const int *txs,
                               const int *tys, const float *sigmas, int n, void *stream)
{
    if (n == 0) return TP_OK;
    if (!s || s->on_device != 1 || s->channels != 1)
        return fail(TP_E_BAD_ARG, "synthetic residuals: a 1-channel device storage is required");
    std::vector<SynthTile> h((size_t)n);
    for (int k = 0; k < n; ++k) {
        if (slots[k] < 0 || slots[k] >= s->capacity) return fail(TP_E_BAD_ARG, "synthetic residuals: slot out of range");
        h[k] = SynthTile{slots[k], synth_key(seed, levels[k], txs[k], tys[k]), sigmas[k]};
    }
    char *dbuf = nullptr;
    int rc = device_scratch(kScratchSynth, sizeof(SynthTile) * (size_t)n, stream, &dbuf);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(dbuf, h.data(), sizeof(SynthTile) * (size_t)n, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail("cudaMemcpyAsync (synthetic residual tiles)", e);
    synth_kernel<<<n, 256, 0, st>>>(reinterpret_cast<const SynthTile *>(dbuf), s->base, s->W, s->pitch, s->slot_stride);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("synth_kernel launch", e);
    return TP_OK;
}

}  // namespace tp
