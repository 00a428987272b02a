// Host side of the learned residual predictor: parameters, activation buffers,
// the forward / backward / Adam sequence of kernel launches, and the step that
// writes predicted residual tiles into a residual storage for the elevation
// kernel.  The net has no counterpart in the reference (it stands in for stored
// residuals below the finest level of a terrain's residual pyramid).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "tp_internal.h"
#include "tp_trace.h"
#include "tp_learned.h"

using namespace tp::learned;

struct tp_learned {
    int W = 0, cap = 0, tiles_x = 0, tiles_y = 0;
    int nparams = 0;
    int woff[kLayers] = {}, boff[kLayers] = {}, emb_off = 0;
    float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr, *mask = nullptr;
    uint8_t *fwd[kLayers] = {}, *bwd[kLayers] = {};
    float *sigma_in = nullptr, *sigma_out = nullptr;
    __nv_bfloat16 *x0 = nullptr, *act[4] = {}, *z[4] = {}, *dz4 = nullptr, *dza = nullptr, *dzb = nullptr;
    float *pred = nullptr, *loss = nullptr, *up = nullptr, *mean = nullptr;
    int *levels = nullptr, *status = nullptr, *aux = nullptr;
    CUtensorMap h_x0, h_act[4], h_dz4, h_dza, h_dzb;  // 10 x 18 halo boxes (convolutions)
    CUtensorMap b_x0, b_act[4], b_dz4, b_dza, b_dzb;  // 8 x 16 block boxes (weight gradients)
    CUtensorMap w_act[4];                             // 12 x 20 halo boxes (fused pairs' inputs)
    bool fused = false;  // inference runs layers (0, 1) and (2, 3) as fused pairs (slower on GB300, kept selectable)
    int step = 0, nimg = 0;
    bool packed = false, trained_forward = false;
    std::vector<void *> allocs;
};

namespace {

template <typename T>
int dev_alloc(tp_learned *net, T **p, size_t count)
{
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return tp::cuda_fail("learned: cudaMalloc", e);
    e = cudaMemset(q, 0, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return tp::cuda_fail("learned: cudaMemset", e);
    net->allocs.push_back(q);
    *p = static_cast<T *>(q);
    return TP_OK;
}

void free_all(tp_learned *net)
{
    for (void *p : net->allocs) cudaFree(p);
    net->allocs.clear();
}

int pack(tp_learned *net, cudaStream_t s)
{
    for (int l = 0; l < kLayers; ++l) launch_pack(net->params + net->woff[l], kCin[l], kCout[l], net->fwd[l], net->bwd[l], s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return tp::cuda_fail("learned: weight packing", e);
    net->packed = true;
    return TP_OK;
}

int check_status(tp_learned *net, cudaStream_t s)
{
    int st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, net->status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return tp::cuda_fail("learned: stream", e);
    if (st != 0) {
        cudaMemsetAsync(net->status, 0, sizeof(int), s);
        return tp::fail(st, "learned: a kernel gave up waiting for its tensor-core or TMA work");
    }
    return TP_OK;
}

ConvLaunch conv_args(tp_learned *net, int n)
{
    ConvLaunch a;
    std::memset(&a, 0, sizeof a);
    a.W = net->W;
    a.nimg = n;
    a.tiles_x = net->tiles_x;
    a.tiles_y = net->tiles_y;
    a.level = net->levels;
    a.status = net->status;
    return a;
}

WgradLaunch wgrad_args(tp_learned *net, int l)
{
    WgradLaunch a;
    std::memset(&a, 0, sizeof a);
    a.W = net->W;
    a.nimg = net->nimg;
    a.tiles_x = net->tiles_x;
    a.tiles_y = net->tiles_y;
    a.gw = net->grads + net->woff[l];
    a.gb = net->grads + net->boff[l];
    a.gemb = l == 0 ? net->grads + net->emb_off : nullptr;
    a.level = net->levels;
    a.status = net->status;
    return a;
}

int forward(tp_learned *net, int n, bool training, cudaStream_t s)
{
    if (!net->packed) {
        int rc = pack(net, s);
        if (rc) return rc;
    }
    // training keeps the first layer's input image (its weight gradient reads it);
    // inference makes the input channels inside the first convolution
    if (training) launch_prep(net->up, net->levels, net->sigma_in, net->sigma_out, net->W, n, net->x0, s);
    else launch_means(net->up, net->W, n, net->mean, s);
    if (!training && net->fused) {
        // layers 0 + 1 and 2 + 3 as fused pairs (their hidden activations stay on chip),
        // then the last layer
        for (int pair = 0; pair < 2; ++pair) {
            FusedLaunch f;
            std::memset(&f, 0, sizeof f);
            f.W = net->W;
            f.nimg = n;
            f.tiles_x = net->tiles_x;
            f.tiles_y = (net->W + kFusedBlockY - 1) / kFusedBlockY;
            f.level = net->levels;
            f.status = net->status;
            const int la = 2 * pair, lb = la + 1;
            f.wpack_a = net->fwd[la];
            f.wpack_b = net->fwd[lb];
            f.bias_a = net->params + net->boff[la];
            f.bias_b = net->params + net->boff[lb];
            f.emb = la == 0 ? net->params + net->emb_off : nullptr;
            f.out = net->act[lb];
            f.up = net->up;
            f.mean = net->mean;
            f.sigma_in = net->sigma_in;
            f.sigma_out = net->sigma_out;
            int rc = launch_fused(pair == 0, f, &net->w_act[pair == 0 ? 0 : la - 1], s);
            if (rc) return rc;
        }
        ConvLaunch a = conv_args(net, n);
        a.wpack = net->fwd[kLayers - 1];
        a.bias = net->params + net->boff[kLayers - 1];
        a.out_f32 = net->pred;
        int rc = launch_conv(kCin[kLayers - 1], kCout[kLayers - 1], kLast, a, &net->h_act[kLayers - 2], s);
        if (rc) return rc;
        net->nimg = n;
        net->trained_forward = false;
        return TP_OK;
    }
    const CUtensorMap *in[kLayers] = {&net->h_x0, &net->h_act[0], &net->h_act[1], &net->h_act[2], &net->h_act[3]};
    for (int l = 0; l < kLayers; ++l) {
        ConvLaunch a = conv_args(net, n);
        a.wpack = net->fwd[l];
        a.bias = net->params + net->boff[l];
        if (l < kLayers - 1) {
            a.emb = l == 0 ? net->params + net->emb_off : nullptr;
            a.out = net->act[l];
            a.zsave = training ? net->z[l] : nullptr;
        } else {
            a.out_f32 = net->pred;
        }
        int mode = l < kLayers - 1 ? kHidden : kLast;
        if (l == 0 && !training) {
            mode = kFirst;
            a.up = net->up;
            a.mean = net->mean;
            a.sigma_in = net->sigma_in;
            a.sigma_out = net->sigma_out;
        }
        int rc = launch_conv(kCin[l], kCout[l], mode, a, in[l], s);
        if (rc) return rc;
    }
    net->nimg = n;
    net->trained_forward = training;
    return TP_OK;
}

int upload_levels(tp_learned *net, const int *levels, int n, cudaStream_t s)
{
    cudaError_t e = cudaMemcpyAsync(net->levels, levels, sizeof(int) * n, cudaMemcpyHostToDevice, s);
    return e == cudaSuccess ? TP_OK : tp::cuda_fail("learned: level upload", e);
}

int check_levels(const int *levels, int n)
{
    for (int i = 0; i < n; ++i)
        if (levels[i] < 0 || levels[i] >= kLevels) return tp::fail(TP_E_BAD_ARG, "learned: level outside the embedding table");
    return TP_OK;
}

}  // namespace

extern "C" int tp_learned_create(int tile_width, int max_batch, tp_learned **out)
{
    if (!out) return tp::fail(TP_E_BAD_ARG, "tp_learned_create: out is NULL");
    *out = nullptr;
    if (tile_width < 8 || tile_width > 1024 || max_batch < 1) return tp::fail(TP_E_BAD_ARG, "tp_learned_create: bad sizes");
    if (!tp_device_available()) return tp::fail(TP_E_NO_DEVICE, "no CUDA device");
    tp_learned *net = new tp_learned;
    net->W = tile_width;
    net->cap = max_batch;
    net->tiles_x = (tile_width + kBlockX - 1) / kBlockX;
    net->tiles_y = (tile_width + kBlockY - 1) / kBlockY;
    int off = 0;
    for (int l = 0; l < kLayers; ++l) {
        net->woff[l] = off;
        off += kCout[l] * 9 * kCin[l];
        net->boff[l] = off;
        off += kCout[l];
    }
    net->emb_off = off;
    off += kLevels * kCout[0];
    net->nparams = off;
    const size_t px = (size_t)(tile_width + 2) * (tile_width + 2) * max_batch;
    const size_t tile = (size_t)tile_width * tile_width * max_batch;
    int rc = TP_OK;
    auto A = [&](auto **p, size_t count) {
        if (rc == TP_OK) rc = dev_alloc(net, p, count);
    };
    A(&net->params, net->nparams);
    A(&net->grads, net->nparams);
    A(&net->m, net->nparams);
    A(&net->v, net->nparams);
    A(&net->mask, net->nparams);
    for (int l = 0; l < kLayers; ++l) {
        A(&net->fwd[l], (size_t)9 * kCin[l] * kCout[l] * 2);
        A(&net->bwd[l], (size_t)9 * kCin[l] * kCout[l] * 2);
    }
    A(&net->sigma_in, kLevels);
    A(&net->sigma_out, kLevels);
    A(&net->x0, px * 16);
    for (int l = 0; l < 4; ++l) {
        A(&net->act[l], px * 32);
        A(&net->z[l], px * 32);
    }
    A(&net->dz4, px * 16);
    A(&net->dza, px * 32);
    A(&net->dzb, px * 32);
    A(&net->pred, tile);
    A(&net->up, tile);
    A(&net->mean, max_batch);
    A(&net->loss, 1);
    A(&net->levels, max_batch);
    A(&net->status, 1);
    A(&net->aux, (size_t)4 * max_batch);
    if (rc == TP_OK) {
        const int W = tile_width, B = max_batch;
        auto M = [&](void *base, int ch, CUtensorMap *h, CUtensorMap *b) {
            if (rc == TP_OK) rc = encode_act_map(base, W, ch, B, kBlockX + 2, kBlockY + 2, h);
            if (rc == TP_OK) rc = encode_act_map(base, W, ch, B, kBlockX, kBlockY, b);
        };
        M(net->x0, 16, &net->h_x0, &net->b_x0);
        for (int l = 0; l < 4; ++l) M(net->act[l], 32, &net->h_act[l], &net->b_act[l]);
        for (int l = 0; l < 4; ++l)
            if (rc == TP_OK) rc = encode_act_map(net->act[l], W, 32, B, kWideX, kWideY, &net->w_act[l]);
        M(net->dz4, 16, &net->h_dz4, &net->b_dz4);
        M(net->dza, 32, &net->h_dza, &net->b_dza);
        M(net->dzb, 32, &net->h_dzb, &net->b_dzb);
    }
    if (rc == TP_OK) {  // unit sigmas until the caller sets the data's
        std::vector<float> one(kLevels, 1.0f);
        cudaMemcpy(net->sigma_in, one.data(), sizeof(float) * kLevels, cudaMemcpyHostToDevice);
        cudaMemcpy(net->sigma_out, one.data(), sizeof(float) * kLevels, cudaMemcpyHostToDevice);
    }
    if (rc != TP_OK) {
        free_all(net);
        delete net;
        return rc;
    }
    *out = net;
    return tp_learned_init(net, 1);
}

extern "C" int tp_learned_destroy(tp_learned *net)
{
    if (!net) return TP_OK;
    cudaDeviceSynchronize();
    free_all(net);
    delete net;
    return TP_OK;
}

extern "C" int tp_learned_param_count(const tp_learned *net) { return net ? net->nparams : 0; }

// He-normal weights over the used input channels, zero biases and embedding; the
// padded channels (inputs 4..15 of layer 0, outputs 1..15 of the last layer) stay
// zero through training (their mask is 0).
extern "C" int tp_learned_init(tp_learned *net, uint32_t seed)
{
    if (!net) return tp::fail(TP_E_BAD_ARG, "tp_learned_init: net is NULL");
    std::mt19937 rng(seed);
    std::vector<float> p(net->nparams, 0.0f), mask(net->nparams, 1.0f);
    for (int l = 0; l < kLayers; ++l) {
        const int cin = kCin[l], cout = kCout[l];
        const int used_in = l == 0 ? kInputChannels : cin;
        const int used_out = l == kLayers - 1 ? 1 : cout;
        std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (9.0f * used_in)) * (l == kLayers - 1 ? 0.1f : 1.0f));
        for (int co = 0; co < cout; ++co)
            for (int t = 0; t < 9; ++t)
                for (int ci = 0; ci < cin; ++ci) {
                    const size_t i = net->woff[l] + ((size_t)co * 9 + t) * cin + ci;
                    const bool used = co < used_out && ci < used_in;
                    p[i] = used ? nd(rng) : 0.0f;
                    mask[i] = used ? 1.0f : 0.0f;
                }
        for (int co = 0; co < cout; ++co) mask[net->boff[l] + co] = co < used_out ? 1.0f : 0.0f;
    }
    cudaError_t e = cudaMemcpy(net->params, p.data(), sizeof(float) * p.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(net->mask, mask.data(), sizeof(float) * mask.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(net->m, 0, sizeof(float) * net->nparams);
    if (e == cudaSuccess) e = cudaMemset(net->v, 0, sizeof(float) * net->nparams);
    if (e != cudaSuccess) return tp::cuda_fail("tp_learned_init", e);
    net->step = 0;
    net->packed = false;
    return TP_OK;
}

extern "C" int tp_learned_get_params(tp_learned *net, float *host, int count)
{
    if (!net || !host || count != net->nparams) return tp::fail(TP_E_BAD_ARG, "tp_learned_get_params: bad arguments");
    cudaError_t e = cudaMemcpy(host, net->params, sizeof(float) * count, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? TP_OK : tp::cuda_fail("tp_learned_get_params", e);
}

extern "C" int tp_learned_set_params(tp_learned *net, const float *host, int count)
{
    if (!net || !host || count != net->nparams) return tp::fail(TP_E_BAD_ARG, "tp_learned_set_params: bad arguments");
    cudaError_t e = cudaMemcpy(net->params, host, sizeof(float) * count, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return tp::cuda_fail("tp_learned_set_params", e);
    net->packed = false;
    return TP_OK;
}

extern "C" int tp_learned_get_grads(tp_learned *net, float *host, int count)
{
    if (!net || !host || count != net->nparams) return tp::fail(TP_E_BAD_ARG, "tp_learned_get_grads: bad arguments");
    cudaError_t e = cudaMemcpy(host, net->grads, sizeof(float) * count, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? TP_OK : tp::cuda_fail("tp_learned_get_grads", e);
}

extern "C" int tp_learned_set_fused(tp_learned *net, int on)
{
    if (!net) return tp::fail(TP_E_BAD_ARG, "tp_learned_set_fused: net is NULL");
    net->fused = on != 0;
    return TP_OK;
}

extern "C" int tp_learned_get_state(tp_learned *net, float *m, float *v, int count, int *step)
{
    if (!net || !m || !v || !step || count != net->nparams) return tp::fail(TP_E_BAD_ARG, "tp_learned_get_state: bad arguments");
    cudaError_t e = cudaMemcpy(m, net->m, sizeof(float) * count, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(v, net->v, sizeof(float) * count, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return tp::cuda_fail("tp_learned_get_state", e);
    *step = net->step;
    return TP_OK;
}

extern "C" int tp_learned_set_state(tp_learned *net, const float *m, const float *v, int count, int step)
{
    if (!net || !m || !v || count != net->nparams || step < 0)
        return tp::fail(TP_E_BAD_ARG, "tp_learned_set_state: bad arguments");
    cudaError_t e = cudaMemcpy(net->m, m, sizeof(float) * count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(net->v, v, sizeof(float) * count, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return tp::cuda_fail("tp_learned_set_state", e);
    net->step = step;
    return TP_OK;
}

extern "C" int tp_learned_get_sigmas(tp_learned *net, float *sigma_in, float *sigma_out, int nlevels)
{
    if (!net || !sigma_in || !sigma_out || nlevels < 1 || nlevels > kLevels)
        return tp::fail(TP_E_BAD_ARG, "tp_learned_get_sigmas: bad arguments");
    cudaError_t e = cudaMemcpy(sigma_in, net->sigma_in, sizeof(float) * nlevels, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(sigma_out, net->sigma_out, sizeof(float) * nlevels, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? TP_OK : tp::cuda_fail("tp_learned_get_sigmas", e);
}

extern "C" int tp_learned_set_sigmas(tp_learned *net, const float *sigma_in, const float *sigma_out, int nlevels)
{
    if (!net || !sigma_in || !sigma_out || nlevels < 1 || nlevels > kLevels)
        return tp::fail(TP_E_BAD_ARG, "tp_learned_set_sigmas: bad arguments");
    for (int i = 0; i < nlevels; ++i)
        if (!(sigma_in[i] > 0.0f) || !(sigma_out[i] > 0.0f)) return tp::fail(TP_E_BAD_ARG, "tp_learned_set_sigmas: sigmas must be positive");
    cudaError_t e = cudaMemcpy(net->sigma_in, sigma_in, sizeof(float) * nlevels, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(net->sigma_out, sigma_out, sizeof(float) * nlevels, cudaMemcpyHostToDevice);
    return e == cudaSuccess ? TP_OK : tp::cuda_fail("tp_learned_set_sigmas", e);
}

extern "C" int tp_learned_forward(tp_learned *net, const float *up_dev, const int *levels, int n, int training,
                                  float *out_dev, void *stream)
{
    tp::TraceScope trace("learned forward", tp::kPhLearned);
    if (!net || !up_dev || !levels || n < 1 || n > net->cap) return tp::fail(TP_E_BAD_ARG, "tp_learned_forward: bad arguments");
    int rc = check_levels(levels, n);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    rc = upload_levels(net, levels, n, s);
    if (rc) return rc;
    cudaError_t e = cudaMemcpyAsync(net->up, up_dev, sizeof(float) * net->W * net->W * n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return tp::cuda_fail("tp_learned_forward: input copy", e);
    rc = forward(net, n, training != 0, s);
    if (rc) return rc;
    if (out_dev) launch_scale_out(net->pred, net->levels, net->sigma_out, net->W, n, out_dev, s);
    // an inference pass is left running on the stream (passes in a row overlap their launch
    // gaps); its kernels' failures are reported by the next call that synchronises
    return training ? check_status(net, s) : TP_OK;
}

extern "C" int tp_learned_check(tp_learned *net, void *stream)
{
    if (!net) return tp::fail(TP_E_BAD_ARG, "tp_learned_check: bad arguments");
    return check_status(net, static_cast<cudaStream_t>(stream));
}

extern "C" int tp_learned_backward(tp_learned *net, const float *target_dev, float *loss, void *stream)
{
    tp::TraceScope trace("learned backward", tp::kPhLearned);
    if (!net || !target_dev) return tp::fail(TP_E_BAD_ARG, "tp_learned_backward: bad arguments");
    if (!net->trained_forward || net->nimg < 1)
        return tp::fail(TP_E_BAD_ARG, "tp_learned_backward: needs a forward pass with training = 1 first");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int n = net->nimg;
    cudaError_t e = cudaMemsetAsync(net->grads, 0, sizeof(float) * net->nparams, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(net->loss, 0, sizeof(float), s);
    if (e != cudaSuccess) return tp::cuda_fail("tp_learned_backward: clear", e);
    launch_loss(net->pred, target_dev, net->levels, net->sigma_out, net->W, n, net->dz4, net->loss, s);
    // layer by layer, last first: weight gradient from (input, dZ), then dZ of the layer below
    const CUtensorMap *xin[kLayers] = {&net->b_x0, &net->b_act[0], &net->b_act[1], &net->b_act[2], &net->b_act[3]};
    __nv_bfloat16 *dz[kLayers] = {net->dzb, net->dza, net->dzb, net->dza, net->dz4};
    const CUtensorMap *dzh[kLayers] = {&net->h_dzb, &net->h_dza, &net->h_dzb, &net->h_dza, &net->h_dz4};
    const CUtensorMap *dzbx[kLayers] = {&net->b_dzb, &net->b_dza, &net->b_dzb, &net->b_dza, &net->b_dz4};
    for (int l = kLayers - 1; l >= 0; --l) {
        int rc = launch_wgrad(kCin[l], kCout[l], wgrad_args(net, l), xin[l], dzbx[l], s);
        if (rc) return rc;
        if (l == 0) break;
        ConvLaunch a = conv_args(net, n);
        a.wpack = net->bwd[l];
        a.zprev = net->z[l - 1];
        a.out = dz[l - 1];
        rc = launch_conv(kCout[l], kCin[l], kBackData, a, dzh[l], s);
        if (rc) return rc;
    }
    int rc = check_status(net, s);
    if (rc) return rc;
    if (loss) {
        float v = 0.0f;
        e = cudaMemcpy(&v, net->loss, sizeof(float), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return tp::cuda_fail("tp_learned_backward: loss", e);
        *loss = v / ((float)net->W * net->W * n);
    }
    return TP_OK;
}

extern "C" int tp_learned_adam(tp_learned *net, float lr, void *stream)
{
    tp::TraceScope trace("learned adam", tp::kPhLearned);
    if (!net || !(lr > 0.0f)) return tp::fail(TP_E_BAD_ARG, "tp_learned_adam: bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ++net->step;
    launch_adam(net->params, net->grads, net->m, net->v, net->mask, net->nparams, lr, 0.9f, 0.999f, 1e-8f, net->step, s);
    return pack(net, s);
}

extern "C" int tp_learned_gather(tp_learned *net, const float *up_src, const float *res_src, int n_src, const int *src,
                                 const int *dihedral, int n, float *up_out, float *res_out, void *stream)
{
    if (!net || !up_src || !res_src || !src || !dihedral || !up_out || !res_out || n < 1 || n > net->cap)
        return tp::fail(TP_E_BAD_ARG, "tp_learned_gather: bad arguments");
    for (int i = 0; i < n; ++i)
        if (src[i] < 0 || src[i] >= n_src || dihedral[i] < 0 || dihedral[i] > 7)
            return tp::fail(TP_E_BAD_ARG, "tp_learned_gather: source index or symmetry out of range");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(net->aux, src, sizeof(int) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(net->aux + n, dihedral, sizeof(int) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return tp::cuda_fail("tp_learned_gather: upload", e);
    launch_gather(up_src, res_src, net->aux, net->aux + n, net->W, n, up_out, res_out, s);
    e = cudaGetLastError();
    return e == cudaSuccess ? TP_OK : tp::cuda_fail("tp_learned_gather", e);
}

extern "C" int tp_learned_predict_residuals(tp_learned *net, tp_storage *elev, const tp_tile_job *jobs, int n,
                                            tp_storage *residuals, void *stream)
{
    tp::TraceScope trace("learned residuals", tp::kPhLearned);
    if (!net || !elev || !jobs || !residuals || n < 1 || n > net->cap)
        return tp::fail(TP_E_BAD_ARG, "tp_learned_predict_residuals: bad arguments");
    if (elev->on_device != 1 || elev->channels != 3 || elev->W != net->W || residuals->on_device != 1 ||
        residuals->channels != 1 || residuals->W != net->W)
        return tp::fail(TP_E_BAD_ARG, "tp_learned_predict_residuals: storages must be device storages of the net's width");
    std::vector<int> h((size_t)4 * n), lv(n);
    for (int i = 0; i < n; ++i) {
        const tp_tile_job &j = jobs[i];
        if (j.level < 1 || j.parent_slot < 0 || j.parent_slot >= elev->capacity || j.residual_slot < 0 ||
            j.residual_slot >= residuals->capacity)
            return tp::fail(TP_E_BAD_ARG, "tp_learned_predict_residuals: each job needs a resident parent and a residual slot");
        h[i] = j.parent_slot;
        h[n + i] = j.tx;
        h[2 * n + i] = j.ty;
        h[3 * n + i] = j.residual_slot;
        lv[i] = j.level;
    }
    int rc = check_levels(lv.data(), n);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(net->aux, h.data(), sizeof(int) * 4 * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return tp::cuda_fail("tp_learned_predict_residuals: upload", e);
    rc = upload_levels(net, lv.data(), n, s);
    if (rc) return rc;
    launch_upsample(elev->base, elev->pitch, elev->plane_stride, elev->slot_stride, net->aux, net->aux + n,
                    net->aux + 2 * n, net->W, n, net->up, s);
    rc = forward(net, n, false, s);
    if (rc) return rc;
    launch_store_residuals(net->pred, net->levels, net->sigma_out, net->W, n, residuals->base, residuals->pitch,
                           residuals->slot_stride, net->aux + 3 * n, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return tp::cuda_fail("tp_learned_predict_residuals", e);
    // the host copies of the slot and level arrays must outlive the uploads
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return tp::cuda_fail("tp_learned_predict_residuals", e);
    return check_status(net, s);
}
