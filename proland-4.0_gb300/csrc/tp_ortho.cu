// Ortho (colour) tile kernel for sm_103a: OrthoProducer::doCreateTile
// (terrain/.../ortho/OrthoProducer.cpp:292-382) with its upsample shader
// (terrain/examples/terrain3/upsampleOrthoShader.glsl) for every tile of a batch,
// in one persistent launch.
//
// Texels are RGBA8 packed in 32-bit words (R in the low byte).  Per tile a CTA
// stages the parent window (the (W/2 + 2)^2 parent texels the 2x upsample reads)
// in shared memory, then each thread produces quads of 4 texels: the parent's
// bilinear (1, 3, 3, 9)/16 mask floored to an integer, the residual
// ((r - 128) * scale, or the root colour at level 0), the rotated noise layer
// (RGB or HSV mode), and the framebuffer's unorm8 rounding -- every float
// operation rounded on its own in the shader's order, so that the bytes equal a
// CPU evaluation without contraction.  Jobs naming their parent's job wait for
// its completion count (acquire, bounded), so a batch may hold parents and
// children; parents must come first.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "tp_internal.h"
#include "tp_div.h"

namespace {

constexpr int kThreads = 256;
constexpr unsigned kDepLimit = 1u << 22;  // dependency polls (64 ns back-off) before giving up

// The library's status word lives in another file's device memory: its address comes
// with the launch.
__device__ __forceinline__ void report(int *status, int code) { atomicCAS(status, 0, code); }

__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ float m_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float a_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float s_(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float d_(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float clamp01(float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); }

// x / y for a divisor known in advance, with z = RN(1 / y): q = RN(x z), the exact
// remainder r = x - q y by one FMA, then RN(q + r z) -- the one-correction scheme
// for known divisors of Brisebarre, Muller and Raina (IEEE Trans. Computers 53(8),
// 2004), which returns the correctly rounded quotient for every x when y passes
// their test.  Outside 2^-96 <= |x| <= 2^96 (and for infinities and NaN) the
// correctly rounded division is called (y > 0).  tp_division_self_test compares it with
// the correctly rounded division over all 2^32 x for the divisors used here.
__device__ __forceinline__ float div_known(float x, float y, float z)
{
    const float ax = fabsf(x);
    if (ax <= 0x1p96f && ax >= 0x1p-96f) {
        const float q = __fmul_rn(x, z);
        const float r = __fmaf_rn(-q, y, x);
        return __fmaf_rn(r, z, q);
    }
    if (ax == 0.0f) return __fmul_rn(x, z);  // +-0 / y = +-0 (y > 0)
    return __fdiv_rn(x, y);
}
constexpr float kInv6 = 1.0f / 6.0f, kInv255 = 1.0f / 255.0f, kInv04 = 1.0f / 0.4f;

// Byte c of w as a float, exactly: the byte placed in the mantissa of 2^23
// (0x4B0000bb) minus 2^23.
__device__ __forceinline__ float byte_of(uint32_t w, int c)
{
    return __fsub_rn(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + c)), 8388608.0f);
}

// An integer 0 <= v < 2^23 as a float, exactly.
__device__ __forceinline__ float int_to_f(uint32_t v) { return __fsub_rn(__uint_as_float(0x4B000000u | v), 8388608.0f); }

// Framebuffer write of result / 255 to an 8-bit channel: clamp(result / 255, 0, 1)
// times 255, rounded to nearest even.  Both roundings move a result in [0, 255]
// by less than 3.1e-5, so away from the half-integers (1e-3 margin) the byte is
// clamp(rint(result)); within the margin the two roundings are evaluated.
__device__ __forceinline__ uint32_t unorm8(float result)
{
    const float t = __fsub_rn(result, floorf(result));
    float v;
    if (fabsf(__fsub_rn(t, 0.5f)) > 1e-3f) {
        v = fminf(fmaxf(result, 0.0f), 255.0f);
    } else {
        v = m_(clamp01(d_(result, 255.0f)), 255.0f);
    }
    // rint by the 1.5 * 2^23 addition (ties to even), the integer in the low bits
    return __float_as_uint(__fadd_rn(v, 12582912.0f)) & 0x1FFu;
}

__device__ __forceinline__ void rgb_to_hsv(const float *rgb, float *hsv)
{
    const float mn = fminf(rgb[0], fminf(rgb[1], rgb[2]));
    const float mx = fmaxf(rgb[0], fmaxf(rgb[1], rgb[2]));
    const float delta = s_(mx, mn);
    hsv[0] = 0.0f;
    hsv[1] = 0.0f;
    hsv[2] = mx;
    if (delta != 0.0f) {
        hsv[1] = d_(delta, mx);
        const float rdelta = __frcp_rn(delta);  // the three quotients below share the divisor
        float d[3];
#pragma unroll
        for (int c = 0; c < 3; ++c)  // delta / 2 exact
            d[c] = tp::div_rcp(a_(div_known(s_(mx, rgb[c]), 6.0f, kInv6), m_(delta, 0.5f)), delta, rdelta);
        if (rgb[0] == mx) hsv[0] = s_(d[2], d[1]);
        else if (rgb[1] == mx) hsv[0] = s_(a_(1.0f / 3.0f, d[0]), d[2]);
        else if (rgb[2] == mx) hsv[0] = s_(a_(2.0f / 3.0f, d[1]), d[0]);
        if (hsv[0] < 0.0f) hsv[0] = a_(hsv[0], 1.0f);
        if (hsv[0] > 1.0f) hsv[0] = s_(hsv[0], 1.0f);
    }
}

__device__ __forceinline__ void hsv_to_rgb(const float *hsv, float *rgb)
{
    rgb[0] = rgb[1] = rgb[2] = hsv[2];
    if (hsv[1] != 0.0f) {
        const float h = m_(hsv[0], 6.0f);
        const float i = floorf(h);
        const float f = s_(h, i);
        const float v1 = m_(hsv[2], s_(1.0f, hsv[1]));
        const float v2 = m_(hsv[2], s_(1.0f, m_(hsv[1], f)));
        const float v3 = m_(hsv[2], s_(1.0f, m_(hsv[1], s_(1.0f, f))));
        if (i == 0.0f) { rgb[0] = hsv[2]; rgb[1] = v3; rgb[2] = v1; }
        else if (i == 1.0f) { rgb[0] = v2; rgb[1] = hsv[2]; rgb[2] = v1; }
        else if (i == 2.0f) { rgb[0] = v1; rgb[1] = hsv[2]; rgb[2] = v3; }
        else if (i == 3.0f) { rgb[0] = v1; rgb[1] = v2; rgb[2] = hsv[2]; }
        else if (i == 4.0f) { rgb[0] = v3; rgb[1] = v1; rgb[2] = hsv[2]; }
        else { rgb[0] = hsv[2]; rgb[1] = v1; rgb[2] = v2; }
    }
}

// One texel: r = residual / root colour / 128 as floats, c = floored parent mask
// sum (when there is a parent), n = noise texel.
__device__ __forceinline__ uint32_t texel(float (&r)[4], const float (&nv)[4], const float (&nc)[4], bool hsv,
                                          const float *inv255)
{
    float out[4];
    if (hsv) {
        float rgb[3], h[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            // k / 255 of the integers 0..255 from the table (the same correctly rounded quotients)
            const bool tab = r[c] >= 0.0f && r[c] <= 255.0f && r[c] == floorf(r[c]);
            rgb[c] = tab ? inv255[(int)r[c]] : d_(r[c], 255.0f);
        }
        rgb_to_hsv(rgb, h);
        // 1 - smoothstep(0.4, 0.8, v); 0.8f - 0.4f is exactly 0.4f
        float t = clamp01(div_known(s_(h[2], 0.4f), 0.4f, kInv04));
        t = m_(m_(t, t), s_(3.0f, m_(2.0f, t)));
        const float k = s_(1.0f, t);
#pragma unroll
        for (int c = 0; c < 3; ++c)
            h[c] = m_(h[c], a_(1.0f, div_known(m_(m_(k, nc[c]), s_(nv[c], 128.0f)), 255.0f, kInv255)));
        h[0] = s_(h[0], floorf(h[0]));
        h[1] = clamp01(h[1]);
        h[2] = clamp01(h[2]);
        hsv_to_rgb(h, rgb);
#pragma unroll
        for (int c = 0; c < 3; ++c) out[c] = m_(rgb[c], 255.0f);
        out[3] = a_(m_(nc[3], s_(nv[3], 128.0f)), r[3]);
    } else {
#pragma unroll
        for (int c = 0; c < 4; ++c) out[c] = a_(m_(nc[c], s_(nv[c], 128.0f)), r[c]);
    }
    return (unorm8(out[0]) & 255u) | ((unorm8(out[1]) & 255u) << 8) | ((unorm8(out[2]) & 255u) << 16) |
           ((unorm8(out[3]) & 255u) << 24);
}

__global__ void __launch_bounds__(kThreads) ortho_kernel(const tp::OrthoLaunch L)
{
    extern __shared__ __align__(16) uint32_t win[];   // parent window, (W/2 + 2) rows of wp words
    __shared__ int unit;
    __shared__ float inv255[256];
    for (int k = threadIdx.x; k < 256; k += kThreads) inv255[k] = __fdiv_rn((float)k, 255.0f);
    const int W = L.W, n = W - 4, wp = L.win_pitch;
    const int NQ = W / 4;
    // t / NQ by a multiply-high with ceil(2^32 / NQ): exact for t < 2^20 and NQ <= 4096
    const uint32_t nq_magic = 0xFFFFFFFFu / (uint32_t)NQ + 1u;
    __shared__ int skip;
    for (;;) {
        if (threadIdx.x == 0) {
            unit = atomicAdd(L.counter, 1);
            skip = 0;
            if (unit < L.njobs) {
                const int pj = L.jobs[unit].parent_job;
#ifdef TP_DEBUG
                // debug builds: the job's indexes before any of them addresses memory
                const tp_ortho_job &J = L.jobs[unit];
                const bool ok = J.out_slot >= 0 && J.out_slot < L.cap && J.level >= 0 && J.level <= 30 &&
                                (J.level == 0 || (J.parent_slot >= 0 && J.parent_slot < L.cap)) &&
                                (J.residual_slot < 0 || J.residual_slot < L.res_cap) && pj >= -1 && pj < unit &&
                                J.noise_layer >= 0 && J.noise_layer < 6 && J.noise_rot >= 0 && J.noise_rot < 4;
                if (!ok) {
                    report(L.status, TP_E_BOUNDS);
                    skip = 1;
                }
                if (pj >= 0 && ok) {
#else
                if (pj >= 0) {
#endif
                    unsigned k = 0;
                    while (ld_acquire(L.done + pj) < 1) {
                        if (++k > kDepLimit) {
                            report(L.status, TP_E_TIMEOUT);
                            break;
                        }
                        __nanosleep(64);
                    }
                    __threadfence();
                }
            }
        }
        __syncthreads();
        const int u = unit;
        if (u >= L.njobs) break;
        if (skip) {  // debug builds: a job that failed its checks counts as done, unproduced
            __syncthreads();
            if (threadIdx.x == 0) {
                __threadfence();
                atomicAdd(L.done + u, 1);
            }
            continue;
        }
        const tp_ortho_job J = L.jobs[u];
        const bool has_parent = J.level > 0;
        const bool has_res = J.residual_slot >= 0;
        const int dx = (J.tx & 1) * (n / 2), dy = (J.ty & 1) * (n / 2);
        const int ww = W / 2 + 2;  // window side
        if (has_parent) {
            // rows dy .. dy + ww - 1, columns dx .. dx + ww - 1 of the parent, by 8-byte
            // L2 loads (the parent may have been written by another CTA of this launch)
            const uint32_t *par = L.tiles + (long long)J.parent_slot * L.slot_stride;
            const int halves = ww / 2;
            for (int t = threadIdx.x; t < ww * halves; t += kThreads) {
                const int r = t / halves, h = t - r * halves;
                const uint2 v = __ldcg(reinterpret_cast<const uint2 *>(par + (long long)(dy + r) * L.pitch + dx) + h);
                *reinterpret_cast<uint2 *>(win + r * wp + 2 * h) = v;
            }
        }
        __syncthreads();
        // noiseColor of the tile (OrthoProducer.cpp:376-380)
        float nc[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            if (L.p.hsv) nc[c] = d_(m_(L.p.noise_color[c], c < 3 ? J.noise_amp : m_(L.p.scale, J.noise_amp)), 255.0f);
            else nc[c] = d_(m_(m_(L.p.noise_color[c], L.p.scale), J.noise_amp), 255.0f);
        }
        const float rscale = has_res ? L.p.scale : -1.0f;  // residualOSH.w
        const bool hsv = L.p.hsv != 0;
        const uint32_t *res = has_res ? L.res + (long long)J.residual_slot * L.res_slot_stride : nullptr;
        const uint32_t *noise = L.noise + (long long)(J.noise_rot * 6 + J.noise_layer) * W * L.pitch;
        uint32_t *out = L.tiles + (long long)J.out_slot * L.slot_stride;
        for (int t = threadIdx.x; t < W * NQ; t += kThreads) {
            const int j = (int)__umulhi((uint32_t)t, nq_magic), q = t - j * NQ, i0 = 4 * q;  // j = t / NQ
            const uint4 nq = __ldg(reinterpret_cast<const uint4 *>(noise + (long long)j * L.pitch + i0));
            uint4 rq = make_uint4(0u, 0u, 0u, 0u);
            if (has_res) rq = __ldg(reinterpret_cast<const uint4 *>(res + (long long)j * L.res_pitch + i0));
            const uint32_t nw[4] = {nq.x, nq.y, nq.z, nq.w}, rw[4] = {rq.x, rq.y, rq.z, rq.w};
            // parent texels of the quad: window columns 2q .. 2q + 3 of rows ly, ly + 1
            uint32_t pa[4], pb[4];
            const int ly = (j + 1) / 2;
            if (has_parent) {
                const uint2 a01 = *reinterpret_cast<const uint2 *>(win + ly * wp + 2 * q);
                const uint2 a23 = *reinterpret_cast<const uint2 *>(win + ly * wp + 2 * q + 2);
                const uint2 b01 = *reinterpret_cast<const uint2 *>(win + (ly + 1) * wp + 2 * q);
                const uint2 b23 = *reinterpret_cast<const uint2 *>(win + (ly + 1) * wp + 2 * q + 2);
                pa[0] = a01.x; pa[1] = a01.y; pa[2] = a23.x; pa[3] = a23.y;
                pb[0] = b01.x; pb[1] = b01.y; pb[2] = b23.x; pb[3] = b23.y;
            }
            uint32_t o[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float r[4], nv[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    r[c] = has_res ? byte_of(rw[k], c) : (has_parent ? 128.0f : m_(L.p.root_color[c], 255.0f));
                    nv[c] = byte_of(nw[k], c);
                }
                if (has_parent) {
                    // masks (1,3,3,9), (3,1,9,3), (3,9,1,3), (9,3,3,1) over the texels
                    // (px, py), (px + 1, py), (px, py + 1), (px + 1, py + 1): the integer
                    // sums (exact, as in float) by byte dot products, channel by channel
                    const int lp = (k + 1) / 2;  // ((i0 + k + 1) / 2) - 2q
                    const int mi = (k & 1) + 2 * (j & 1);
                    const uint32_t mw = mi == 0 ? 0x09030301u : mi == 1 ? 0x03090103u : mi == 2 ? 0x03010903u
                                                                                            : 0x01030309u;
                    // transpose the four texels into four channel words [t0, t1, t2, t3]
                    const uint32_t t0 = pa[lp], t1 = pa[lp + 1], t2 = pb[lp], t3 = pb[lp + 1];
                    const uint32_t lo01 = __byte_perm(t0, t1, 0x5140u), hi01 = __byte_perm(t0, t1, 0x7362u);
                    const uint32_t lo23 = __byte_perm(t2, t3, 0x5140u), hi23 = __byte_perm(t2, t3, 0x7362u);
                    const uint32_t ch[4] = {__byte_perm(lo01, lo23, 0x5410u), __byte_perm(lo01, lo23, 0x7632u),
                                            __byte_perm(hi01, hi23, 0x5410u), __byte_perm(hi01, hi23, 0x7632u)};
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const float cc = int_to_f((uint32_t)__dp4a(ch[c], mw, 0u) >> 4);   // floor(s / 16)
                        r[c] = a_(m_(s_(r[c], 128.0f), rscale), cc);
                    }
                }
                o[k] = texel(r, nv, nc, hsv, inv255);
            }
            *reinterpret_cast<uint4 *>(out + (long long)j * L.pitch + i0) = make_uint4(o[0], o[1], o[2], o[3]);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(L.done + u, 1);
        }
    }
}

}  // namespace

namespace tp {

int ortho_smem_bytes(int W, int *win_pitch)
{
    const int ww = W / 2 + 2;
    *win_pitch = round_up(ww, 4);
    return (int)sizeof(uint32_t) * ww * *win_pitch;
}

int launch_ortho(const OrthoLaunch &L, void *stream)
{
    // per device: SM count, the shared-memory limit set on the kernel, CTAs per SM
    struct DevState {
        int sms = 0, per_sm = 0, smem_set = 0;
    };
    static std::mutex mu;
    static std::map<int, DevState> states;
    int pitch = 0;
    const int smem = ortho_smem_bytes(L.W, &pitch);
    int dev = 0;
    cudaGetDevice(&dev);
    int grid = 1;
    {
        std::lock_guard<std::mutex> lk(mu);
        DevState &st = states[dev];
        if (st.sms == 0) cudaDeviceGetAttribute(&st.sms, cudaDevAttrMultiProcessorCount, dev);
        if (smem > st.smem_set) {
            cudaError_t e = cudaFuncSetAttribute(ortho_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return cuda_fail("cudaFuncSetAttribute (ortho)", e);
            st.smem_set = smem;
            st.per_sm = 0;
        }
        if (st.per_sm == 0) {
            cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&st.per_sm, ortho_kernel, kThreads, st.smem_set);
            if (e != cudaSuccess) return cuda_fail("occupancy (ortho)", e);
            if (st.per_sm < 1) return fail(TP_E_BAD_ARG, "ortho: the parent window does not fit in shared memory");
        }
        grid = std::max(1, std::min(L.njobs, st.per_sm * st.sms));
    }
    ortho_kernel<<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(L);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("ortho kernel launch", e);
    return TP_OK;
}

}  // namespace tp

namespace {

__global__ void division_check_kernel(float y, float z, unsigned long long *mismatches, uint32_t *first)
{
    unsigned long long bad = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b <= 0xFFFFFFFFull; b += stride) {
        const float x = __uint_as_float((uint32_t)b);
        const float f = div_known(x, y, z), e = __fdiv_rn(x, y);
        const bool same = __float_as_uint(f) == __float_as_uint(e) || (f != f && e != e);
        if (!same) {
            ++bad;
            atomicMin(first, (uint32_t)b);
        }
    }
    if (bad) atomicAdd(mismatches, bad);
}

}  // namespace

extern "C" int tp_division_self_test(float divisor, unsigned long long *mismatches, uint32_t *first_mismatch)
{
    if (!mismatches || !(divisor > 0.0f) || !(divisor < 1e30f))
        return tp::fail(TP_E_BAD_ARG, "tp_division_self_test: bad arguments");
    unsigned long long *d_count = nullptr;
    cudaError_t e = cudaMalloc(&d_count, sizeof(unsigned long long) + sizeof(uint32_t));
    if (e != cudaSuccess) return tp::cuda_fail("cudaMalloc (division check)", e);
    uint32_t *d_first = reinterpret_cast<uint32_t *>(d_count + 1);
    const unsigned long long zero = 0;
    const uint32_t none = 0xFFFFFFFFu;
    cudaMemcpy(d_count, &zero, sizeof zero, cudaMemcpyHostToDevice);
    cudaMemcpy(d_first, &none, sizeof none, cudaMemcpyHostToDevice);
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const float z = 1.0f / divisor;  // correctly rounded on the host as on the device
    division_check_kernel<<<sms * 8, 256>>>(divisor, z, d_count, d_first);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(mismatches, d_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    uint32_t first = none;
    if (e == cudaSuccess) e = cudaMemcpy(&first, d_first, sizeof first, cudaMemcpyDeviceToHost);
    cudaFree(d_count);
    if (e != cudaSuccess) return tp::cuda_fail("division check", e);
    if (first_mismatch) *first_mismatch = first;
    return TP_OK;
}
