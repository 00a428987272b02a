// Kernels of the learned residual predictor (sm_103a).
//
// Convolutions are implicit GEMMs on the 5th-generation tensor cores: a CTA owns a
// block of 8 x 16 output pixels (M = 128 rows of one tcgen05.mma), TMA stages the
// block's input halo (10 x 18 pixels, zero-filled outside the image) into shared
// memory as one plane of 8-channel rows per channel group, and each of the nine
// taps is a descriptor offset into that halo -- no im2col copy.  K runs over
// (tap, 16-channel step); the weights are the B operand, packed once per update in
// the canonical no-swizzle K-major layout.  Accumulators live in tensor memory and
// are read back with tcgen05.ld for a fused epilogue (bias, level embedding, GELU,
// or the GELU derivative of the backward pass).
//
// The weight gradient is a GEMM over pixels: D[(tap, ci)][co] += X[p + tap][ci] *
// dZ[p][co] with both operands MN-major (pixels along K), each 8-pixel row of an
// operand tile brought in by TMA at the tap's offset; a CTA accumulates its blocks
// in tensor memory and adds its sums to the gradient once at the end.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <map>
#include <mutex>

#include "tp_internal.h"
#include "tp_learned.h"
#include "tp_sm100.h"
#include "tp_stencil.h"

namespace tp {
namespace learned {
namespace {

using namespace tp::sm100;

constexpr int kHaloX = kBlockX + 2, kHaloY = kBlockY + 2;
constexpr int kRowStride = kHaloX * 16;                     // bytes per halo row of one channel group
constexpr int kHaloBytes = kRowStride * kHaloY;             // one channel group: 2880
constexpr int kGroupStride = (kHaloBytes + 127) / 128 * 128;  // 2944: TMA destinations 128-byte aligned
constexpr int kBoxBytes = 8 * kBlockX * kBlockY * 2;        // one 8-channel group of a block: 2048

// GELU in its tanh form, 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))), on channel
// pairs: the polynomial in packed f32x2 arithmetic, tanh on the SFU as one
// tanh.approx.f16x2 per pair (the precision class of tanh.approx.f32, about 2^-11
// relative), the result back in f32.
__device__ __forceinline__ uint64_t pk2(float a, float b)
{
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk2(uint64_t r, float &a, float &b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b)
{
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b)
{
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c)
{
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t tanh2(uint64_t x)
{
    float a, b;
    upk2(x, a, b);
    __half2 h = __floats2half2_rn(a, b);
    uint32_t u = *reinterpret_cast<uint32_t *>(&h), t;
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(t) : "r"(u));
    const float2 f = __half22float2(*reinterpret_cast<__half2 *>(&t));
    return pk2(f.x, f.y);
}
__device__ __forceinline__ uint64_t splat2(float v) { return pk2(v, v); }

// (v[j], v[j+1]) <- gelu(v[j], v[j+1])
__device__ __forceinline__ void gelu_pair(float &x, float &y)
{
    const uint64_t z = pk2(x, y);
    const uint64_t z3 = mul2(mul2(z, z), z);
    const uint64_t u = mul2(fma2(z3, splat2(0.044715f), z), splat2(0.7978845608028654f));
    const uint64_t t = tanh2(u);
    const uint64_t h = mul2(z, splat2(0.5f));
    upk2(fma2(h, t, h), x, y);  // 0.5 z + 0.5 z t
}

// (g[j], g[j+1]) <- g * gelu'(z) with gelu'(z) = 0.5 (1 + t) + 0.5 z (1 - t^2) sqrt(2/pi) (1 + 0.134145 z^2)
__device__ __forceinline__ void gelu_grad_pair(float &gx, float &gy, float zx, float zy)
{
    const uint64_t z = pk2(zx, zy);
    const uint64_t z2 = mul2(z, z);
    const uint64_t u = mul2(fma2(mul2(z2, z), splat2(0.044715f), z), splat2(0.7978845608028654f));
    const uint64_t t = tanh2(u);
    const uint64_t half_ = splat2(0.5f);
    const uint64_t a = fma2(half_, t, half_);                                          // 0.5 (1 + t)
    const uint64_t omt2 = fma2(mul2(t, t), splat2(-1.0f), splat2(1.0f));               // 1 - t^2
    const uint64_t p = fma2(z2, splat2(0.134145f), splat2(1.0f));                       // 1 + 0.134145 z^2
    const uint64_t b = mul2(mul2(mul2(z, half_), omt2), mul2(p, splat2(0.7978845608028654f)));
    upk2(mul2(add2(a, b), pk2(gx, gy)), gx, gy);
}

__device__ __forceinline__ uint32_t pack2(float a, float b)
{
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&h);
}

// Activations are stored per 8-channel group: image `img` of C channels is C / 8
// planes of (W + 2)^2 pixels of 16 bytes (one pixel's 8 channels), so that a TMA box
// of one channel group reads whole 16-byte pixels of contiguous rows.  `plane` is
// (W + 2)^2 and `pix` the pixel's index in its plane.
template <int C>
__device__ __forceinline__ void store_bf16(__nv_bfloat16 *base, int img, size_t plane, size_t pix, const float *v)
{
#pragma unroll
    for (int q = 0; q < C / 8; ++q) {
        uint4 u;
        u.x = pack2(v[8 * q + 0], v[8 * q + 1]);
        u.y = pack2(v[8 * q + 2], v[8 * q + 3]);
        u.z = pack2(v[8 * q + 4], v[8 * q + 5]);
        u.w = pack2(v[8 * q + 6], v[8 * q + 7]);
        *reinterpret_cast<uint4 *>(base + (((size_t)img * (C / 8) + q) * plane + pix) * 8) = u;
    }
}

template <int C>
__device__ __forceinline__ void load_bf16(const __nv_bfloat16 *base, int img, size_t plane, size_t pix, float *v)
{
#pragma unroll
    for (int q = 0; q < C / 8; ++q) {
        uint4 u = *reinterpret_cast<const uint4 *>(base + (((size_t)img * (C / 8) + q) * plane + pix) * 8);
        const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            float2 f = __bfloat1622float2(h[e]);
            v[8 * q + 2 * e] = f.x;
            v[8 * q + 2 * e + 1] = f.y;
        }
    }
}

// Roles of a CTA: warp 0 issues the TMA copies, warp 1 the tensor-core MMAs (and owns
// the tensor memory), warps 2-5 (one per tensor-memory lane quadrant) run the epilogue.
constexpr int kRoleThreads = 192;
constexpr int kConvStages = 3;
// The first layer of an inference pass makes its input channels itself: a second
// producer warp (warp 6) takes every other block, so that one block's loads overlap
// another's arithmetic.
template <int MODE>
constexpr int conv_threads() { return MODE == kFirst ? kRoleThreads + 32 : kRoleThreads; }

template <int CIN, int COUT>
constexpr int conv_smem_bytes()
{
    return kConvStages * (CIN / 8) * kGroupStride + 9 * CIN * COUT * 2 + 128 + COUT * 4;
}

// Tiles this CTA takes from a persistent loop over `total` tiles.
__device__ __forceinline__ int my_tiles(int total) { return (total - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x; }

template <int CIN, int COUT, int MODE>
__global__ void __launch_bounds__(conv_threads<MODE>()) conv_kernel(const __grid_constant__ CUtensorMap xmap,
                                                                    const ConvLaunch a)
{
    constexpr int kThreadsC = conv_threads<MODE>();
    extern __shared__ __align__(1024) uint8_t smem[];
    constexpr int NCG = CIN / 8, KSTEPS = CIN / 16, NMMA = 9 * KSTEPS;
    constexpr int STAGE = NCG * kGroupStride;
    constexpr int BBYTES = NMMA * COUT * 32;
    uint8_t *halo = smem;
    uint8_t *bsm = smem + kConvStages * STAGE;
    uint64_t *full = reinterpret_cast<uint64_t *>(bsm + BBYTES);
    uint64_t *empty = full + kConvStages;
    uint64_t *acc_full = empty + kConvStages;
    uint64_t *acc_empty = acc_full + 2;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(acc_empty + 2);
    volatile int *abort = reinterpret_cast<volatile int *>(tslot + 1);
    float *bias_s = reinterpret_cast<float *>(tslot + 4);  // 16-byte aligned, COUT floats
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    for (int i = tid; i < BBYTES / 16; i += kThreadsC)
        reinterpret_cast<uint4 *>(bsm)[i] = reinterpret_cast<const uint4 *>(a.wpack)[i];
    if (tid < COUT) bias_s[tid] = a.bias ? a.bias[tid] : 0.0f;
    if (MODE == kFirst)  // channels 8-15 of every stage are zero (before any MMA reads a stage)
        for (int i = tid; i < kConvStages * kHaloX * kHaloY; i += kThreadsC) {
            const int st = i / (kHaloX * kHaloY), p = i - st * (kHaloX * kHaloY);
            *reinterpret_cast<uint4 *>(halo + st * STAGE + kGroupStride + p * 16) = make_uint4(0u, 0u, 0u, 0u);
        }
    if (tid == 0) {
        for (int s = 0; s < kConvStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 128);
        }
        *abort = 0;
    }
    if (warp == 1) tmem_alloc(tslot, 64);
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const int per_img = a.tiles_x * a.tiles_y, total = a.nimg * per_img;
    const int mine = my_tiles(total);

    if (MODE == kFirst && (warp == 0 || warp == 6)) {
        // producers: the input channels of tile i's halo made from the upsampled parent
        // (the values launch_prep writes: (up - mean) / sigma_in, x and y parity, 1, the
        // second differences along x and y over sigma_out; 0 outside the image), written
        // as bf16 into stage i % kConvStages; warp 0 makes the even tiles, warp 6 the odd
        int i = warp == 0 ? 0 : 1;
        for (; i < mine; i += 2) {
            const int s = i % kConvStages;
            if (i >= kConvStages &&
                !__all_sync(0xffffffffu, mbar_wait_abortable(&empty[s], ((i / kConvStages) - 1) & 1, abort)))
                break;
            const int t = blockIdx.x + i * gridDim.x;
            const int img = t / per_img, rem = t - img * per_img;
            const int by = rem / a.tiles_x, bx = rem - by * a.tiles_x;
            const float *u = a.up + (size_t)img * a.W * a.W;
            // all loads of the tile first (one latency), then the conversions
            constexpr int kPer = (kHaloX * kHaloY + 31) / 32;
            float val[kPer], d2x[kPer], d2y[kPer];
            int xs[kPer], ys[kPer];
            const float mean = __ldg(a.mean + img);
            const int lv = __ldg(a.level + img);
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                const int p = lane + 32 * k;
                const int hy = p / kHaloX, hx = p - hy * kHaloX;
                xs[k] = bx * kBlockX + hx - 1;
                ys[k] = by * kBlockY + hy - 1;
                const bool in = p < kHaloX * kHaloY && xs[k] >= 0 && ys[k] >= 0 && xs[k] < a.W && ys[k] < a.W;
                const float *c = u + (size_t)ys[k] * a.W + xs[k];
                val[k] = in ? __ldg(c) : 0.0f;
                const bool ix = in && xs[k] > 0 && xs[k] < a.W - 1, iy = in && ys[k] > 0 && ys[k] < a.W - 1;
                d2x[k] = ix ? __fadd_rn(__ldg(c - 1), __ldg(c + 1)) : 0.0f;
                d2y[k] = iy ? __fadd_rn(__ldg(c - a.W), __ldg(c + a.W)) : 0.0f;
                if (ix) d2x[k] = __fsub_rn(d2x[k], __fmul_rn(2.0f, val[k]));
                if (iy) d2y[k] = __fsub_rn(d2y[k], __fmul_rn(2.0f, val[k]));
                if (!in) xs[k] = -1;
            }
            const int lc = min(max(lv, 0), kLevels - 1);
            const float inv = 1.0f / __ldg(a.sigma_in + lc), inv2 = 1.0f / __ldg(a.sigma_out + lc);
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                const int p = lane + 32 * k;
                if (p >= kHaloX * kHaloY) break;
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (xs[k] >= 0) {
                    v.x = pack2((val[k] - mean) * inv, (float)(xs[k] & 1));
                    v.y = pack2((float)(ys[k] & 1), 1.0f);
                    v.z = pack2(__fmul_rn(d2x[k], inv2), __fmul_rn(d2y[k], inv2));
                }
                *reinterpret_cast<uint4 *>(halo + s * STAGE + p * 16) = v;
            }
            fence_proxy_async_smem();  // the generic-proxy writes, before the tensor cores read them
            __syncwarp();
            if (lane == 0) mbar_arrive(&full[s]);
        }
    } else if (warp == 0) {
        if (lane == 0) {  // producer: halo of tile i into stage i % kConvStages
            int i = 0;
            for (; i < mine; ++i) {
                const int s = i % kConvStages;
                if (i >= kConvStages && !mbar_wait_abortable(&empty[s], ((i / kConvStages) - 1) & 1, abort)) break;
                const int t = blockIdx.x + i * gridDim.x;
                const int img = t / per_img, rem = t - img * per_img;
                const int by = rem / a.tiles_x, bx = rem - by * a.tiles_x;
                mbar_expect_tx(&full[s], NCG * kHaloBytes);
#pragma unroll
                for (int cg = 0; cg < NCG; ++cg)
                    tma_load_3d(halo + s * STAGE + cg * kGroupStride, &xmap, bx * kBlockX * 8, by * kBlockY,
                                img * NCG + cg, &full[s]);
            }
            if (*abort)  // copies in flight land before the CTA leaves
                for (int k = i > kConvStages ? i - kConvStages : 0; k < i; ++k)
                    mbar_wait(&full[k % kConvStages], (k / kConvStages) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer: tile i into accumulator i % 2
            constexpr uint32_t idesc = idesc_bf16(128, COUT, 0, 0);
            const uint32_t b_a = smem_u32(bsm);
            int i = 0;
            for (; i < mine; ++i) {
                const int s = i % kConvStages, b = i & 1;
                if (!mbar_wait_abortable(&full[s], (i / kConvStages) & 1, abort)) break;
                if (i >= 2 && !mbar_wait_abortable(&acc_empty[b], ((i >> 1) - 1) & 1, abort)) break;
                tc_fence_after();
                const uint32_t h_a = smem_u32(halo + s * STAGE);
#pragma unroll
                for (int q = 0; q < NMMA; ++q) {
                    const int tap = q / KSTEPS, st = q - tap * KSTEPS;
                    const int dy = tap / 3, dx = tap - dy * 3;
                    const uint64_t ad = sdesc(h_a + 2 * st * kGroupStride + dy * kRowStride + dx * 16, kGroupStride,
                                              kRowStride);
                    const uint64_t bd = sdesc(b_a + q * COUT * 32, 128, 256);
                    mma_bf16(tmem + b * 32, ad, bd, idesc, q > 0 ? 1u : 0u);
                }
                mma_commit(&empty[s]);
                mma_commit(&acc_full[b]);
            }
            if (*abort && i > 0) mbar_wait(&empty[(i - 1) % kConvStages], ((i - 1) / kConvStages) & 1);
        }
    } else {  // epilogue: rows 32 q .. 32 q + 31 of the accumulator
        const int q = warp & 3;
        const int Wp = a.W + 2;
        for (int i = 0; i < mine; ++i) {
            const int b = i & 1;
            if (!__all_sync(0xffffffffu, mbar_wait_abortable(&acc_full[b], (i >> 1) & 1, abort))) break;
            tc_fence_after();
            float acc[COUT];
            const uint32_t taddr = tmem + b * 32 + ((uint32_t)(q * 32) << 16);
            if (COUT == 32)
                tmem_ld32(taddr, acc);
            else
                tmem_ld16(taddr, acc);
            tc_fence_before();
            mbar_arrive(&acc_empty[b]);
            const int t = blockIdx.x + i * gridDim.x;
            const int img = t / per_img, rem = t - img * per_img;
            const int by = rem / a.tiles_x, bx = rem - by * a.tiles_x;
            const int m = q * 32 + lane;
            const int px = bx * kBlockX + (m & 7), py = by * kBlockY + (m >> 3);
            if (px < a.W && py < a.W) {
                const size_t plane = (size_t)Wp * Wp, pix = (size_t)(py + 1) * Wp + (px + 1);
                if (MODE == kHidden || MODE == kFirst) {
                    const float2 *b2 = reinterpret_cast<const float2 *>(bias_s);
                    if (a.emb) {
                        const float2 *e2 = reinterpret_cast<const float2 *>(
                            a.emb + (size_t)min(max(a.level[img], 0), kLevels - 1) * COUT);
#pragma unroll
                        for (int j = 0; j < COUT / 2; ++j) {
                            const float2 bb = b2[j], ee = __ldg(e2 + j);
                            upk2(add2(pk2(acc[2 * j], acc[2 * j + 1]), add2(pk2(bb.x, bb.y), pk2(ee.x, ee.y))),
                                 acc[2 * j], acc[2 * j + 1]);
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < COUT / 2; ++j) {
                            const float2 bb = b2[j];
                            upk2(add2(pk2(acc[2 * j], acc[2 * j + 1]), pk2(bb.x, bb.y)), acc[2 * j], acc[2 * j + 1]);
                        }
                    }
                    if (a.zsave) store_bf16<COUT>(a.zsave, img, plane, pix, acc);
#pragma unroll
                    for (int j = 0; j < COUT; j += 2) gelu_pair(acc[j], acc[j + 1]);
                    store_bf16<COUT>(a.out, img, plane, pix, acc);
                } else if (MODE == kLast) {
                    a.out_f32[((size_t)img * a.W + py) * a.W + px] = acc[0] + bias_s[0];
                } else {
                    float z[COUT];
                    load_bf16<COUT>(a.zprev, img, plane, pix, z);
#pragma unroll
                    for (int j = 0; j < COUT; j += 2) gelu_grad_pair(acc[j], acc[j + 1], z[j], z[j + 1]);
                    store_bf16<COUT>(a.out, img, plane, pix, acc);
                }
            }
        }
    }
    __syncthreads();
    if (tid == 0 && *abort) atomicExch(a.status, TP_E_TIMEOUT);
    tc_fence_after();
    if (warp == 1) tmem_dealloc(tmem, 64);
}

// ---------------------------------------------------------------- fused pairs (inference)
// Two consecutive convolutions in one launch.  For the 8 x 14 output block of the
// second layer (B), the first layer (A) is computed on the block's 10 x 16 halo as
// two overlapping 8 x 16 MMA tiles, at columns 0 and 2 of that halo, from a 12 x 18
// input halo; the second tile contributes columns 8 and 9 only, whose 8 rows per warp
// the epilogue gathers across the warp's 32 lanes before the GELU.  A's epilogue
// (bias, level embedding, GELU, bf16) writes its outputs into shared memory in the
// K-major layout B's MMAs read, zero outside the image as the activation image's
// border is, so the hidden activations never reach HBM.
//
// Roles: warp 0 stages the input halos, warp 1 issues the MMAs (A(i), then B(i - 1)),
// warps 2-5 and 6-9 are two epilogue groups: group i % 2 finishes block i (A's
// epilogue, then B's), so that two blocks' epilogue chains run at once.  Each group
// owns 128 tensor-memory columns (A's two tiles, B's tile) and one B-operand halo.
// Every wait is bounded (abort flag).
constexpr int kFusedStages = 3;
constexpr int kFusedThreads = 320;
constexpr int kWideRow = kWideX * 16;                                // 192 bytes per row of one channel group
constexpr int kWideGroup = (kWideRow * kWideY + 127) / 128 * 128;    // 3456
constexpr int kWinX = kWideX + 2, kWinY = kWideY + 2;                // fp32 window of the first pair's producer
constexpr uint32_t kFusedCols = 256;

template <int CINA>
constexpr int fused_smem_bytes()
{
    return kFusedStages * (CINA / 8) * kWideGroup + 2 * 4 * kGroupStride + 9 * CINA * 32 * 2 + 9 * 32 * 32 * 2 +
           kWinX * kWinY * 4 + 512;
}

// bias (+ level embedding), GELU: the kHidden / kFirst epilogue's operations, on the
// channels [c0, c0 + N) held in acc[0, N)
template <int N>
__device__ __forceinline__ void hidden_epilogue(float *acc, const float *bias, const float *emb_row)
{
    if (emb_row) {
#pragma unroll
        for (int j = 0; j < N; j += 2)
            upk2(add2(pk2(acc[j], acc[j + 1]), add2(pk2(bias[j], bias[j + 1]), pk2(__ldg(emb_row + j), __ldg(emb_row + j + 1)))),
                 acc[j], acc[j + 1]);
    } else {
#pragma unroll
        for (int j = 0; j < N; j += 2) upk2(add2(pk2(acc[j], acc[j + 1]), pk2(bias[j], bias[j + 1])), acc[j], acc[j + 1]);
    }
#pragma unroll
    for (int j = 0; j < N; j += 2) gelu_pair(acc[j], acc[j + 1]);
}

template <bool FIRST>
__global__ void __launch_bounds__(kFusedThreads, 2) fused_kernel(const __grid_constant__ CUtensorMap xmap,
                                                                 const FusedLaunch a)
{
    constexpr int CINA = FIRST ? 16 : 32;
    constexpr int NCGA = CINA / 8, KSA = CINA / 16, NMMA_A = 9 * KSA, NMMA_B = 18;
    constexpr int STAGE = NCGA * kWideGroup;
    constexpr int HB = 4 * kGroupStride;                           // one B-operand halo, 32 channels
    constexpr int WA = NMMA_A * 32 * 32, WB = NMMA_B * 32 * 32;    // packed weights, bytes
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *ha = smem;
    uint8_t *hb = ha + kFusedStages * STAGE;
    uint8_t *wa = hb + 2 * HB;
    uint8_t *wb = wa + WA;
    float *win = reinterpret_cast<float *>(wb + WB);
    uint64_t *full = reinterpret_cast<uint64_t *>(win + kWinX * kWinY);
    uint64_t *empty = full + kFusedStages;
    uint64_t *accA_full = empty + kFusedStages, *accA_empty = accA_full + 2;
    uint64_t *hb_full = accA_empty + 2, *hb_empty = hb_full + 2;
    uint64_t *accB_full = hb_empty + 2, *accB_empty = accB_full + 2;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(accB_empty + 2);
    volatile int *abort = reinterpret_cast<volatile int *>(tslot + 1);
    float *bias_s = reinterpret_cast<float *>(tslot + 4);  // [64]: layer A's then layer B's biases
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    for (int i = tid; i < WA / 16; i += kFusedThreads)
        reinterpret_cast<uint4 *>(wa)[i] = reinterpret_cast<const uint4 *>(a.wpack_a)[i];
    for (int i = tid; i < WB / 16; i += kFusedThreads)
        reinterpret_cast<uint4 *>(wb)[i] = reinterpret_cast<const uint4 *>(a.wpack_b)[i];
    if (tid < 32) {
        bias_s[tid] = a.bias_a[tid];
        bias_s[32 + tid] = a.bias_b[tid];
    }
    // rows 16 and 17 of B's operand halo feed only the two unused rows of B's MMA tile
    for (int i = tid; i < 2 * 4 * 2 * kHaloX; i += kFusedThreads) {
        const int px = i % kHaloX, row = 16 + (i / kHaloX) % 2, g = (i / (2 * kHaloX)) % 4, h = i / (8 * kHaloX);
        *reinterpret_cast<uint4 *>(hb + h * HB + g * kGroupStride + row * kRowStride + px * 16) = make_uint4(0u, 0u, 0u, 0u);
    }
    if (tid == 0) {
        for (int s = 0; s < kFusedStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&accA_full[b], 1);
            mbar_init(&accA_empty[b], 128);
            mbar_init(&hb_full[b], 128);
            mbar_init(&hb_empty[b], 1);
            mbar_init(&accB_full[b], 1);
            mbar_init(&accB_empty[b], 128);
        }
        *abort = 0;
    }
    if (warp == 1) tmem_alloc(tslot, kFusedCols);
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const int per_img = a.tiles_x * a.tiles_y, total = a.nimg * per_img;
    const int mine = my_tiles(total);

    if (FIRST && warp == 0) {
        // producer: layer 0's input channels on the 12 x 18 halo, from a 14 x 20 window of
        // the upsampled tile staged in shared memory (the same values and operations as the
        // kFirst producer); channels 8-15 are zero in every stage
        for (int s = 0; s < kFusedStages; ++s)
            for (int p = lane; p < kWideX * kWideY; p += 32)
                *reinterpret_cast<uint4 *>(ha + s * STAGE + kWideGroup + p * 16) = make_uint4(0u, 0u, 0u, 0u);
        for (int i = 0; i < mine; ++i) {
            const int s = i % kFusedStages;
            if (i >= kFusedStages &&
                !__all_sync(0xffffffffu, mbar_wait_abortable(&empty[s], ((i / kFusedStages) - 1) & 1, abort)))
                break;
            const int t = blockIdx.x + i * gridDim.x;
            const int img = t / per_img, rem = t - img * per_img;
            const int by = rem / a.tiles_x, bx = rem - by * a.tiles_x;
            const float *u = a.up + (size_t)img * a.W * a.W;
            const int x0 = bx * kBlockX - 3, y0 = by * kFusedBlockY - 3;  // window origin (image pixels)
            {
                constexpr int kWinPer = (kWinX * kWinY + 31) / 32;
                float w[kWinPer];
#pragma unroll
                for (int k = 0; k < kWinPer; ++k) {  // all loads first (one latency), then the stores
                    const int p = lane + 32 * k;
                    const int wy = p / kWinX, wx = p - wy * kWinX;
                    const int gx = x0 + wx, gy = y0 + wy;
                    w[k] = p < kWinX * kWinY && gx >= 0 && gy >= 0 && gx < a.W && gy < a.W
                               ? __ldg(u + (size_t)gy * a.W + gx) : 0.0f;
                }
#pragma unroll
                for (int k = 0; k < kWinPer; ++k)
                    if (lane + 32 * k < kWinX * kWinY) win[lane + 32 * k] = w[k];
            }
            __syncwarp();
            const float mean = __ldg(a.mean + img);
            const int lc = min(max(__ldg(a.level + img), 0), kLevels - 1);
            const float inv = 1.0f / __ldg(a.sigma_in + lc), inv2 = 1.0f / __ldg(a.sigma_out + lc);
            for (int p = lane; p < kWideX * kWideY; p += 32) {
                const int hy = p / kWideX, hx = p - hy * kWideX;
                const int gx = x0 + 1 + hx, gy = y0 + 1 + hy;
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (gx >= 0 && gy >= 0 && gx < a.W && gy < a.W) {
                    const int c = (hy + 1) * kWinX + hx + 1;
                    const float val = win[c];
                    const float d2x = gx > 0 && gx < a.W - 1
                                          ? __fsub_rn(__fadd_rn(win[c - 1], win[c + 1]), __fmul_rn(2.0f, val)) : 0.0f;
                    const float d2y = gy > 0 && gy < a.W - 1
                                          ? __fsub_rn(__fadd_rn(win[c - kWinX], win[c + kWinX]), __fmul_rn(2.0f, val))
                                          : 0.0f;
                    v.x = pack2((val - mean) * inv, (float)(gx & 1));
                    v.y = pack2((float)(gy & 1), 1.0f);
                    v.z = pack2(__fmul_rn(d2x, inv2), __fmul_rn(d2y, inv2));
                }
                *reinterpret_cast<uint4 *>(ha + s * STAGE + p * 16) = v;
            }
            fence_proxy_async_smem();  // the generic-proxy writes, before the tensor cores read them
            __syncwarp();              // and every lane is done with the window before it is refilled
            if (lane == 0) mbar_arrive(&full[s]);
        }
    } else if (warp == 0) {
        if (lane == 0) {  // producer: the 12 x 18 input halo of block i, 4 channel groups
            int i = 0;
            for (; i < mine; ++i) {
                const int s = i % kFusedStages;
                if (i >= kFusedStages && !mbar_wait_abortable(&empty[s], ((i / kFusedStages) - 1) & 1, abort)) break;
                const int t = blockIdx.x + i * gridDim.x;
                const int img = t / per_img, rem = t - img * per_img;
                const int by = rem / a.tiles_x, bx = rem - by * a.tiles_x;
                mbar_expect_tx(&full[s], 4 * kWideRow * kWideY);
#pragma unroll
                for (int cg = 0; cg < 4; ++cg)  // the bordered image's pixel (bx 8 - 1, by 14 - 1): image pixel - 2
                    tma_load_3d(ha + s * STAGE + cg * kWideGroup, &xmap, (bx * kBlockX - 1) * 8, by * kFusedBlockY - 1,
                                img * 4 + cg, &full[s]);
            }
            if (*abort)  // copies in flight land before the CTA leaves
                for (int k = i > kFusedStages ? i - kFusedStages : 0; k < i; ++k)
                    mbar_wait(&full[k % kFusedStages], (k / kFusedStages) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer: A(i) and B(j) each as soon as their inputs are ready
            constexpr uint32_t idesc = idesc_bf16(128, 32, 0, 0);
            const uint32_t wa_a = smem_u32(wa), wb_a = smem_u32(wb);
            int na = 0, nb = 0;  // the next blocks of layer A and of layer B to issue
            unsigned idle = 0;
            while (nb < mine) {
                bool issued = false;
                // B first: it unblocks an epilogue chain, and MMAs run in issue order
                if (nb < na) {
                    const int h = nb & 1;
                    if (mbar_try(&hb_full[h], (nb >> 1) & 1) && (nb < 2 || mbar_try(&accB_empty[h], ((nb >> 1) - 1) & 1))) {
                        tc_fence_after();
                        const uint32_t h_a = smem_u32(hb + h * HB);
#pragma unroll
                        for (int q = 0; q < NMMA_B; ++q) {
                            const int tap = q / 2, st = q - tap * 2;
                            const int dy = tap / 3, dx = tap - dy * 3;
                            const uint64_t ad =
                                sdesc(h_a + 2 * st * kGroupStride + dy * kRowStride + dx * 16, kGroupStride, kRowStride);
                            const uint64_t bd = sdesc(wb_a + q * 32 * 32, 128, 256);
                            mma_bf16(tmem + 128 * h + 64, ad, bd, idesc, q > 0 ? 1u : 0u);
                        }
                        mma_commit(&hb_empty[h]);
                        mma_commit(&accB_full[h]);
                        ++nb;
                        issued = true;
                    }
                }
                if (na < mine) {
                    const int s = na % kFusedStages, b = na & 1;
                    if (mbar_try(&full[s], (na / kFusedStages) & 1) &&
                        (na < 2 || mbar_try(&accA_empty[b], ((na >> 1) - 1) & 1))) {
                        tc_fence_after();
                        const uint32_t h_a = smem_u32(ha + s * STAGE);
#pragma unroll
                        for (int T = 0; T < 2; ++T) {
                            const int o = 2 * T;  // tile origin: column o, row 0 of the 10 x 16 region
#pragma unroll
                            for (int q = 0; q < NMMA_A; ++q) {
                                const int tap = q / KSA, st = q - tap * KSA;
                                const int dy = tap / 3, dx = tap - dy * 3;
                                const uint64_t ad = sdesc(h_a + 2 * st * kWideGroup + dy * kWideRow + (o + dx) * 16,
                                                          kWideGroup, kWideRow);
                                const uint64_t bd = sdesc(wa_a + q * 32 * 32, 128, 256);
                                mma_bf16(tmem + 128 * b + 32 * T, ad, bd, idesc, q > 0 ? 1u : 0u);
                            }
                        }
                        mma_commit(&empty[s]);
                        mma_commit(&accA_full[b]);
                        ++na;
                        issued = true;
                    }
                }
                if (issued) {
                    idle = 0;
                } else if (*abort) {
                    break;
                } else if (++idle > (1u << 22)) {  // nothing became ready: give up
                    *abort = 1;
                    break;
                }
            }
            if (*abort) {  // the MMAs issued complete before the tensor memory is freed
                if (na > 0) mbar_wait(&empty[(na - 1) % kFusedStages], ((na - 1) / kFusedStages) & 1);
                if (nb > 0) mbar_wait(&hb_empty[(nb - 1) & 1], ((nb - 1) >> 1) & 1);
            }
        }
    } else {  // epilogue group g = block parity; rows 32 q .. 32 q + 31 of each accumulator
        const int g = (warp - 2) >> 2, q = warp & 3, m = q * 32 + lane;
        const uint32_t lanes = (uint32_t)(q * 32) << 16;
        const int Wp = a.W + 2;
        const size_t plane = (size_t)Wp * Wp;
        uint8_t *dst = hb + g * HB;
        for (int i = g; i < mine; i += 2) {
            // layer A's two tiles
            if (!__all_sync(0xffffffffu, mbar_wait_abortable(&accA_full[g], (i >> 1) & 1, abort))) break;
            if (i >= 2 && !__all_sync(0xffffffffu, mbar_wait_abortable(&hb_empty[g], ((i >> 1) - 1) & 1, abort))) break;
            tc_fence_after();
            const int t = blockIdx.x + i * gridDim.x;
            const int img = t / per_img, rem = t - img * per_img;
            const int by = rem / a.tiles_x, bx = rem - by * a.tiles_x;
            const float *emb_row = a.emb ? a.emb + (size_t)min(max(__ldg(a.level + img), 0), kLevels - 1) * 32 : nullptr;
            float acc[32];
            tmem_ld32(tmem + 128 * g + lanes, acc);
            {  // first tile: the region's columns 0-7, rows 0-15, one pixel per thread
                const int rx = m & 7, ry = m >> 3;
                const int gx = bx * kBlockX - 1 + rx, gy = by * kFusedBlockY - 1 + ry;
                uint4 u[4] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u),
                              make_uint4(0u, 0u, 0u, 0u)};
                if (gx >= 0 && gy >= 0 && gx < a.W && gy < a.W) {
                    hidden_epilogue<32>(acc, bias_s, emb_row);
#pragma unroll
                    for (int c = 0; c < 4; ++c)
                        u[c] = make_uint4(pack2(acc[8 * c + 0], acc[8 * c + 1]), pack2(acc[8 * c + 2], acc[8 * c + 3]),
                                          pack2(acc[8 * c + 4], acc[8 * c + 5]), pack2(acc[8 * c + 6], acc[8 * c + 7]));
                }
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    *reinterpret_cast<uint4 *>(dst + c * kGroupStride + ry * kRowStride + rx * 16) = u[c];
            }
            tmem_ld32(tmem + 128 * g + 32 + lanes, acc);
            tc_fence_before();
            mbar_arrive(&accA_empty[g]);
            {  // second tile: only its rows at columns 8 and 9 of the region (lanes 6, 7 of each
               // 8-lane row group: 8 rows per warp), spread over the warp: lane l takes row
               // (l >> 2) of those 8 and channels 8 (l & 3) .. 8 (l & 3) + 7
                const int j = lane >> 2, cg = lane & 3;
                const int src = 8 * (j >> 1) + 6 + (j & 1);
                float v[8];
#pragma unroll
                for (int c = 0; c < 32; ++c) {
                    const float x = __shfl_sync(0xffffffffu, acc[c], src);
                    if ((c >> 3) == cg) v[c & 7] = x;
                }
                const int ms = q * 32 + src;
                const int rx = 2 + (ms & 7), ry = ms >> 3;  // rx is 8 or 9
                const int gx = bx * kBlockX - 1 + rx, gy = by * kFusedBlockY - 1 + ry;
                uint4 u = make_uint4(0u, 0u, 0u, 0u);
                if (gx >= 0 && gy >= 0 && gx < a.W && gy < a.W) {
                    hidden_epilogue<8>(v, bias_s + 8 * cg, emb_row ? emb_row + 8 * cg : nullptr);
                    u = make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]), pack2(v[4], v[5]), pack2(v[6], v[7]));
                }
                *reinterpret_cast<uint4 *>(dst + cg * kGroupStride + ry * kRowStride + rx * 16) = u;
            }
            fence_proxy_async_smem();  // generic writes of B's operand, before the tensor cores read it
            mbar_arrive(&hb_full[g]);
            // layer B
            if (!__all_sync(0xffffffffu, mbar_wait_abortable(&accB_full[g], (i >> 1) & 1, abort))) break;
            tc_fence_after();
            tmem_ld32(tmem + 128 * g + 64 + lanes, acc);
            tc_fence_before();
            mbar_arrive(&accB_empty[g]);
            const int px = bx * kBlockX + (m & 7), py = by * kFusedBlockY + (m >> 3);
            if ((m >> 3) < kFusedBlockY && px < a.W && py < a.W) {
                hidden_epilogue<32>(acc, bias_s + 32, nullptr);
                store_bf16<32>(a.out, img, plane, (size_t)(py + 1) * Wp + (px + 1), acc);
            }
        }
    }
    __syncthreads();
    if (tid == 0 && *abort) atomicExch(a.status, TP_E_TIMEOUT);
    tc_fence_after();
    if (warp == 1) tmem_dealloc(tmem, kFusedCols);
}

template <int CIN, int COUT>
constexpr int wgrad_tiles()
{
    return (9 * CIN / 8 + 15) / 16;
}
template <int CIN, int COUT>
constexpr int wgrad_stage_bytes()
{
    return wgrad_tiles<CIN, COUT>() * 16 * kBoxBytes + (COUT / 8) * kBoxBytes;
}
template <int CIN, int COUT>
constexpr int wgrad_smem_bytes()
{
    return 2 * wgrad_stage_bytes<CIN, COUT>() + 128;
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(kRoleThreads) wgrad_kernel(const __grid_constant__ CUtensorMap xmap,
                                                             const __grid_constant__ CUtensorMap zmap, const WgradLaunch a)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    constexpr int NCG = CIN / 8, NGO = COUT / 8, NG = 9 * NCG;
    constexpr int NMT = wgrad_tiles<CIN, COUT>();
    constexpr int ABYTES = NMT * 16 * kBoxBytes;
    constexpr int STAGE = wgrad_stage_bytes<CIN, COUT>();
    constexpr uint32_t TCOLS = NMT * 32 <= 32 ? 32 : (NMT * 32 <= 64 ? 64 : 128);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + 2 * STAGE);
    uint64_t *empty = full + 2;
    uint64_t *done = empty + 2;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
    volatile int *abort = reinterpret_cast<volatile int *>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // rows of the last M tile past the real (tap, channel) groups are never loaded
    for (int s = 0; s < 2; ++s)
        for (int i = NG * kBoxBytes / 16 + tid; i < ABYTES / 16; i += kRoleThreads)
            reinterpret_cast<uint4 *>(smem + s * STAGE)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1 + 128);  // the MMAs' commit and the 128 bias threads
        }
        mbar_init(done, 1);
        *abort = 0;
    }
    if (warp == 1) tmem_alloc(tslot, TCOLS);
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const int per_img = a.tiles_x * a.tiles_y, total = a.nimg * per_img;
    const int mine = my_tiles(total);

    if (warp == 0) {
        if (lane == 0) {
            int i = 0;
            for (; i < mine; ++i) {
                const int s = i & 1;
                if (i >= 2 && !mbar_wait_abortable(&empty[s], ((i >> 1) - 1) & 1, abort)) break;
                const int t = blockIdx.x + i * gridDim.x;
                const int img = t / per_img, rem = t - img * per_img;
                const int by = rem / a.tiles_x, bx = rem - by * a.tiles_x;
                const int x0 = bx * kBlockX, y0 = by * kBlockY;
                uint8_t *st = smem + s * STAGE;
                mbar_expect_tx(&full[s], (NG + NGO) * kBoxBytes);
                for (int g = 0; g < NG; ++g) {
                    const int tap = g / NCG, cg = g - tap * NCG;
                    const int dy = tap / 3, dx = tap - dy * 3;
                    tma_load_3d(st + g * kBoxBytes, &xmap, (x0 + dx) * 8, y0 + dy, img * NCG + cg, &full[s]);
                }
#pragma unroll
                for (int go = 0; go < NGO; ++go)
                    tma_load_3d(st + ABYTES + go * kBoxBytes, &zmap, (x0 + 1) * 8, y0 + 1, img * NGO + go, &full[s]);
            }
            if (*abort)
                for (int k = i > 2 ? i - 2 : 0; k < i; ++k) mbar_wait(&full[k & 1], (k >> 1) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16(128, COUT, 1, 1);
            int i = 0;
            for (; i < mine; ++i) {
                const int s = i & 1;
                if (!mbar_wait_abortable(&full[s], (i >> 1) & 1, abort)) break;
                tc_fence_after();
                const uint32_t a_a = smem_u32(smem + s * STAGE), b_a = a_a + ABYTES;
#pragma unroll
                for (int mt = 0; mt < NMT; ++mt)
#pragma unroll
                    for (int k = 0; k < kBlockY / 2; ++k) {
                        const uint64_t ad = sdesc(a_a + mt * 16 * kBoxBytes + k * 256, 128, kBoxBytes);
                        const uint64_t bd = sdesc(b_a + k * 256, 128, kBoxBytes);
                        mma_bf16(tmem + mt * 32, ad, bd, idesc, (i > 0 || k > 0) ? 1u : 0u);
                    }
                mma_commit(&empty[s]);
            }
            mma_commit(done);  // every MMA of this CTA
            if (*abort && i > 0) mbar_wait(&empty[(i - 1) & 1], ((i - 1) >> 1) & 1);
        }
    } else {
        const int bt = tid - 64, bn = bt % COUT;
        const int q = warp & 3;
        int i = 0;
        for (; i < mine; ++i) {
            const int s = i & 1;
            if (!__all_sync(0xffffffffu, mbar_wait_abortable(&full[s], (i >> 1) & 1, abort))) break;
            // bias (and level-embedding) gradient of this block from the staged dZ tile
            const __nv_bfloat16 *bz = reinterpret_cast<const __nv_bfloat16 *>(smem + s * STAGE + ABYTES);
            float sum = 0.0f;
            for (int k = bt / COUT; k < kBlockX * kBlockY; k += 128 / COUT)
                sum += __bfloat162float(bz[((bn >> 3) * kBoxBytes + (k >> 3) * 128 + (k & 7) * 16) / 2 + (bn & 7)]);
            const int t = blockIdx.x + i * gridDim.x;
            const int img = t / per_img;
            atomicAdd(a.gb + bn, sum);
            if (a.gemb) atomicAdd(a.gemb + (size_t)min(max(a.level[img], 0), kLevels - 1) * COUT + bn, sum);
            mbar_arrive(&empty[s]);
        }
        if (i == mine && mine > 0 && __all_sync(0xffffffffu, mbar_wait_abortable(done, 0, abort))) {
            tc_fence_after();
#pragma unroll
            for (int mt = 0; mt < NMT; ++mt) {
                float v[COUT];
                const uint32_t taddr = tmem + mt * 32 + ((uint32_t)(q * 32) << 16);
                if (COUT == 32)
                    tmem_ld32(taddr, v);
                else
                    tmem_ld16(taddr, v);
                const int m = mt * 128 + q * 32 + lane;
                if (m < 9 * CIN)
#pragma unroll
                    for (int n = 0; n < COUT; ++n) atomicAdd(a.gw + (size_t)n * 9 * CIN + m, v[n]);
            }
        }
    }
    __syncthreads();
    if (tid == 0 && *abort) atomicExch(a.status, TP_E_TIMEOUT);
    tc_fence_after();
    if (warp == 1) tmem_dealloc(tmem, TCOLS);
}

// ---------------------------------------------------------------- launch helpers
int sm_count() { return tp::device_sm_count(); }

// CTAs of `kernel` resident on one SM, from its shared memory, registers, threads
// and tensor-memory columns.  The runtime's occupancy query assumes one CTA per SM
// for kernels that allocate tensor memory; on GB300 several run together as long
// as their columns fit in the SM's 512.  An overestimate only queues CTAs (they
// never wait on one another).
template <typename K>
int grid_for(K kernel, int smem, int tmem_cols, int units, int *grid, int threads = kRoleThreads)
{
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, int> cache;  // per device and kernel instance
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    int &per_sm = cache[std::make_pair(dev, reinterpret_cast<const void *>(kernel))];
    if (!per_sm) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return tp::cuda_fail("cudaFuncSetAttribute (learned)", e);
        cudaFuncAttributes fa;
        e = cudaFuncGetAttributes(&fa, kernel);
        if (e != cudaSuccess) return tp::cuda_fail("cudaFuncGetAttributes (learned)", e);
        int dev = 0, smem_sm = 0, regs_sm = 0, reserved = 0, threads_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
        cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
        const int warps = (threads + 31) / 32;
        const int regs_warp = (fa.numRegs * 32 + 255) / 256 * 256;
        int n = smem_sm / (smem + (int)fa.sharedSizeBytes + reserved);
        n = std::min(n, regs_sm / std::max(1, regs_warp * warps));
        n = std::min(n, threads_sm / threads);
        n = std::min(n, 512 / tmem_cols);
        if (n < 1) return tp::fail(TP_E_BAD_ARG, "learned: kernel does not fit on an SM");
        per_sm = n;
    }
    *grid = std::max(1, std::min(units, per_sm * sm_count()));
    return TP_OK;
}

template <int CIN, int COUT, int MODE>
int conv_instance(const ConvLaunch &a, const CUtensorMap *halo, cudaStream_t s)
{
    const int units = a.nimg * a.tiles_x * a.tiles_y;
    if (units <= 0) return TP_OK;
    constexpr int smem = conv_smem_bytes<CIN, COUT>();
    int grid = 0;
    int rc = grid_for(conv_kernel<CIN, COUT, MODE>, smem, 64, units, &grid, conv_threads<MODE>());
    if (rc) return rc;
    conv_kernel<CIN, COUT, MODE><<<grid, conv_threads<MODE>(), smem, s>>>(*halo, a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TP_OK : tp::cuda_fail("conv kernel launch", e);
}

template <bool FIRST>
int fused_instance(const FusedLaunch &a, const CUtensorMap *wide, cudaStream_t s)
{
    const int units = a.nimg * a.tiles_x * a.tiles_y;
    if (units <= 0) return TP_OK;
    constexpr int smem = fused_smem_bytes<FIRST ? 16 : 32>();
    int grid = 0;
    int rc = grid_for(fused_kernel<FIRST>, smem, (int)kFusedCols, units, &grid, kFusedThreads);
    if (rc) return rc;
    fused_kernel<FIRST><<<grid, kFusedThreads, smem, s>>>(*wide, a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TP_OK : tp::cuda_fail("fused convolution launch", e);
}

template <int CIN, int COUT>
int wgrad_instance(const WgradLaunch &a, const CUtensorMap *xb, const CUtensorMap *zb, cudaStream_t s)
{
    const int units = a.nimg * a.tiles_x * a.tiles_y;
    if (units <= 0) return TP_OK;
    constexpr int smem = wgrad_smem_bytes<CIN, COUT>();
    int grid = 0;
    constexpr int NMT = wgrad_tiles<CIN, COUT>();
    int rc = grid_for(wgrad_kernel<CIN, COUT>, smem, NMT * 32 <= 32 ? 32 : (NMT * 32 <= 64 ? 64 : 128), units, &grid);
    if (rc) return rc;
    wgrad_kernel<CIN, COUT><<<grid, kRoleThreads, smem, s>>>(*xb, *zb, a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TP_OK : tp::cuda_fail("weight-gradient kernel launch", e);
}

// ---------------------------------------------------------------- small kernels
__global__ void pack_kernel(const float *w, int cin, int cout, uint8_t *fwd, uint8_t *bwd)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cout * 9 * cin) return;
    const int co = i / (9 * cin), rem = i - co * 9 * cin, tap = rem / cin, ci = rem - tap * cin;
    const __nv_bfloat16 v = __float2bfloat16_rn(w[i]);
    {  // forward: B[n = co][k = (tap, ci)], 16-channel K steps
        const int q = tap * (cin / 16) + ci / 16, kk = ci % 16;
        const size_t off = (size_t)q * cout * 32 + (co / 8) * 256 + (kk / 8) * 128 + (co % 8) * 16 + (kk % 8) * 2;
        *reinterpret_cast<__nv_bfloat16 *>(fwd + off) = v;
    }
    {  // data gradient: a convolution of dZ with B'[n = ci][k = (8 - tap, co)]
        const int tp_ = 8 - tap;
        const int q = tp_ * (cout / 16) + co / 16, kk = co % 16;
        const size_t off = (size_t)q * cin * 32 + (ci / 8) * 256 + (kk / 8) * 128 + (ci % 8) * 16 + (kk % 8) * 2;
        *reinterpret_cast<__nv_bfloat16 *>(bwd + off) = v;
    }
}

// Mean of one tile by a block of 256 threads: strided per-thread sums in double, then
// a tree over the threads (the same order wherever it is used).
__device__ float tile_mean(const float *u, int n)
{
    __shared__ double part[256];
    double s = 0.0;
    // each thread's values in the same order as one strided loop, loaded 8 at a time
    // ahead of the (dependent) additions
    int i = threadIdx.x;
    for (; i + 7 * (int)blockDim.x < n; i += 8 * blockDim.x) {
        float v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = __ldg(u + i + k * blockDim.x);
#pragma unroll
        for (int k = 0; k < 8; ++k) s += v[k];
    }
    for (; i < n; i += blockDim.x) s += u[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) part[threadIdx.x] += part[threadIdx.x + k];
        __syncthreads();
    }
    return (float)(part[0] / n);
}

__global__ void mean_kernel(const float *up, int W, float *mean)
{
    const int n = W * W;
    const float m = tile_mean(up + (size_t)blockIdx.x * n, n);
    if (threadIdx.x == 0) mean[blockIdx.x] = m;
}

__global__ void prep_kernel(const float *up, const int *level, const float *sigma_in, const float *sigma_out, int W,
                            __nv_bfloat16 *x0)
{
    const int img = blockIdx.x, n = W * W;
    const float *u = up + (size_t)img * n;
    const float mean = tile_mean(u, n);
    const int lc = min(max(level[img], 0), kLevels - 1);
    const float inv = 1.0f / sigma_in[lc], inv2 = 1.0f / sigma_out[lc];
    const int Wp = W + 2;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int y = i / W, x = i - y * W;
        // second differences in fp32 (0 on the tile's edge rows / columns)
        const float d2x = x > 0 && x < W - 1 ? __fsub_rn(__fadd_rn(u[i - 1], u[i + 1]), __fmul_rn(2.0f, u[i])) : 0.0f;
        const float d2y = y > 0 && y < W - 1 ? __fsub_rn(__fadd_rn(u[i - W], u[i + W]), __fmul_rn(2.0f, u[i])) : 0.0f;
        float v[16] = {(u[i] - mean) * inv, (float)(x & 1), (float)(y & 1), 1.0f, __fmul_rn(d2x, inv2),
                       __fmul_rn(d2y, inv2)};
        store_bf16<16>(x0, img, (size_t)Wp * Wp, (size_t)(y + 1) * Wp + x + 1, v);
    }
}

__global__ void loss_kernel(const float *pred, const float *target, const int *level, const float *sigma_out, int W,
                            int nimg, float scale, __nv_bfloat16 *dz, float *loss)
{
    const size_t n = (size_t)W * W;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    float d2 = 0.0f;
    if (i < n * nimg) {
        const int img = (int)(i / n), p = (int)(i - (size_t)img * n), y = p / W, x = p - y * W;
        const float t = target[i] / sigma_out[min(max(level[img], 0), kLevels - 1)];
        const float d = pred[i] - t;
        d2 = d * d;
        float v[16] = {2.0f * d * scale};
        const int Wp = W + 2;
        store_bf16<16>(dz, img, (size_t)Wp * Wp, (size_t)(y + 1) * Wp + x + 1, v);
    }
    for (int o = 16; o > 0; o >>= 1) d2 += __shfl_xor_sync(0xffffffffu, d2, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, d2);
}

__global__ void adam_kernel(float *p, const float *g, float *m, float *v, const float *mask, int n, float lr, float b1,
                            float b2, float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] * mask[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] = mask[i] * (p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps));
}

__global__ void scale_kernel(const float *pred, const int *level, const float *sigma_out, int W, int nimg, float *out)
{
    const size_t n = (size_t)W * W;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * nimg) return;
    out[i] = pred[i] * sigma_out[min(max(level[i / n], 0), kLevels - 1)];
}

// the eight symmetries of the square: bit 2 transposes, bit 0 mirrors x, bit 1 mirrors y
__global__ void gather_kernel(const float *up, const float *res, const int *src, const int *dihedral, int W, int n,
                              float *up_out, float *res_out)
{
    const size_t np = (size_t)W * W;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np * n) return;
    const int s = (int)(i / np), p = (int)(i - (size_t)s * np), y = p / W, x = p - y * W;
    const int d = dihedral[s];
    int u = x, v = y;
    if (d & 4) {
        u = y;
        v = x;
    }
    if (d & 1) u = W - 1 - u;
    if (d & 2) v = W - 1 - v;
    const size_t o = (size_t)src[s] * np + (size_t)v * W + u;
    up_out[i] = up[o];
    res_out[i] = res[o];
}

__global__ void upsample_kernel(const float *elev, int pitch, long long plane_stride, long long slot_stride,
                                const int *parent_slot, const int *tx, const int *ty, int W, int n, float *up)
{
    const size_t np = (size_t)W * W;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np * n) return;
    const int s = (int)(i / np), p = (int)(i - (size_t)s * np), j = p / W, c = p - j * W;
    const int ts = W - 5;
    const float *P = elev + (long long)parent_slot[s] * slot_stride;  // plane 0: zf
    up[i] = tp::upsample_cpu_order(P, pitch, c, j, 1 + (tx[s] & 1) * ts / 2, 1 + (ty[s] & 1) * ts / 2);
    (void)plane_stride;
}

__global__ void store_residuals_kernel(const float *pred, const int *level, const float *sigma_out, int W, int n,
                                       float *res, int pitch, long long slot_stride, const int *slots)
{
    const size_t np = (size_t)W * W;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np * n) return;
    const int s = (int)(i / np), p = (int)(i - (size_t)s * np), y = p / W, x = p - y * W;
    res[(long long)slots[s] * slot_stride + (long long)y * pitch + x] =
        pred[i] * sigma_out[min(max(level[s], 0), kLevels - 1)];
}

inline unsigned blocks_for(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

int launch_conv(int cin, int cout, int mode, const ConvLaunch &a, const CUtensorMap *halo, cudaStream_t s)
{
    if (cin == 16 && cout == 32 && mode == kHidden) return conv_instance<16, 32, kHidden>(a, halo, s);
    if (cin == 16 && cout == 32 && mode == kFirst) return conv_instance<16, 32, kFirst>(a, halo, s);
    if (cin == 32 && cout == 32 && mode == kHidden) return conv_instance<32, 32, kHidden>(a, halo, s);
    if (cin == 32 && cout == 16 && mode == kLast) return conv_instance<32, 16, kLast>(a, halo, s);
    if (cin == 16 && cout == 32 && mode == kBackData) return conv_instance<16, 32, kBackData>(a, halo, s);
    if (cin == 32 && cout == 32 && mode == kBackData) return conv_instance<32, 32, kBackData>(a, halo, s);
    return tp::fail(TP_E_BAD_ARG, "learned: no convolution instance for this shape");
}

int launch_fused(bool first, const FusedLaunch &a, const CUtensorMap *wide, cudaStream_t s)
{
    return first ? fused_instance<true>(a, wide, s) : fused_instance<false>(a, wide, s);
}

int launch_wgrad(int cin, int cout, const WgradLaunch &a, const CUtensorMap *xb, const CUtensorMap *zb, cudaStream_t s)
{
    if (cin == 16 && cout == 32) return wgrad_instance<16, 32>(a, xb, zb, s);
    if (cin == 32 && cout == 32) return wgrad_instance<32, 32>(a, xb, zb, s);
    if (cin == 32 && cout == 16) return wgrad_instance<32, 16>(a, xb, zb, s);
    return tp::fail(TP_E_BAD_ARG, "learned: no weight-gradient instance for this shape");
}

void launch_pack(const float *w, int cin, int cout, uint8_t *fwd, uint8_t *bwd, cudaStream_t s)
{
    const int n = cout * 9 * cin;
    pack_kernel<<<blocks_for(n, 256), 256, 0, s>>>(w, cin, cout, fwd, bwd);
}

void launch_prep(const float *up, const int *level, const float *sigma_in, const float *sigma_out, int W, int nimg,
                 __nv_bfloat16 *x0,
                 cudaStream_t s)
{
    if (nimg > 0) prep_kernel<<<nimg, 256, 0, s>>>(up, level, sigma_in, sigma_out, W, x0);
}

void launch_means(const float *up, int W, int nimg, float *mean, cudaStream_t s)
{
    if (nimg > 0) mean_kernel<<<nimg, 256, 0, s>>>(up, W, mean);
}

void launch_loss(const float *pred, const float *target, const int *level, const float *sigma_out, int W, int nimg,
                 __nv_bfloat16 *dz, float *loss, cudaStream_t s)
{
    const size_t n = (size_t)W * W * nimg;
    if (n) loss_kernel<<<blocks_for(n, 256), 256, 0, s>>>(pred, target, level, sigma_out, W, nimg, 1.0f / (float)n, dz, loss);
}

void launch_adam(float *p, const float *g, float *m, float *v, const float *mask, int n, float lr, float b1, float b2,
                 float eps, int step, cudaStream_t s)
{
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    adam_kernel<<<blocks_for(n, 256), 256, 0, s>>>(p, g, m, v, mask, n, lr, b1, b2, eps, c1, c2);
}

void launch_scale_out(const float *pred, const int *level, const float *sigma_out, int W, int nimg, float *out,
                      cudaStream_t s)
{
    const size_t n = (size_t)W * W * nimg;
    if (n) scale_kernel<<<blocks_for(n, 256), 256, 0, s>>>(pred, level, sigma_out, W, nimg, out);
}

void launch_gather(const float *up, const float *res, const int *src, const int *dihedral, int W, int n, float *up_out,
                   float *res_out, cudaStream_t s)
{
    const size_t t = (size_t)W * W * n;
    if (t) gather_kernel<<<blocks_for(t, 256), 256, 0, s>>>(up, res, src, dihedral, W, n, up_out, res_out);
}

void launch_upsample(const float *elev, int pitch, long long plane_stride, long long slot_stride, const int *parent_slot,
                     const int *tx, const int *ty, int W, int n, float *up, cudaStream_t s)
{
    const size_t t = (size_t)W * W * n;
    if (t) upsample_kernel<<<blocks_for(t, 256), 256, 0, s>>>(elev, pitch, plane_stride, slot_stride, parent_slot, tx, ty, W, n, up);
}

void launch_store_residuals(const float *pred, const int *level, const float *sigma_out, int W, int n, float *res,
                            int pitch, long long slot_stride, const int *slots, cudaStream_t s)
{
    const size_t t = (size_t)W * W * n;
    if (t) store_residuals_kernel<<<blocks_for(t, 256), 256, 0, s>>>(pred, level, sigma_out, W, n, res, pitch, slot_stride, slots);
}

}  // namespace learned
}  // namespace tp
