// Persistent, double-buffered elevation + normal tile kernel for sm_103a.
//
// A frame is a list of work units: one band of rows [j0, j1) of one child tile
// (a whole 101-wide tile, or a quarter of a 197-wide one), for up to two tile
// widths.  A grid of resident CTAs pulls units from a device counter in frame
// order; because the host lists parents before children, a unit's parent tile
// has always been taken by a running CTA, and a per-job completion counter
// (release on the producer side, acquire + bounded wait on the consumer side)
// orders a child after its parent inside the single launch.
//
// Per unit, one thread issues two TMA copies into a shared-memory stage,
// completing on that stage's mbarrier:
//   * the residual rows [j0 - 1, j1 + 1) of the tile's residual window, and
//   * the parent zf window those rows' stencil reads;
// every thread adds cp.async copies of the parent zm at the coarse-mesh
// vertices zc interpolates.  Two stages alternate: the copies of the next unit
// are in flight while the current one is computed.
//
// Phase A computes zf, zc, zm of rows [j0 - 1, j1] (the band plus one halo row
// each side), writing the band rows to HBM with 16-byte stores and each row's zm
// over its residual in shared memory; every thread sweeps one column quad down a
// strip of rows holding the four parent rows its stencil reads in registers.
// Phase B forms the normals of the band rows from that zm: each lane reads the
// 8 columns around its quad of normals from the row and the rows above and below.
//
// Arithmetic follows the reference exactly:
//  * stencil: CPUElevationProducer.cpp:202-238 (the same loops as
//    ResidualProducer.cpp:342-384 and HeightMipmap.cpp:449-497), in that
//    operation order, each operation rounded on its own (__f*_rn), so the result
//    is bit-identical to a CPU build without floating-point contraction;
//  * residual, noise, zc, zm: upsampleShader.glsl main()
//    (terrain/examples/terrain1/upsampleShader.glsl:81-125; flip variant
//    terrain/examples/terrain4/upsampleShader.glsl:112-127; modulated noise
//    demo/shaders/elevation/upsampleShader.glsl:140-203);
//  * normals: terrain/examples/terrain1/normalShader.glsl:57-74, point sampling
//    of the zm channel.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <type_traits>

#include "tp_internal.h"

__device__ int g_tp_status = 0;  // TP_OK, or the first TP_E_* a kernel reported

namespace {

constexpr int kThreads = tp::kFrameThreads;
constexpr int kWarps = kThreads / 32;
constexpr unsigned kWaitLimit = 1u << 22;   // mbarrier polls before a copy wait is declared failed
constexpr unsigned kDepLimit = 1u << 22;    // dependency polls (64 ns back-off) before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity)
{
    for (unsigned k = 0; k < kWaitLimit; ++k)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y, int z)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void cp_async4(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all_but_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void fence_proxy_async_global()
{
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int floordiv(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// floor(a / (2g)) and a mod 2g: a shift and a mask when g is a power of two
// (gshift = log2(2g)), a division otherwise (gshift < 0).
__device__ __forceinline__ int fdiv2g(int a, int g, int gshift) { return gshift >= 0 ? a >> gshift : floordiv(a, 2 * g); }
__device__ __forceinline__ int fmod2g(int a, int g, int gshift)
{
    return gshift >= 0 ? a & ((1 << gshift) - 1) : a - 2 * g * floordiv(a, 2 * g);
}

// 4x4 operators of the modulated-noise shader, entry k weighing parent sample
// (x0 + k % 4, y0 + k / 4) (demo/shaders/elevation/upsampleShader.glsl:60-115).
__constant__ float c_slopex[4][16] = {
    {0, 0, 0, 0, 1, 0, -1, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0.5f, 0.5f, -0.5f, -0.5f, 0, 0, 0, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0.5f, 0, -0.5f, 0, 0.5f, 0, -0.5f, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0.25f, 0.25f, -0.25f, -0.25f, 0.25f, 0.25f, -0.25f, -0.25f, 0, 0, 0, 0}};
__constant__ float c_slopey[4][16] = {
    {0, 1, 0, 0, 0, 0, 0, 0, 0, -1, 0, 0, 0, 0, 0, 0},
    {0, 0.5f, 0.5f, 0, 0, 0, 0, 0, 0, -0.5f, -0.5f, 0, 0, 0, 0, 0},
    {0, 0.5f, 0, 0, 0, 0.5f, 0, 0, 0, -0.5f, 0, 0, 0, -0.5f, 0, 0},
    {0, 0.25f, 0.25f, 0, 0, 0.25f, 0.25f, 0, 0, -0.25f, -0.25f, 0, 0, -0.25f, -0.25f, 0}};
__constant__ float c_curv[4][16] = {
    {0, -1, 0, 0, -1, 4, -1, 0, 0, -1, 0, 0, 0, 0, 0, 0},
    {0, -0.5f, -0.5f, 0, -0.5f, 1.5f, 1.5f, -0.5f, 0, -0.5f, -0.5f, 0, 0, 0, 0, 0},
    {0, -0.5f, 0, 0, -0.5f, 1.5f, -0.5f, 0, -0.5f, 1.5f, -0.5f, 0, 0, -0.5f, 0, 0},
    {0, -0.25f, -0.25f, 0, -0.25f, 0.5f, 0.5f, -0.25f, -0.25f, 0.5f, 0.5f, -0.25f, 0, -0.25f, -0.25f, 0}};

// mdot: four column dot products, each left to right, summed left to right.
__device__ __forceinline__ float mdot16(const float *cz, const float *M)
{
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float d = __fmul_rn(cz[4 * c], M[4 * c]);
        d = __fadd_rn(d, __fmul_rn(cz[4 * c + 1], M[4 * c + 1]));
        d = __fadd_rn(d, __fmul_rn(cz[4 * c + 2], M[4 * c + 2]));
        d = __fadd_rn(d, __fmul_rn(cz[4 * c + 3], M[4 * c + 3]));
        s = c == 0 ? d : __fadd_rn(s, d);
    }
    return s;
}

__device__ __forceinline__ float demo_modulation(const float *cz, int mi, float mps)
{
    float sx = mdot16(cz, c_slopex[mi]);
    float sy = mdot16(cz, c_slopey[mi]);
    float nz = __fmul_rn(2.0f, mps);
    float slope = __fdiv_rn(__fsqrt_rn(__fadd_rn(__fmul_rn(sx, sx), __fmul_rn(sy, sy))), nz);
    float curv = __fdiv_rn(mdot16(cz, c_curv[mi]), mps);
    float a = __fmul_rn(4.0f, curv);
    a = a < 0.0f ? 0.0f : (a > 1.5f ? 1.5f : a);
    float b = __fsub_rn(__fmul_rn(2.0f, slope), 0.5f);
    b = b < 0.1f ? 0.1f : (b > 4.0f ? 4.0f : b);
    return a > b ? a : b;
}

__device__ __forceinline__ void report(int code) { atomicCAS(&g_tp_status, 0, code); }

// A unit as decoded by thread 0 and shared with the CTA.
struct UnitInfo {
    int valid;    // 0: past the end of the frame
    int job;      // job index
    int band;
    int skip;     // debug builds: the job failed its index checks and is not produced
};

#ifdef TP_DEBUG
// Debug builds: a job's indexes against the storages and the job list before any of
// them addresses memory; a bad job sets the status word to TP_E_BOUNDS.
__device__ bool job_in_bounds(const tp::ClassLaunch &c, int job)
{
    const tp_tile_job &J = c.jobs[job];
    const bool ok = J.out_slot >= 0 && J.out_slot < c.elev_cap && J.level >= 0 && J.level <= 30 &&
                    (J.level == 0 || (J.parent_slot >= 0 && J.parent_slot < c.elev_cap)) &&
                    (J.residual_slot < 0 || J.residual_slot < c.res_cap) &&
                    (J.normal_slot < 0 || c.nrm == nullptr || J.normal_slot < c.nrm_cap) &&
                    J.parent_job >= -1 && J.parent_job < job && J.noise_layer >= 0 && J.noise_layer < 6 &&
                    J.noise_rot >= 0 && J.noise_rot < 4;
    if (!ok) report(TP_E_BOUNDS);
    return ok;
}
#endif

// Thread 0: wait (bounded) until the parent job's bands are complete, then issue
// the TMA copies of unit (job, band) into `stage`, completing on `bar`.
__device__ void issue_copies(const tp::ClassLaunch &c, const CUtensorMap *pmap, const CUtensorMap *rmap, int job,
                             int band, float *stage, uint64_t *bar)
{
    const tp_tile_job &J = c.jobs[job];
    if (J.parent_job >= 0) {
        unsigned k = 0;
        while (ld_acquire(c.done + J.parent_job) < c.bands) {
            if (++k > kDepLimit) {
                report(TP_E_TIMEOUT);
                break;
            }
            __nanosleep(64);
        }
        fence_proxy_async_global();  // the parent's generic-proxy writes before our async-proxy reads
    }
    const int n = c.W - 5;
    const int dx = (J.tx & 1) * (n / 2), dy = (J.ty & 1) * (n / 2);
    const int j0 = band * c.band_rows;
    const int ja = max(j0 - 1, 0);
    const bool has_parent = J.level > 0, has_res = J.residual_slot >= 0;
    uint32_t bytes = 0;
    if (has_res) bytes += c.res_box_bytes;
    if (has_parent) bytes += c.par_box_bytes;
    if (bytes == 0) {
        mbar_arrive(bar);
        return;
    }
    mbar_expect_tx(bar, bytes);
    if (has_res) tma_load_3d(stage, rmap, bar, J.rx, J.ry + j0 - 1, J.residual_slot);
    if (has_parent) tma_load_3d(stage + c.buf_floats, pmap, bar, dx, ja / 2 + dy, J.parent_slot * 3 + 0);
}

// All threads: cp.async copies of the coarse-mesh lattice (parent zm) of a job.
__device__ __forceinline__ void issue_lattice(const tp::ClassLaunch &c, int job, float *stage)
{
    const tp_tile_job &J = c.jobs[job];
    if (J.level <= 0) return;
    const int W = c.W, n = W - 5;
    const int dx = (J.tx & 1) * (n / 2), dy = (J.ty & 1) * (n / 2);
    const float *pzm = c.elev + (long long)J.parent_slot * c.slot_stride + 2 * c.plane_stride;
    float *lat = stage + c.buf_floats + c.par_floats;
    for (int t = threadIdx.x; t < c.ck * c.ck; t += kThreads) {
        const int ky = t / c.ck - 1, kx = t - (ky + 1) * c.ck - 1;
        const int X = clampi(2 + dx + c.g * kx, 0, W - 1), Y = clampi(2 + dy + c.g * ky, 0, W - 1);
        cp_async4(lat + t, pzm + (long long)Y * c.pitch + X);
    }
}

// All threads: produce unit (job, band) from `stage` (its copies complete).
// MOD: the class uses the slope/curvature-modulated noise (a separate kernel
// instantiation keeps its 4x4 neighbourhood out of the common path's registers).
// `release` (the job's completion counter, or null when no job of the launch waits
// on another): incremented once the band's elevation rows are written, before the
// normal phase -- a child reads only its parent's zf and zm, so it can start while
// the parent forms its normals.
template <bool MOD>
__device__ __forceinline__ void compute_unit(const tp::ClassLaunch &c, int job, int band, float *stage,
                                             int *release)
{
    const tp_tile_job J = c.jobs[job];
    const int W = c.W, n = W - 5, PE = c.pitch, g = c.g, gs = c.gshift;
    const int dx = (J.tx & 1) * (n / 2), dy = (J.ty & 1) * (n / 2);
    const bool has_parent = J.level > 0, has_res = J.residual_slot >= 0;
    const int j0 = band * c.band_rows, j1 = min(j0 + c.band_rows, W);
    const int ja = max(j0 - 1, 0), jb = min(j1, W - 1);
    const int pr0 = ja / 2 + dy;  // first parent row of the window
    float *sbuf = stage;                        // residual rows, then zm rows
    const float *spar = stage + c.buf_floats;   // parent zf window
    const float *slat = spar + c.par_floats;    // parent zm at the coarse-mesh vertices

    // ---- phase A: elevation of rows [ja, jb].  Thread t sweeps one column quad
    // (4 samples) down a strip of S rows (S even, so every lane of a warp sees the
    // same row parity), keeping the four parent rows its stencil reads in
    // registers: one new parent row (5 samples) per two child rows.
    const int NQ = PE / 4;
    const int nseg = max(1, kThreads / NQ);
    const int nrows = jb - ja + 1;
    const int S = ((nrows + nseg - 1) / nseg + 1) & ~1;
    if (threadIdx.x < NQ * nseg) {
        const int q = threadIdx.x % NQ, seg = threadIdx.x / NQ;
        const int i0 = 4 * q;
        const int rbeg = ja + seg * S, rend = min(rbeg + S, jb + 1);
        const int out_slot = J.out_slot;
        const bool noisy = J.noise_amp != 0.0f;
        const bool modulated = MOD && J.noise_amp > 0.0f;
        const int nzo = (J.noise_rot * 6 + J.noise_layer) * W * PE + i0;  // offset of the quad in the noise table
        // zf + |amp| N (terrain1), or zf - amp N (modulated shader, amp < 0): -(amp N) == (-amp) N exactly
        const float namp = c.noise_mode == 0 ? fabsf(J.noise_amp) : -J.noise_amp;
        const float rscale = J.rscale;
        // coarse-mesh lattice columns of the quad's samples: for g >= 2 four
        // consecutive columns span at most two lattice cells, (A, B) with a selector
        // (g == 1 falls back to per-sample lattice reads)
        // packed in one register: xr0 | xr3 << 8 | xf0 << 16 | xf3 << 24 (lattice sides <= 255)
        uint32_t xcells;
        unsigned selr = 0, self_ = 0;  // bit k: sample k uses cell B
        {
            const int xr0 = fdiv2g(min(i0, W - 1) - 2 + g, g, gs) + 1, xr3 = fdiv2g(min(i0 + 3, W - 1) - 2 + g, g, gs) + 1;
            const int xf0 = fdiv2g(min(i0, W - 1) - 2, g, gs) + 1, xf3 = fdiv2g(min(i0 + 3, W - 1) - 2, g, gs) + 1;
            xcells = (uint32_t)xr0 | ((uint32_t)xr3 << 8) | ((uint32_t)xf0 << 16) | ((uint32_t)xf3 << 24);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int cx = min(i0 + k, W - 1) - 2;
                if (fdiv2g(cx + g, g, gs) + 1 != xr0) selr |= 1u << k;
                if (fdiv2g(cx, g, gs) + 1 != xf0) self_ |= 1u << k;
            }
        }
        const bool two_cells = g >= 2;
        float P[4][5];
        int wr0 = -1000;
        float zcv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        int zkey = -1;
        const float *pcol = spar + 2 * q;
        auto load_row = [&](float(&dst)[5], int r) {
            const float *src = pcol + r * c.par_pitch;
            const float2 a01 = *reinterpret_cast<const float2 *>(src);
            const float2 a23 = *reinterpret_cast<const float2 *>(src + 2);
            dst[0] = a01.x; dst[1] = a01.y; dst[2] = a23.x; dst[3] = a23.y; dst[4] = src[4];
        };
        auto advance = [&](int pc) {
            if (wr0 == pc - 1) return;
            if (wr0 + 1 == pc - 1) {
#pragma unroll
                for (int cc = 0; cc < 5; ++cc) { P[0][cc] = P[1][cc]; P[1][cc] = P[2][cc]; P[2][cc] = P[3][cc]; }
                load_row(P[3], pc + 2);
            } else {
                load_row(P[0], pc - 1);
                load_row(P[1], pc);
                load_row(P[2], pc + 1);
                load_row(P[3], pc + 2);
            }
            wr0 = pc - 1;
        };
        const bool edge = i0 + 3 >= W;  // the quad holding the last sample column and the padding
        // HP_ (the tile has a parent) and NZ_ (noise amplitude non-zero) are uniform per
        // tile: the row code is specialised on them (no per-row tests of either)
        auto row = [&](int j, const uint2 h, auto odd_tag, auto hp_tag, auto nz_tag) {
            constexpr bool ODD = decltype(odd_tag)::value;
            constexpr bool HP_ = decltype(hp_tag)::value;
            constexpr bool NZ_ = decltype(nz_tag)::value;
            float *brow = sbuf + (j - j0 + 1) * PE + i0;
            const float4 r4 = *reinterpret_cast<const float4 *>(brow);
            // (a tile without residual has a zeroed buffer: rscale * 0 == 0)
            float zf[4];
            zf[0] = __fmul_rn(rscale, r4.x);
            zf[1] = __fmul_rn(rscale, r4.y);
            zf[2] = __fmul_rn(rscale, r4.z);
            zf[3] = __fmul_rn(rscale, r4.w);
            if constexpr (NZ_) {
                const float2 n01 = __half22float2(*reinterpret_cast<const __half2 *>(&h.x));
                const float2 n23 = __half22float2(*reinterpret_cast<const __half2 *>(&h.y));
                const float nv[4] = {n01.x, n01.y, n23.x, n23.y};
                if (!MOD || !modulated) {
#pragma unroll
                    for (int k = 0; k < 4; ++k) zf[k] = __fadd_rn(zf[k], __fmul_rn(namp, nv[k]));
                } else if constexpr (MOD) {
                    const float mps = __fdiv_rn(J.tile_meters, (float)n);
#pragma unroll 1
                    for (int k = 0; k < 4; ++k) {
                        const int i = i0 + k;
                        float cz[16];
#pragma unroll
                        for (int t = 0; t < 16; ++t) {
                            const int X = clampi(i / 2 + dx + t % 4, 0, W - 1) - dx;
                            const int Y = clampi(j / 2 + dy + t / 4, 0, W - 1) - pr0;
                            cz[t] = has_parent ? spar[Y * c.par_pitch + X] : 0.0f;
                        }
                        const float m = demo_modulation(cz, (i & 1) + 2 * (j & 1), mps);
                        zf[k] = __fadd_rn(zf[k], __fmul_rn(__fmul_rn(m, J.noise_amp), nv[k]));
                    }
                }
            }
            float zc[4] = {zf[0], zf[1], zf[2], zf[3]};
            if constexpr (HP_) {
                float up[4];
                if constexpr (!ODD) {
                    up[0] = P[1][1];
                    up[1] = __fmul_rn(__fsub_rn(__fmul_rn(__fadd_rn(P[1][1], P[1][2]), 9.0f), __fadd_rn(P[1][0], P[1][3])), 0.0625f);
                    up[2] = P[1][2];
                    up[3] = __fmul_rn(__fsub_rn(__fmul_rn(__fadd_rn(P[1][2], P[1][3]), 9.0f), __fadd_rn(P[1][1], P[1][4])), 0.0625f);
                } else {
                    up[0] = __fmul_rn(__fsub_rn(__fmul_rn(__fadd_rn(P[1][1], P[2][1]), 9.0f), __fadd_rn(P[0][1], P[3][1])), 0.0625f);
                    up[2] = __fmul_rn(__fsub_rn(__fmul_rn(__fadd_rn(P[1][2], P[2][2]), 9.0f), __fadd_rn(P[0][2], P[3][2])), 0.0625f);
                    // odd/odd: the reference sums the 16 products f*g*z one by one, rows outer
                    constexpr float w[4] = {-1.0f / 16.0f, 9.0f / 16.0f, 9.0f / 16.0f, -1.0f / 16.0f};
                    float z1 = 0.0f, z3 = 0.0f;
#pragma unroll
                    for (int dj = 0; dj < 4; ++dj)
#pragma unroll
                        for (int di = 0; di < 4; ++di) {
                            z1 = __fadd_rn(z1, __fmul_rn(w[dj] * w[di], P[dj][di]));
                            z3 = __fadd_rn(z3, __fmul_rn(w[dj] * w[di], P[dj][di + 1]));
                        }
                    up[1] = z1;
                    up[3] = z3;
                }
                // zc from the parent zm lattice: constant between lattice rows, so the
                // four values are cached and recomputed only when the row's cells change
                const int cy = j - 2;
                const int kyr = fdiv2g(cy + g, g, gs) + 1, kyf = fdiv2g(cy, g, gs) + 1;
                const int key = (kyr << 16) | kyf;
                if (key != zkey) {
                    zkey = key;
                    const int yr = kyr * c.ck, yf = kyf * c.ck;
                    float r1[4], r3[4];
                    if (two_cells) {
                        const float a1 = slat[yf + (int)(xcells & 255u)], b1 = slat[yf + (int)((xcells >> 8) & 255u)];
                        const float a3 = slat[yr + (int)((xcells >> 16) & 255u)], b3 = slat[yr + (int)(xcells >> 24)];
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            r1[k] = (selr >> k) & 1u ? b1 : a1;
                            r3[k] = (self_ >> k) & 1u ? b3 : a3;
                        }
                    } else {
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            const int cx = min(i0 + k, W - 1) - 2;
                            r1[k] = slat[yf + fdiv2g(cx + g, g, gs) + 1];
                            r3[k] = slat[yr + fdiv2g(cx, g, gs) + 1];
                        }
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k) zcv[k] = __fmul_rn(__fadd_rn(r1[k], r3[k]), 0.5f);
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    zf[k] = __fadd_rn(zf[k], up[k]);
                    zc[k] = zcv[k];
                }
                if (c.flip && fmod2g(cy, g, gs) == g) {  // cell-centre rows of a flipped mesh
                    const int yr = kyr * c.ck, yf = kyf * c.ck;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int cx = min(i0 + k, W - 1) - 2;
                        if (fmod2g(cx, g, gs) == g) {
                            const int xr = fdiv2g(cx + g, g, gs) + 1, xf = fdiv2g(cx, g, gs) + 1;
                            const float zc1 = slat[yf + xr], zc3 = slat[yr + xf];
                            const float zc0 = slat[yf + xf], zc2 = slat[yr + xr];
                            const float s13 = __fadd_rn(zc3, zc1), s02 = __fadd_rn(zc0, zc2);
                            zc[k] = __fmul_rn(s13 >= s02 ? __fadd_rn(zc1, zc3) : s02, 0.5f);
                        }
                    }
                }
            }
            float vf[4], vc[4], vm[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                vf[k] = zf[k];
                vc[k] = zc[k];
                vm[k] = c.no_clamp ? zf[k] : (zf[k] > 0.0f ? zf[k] : 0.0f);
            }
            if (edge) {
#pragma unroll
                for (int k = 1; k < 4; ++k)
                    if (i0 + k >= W) vf[k] = vc[k] = vm[k] = 0.0f;
            }
            if (j >= j0 && j < j1) {
                float *o = c.elev + (long long)out_slot * c.slot_stride + (j * PE + i0);
                *reinterpret_cast<float4 *>(o) = make_float4(vf[0], vf[1], vf[2], vf[3]);
                *reinterpret_cast<float4 *>(o + c.plane_stride) = make_float4(vc[0], vc[1], vc[2], vc[3]);
                *reinterpret_cast<float4 *>(o + 2 * c.plane_stride) = make_float4(vm[0], vm[1], vm[2], vm[3]);
            }
            *reinterpret_cast<float4 *>(brow) = make_float4(vm[0], vm[1], vm[2], vm[3]);
        };
        using Even = std::integral_constant<bool, false>;
        using Odd = std::integral_constant<bool, true>;
        // noise rows come from L2, each fetched one row ahead
        auto strip = [&](auto hp_tag, auto nz_tag) {
            constexpr bool HP_ = decltype(hp_tag)::value;
            constexpr bool NZ_ = decltype(nz_tag)::value;
            uint2 nzh = make_uint2(0u, 0u);
            if constexpr (NZ_) {
                if (rbeg < rend) nzh = __ldg(reinterpret_cast<const uint2 *>(c.noise + nzo + rbeg * PE));
            }
            auto step = [&](int j, auto odd_tag) {
                const uint2 h = nzh;
                if constexpr (NZ_) {
                    if (j + 1 < rend) nzh = __ldg(reinterpret_cast<const uint2 *>(c.noise + nzo + (j + 1) * PE));
                }
                if constexpr (HP_) advance(j / 2 + 1 + dy - pr0);  // (even, odd) rows share the stencil centre row
                row(j, h, odd_tag, hp_tag, nz_tag);
            };
#pragma unroll 1
            for (int j = rbeg; j < rend; ++j) {
                if (j & 1) step(j, Odd{});
                else step(j, Even{});
            }
        };
        using T_ = std::integral_constant<bool, true>;
        using F_ = std::integral_constant<bool, false>;
        if (has_parent) {
            if (noisy) strip(T_{}, T_{});
            else strip(T_{}, F_{});
        } else {
            if (noisy) strip(F_{}, T_{});
            else strip(F_{}, F_{});
        }
    }
    if (release) fence_proxy_async_global();  // our generic-proxy writes before a child's TMA reads
    __syncthreads();
    if (release && threadIdx.x == 0) {
        __threadfence();
        atomicAdd(release, 1);  // release: this band's elevation rows are complete
    }

    // ---- phase B: normals of rows jn in [max(j0, 2), min(j1, W - 2)): the (row, column
    // quad) items of the band spread over all threads, so that every lane has a quad
    // (one warp per row left 7 of 32 lanes idle on a 25-quad row)
    if (c.nrm != nullptr && J.normal_slot >= 0) {
        const int Wn = W - 4, NQn = c.nrm_pitch / 4;
        float *onx = c.nrm + (long long)J.normal_slot * c.nrm_slot_stride;
        float *ony = onx + c.nrm_plane_stride;
        const float h2 = __fmul_rn(2.0f, __fdiv_rn(J.tile_meters, (float)n));
        const float hh = h2 * h2;
        const int jn0 = max(j0, 2), items = max(min(j1, W - 2) - jn0, 0) * NQn;
        // idx / NQn by a multiply-high with ceil(2^32 / NQn): exact for 2 <= NQn <= 64 and
        // idx < 2^16 (rows <= 253 of at most 64 quads)
        const uint32_t mq = NQn > 1 ? 0xFFFFFFFFu / (uint32_t)NQn + 1u : 0u;
        for (int idx = threadIdx.x; idx < items; idx += kThreads) {
            const int r = NQn > 1 ? (int)__umulhi((uint32_t)idx, mq) : idx, m = idx - r * NQn;
            const int jn = jn0 + r;
            const float *cr = sbuf + (jn - j0 + 1) * PE;
            const float *up = cr + PE, *dn = cr - PE;
            // elevation columns b .. b + 7 of the three rows as two aligned 16-byte loads
            // each; this quad's normals sit at columns b + 2 .. b + 5 and read b + 1 .. b + 6.
            // b2 stays inside the row: a quad past the last normal column (its values
            // unused) reads the row's last 16 bytes instead.
            const int b = 4 * m, b2 = min(b + 4, PE - 4);
            const float4 cA = *reinterpret_cast<const float4 *>(cr + b);
            const float4 cB = *reinterpret_cast<const float4 *>(cr + b2);
            const float4 uA = *reinterpret_cast<const float4 *>(up + b);
            const float4 uB = *reinterpret_cast<const float4 *>(up + b2);
            const float4 dA = *reinterpret_cast<const float4 *>(dn + b);
            const float4 dB = *reinterpret_cast<const float4 *>(dn + b2);
            const float zr[6] = {cA.y, cA.z, cA.w, cB.x, cB.y, cB.z};
            const float zu[4] = {uA.z, uA.w, uB.x, uB.y};
            const float zd[4] = {dA.z, dA.w, dB.x, dB.y};
            float nx[4], ny[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float ax = -__fsub_rn(zr[k + 2], zr[k]);
                const float ay = -__fsub_rn(zu[k], zd[k]);
                const float inv = rsqrtf(ax * ax + ay * ay + hh);
                nx[k] = ax * inv;
                ny[k] = ay * inv;
            }
            if (4 * m + 3 >= Wn) {
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (4 * m + k >= Wn) nx[k] = ny[k] = 0.0f;
            }
            const int o = (jn - 2) * c.nrm_pitch + 4 * m;
            *reinterpret_cast<float4 *>(onx + o) = make_float4(nx[0], nx[1], nx[2], nx[3]);
            *reinterpret_cast<float4 *>(ony + o) = make_float4(ny[0], ny[1], ny[2], ny[3]);
        }
    }
}

template <int MINB, bool MOD>
__global__ void __launch_bounds__(kThreads, MINB)
frame_kernel(const __grid_constant__ CUtensorMap pmap, const __grid_constant__ CUtensorMap rmap,
             const tp::FrameLaunch f)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t bar;
    __shared__ UnitInfo info;
    __shared__ int timed_out;
    const uint32_t raw = smem_u32(smem_raw);
    float *const stage = reinterpret_cast<float *>(smem_raw + (((raw + 127u) & ~127u) - raw));
    const tp::ClassLaunch &c = f.c;
    const int units = c.njobs * c.bands;

    __shared__ int reserved;  // unit index taken ahead, while the current unit is computed
    if (threadIdx.x == 0) {
        timed_out = 0;
        mbar_init(&bar, 1);
        reserved = atomicAdd(f.counter, 1);
    }
    for (uint32_t phase = 0;; phase ^= 1u) {
        // start the reserved unit; its parent has a smaller index, taken earlier by a
        // running CTA, so waiting for it (bounded) cannot deadlock
        if (threadIdx.x == 0) {
            UnitInfo x{0, 0, 0, 0};
            const int u = reserved;
            if (u < units) {
                x.valid = 1;
                x.job = u / c.bands;
                x.band = u - x.job * c.bands;
#ifdef TP_DEBUG
                x.skip = job_in_bounds(c, x.job) ? 0 : 1;
                if (x.skip) mbar_arrive(&bar);  // the unit's phase completes with no copy
                else
#endif
                    issue_copies(c, &pmap, &rmap, x.job, x.band, stage, &bar);
            }
            info = x;
        }
        __syncthreads();
        const UnitInfo x = info;
        if (!x.valid) break;
        if (threadIdx.x == 0) reserved = atomicAdd(f.counter, 1);
        if (!x.skip) issue_lattice(c, x.job, stage);
        cp_async_commit();
        // warp 0 polls the mbarrier; the other warps wait at the CTA barrier below
        if (threadIdx.x < 32) {
            if (!mbar_wait_bounded(&bar, phase)) {
                report(TP_E_TIMEOUT);
                mbar_wait_bounded(&bar, phase);  // the copies get a second chance to land
                timed_out = 1;
            }
        }
        cp_async_wait_all();
        const bool no_res = c.jobs[x.job].residual_slot < 0;
        __syncthreads();
        if (timed_out) break;
        if (no_res) {
            for (int t = threadIdx.x; t < c.buf_floats; t += kThreads) stage[t] = 0.0f;
            __syncthreads();
        }
        if (!x.skip) compute_unit<MOD>(c, x.job, x.band, stage, f.any_deps ? c.done + x.job : nullptr);
        __syncthreads();  // the stage is free again
        if (x.skip && f.any_deps && threadIdx.x == 0) atomicAdd(c.done + x.job, 1);  // a skipped unit is complete
    }
    cp_async_wait_all();
}

// Double-buffered variant: two stages per CTA; the copies of the next unit are
// issued before the current one is computed (unless the next unit's parent is
// still in production, possibly by this CTA: then they are issued after it).
__device__ __forceinline__ bool parent_ready(const tp::ClassLaunch &c, int job)
{
    const int pj = c.jobs[job].parent_job;
    return pj < 0 || ld_acquire(c.done + pj) >= c.bands;
}

template <int MINB, bool MOD>
__global__ void __launch_bounds__(kThreads, MINB)
frame_kernel2(const __grid_constant__ CUtensorMap pmap, const __grid_constant__ CUtensorMap rmap,
              const tp::FrameLaunch f)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t bars[2];
    __shared__ UnitInfo info[2];
    __shared__ int issued[2];
    __shared__ int timed_out;
    const uint32_t raw = smem_u32(smem_raw);
    float *const stage0 = reinterpret_cast<float *>(smem_raw + (((raw + 127u) & ~127u) - raw));
    float *const stage1 = stage0 + f.stage_floats;
    const tp::ClassLaunch &c = f.c;
    const int units = c.njobs * c.bands;
    auto take = [&]() {
        UnitInfo x{0, 0, 0};
        const int u = atomicAdd(f.counter, 1);
        if (u < units) {
            x.valid = 1;
            x.job = u / c.bands;
            x.band = u - x.job * c.bands;
        }
        return x;
    };

    if (threadIdx.x == 0) {
        timed_out = 0;
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        const UnitInfo x = take();
        // the first unit's parent was taken earlier by a running CTA: waiting is safe
        if (x.valid) issue_copies(c, &pmap, &rmap, x.job, x.band, stage0, &bars[0]);
        info[0] = x;
        issued[0] = 1;
    }
    __syncthreads();
    if (info[0].valid) issue_lattice(c, info[0].job, stage0);
    cp_async_commit();

    uint32_t phases = 0u;  // bit s: parity of stage s's next completion
    for (int cur = 0;; cur ^= 1) {
        const int nxt = cur ^ 1;
        float *const scur = cur ? stage1 : stage0;
        float *const snxt = cur ? stage0 : stage1;
        const UnitInfo x = info[cur];
        if (!x.valid) break;
        if (threadIdx.x == 0) {
            const UnitInfo y = take();
            int iss = 0;
            if (y.valid && parent_ready(c, y.job)) {
                issue_copies(c, &pmap, &rmap, y.job, y.band, snxt, &bars[nxt]);
                iss = 1;
            }
            info[nxt] = y;
            issued[nxt] = iss;
        }
        __syncthreads();
        const bool y_valid = info[nxt].valid != 0, y_issued = issued[nxt] != 0;
        if (y_valid && y_issued) issue_lattice(c, info[nxt].job, snxt);
        cp_async_commit();
        if (threadIdx.x < 32) {
            if (!mbar_wait_bounded(&bars[cur], (phases >> cur) & 1u)) {
                report(TP_E_TIMEOUT);
                mbar_wait_bounded(&bars[cur], (phases >> cur) & 1u);
                timed_out = 1;
            }
        }
        phases ^= 1u << cur;
        cp_async_wait_all_but_one();
        const bool no_res = c.jobs[x.job].residual_slot < 0;
        __syncthreads();
        if (timed_out) break;
        if (no_res) {
            for (int t = threadIdx.x; t < c.buf_floats; t += kThreads) scur[t] = 0.0f;
            __syncthreads();
        }
        compute_unit<MOD>(c, x.job, x.band, scur, f.any_deps ? c.done + x.job : nullptr);
        __syncthreads();
        if (threadIdx.x == 0) {
            if (y_valid && !y_issued) {
                issue_copies(c, &pmap, &rmap, info[nxt].job, info[nxt].band, snxt, &bars[nxt]);
                issued[nxt] = 1;
            }
        }
        if (y_valid && !y_issued) {
            __syncthreads();  // thread 0 has seen the parent complete
            issue_lattice(c, info[nxt].job, snxt);
            cp_async_commit();
        }
    }
    cp_async_wait_all();
}

}  // namespace

namespace tp {

static size_t frame_smem(int stage_floats, int stages) { return sizeof(float) * (size_t)stage_floats * stages + 128; }

using KernelFn = void (*)(const CUtensorMap, const CUtensorMap, const FrameLaunch);

// The kernel instance of a (stages, CTAs-per-SM target, modulated-noise) choice.
static KernelFn pick(int stages, int minb, bool mod)
{
#ifdef TP_DEBUG
    stages = 1;  // the index checks are in the single-stage kernel
#endif
    if (stages >= 2) {
        if (minb >= 3) return mod ? frame_kernel2<3, true> : frame_kernel2<3, false>;
        return mod ? frame_kernel2<2, true> : frame_kernel2<2, false>;
    }
    if (minb >= 3) return mod ? frame_kernel<3, true> : frame_kernel<3, false>;
    return mod ? frame_kernel<2, true> : frame_kernel<2, false>;
}

// Raises a kernel's dynamic shared-memory limit (a host-side attribute, set
// before any stream capture that launches the kernel).
static int ensure_smem_attr(KernelFn fn, size_t smem)
{
    static std::mutex mu;
    static std::map<std::pair<int, KernelFn>, size_t> have;  // per device and kernel
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    size_t &h = have[std::make_pair(dev, fn)];
    if (smem <= h) return TP_OK;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail("cudaFuncSetAttribute", e);
    h = smem;
    return TP_OK;
}

int launch_frame(const FrameLaunch &f, const CUtensorMap *pmap, const CUtensorMap *rmap, int grid, void *stream)
{
    if (f.c.njobs <= 0) return TP_OK;
    const KernelFn fn = pick(f.stages, f.minb, f.c.noise_mode == 1);
    const size_t smem = frame_smem(f.stage_floats, f.stages);
    int rc = ensure_smem_attr(fn, smem);
    if (rc) return rc;
    fn<<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(*pmap, *rmap, f);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("frame kernel launch", e);
    return TP_OK;
}

int frame_occupancy(int stage_floats, int stages, int minb, bool mod, int *blocks_per_sm)
{
    const KernelFn fn = pick(stages, minb, mod);
    const size_t smem = frame_smem(stage_floats, stages);
    int rc = ensure_smem_attr(fn, smem);
    if (rc) return rc;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, kThreads, smem);
    if (e != cudaSuccess) return cuda_fail("cudaOccupancyMaxActiveBlocksPerMultiprocessor", e);
    return TP_OK;
}

int status_device_ptr(int **out)
{
    static std::mutex mu;
    static std::map<int, int *> ptrs;  // per device
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail("cudaGetDevice (status)", e);
    std::lock_guard<std::mutex> lk(mu);
    int *&p = ptrs[dev];
    if (!p) {
        void *q = nullptr;
        e = cudaGetSymbolAddress(&q, g_tp_status);
        if (e != cudaSuccess) return cuda_fail("cudaGetSymbolAddress (status)", e);
        p = static_cast<int *>(q);
    }
    *out = p;
    return TP_OK;
}

int read_status(int *status, bool clear)
{
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_tp_status, sizeof(int));
    if (e != cudaSuccess) return cuda_fail("cudaMemcpyFromSymbol (status)", e);
    if (clear && v != 0) {
        int z = 0;
        e = cudaMemcpyToSymbol(g_tp_status, &z, sizeof(int));
        if (e != cudaSuccess) return cuda_fail("cudaMemcpyToSymbol (status)", e);
    }
    *status = v;
    return TP_OK;
}

}  // namespace tp
