// Fused elevation + normal tile kernel for sm_103a.
//
// Work unit: one band of rows [j0, j1) of one child tile (a whole 101-wide tile,
// or a quarter of a 197-wide one; the band height is a launch parameter).  Per
// unit, one thread issues two TMA copies into shared memory, completing on one
// mbarrier:
//   * the residual rows [j0 - 1, j1 + 1) of the tile's residual window
//     (cp.async.bulk.tensor.3d over the residual slot pool), and
//   * the parent zf window the stencil of those rows reads (over the elevation
//     slot pool, plane zf of the parent slot);
// while the copies fly, the other threads fetch the parent zm at the coarse-mesh
// vertices zc interpolates (a 14 x 14 lattice for the default grid).
// Phase A then computes zf, zc, zm of rows [j0 - 1, j1] (the band plus one halo
// row each side), writing the band rows to HBM with 16-byte stores and every
// row's zm back over its residual in shared memory.  Phase B forms the normals
// of the band rows from that zm: vertical neighbours from the rows above and
// below, horizontal neighbours across quad boundaries by warp shuffles.
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

#include "tp_internal.h"

__device__ int g_tp_status = 0;  // TP_OK, or the first TP_E_* a kernel reported

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr unsigned kWaitLimit = 1u << 22;  // mbarrier polls before a wait is declared failed

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

// Waits for phase `parity` of the barrier with a bounded number of polls.
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

__device__ __forceinline__ int floordiv(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// floor(a / (2g)) for a grid step g known at compile time (power of two) or not (G == 0)
template <int G>
__device__ __forceinline__ int fdiv2g(int a, int g)
{
    if constexpr (G == 4) return a >> 3;
    else if constexpr (G == 8) return a >> 4;
    else return floordiv(a, 2 * g);
}
template <int G>
__device__ __forceinline__ int fmod2g(int a, int g)
{
    if constexpr (G == 4) return a & 7;
    else if constexpr (G == 8) return a & 15;
    else return a - 2 * g * floordiv(a, 2 * g);
}

// Stencil of one child sample; `c` points at the parent sample (i/2 + px, j/2 + py)
// in the staged window, `ww` is the window row pitch.
__device__ __forceinline__ float upsample_at(const float *c, int ww, int i, int j)
{
    if ((j & 1) == 0) {
        if ((i & 1) == 0) return c[0];
        return __fmul_rn(__fsub_rn(__fmul_rn(__fadd_rn(c[0], c[1]), 9.0f), __fadd_rn(c[-1], c[2])), 0.0625f);
    }
    if ((i & 1) == 0)
        return __fmul_rn(__fsub_rn(__fmul_rn(__fadd_rn(c[0], c[ww]), 9.0f), __fadd_rn(c[-ww], c[2 * ww])), 0.0625f);
    // odd/odd: the reference sums the 16 products f*g*z one by one, rows outer
    constexpr float w[4] = {-1.0f / 16.0f, 9.0f / 16.0f, 9.0f / 16.0f, -1.0f / 16.0f};
    float z = 0.0f;
#pragma unroll
    for (int dj = 0; dj < 4; ++dj)
#pragma unroll
        for (int di = 0; di < 4; ++di)
            z = __fadd_rn(z, __fmul_rn(w[dj] * w[di], c[(di - 1) + (dj - 1) * ww]));
    return z;
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

__device__ __noinline__ float demo_modulation(const float *cz, int mi, float mps)
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

template <int G>
__global__ void __launch_bounds__(kThreads, 3)
elevation_kernel(const __grid_constant__ CUtensorMap parent_map, const __grid_constant__ CUtensorMap res_map,
                 const tp::ElevLaunch a)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t bar;
    // TMA destinations on 128-byte boundaries (the launch adds 128 bytes of slack)
    const uint32_t raw = smem_u32(smem_raw);
    float *sbuf = reinterpret_cast<float *>(smem_raw + (((raw + 127u) & ~127u) - raw));  // residual rows, then zm rows
    float *spar = sbuf + a.buf_floats;                      // parent zf window
    float *scoarse = spar + a.par_floats;                   // parent zm at the coarse-mesh vertices

    const int unit = a.first + blockIdx.x;
    const int jslot = unit / a.bands;
    const int band = unit - jslot * a.bands;
    const int jidx = a.order ? a.order[jslot] : jslot;
    const tp_tile_job &J = a.jobs[jidx];
    const int W = a.W, n = W - 5, PE = a.pitch, g = G ? G : a.g;
    const int level = J.level, tx = J.tx, ty = J.ty;
    const int dx = (tx & 1) * (n / 2), dy = (ty & 1) * (n / 2);
    const bool has_parent = level > 0, has_res = J.residual_slot >= 0;
    const int j0 = (band * W) / a.bands, j1 = ((band + 1) * W) / a.bands;
    const int ja = max(j0 - 1, 0), jb = min(j1, W - 1);
    const int pr0 = ja / 2 + dy;  // first parent row of the window

    // ---- issue the copies
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        uint32_t bytes = 0;
        if (has_res) bytes += a.res_box_bytes;
        if (has_parent) bytes += a.par_box_bytes;
        mbar_expect_tx(&bar, bytes);
        if (has_res) tma_load_3d(sbuf, &res_map, &bar, J.rx, J.ry + j0 - 1, J.residual_slot);
        if (has_parent) tma_load_3d(spar, &parent_map, &bar, dx, pr0, J.parent_slot * 3 + 0);
    }
    // coarse-mesh vertices (parent zm, CLAMP_TO_EDGE) with plain loads meanwhile
    if (has_parent) {
        const float *pzm = a.elev + (long long)J.parent_slot * a.slot_stride + 2 * a.plane_stride;
        for (int t = threadIdx.x; t < a.ck * a.ck; t += kThreads) {
            const int ky = t / a.ck - 1, kx = t - (ky + 1) * a.ck - 1;
            const int X = clampi(2 + dx + g * kx, 0, W - 1), Y = clampi(2 + dy + g * ky, 0, W - 1);
            scoarse[t] = __ldg(pzm + (long long)Y * PE + X);
        }
    }
    __syncthreads();  // barrier initialised, coarse lattice written
    if (has_res || has_parent) {
        if (!mbar_wait_bounded(&bar, 0)) {
            report(TP_E_TIMEOUT);
            mbar_wait_bounded(&bar, 0);  // give the copies a second chance to land before leaving
            return;
        }
    }
    if (!has_res) {
        for (int t = threadIdx.x; t < a.buf_floats; t += kThreads) sbuf[t] = 0.0f;
        __syncthreads();
    }

    // ---- phase A: elevation of rows [ja, jb], quads of 4 samples
    const int NQ = PE / 4;
    float *ozf = a.elev + (long long)J.out_slot * a.slot_stride;
    float *ozc = ozf + a.plane_stride;
    float *ozm = ozf + 2 * a.plane_stride;
    const bool noisy = J.noise_amp != 0.0f;
    const __half *nz_base = a.noise + (long long)(J.noise_rot * 6 + J.noise_layer) * W * PE;
    const float abs_amp = fabsf(J.noise_amp);
    const int nitems = (jb - ja + 1) * NQ;
    for (int it = threadIdx.x; it < nitems; it += kThreads) {
        const int rr = it / NQ, q = it - rr * NQ;
        const int j = ja + rr, i0 = 4 * q;
        float *brow = sbuf + (j - j0 + 1) * PE;
        const float4 r4 = *reinterpret_cast<const float4 *>(brow + i0);
        const float rv[4] = {r4.x, r4.y, r4.z, r4.w};
        float nv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (noisy) {
            const uint2 h = __ldg(reinterpret_cast<const uint2 *>(nz_base + (long long)j * PE + i0));
            const float2 n01 = __half22float2(*reinterpret_cast<const __half2 *>(&h.x));
            const float2 n23 = __half22float2(*reinterpret_cast<const __half2 *>(&h.y));
            nv[0] = n01.x; nv[1] = n01.y; nv[2] = n23.x; nv[3] = n23.y;
        }
        const float *prow = spar + (j / 2 + 1 + dy - pr0) * a.par_pitch;
        const int cy = j - 2;
        const int kyr = fdiv2g<G>(cy + g, g) + 1, kyf = fdiv2g<G>(cy, g) + 1;
        const bool flip_row = a.flip && fmod2g<G>(cy, g) == g;
        float vf[4], vc[4], vm[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = min(i0 + k, W - 1);
            float zf = has_res ? __fmul_rn(J.rscale, rv[k]) : 0.0f;
            if (noisy) {
                if (a.noise_mode == 0) {
                    zf = __fadd_rn(zf, __fmul_rn(abs_amp, nv[k]));
                } else if (J.noise_amp < 0.0f) {
                    zf = __fsub_rn(zf, __fmul_rn(J.noise_amp, nv[k]));
                } else {
                    float cz[16];
#pragma unroll
                    for (int t = 0; t < 16; ++t) {
                        const int X = clampi(i / 2 + dx + t % 4, 0, W - 1) - dx;
                        const int Y = clampi(j / 2 + dy + t / 4, 0, W - 1) - pr0;
                        cz[t] = has_parent ? spar[Y * a.par_pitch + X] : 0.0f;
                    }
                    const float mps = __fdiv_rn(J.tile_meters, (float)n);
                    const float m = demo_modulation(cz, (i & 1) + 2 * (j & 1), mps);
                    zf = __fadd_rn(zf, __fmul_rn(__fmul_rn(m, J.noise_amp), nv[k]));
                }
            }
            float zc = zf;
            if (has_parent) {
                zf = __fadd_rn(zf, upsample_at(prow + (i / 2 + 1), a.par_pitch, i, j));
                const int cx = i - 2;
                const int kxr = fdiv2g<G>(cx + g, g) + 1, kxf = fdiv2g<G>(cx, g) + 1;
                const float zc1 = scoarse[kyf * a.ck + kxr];
                const float zc3 = scoarse[kyr * a.ck + kxf];
                if (flip_row && fmod2g<G>(cx, g) == g) {
                    const float zc0 = scoarse[kyf * a.ck + kxf];
                    const float zc2 = scoarse[kyr * a.ck + kxr];
                    const float s13 = __fadd_rn(zc3, zc1), s02 = __fadd_rn(zc0, zc2);
                    zc = __fmul_rn(s13 >= s02 ? __fadd_rn(zc1, zc3) : s02, 0.5f);
                } else {
                    zc = __fmul_rn(__fadd_rn(zc1, zc3), 0.5f);
                }
            }
            const float zm = a.no_clamp ? zf : (zf > 0.0f ? zf : 0.0f);
            const bool pad = i0 + k >= W;
            vf[k] = pad ? 0.0f : zf;
            vc[k] = pad ? 0.0f : zc;
            vm[k] = pad ? 0.0f : zm;
        }
        if (j >= j0 && j < j1) {
            const long long o = (long long)j * PE + i0;
            *reinterpret_cast<float4 *>(ozf + o) = make_float4(vf[0], vf[1], vf[2], vf[3]);
            *reinterpret_cast<float4 *>(ozc + o) = make_float4(vc[0], vc[1], vc[2], vc[3]);
            *reinterpret_cast<float4 *>(ozm + o) = make_float4(vm[0], vm[1], vm[2], vm[3]);
        }
        *reinterpret_cast<float4 *>(brow + i0) = make_float4(vm[0], vm[1], vm[2], vm[3]);
    }
    if (a.nrm == nullptr || J.normal_slot < 0) return;
    __syncthreads();

    // ---- phase B: normals of rows jn in [max(j0, 2), min(j1, W - 2)), one warp per row
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int Wn = W - 4, NQn = a.nrm_pitch / 4;
    float *onx = a.nrm + (long long)J.normal_slot * a.nrm_slot_stride;
    float *ony = onx + a.nrm_plane_stride;
    const float h2 = __fmul_rn(2.0f, __fdiv_rn(J.tile_meters, (float)n));
    const float hh = h2 * h2;
    for (int jn = max(j0, 2) + warp; jn < min(j1, W - 2); jn += kWarps) {
        const float *c = sbuf + (jn - j0 + 1) * PE;
        const float *up = c + PE, *dn = c - PE;
        for (int base = 0; base < NQn; base += 32) {
            const int m = base + lane;
            const bool act = m < NQn;
            const int e = act ? 4 * m + 2 : 2;  // elevation column of this quad's first normal
            const float2 c01 = *reinterpret_cast<const float2 *>(c + e);
            const float2 c23 = *reinterpret_cast<const float2 *>(c + e + 2);
            const float2 u01 = *reinterpret_cast<const float2 *>(up + e);
            const float2 u23 = *reinterpret_cast<const float2 *>(up + e + 2);
            const float2 d01 = *reinterpret_cast<const float2 *>(dn + e);
            const float2 d23 = *reinterpret_cast<const float2 *>(dn + e + 2);
            // horizontal neighbours e - 1 and e + 4 live in the adjacent lanes' quads
            float left = __shfl_up_sync(0xffffffffu, c23.y, 1);
            float right = __shfl_down_sync(0xffffffffu, c01.x, 1);
            if (lane == 0) left = c[e - 1];
            if (lane == 31 || m == NQn - 1) right = c[min(e + 4, PE - 1)];
            const float zc_[6] = {left, c01.x, c01.y, c23.x, c23.y, right};
            const float zu[4] = {u01.x, u01.y, u23.x, u23.y};
            const float zd[4] = {d01.x, d01.y, d23.x, d23.y};
            float nx[4], ny[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float ax = -__fsub_rn(zc_[k + 2], zc_[k]);
                const float ay = -__fsub_rn(zu[k], zd[k]);
                const float inv = rsqrtf(ax * ax + ay * ay + hh);
                const bool pad = 4 * m + k >= Wn;
                nx[k] = pad ? 0.0f : ax * inv;
                ny[k] = pad ? 0.0f : ay * inv;
            }
            if (act) {
                const long long o = (long long)(jn - 2) * a.nrm_pitch + 4 * m;
                *reinterpret_cast<float4 *>(onx + o) = make_float4(nx[0], nx[1], nx[2], nx[3]);
                *reinterpret_cast<float4 *>(ony + o) = make_float4(ny[0], ny[1], ny[2], ny[3]);
            }
        }
    }
}

template <int G>
int launch_g(const tp::ElevLaunch &a, cudaStream_t s)
{
    const size_t smem = a.smem_bytes + 128;
    cudaError_t e = cudaFuncSetAttribute(elevation_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return tp::cuda_fail("cudaFuncSetAttribute", e);
    elevation_kernel<G><<<a.count, kThreads, smem, s>>>(*a.parent_map, *a.res_map, a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return tp::cuda_fail("elevation kernel launch", e);
    return TP_OK;
}

}  // namespace

namespace tp {

int launch_elevation(const ElevLaunch &a, void *stream)
{
    if (a.count <= 0) return TP_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (a.g == 4) return launch_g<4>(a, s);
    if (a.g == 8) return launch_g<8>(a, s);
    return launch_g<0>(a, s);
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
