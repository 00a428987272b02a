// Fused elevation + normal tile kernel for sm_103a.
//
// One CTA produces one tile.  The parent's zf and zm planes over the window the
// child reads are staged in shared memory; each warp then sweeps a band of rows
// of the child tile, every lane owning SPL consecutive columns (SPL = 4 for
// 101-wide tiles, 8 for 197-wide: one lane row covers the padded pitch).  Per
// row a lane computes zf / zc / zm, writes them with 16-byte stores, and keeps
// the last three zm rows in registers; the normal of the row before the current
// one is then formed from those registers, the horizontal neighbours crossing
// lane boundaries by warp shuffles.
//
// Arithmetic follows the reference exactly:
//  * stencil: CPUElevationProducer.cpp:202-238 (the same loops as
//    ResidualProducer.cpp:342-384 and HeightMipmap.cpp:449-497), in that
//    operation order, each operation rounded on its own (__f*_rn) so the result
//    is bit-identical to a CPU build without floating-point contraction;
//  * residual, noise, zc, zm: upsampleShader.glsl main()
//    (terrain/examples/terrain1/upsampleShader.glsl:81-125; flip variant
//    terrain/examples/terrain4/upsampleShader.glsl:112-127; modulated noise
//    demo/shaders/elevation/upsampleShader.glsl:140-203);
//  * normals: terrain/examples/terrain1/normalShader.glsl:57-74 with point
//    sampling of the zm channel.
#include <cuda_runtime.h>

#include "tp_internal.h"

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int floordiv(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Stencil of one child sample.  `c` points at the parent sample (i/2 + px, j/2 + py)
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

__device__ float demo_modulation(const float *cz, int mi, float mps)
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

// Noise texel of sample (i, j) under rotation `rot` (the shader reads
// (uvs[rot], uvs[(rot+1)%4]) with uvs = (u, v, 1-u, 1-v), u = (i+0.5)/W).
__device__ __forceinline__ int noise_index(int W, int rot, int i, int j)
{
    switch (rot & 3) {
    case 0: return i + j * W;
    case 1: return j + (W - 1 - i) * W;
    case 2: return (W - 1 - i) + (W - 1 - j) * W;
    default: return (W - 1 - j) + i * W;
    }
}

template <int SPL>
__device__ __forceinline__ void store_row(float *dst, const float (&v)[SPL])
{
#pragma unroll
    for (int q = 0; q < SPL / 4; ++q)
        reinterpret_cast<float4 *>(dst)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}

template <int SPL>
__global__ void __launch_bounds__(kThreads)
elevation_kernel(const tp::ElevLaunch a)
{
    extern __shared__ float4 smem4[];
    float *szf = reinterpret_cast<float *>(smem4);
    float *szm = szf + a.ww * a.wh;

    const int jidx = a.order ? a.order[a.first + blockIdx.x] : a.first + blockIdx.x;
    const tp_tile_job J = a.jobs[jidx];
    const int W = a.W, n = W - 5;
    const int dx = (J.tx & 1) * (n / 2), dy = (J.ty & 1) * (n / 2);
    const bool has_parent = J.level > 0;

    // ---- stage the parent window: parent samples [d + wlo, d + wlo + ww) on both axes,
    // clamped to the tile (CLAMP_TO_EDGE for the coarse-mesh lookups of zc)
    if (has_parent) {
        const float *pzf = a.elev + (long long)J.parent_slot * a.slot_stride;
        const float *pzm = pzf + 2 * a.plane_stride;
        const int wx0 = dx + a.wlo, wy0 = dy + a.wlo;
        const int total = a.ww * a.wh;
        for (int e = threadIdx.x; e < total; e += kThreads) {
            int r = e / a.ww, c = e - r * a.ww;
            int gx = clampi(wx0 + c, 0, W - 1), gy = clampi(wy0 + r, 0, W - 1);
            long long o = (long long)gy * a.pitch + gx;
            szf[e] = __ldg(pzf + o);
            szm[e] = __ldg(pzm + o);
        }
    }
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int kWarps = kThreads / 32;
    const int r0 = (warp * W) / kWarps, r1 = ((warp + 1) * W) / kWarps;
    const int i0 = lane * SPL;
    const bool store_lane = i0 < a.pitch;
    // lanes past the last sample column compute on the last in-tile quad so that
    // every load of theirs stays inside the tile (their results are not stored)
    const int i0c = min(i0, ((W - 1) / SPL) * SPL);

    float *ozf = a.elev + (long long)J.out_slot * a.slot_stride;
    float *ozc = ozf + a.plane_stride;
    float *ozm = ozf + 2 * a.plane_stride;
    const float *R = J.residual_slot >= 0 ? a.res + (long long)J.residual_slot * a.res_slot_stride : nullptr;
    const float *NZ = J.noise_amp != 0.0f ? a.noise + (long long)J.noise_layer * W * W : nullptr;
    const bool want_normals = a.nrm != nullptr && J.normal_slot >= 0;
    float *onx = want_normals ? a.nrm + (long long)J.normal_slot * a.nrm_slot_stride : nullptr;
    float *ony = want_normals ? onx + a.nrm_plane_stride : nullptr;
    const int Wn = W - 4;
    const float h2 = __fmul_rn(2.0f, __fdiv_rn(J.tile_meters, (float)n));
    const float abs_amp = fabsf(J.noise_amp);
    const int g = a.g;

    float zmA[SPL], zmB[SPL], zmC[SPL];
#pragma unroll
    for (int k = 0; k < SPL; ++k) zmA[k] = zmB[k] = zmC[k] = 0.0f;

    const int ja = max(r0 - 1, 0), jb = min(r1, W - 1);
    for (int j = ja; j <= jb; ++j) {
        float vf[SPL], vc[SPL], vm[SPL];
        // residual: one or two aligned 16-byte loads per lane
        float res[SPL];
        if (R) {
            const float4 *rp = reinterpret_cast<const float4 *>(R + (long long)(j + J.ry) * a.res_pitch + i0c + J.rx);
#pragma unroll
            for (int q = 0; q < SPL / 4; ++q) {
                float4 t = __ldg(rp + q);
                res[4 * q] = t.x; res[4 * q + 1] = t.y; res[4 * q + 2] = t.z; res[4 * q + 3] = t.w;
            }
        }
        const float *crow = szf + (j / 2 + 1 - a.wlo) * a.ww;
#pragma unroll
        for (int k = 0; k < SPL; ++k) {
            const int i = min(i0 + k, W - 1);
            float zf = R ? __fmul_rn(J.rscale, res[k]) : 0.0f;
            if (NZ) {
                float N = __ldg(NZ + noise_index(W, J.noise_rot, i, j));
                if (a.noise_mode == 0) {
                    zf = __fadd_rn(zf, __fmul_rn(abs_amp, N));
                } else if (J.noise_amp < 0.0f) {
                    zf = __fsub_rn(zf, __fmul_rn(J.noise_amp, N));
                } else {
                    float cz[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q)
                        cz[q] = has_parent ? szf[(j / 2 - a.wlo + q / 4) * a.ww + (i / 2 - a.wlo + q % 4)] : 0.0f;
                    float mps = __fdiv_rn(J.tile_meters, (float)n);
                    float m = demo_modulation(cz, (i & 1) + 2 * (j & 1), mps);
                    zf = __fadd_rn(zf, __fmul_rn(__fmul_rn(m, J.noise_amp), N));
                }
            }
            float zc = zf;
            if (has_parent) {
                zf = __fadd_rn(zf, upsample_at(crow + (i / 2 + 1 - a.wlo), a.ww, i, j));
                // coarse-mesh elevation (zc) from the parent zm plane
                const int cx = i - 2, cy = j - 2;
                const int kxr = floordiv(cx + g, 2 * g), kxf = floordiv(cx, 2 * g);
                const int kyr = floordiv(cy + g, 2 * g), kyf = floordiv(cy, 2 * g);
                const int Xr = clampi(2 + dx + g * kxr, 0, W - 1) - dx - a.wlo;
                const int Xf = clampi(2 + dx + g * kxf, 0, W - 1) - dx - a.wlo;
                const int Yr = clampi(2 + dy + g * kyr, 0, W - 1) - dy - a.wlo;
                const int Yf = clampi(2 + dy + g * kyf, 0, W - 1) - dy - a.wlo;
                const float zc1 = szm[Yf * a.ww + Xr];
                const float zc3 = szm[Yr * a.ww + Xf];
                bool flipped = false;
                if (a.flip) {
                    const int mx = ((cx % (2 * g)) + 2 * g) % (2 * g), my = ((cy % (2 * g)) + 2 * g) % (2 * g);
                    if (mx == g && my == g) {
                        const float zc0 = szm[Yf * a.ww + Xf];
                        const float zc2 = szm[Yr * a.ww + Xr];
                        const float s13 = __fadd_rn(zc3, zc1), s02 = __fadd_rn(zc0, zc2);
                        zc = __fmul_rn(s13 >= s02 ? __fadd_rn(zc1, zc3) : s02, 0.5f);
                        flipped = true;
                    }
                }
                if (!flipped) zc = __fmul_rn(__fadd_rn(zc1, zc3), 0.5f);
            }
            const float zm = a.no_clamp ? zf : (zf > 0.0f ? zf : 0.0f);
            const bool pad = i0 + k >= W;
            vf[k] = pad ? 0.0f : zf;
            vc[k] = pad ? 0.0f : zc;
            vm[k] = pad ? 0.0f : zm;
        }
        if (j >= r0 && j < r1 && store_lane) {
            const long long o = (long long)j * a.pitch + i0;
            store_row<SPL>(ozf + o, vf);
            store_row<SPL>(ozc + o, vc);
            store_row<SPL>(ozm + o, vm);
        }
#pragma unroll
        for (int k = 0; k < SPL; ++k) {
            zmA[k] = zmB[k];
            zmB[k] = zmC[k];
            zmC[k] = vm[k];
        }
        // ---- normals of row jn = j - 1 from zm rows j-2, j-1, j
        const int jn = j - 1;
        if (want_normals && jn >= max(r0, 2) && jn < min(r1, W - 2)) {
            const float left = __shfl_up_sync(0xffffffffu, zmB[SPL - 1], 1);
            const float right = __shfl_down_sync(0xffffffffu, zmB[0], 1);
            float nx[SPL], ny[SPL];
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                const float zl = k == 0 ? left : zmB[k - 1];
                const float zr = k == SPL - 1 ? right : zmB[k + 1];
                const float ax = -__fsub_rn(zr, zl);
                const float ay = -__fsub_rn(zmC[k], zmA[k]);
                const float inv = rsqrtf(ax * ax + ay * ay + h2 * h2);
                nx[k] = ax * inv;
                ny[k] = ay * inv;
            }
            // normal column p sits at elevation column p + 2: lane m stores normal
            // columns [SPL m, SPL m + SPL) = its own k = 2.. and lane m+1's k = 0, 1
            const float nx0 = __shfl_down_sync(0xffffffffu, nx[0], 1);
            const float nx1 = __shfl_down_sync(0xffffffffu, nx[1], 1);
            const float ny0 = __shfl_down_sync(0xffffffffu, ny[0], 1);
            const float ny1 = __shfl_down_sync(0xffffffffu, ny[1], 1);
            float sx[SPL], sy[SPL];
#pragma unroll
            for (int k = 0; k < SPL; ++k) {
                float vx = k < SPL - 2 ? nx[k + 2] : (k == SPL - 2 ? nx0 : nx1);
                float vy = k < SPL - 2 ? ny[k + 2] : (k == SPL - 2 ? ny0 : ny1);
                const bool pad = i0 + k >= Wn;
                sx[k] = pad ? 0.0f : vx;
                sy[k] = pad ? 0.0f : vy;
            }
            if (i0 < a.nrm_pitch) {
                const long long o = (long long)(jn - 2) * a.nrm_pitch + i0;
                store_row<SPL>(onx + o, sx);
                store_row<SPL>(ony + o, sy);
            }
        }
    }
}

}  // namespace

namespace tp {

int launch_elevation(const ElevLaunch &a, void *stream)
{
    if (a.count <= 0) return TP_OK;
    const size_t smem = sizeof(float) * 2 * (size_t)a.ww * a.wh;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    if (a.pitch <= 32 * 4) {
        e = cudaFuncSetAttribute(elevation_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_fail("cudaFuncSetAttribute", e);
        elevation_kernel<4><<<a.count, kThreads, smem, s>>>(a);
    } else if (a.pitch <= 32 * 8) {
        e = cudaFuncSetAttribute(elevation_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_fail("cudaFuncSetAttribute", e);
        elevation_kernel<8><<<a.count, kThreads, smem, s>>>(a);
    } else {
        return fail(TP_E_BAD_ARG, "tile width above 256 is not supported by the batch kernel");
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail("elevation kernel launch", e);
    return TP_OK;
}

}  // namespace tp
