// Device form of the terrain preprocess that builds residual pyramids
// (HeightMipmap::buildMipmapLevel / buildResiduals, HeightMipmap.cpp:199-323):
//
//  * a procedural value-noise fBm height field sampled on the base grid of
//    tile_size * 2^max_level + 1 samples and quantised to int16 (the input map);
//  * level l samples are the base samples at stride 2^(max_level - l)
//    (decimation, HeightMipmap.cpp:231), read with coordinates clamped to the level
//    (AbstractTileCache::getTileHeight, AbstractTileCache.cpp:73-92) and divided by
//    the residual scale (HeightMipmap::getTile, :399-407);
//  * per tile of level l >= 1: upsample the parent's approximate tile with the
//    interpolating stencil, residual = sample - upsample rounded to int16
//    (computeResidual / encodeResidual, :449-513), approximate tile = upsample +
//    rounded residual (computeApproxTile, :515-559), kept for the next level.
//
// One CTA per tile; every tile of a level in one launch.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <vector>

#include "tp_internal.h"
#include "tp_stencil.h"

namespace {

// Integer hash of a lattice point (a 32-bit avalanche mix), and its value in [-1, 1).
__device__ __forceinline__ float lattice(uint32_t x, uint32_t y, uint32_t z)
{
    uint32_t h = x * 0x8da6b343u ^ y * 0xd8163841u ^ z * 0xcb1ab31fu;
    h ^= h >> 16;
    h *= 0x7feb352du;
    h ^= h >> 15;
    h *= 0x846ca68bu;
    h ^= h >> 16;
    return __fsub_rn(__fmul_rn((float)(h >> 8), 1.0f / 8388608.0f), 1.0f);
}

__global__ void fbm_kernel(int size, int octaves, int base_cells, float norm, float quantum, uint32_t seed, int16_t *out)
{
    const size_t n = (size_t)size * size;
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int y = (int)(i / size), x = (int)(i - (size_t)y * size);
    const float u = __fdiv_rn((float)x, (float)(size - 1)), v = __fdiv_rn((float)y, (float)(size - 1));
    float sum = 0.0f, amp = 1.0f;
    for (int o = 0; o < octaves; ++o) {
        const float cells = (float)(base_cells << o);
        const float gx = __fmul_rn(u, cells), gy = __fmul_rn(v, cells);
        const float fx0 = floorf(gx), fy0 = floorf(gy);
        const uint32_t ix = (uint32_t)(int)fx0, iy = (uint32_t)(int)fy0, oz = seed * 977u + (uint32_t)o;
        float fx = __fsub_rn(gx, fx0), fy = __fsub_rn(gy, fy0);
        fx = __fmul_rn(__fmul_rn(fx, fx), __fsub_rn(3.0f, __fmul_rn(2.0f, fx)));
        fy = __fmul_rn(__fmul_rn(fy, fy), __fsub_rn(3.0f, __fmul_rn(2.0f, fy)));
        const float v00 = lattice(ix, iy, oz), v10 = lattice(ix + 1, iy, oz);
        const float v01 = lattice(ix, iy + 1, oz), v11 = lattice(ix + 1, iy + 1, oz);
        const float a0 = __fadd_rn(v00, __fmul_rn(__fsub_rn(v10, v00), fx));
        const float a1 = __fadd_rn(v01, __fmul_rn(__fsub_rn(v11, v01), fx));
        sum = __fadd_rn(sum, __fmul_rn(amp, __fadd_rn(a0, __fmul_rn(__fsub_rn(a1, a0), fy))));
        amp *= 0.5f;
    }
    const float q = rintf(__fdiv_rn(__fmul_rn(sum, norm), quantum));
    out[i] = (int16_t)fminf(fmaxf(q, -32767.0f), 32767.0f);
}

__global__ void level_kernel(const int16_t *base, int base_size, int ts, int max_level, int level, float scale,
                             const float *parent, float *approx, float *up, float *res, int16_t *enc)
{
    const int W = ts + 5, side = 1 << level;
    const int t = blockIdx.x, tx = t % side, ty = t / side;
    const int width = ts << level, shift = max_level - level;
    const size_t o0 = (size_t)t * W * W;
    const float *P = level > 0 ? parent + ((size_t)(ty / 2) * (side / 2) + tx / 2) * W * W : nullptr;
    const int px = 1 + (tx % 2) * ts / 2, py = 1 + (ty % 2) * ts / 2;
    for (int p = threadIdx.x; p < W * W; p += blockDim.x) {
        const int j = p / W, i = p - j * W;
        const int x = min(max(i + ts * tx - 2, 0), width), y = min(max(j + ts * ty - 2, 0), width);
        const float v = __fdiv_rn((float)base[((size_t)y << shift) * base_size + ((size_t)x << shift)], scale);
        const size_t o = o0 + p;
        if (level == 0) {
            approx[o] = v;
            continue;
        }
        const float z = tp::upsample_cpu_order(P, W, i, j, px, py);
        const short q = (short)roundf(__fsub_rn(v, z));
        approx[o] = __fadd_rn(z, (float)q);
        if (up) up[o] = z;
        if (res) res[o] = (float)q;
        if (enc) enc[o] = q;
    }
}

}  // namespace

namespace {

// The same procedural fBm as fbm_kernel, evaluated in double precision at domain
// point (u, v) and returned in metres (no quantisation): deep levels sample it far
// below the finest octave's cells, where single-precision coordinates would add
// noise larger than the residuals.
__device__ double fbm_f64(double u, double v, int octaves, int base_cells, double norm, uint32_t seed)
{
    double sum = 0.0, amp = 1.0;
    for (int o = 0; o < octaves; ++o) {
        const double cells = (double)(base_cells << o);
        const double gx = __dmul_rn(u, cells), gy = __dmul_rn(v, cells);
        const double fx0 = floor(gx), fy0 = floor(gy);
        const uint32_t ix = (uint32_t)(long long)fx0, iy = (uint32_t)(long long)fy0, oz = seed * 977u + (uint32_t)o;
        double fx = __dsub_rn(gx, fx0), fy = __dsub_rn(gy, fy0);
        fx = __dmul_rn(__dmul_rn(fx, fx), __dsub_rn(3.0, __dmul_rn(2.0, fx)));
        fy = __dmul_rn(__dmul_rn(fy, fy), __dsub_rn(3.0, __dmul_rn(2.0, fy)));
        const double v00 = lattice(ix, iy, oz), v10 = lattice(ix + 1, iy, oz);
        const double v01 = lattice(ix, iy + 1, oz), v11 = lattice(ix + 1, iy + 1, oz);
        const double a0 = __dadd_rn(v00, __dmul_rn(__dsub_rn(v10, v00), fx));
        const double a1 = __dadd_rn(v01, __dmul_rn(__dsub_rn(v11, v01), fx));
        sum = __dadd_rn(sum, __dmul_rn(amp, __dadd_rn(a0, __dmul_rn(__dsub_rn(a1, a0), fy))));
        amp *= 0.5;
    }
    return __dmul_rn(sum, norm);
}

struct PairTile {
    int level, tx, ty;
};

// One CTA per pair: the parent tile (level - 1) of the field into shared memory (fp32,
// as a produced parent tile is), then the child tile: up = stencil of the parent
// (CPUElevationProducer order, fp32), res = the field's child sample (double) - up,
// rounded once to fp32: at deep levels the residual is far below the fp32 spacing of
// km-scale heights, so it is formed before any rounding of the child sample.
// Sample (i, j) of tile (level, tx, ty) is the field at
// ((i + ts tx - 2), (j + ts ty - 2)) / (ts 2^level).
__global__ void __launch_bounds__(256) pair_kernel(const PairTile *tiles, int ts, int octaves, int base_cells,
                                                   double norm, uint32_t seed, float *up, float *res, float *fine)
{
    extern __shared__ float parent[];
    const PairTile T = tiles[blockIdx.x];
    const int W = ts + 5;
    const int ptx = T.tx / 2, pty = T.ty / 2;
    const double ps = 1.0 / ((double)ts * (double)(1u << (T.level - 1))), cs = 1.0 / ((double)ts * (double)(1u << T.level));
    for (int p = threadIdx.x; p < W * W; p += blockDim.x) {
        const int j = p / W, i = p - j * W;
        parent[p] = (float)fbm_f64(__dmul_rn((double)(i + ts * ptx - 2), ps), __dmul_rn((double)(j + ts * pty - 2), ps),
                                   octaves, base_cells, norm, seed);
    }
    __syncthreads();
    const int px = 1 + (T.tx % 2) * ts / 2, py = 1 + (T.ty % 2) * ts / 2;
    const size_t o0 = (size_t)blockIdx.x * W * W;
    for (int p = threadIdx.x; p < W * W; p += blockDim.x) {
        const int j = p / W, i = p - j * W;
        const double f = fbm_f64(__dmul_rn((double)(i + ts * T.tx - 2), cs), __dmul_rn((double)(j + ts * T.ty - 2), cs),
                                 octaves, base_cells, norm, seed);
        const float z = tp::upsample_cpu_order(parent, W, i, j, px, py);
        up[o0 + p] = z;
        res[o0 + p] = (float)__dsub_rn(f, (double)z);  // the residual in double, then rounded once
        if (fine) fine[o0 + p] = (float)f;
    }
}

}  // namespace

extern "C" int tp_fbm_pairs(int octaves, int base_cells, float amplitude, uint32_t seed, int tile_size, const int *levels,
                            const int *txs, const int *tys, int n, float *up_dev, float *res_dev, float *fine_dev,
                            void *stream)
{
    if (octaves < 1 || octaves > 20 || base_cells < 1 || ((long long)base_cells << (octaves - 1)) > (1 << 24) ||
        tile_size < 8 || tile_size % 2 != 0 || tile_size > 252 || n < 0 || (n > 0 && (!levels || !txs || !tys)) ||
        (n > 0 && (!up_dev || !res_dev)))
        return tp::fail(TP_E_BAD_ARG, "tp_fbm_pairs: bad arguments");
    if (n == 0) return TP_OK;
    std::vector<PairTile> h((size_t)n);
    for (int k = 0; k < n; ++k) {
        if (levels[k] < 1 || levels[k] > 24 || txs[k] < 0 || tys[k] < 0 || (txs[k] >> levels[k]) != 0 ||
            (tys[k] >> levels[k]) != 0)
            return tp::fail(TP_E_BAD_ARG, "tp_fbm_pairs: bad tile");
        h[k] = PairTile{levels[k], txs[k], tys[k]};
    }
    char *dbuf = nullptr;
    int rc = tp::device_scratch(tp::kScratchPairs, sizeof(PairTile) * (size_t)n, stream, &dbuf);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(dbuf, h.data(), sizeof(PairTile) * (size_t)n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return tp::cuda_fail("tp_fbm_pairs: tile copy", e);
    const int W = tile_size + 5;
    const size_t smem = sizeof(float) * (size_t)W * W;
    e = cudaFuncSetAttribute(pair_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return tp::cuda_fail("tp_fbm_pairs: shared memory", e);
    const double norm = (double)amplitude / (2.0 - std::ldexp(1.0, 1 - octaves));
    pair_kernel<<<n, 256, smem, s>>>(reinterpret_cast<const PairTile *>(dbuf), tile_size, octaves, base_cells, norm, seed,
                                     up_dev, res_dev, fine_dev);
    e = cudaGetLastError();
    return e == cudaSuccess ? TP_OK : tp::cuda_fail("tp_fbm_pairs", e);
}

extern "C" int tp_fbm_heights(int size, int octaves, int base_cells, float amplitude, float quantum, uint32_t seed,
                              int16_t *out_dev, void *stream)
{
    if (size < 2 || octaves < 1 || octaves > 20 || base_cells < 1 || ((long long)base_cells << (octaves - 1)) > (1 << 24) ||
        !(quantum > 0.0f) || !out_dev)
        return tp::fail(TP_E_BAD_ARG, "tp_fbm_heights: bad arguments");
    // octave amplitudes 1, 1/2, 1/4, ... normalised so that their sum is `amplitude`
    const float norm = (float)((double)amplitude / (2.0 - std::ldexp(1.0, 1 - octaves)));
    const size_t n = (size_t)size * size;
    fbm_kernel<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(size, octaves, base_cells, norm,
                                                                                          quantum, seed, out_dev);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TP_OK : tp::cuda_fail("tp_fbm_heights", e);
}

extern "C" int tp_preprocess_level(const int16_t *base_dev, int tile_size, int max_level, int level, float scale,
                                   const float *parent_approx_dev, float *approx_dev, float *upsampled_dev,
                                   float *residual_dev, int16_t *encoded_dev, void *stream)
{
    if (!base_dev || tile_size < 8 || tile_size % 2 != 0 || max_level < 0 || max_level > 14 || level < 0 ||
        level > max_level || !(scale > 0.0f) || !approx_dev || (level > 0 && !parent_approx_dev))
        return tp::fail(TP_E_BAD_ARG, "tp_preprocess_level: bad arguments");
    const int base_size = (tile_size << max_level) + 1;
    level_kernel<<<1u << (2 * level), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        base_dev, base_size, tile_size, max_level, level, scale, parent_approx_dev, approx_dev, upsampled_dev,
        residual_dev, encoded_dev);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TP_OK : tp::cuda_fail("tp_preprocess_level", e);
}
