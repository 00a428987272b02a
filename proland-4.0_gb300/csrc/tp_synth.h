// Synthetic residual tiles: iid samples of zero mean and variance sigma^2 per
// tile, the stand-in for a residual pyramid that the benchmark configurations use
// (residuals N(0, (sigma0 * ratio^level)^2)).  Counter-based, so any tile can be
// made on the host or the device, in any order, with the same bits:
//
//   key(seed, level, tx, ty) = h(seed ^ h(level ^ h(tx ^ h(ty))))
//   sample (i, j) of a W-wide tile, s = i + j * W:
//     u_m = ((h(key + 6 s + m) >> 16) + 0.5) / 65536  and the same of its low half, m = 0..5
//     r = (sum of the 12 u - 6) * sigma
//
// h is a 32-bit integer finaliser (xor-shift / multiply, constants 0x7feb352d and
// 0x846ca68b).  The sum of twelve uniforms (Irwin-Hall) has mean 6 and variance 1:
// approximately normal, bounded by 6 sigma.  Each u is a multiple of 2^-17 below 1,
// so every partial sum is exact in fp32 and only the final product rounds.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define TP_HD __host__ __device__ __forceinline__
#else
#define TP_HD inline
#endif

namespace tp {

TP_HD uint32_t synth_hash(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

TP_HD uint32_t synth_key(uint32_t seed, int level, int tx, int ty)
{
    return synth_hash(seed ^ synth_hash((uint32_t)level ^ synth_hash((uint32_t)tx ^ synth_hash((uint32_t)ty))));
}

// unit-variance sample s of the tile with key `key` (exact: a multiple of 2^-17)
TP_HD float synth_unit(uint32_t key, uint32_t s)
{
    float acc = 0.0f;
    for (uint32_t m = 0; m < 6; ++m) {
        const uint32_t h = synth_hash(key + 6u * s + m);
        acc += ((float)(h >> 16) + 0.5f) * (1.0f / 65536.0f);
        acc += ((float)(h & 0xffffu) + 0.5f) * (1.0f / 65536.0f);
    }
    return acc - 6.0f;
}

}  // namespace tp
