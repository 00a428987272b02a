// The child samples of the (-1, 9, 9, -1)/16 interpolating stencil in the order of
// CPUElevationProducer::doCreateTile (CPUElevationProducer.cpp:194-245) and
// HeightMipmap::computeResidual (HeightMipmap.cpp:449-497), each operation rounded
// as written (no contraction), for parent samples P of row pitch `pitch` and the
// child quadrant offsets px = 1 + (tx % 2) n / 2, py = 1 + (ty % 2) n / 2.
#pragma once

namespace tp {

__device__ __forceinline__ float upsample_cpu_order(const float *P, int pitch, int i, int j, int px, int py)
{
    const int ci = i / 2 + px, cj = j / 2 + py;
    if ((j & 1) == 0) {
        if ((i & 1) == 0) return P[cj * pitch + ci];
        const float *r = P + cj * pitch + ci;
        return __fdiv_rn(__fsub_rn(__fmul_rn(__fadd_rn(r[0], r[1]), 9.0f), __fadd_rn(r[-1], r[2])), 16.0f);
    }
    if ((i & 1) == 0) {
        const float *c = P + cj * pitch + ci;
        return __fdiv_rn(__fsub_rn(__fmul_rn(__fadd_rn(c[0], c[pitch]), 9.0f), __fadd_rn(c[-pitch], c[2 * pitch])), 16.0f);
    }
    float z = 0.0f;
#pragma unroll
    for (int dj = -1; dj <= 2; ++dj) {
        const float f = (dj == -1 || dj == 2) ? -0.0625f : 0.5625f;
#pragma unroll
        for (int di = -1; di <= 2; ++di) {
            const float g = (di == -1 || di == 2) ? -0.0625f : 0.5625f;
            z = __fadd_rn(z, __fmul_rn(__fmul_rn(f, g), P[(cj + dj) * pitch + ci + di]));
        }
    }
    return z;
}

}  // namespace tp
