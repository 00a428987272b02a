// Quotients that share a divisor: one correctly rounded reciprocal, then one
// exact-remainder correction per quotient (used by the sphere normals and the ortho
// HSV conversion; tp_sphere_division_self_test checks it against __fdiv_rn).
#pragma once
#include <cuda_runtime.h>

namespace tp {

// x / y correctly rounded, given z = RN(1 / y) (__frcp_rn): q = RN(x z) is within one
// ulp of x / y, the remainder x - q y is exact (one FMA), and RN(q + r z) is the
// correctly rounded quotient (Markstein's theorem, round to nearest).  x or y outside
// [2^-60, 2^60] in magnitude take the division itself: inside, the quotient and the
// remainder stay normal numbers, as the theorem assumes.  tp_sphere_division_self_test
// compares it with __fdiv_rn.
__device__ __forceinline__ float div_rcp(float x, float y, float z)
{
    const float ax = fabsf(x), ay = fabsf(y);
    if (ax <= 0x1p60f && ax >= 0x1p-60f && ay <= 0x1p60f && ay >= 0x1p-60f) {
        const float q = __fmul_rn(x, z);
        const float r = __fmaf_rn(-q, y, x);
        return __fmaf_rn(r, z, q);
    }
    if (ax == 0.0f && ay != 0.0f) return __fmul_rn(x, z);  // +-0 / y: the sign of x / y
    return __fdiv_rn(x, y);
}

}  // namespace tp
