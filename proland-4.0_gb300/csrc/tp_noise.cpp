// Host-side noise: the DEM noise table, the Perlin noise whose sign picks a
// tile's noise layer, and the per-tile layer/rotation choice.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "tp_internal.h"

namespace {

using tp::Lcg;

// 2D gradient noise with period 0 (math/noise.cpp:60-165).  Only the sign of its
// value matters to the elevation producer.
class GradientNoise2 {
public:
    GradientNoise2()
    {
        Lcg rng(12345);
        int k;
        for (k = 0; k < 256; ++k) {
            perm_[k] = k;
            rng.next();  // 1D gradient of the reference's shared table build
            float gx = (float)((int)(rng.next() % 512) - 256) / 256;
            float gy = (float)((int)(rng.next() % 512) - 256) / 256;
            float len = std::sqrt(gx * gx + gy * gy);
            grad_[k][0] = gx / len;
            grad_[k][1] = gy / len;
            rng.next();  // 3D gradient, three draws
            rng.next();
            rng.next();
        }
        for (k = 255; k >= 1; --k) {
            int other = (int)(rng.next() % 256);
            std::swap(perm_[k], perm_[other]);
        }
        for (k = 0; k < 258; ++k) {
            perm_[256 + k] = perm_[k];
            grad_[256 + k][0] = grad_[k][0];
            grad_[256 + k][1] = grad_[k][1];
        }
    }

    float operator()(float x, float y) const
    {
        int ix0, ix1, iy0, iy1;
        float fx0, fx1, fy0, fy1;
        lattice(x, &ix0, &ix1, &fx0, &fx1);
        lattice(y, &iy0, &iy1, &fy0, &fy1);
        const int a = perm_[ix0], b = perm_[ix1];
        const float *g00 = grad_[perm_[a + iy0]], *g10 = grad_[perm_[b + iy0]];
        const float *g01 = grad_[perm_[a + iy1]], *g11 = grad_[perm_[b + iy1]];
        const float sx = fade(fx0), sy = fade(fy0);
        float lo0 = fx0 * g00[0] + fy0 * g00[1];
        float lo1 = fx1 * g10[0] + fy0 * g10[1];
        const float bottom = lo0 + sx * (lo1 - lo0);
        float hi0 = fx0 * g01[0] + fy1 * g01[1];
        float hi1 = fx1 * g11[0] + fy1 * g11[1];
        const float top = hi0 + sx * (hi1 - hi0);
        return bottom + sy * (top - bottom);
    }

private:
    static float fade(float t) { return t * t * (3.0f - 2.0f * t); }
    static void lattice(float v, int *i0, int *i1, float *f0, float *f1)
    {
        const float t = v + 0x1000;
        *i0 = ((int)t) & 0xFF;
        *i1 = (*i0 + 1) & 0xFF;
        *f0 = t - (int)std::floor(t);
        *f1 = *f0 - 1.0f;
    }
    int perm_[2 * 256 + 2];
    float grad_[2 * 256 + 2][2];
};

const GradientNoise2 &gradient_noise()
{
    static const GradientNoise2 g;
    return g;
}

std::mutex g_noise_mu;
std::map<std::pair<int, int>, __half *> g_noise_tables;  // (device, W) -> device table

}  // namespace

namespace tp {

// createDemNoise (terrain/.../dem/ElevationProducer.cpp:50-133).  Each of the six
// layers has a 5-sample frame of border bands: each band is drawn from one of two
// fixed seeds chosen by the layer's bit for that edge and written twice,
// mirrored, so that two neighbouring tiles that use layers with equal edge bits
// agree along their shared edge.  The interior comes from one seed that keeps
// running from layer to layer.  Values are uniform in [-1, 1), rounded to half
// precision as the reference's R16F texture stores them.
void build_dem_noise(int W, float *out)
{
    static const int kEdgeBits[6] = {0, 1, 3, 5, 7, 15};
    Lcg interior(1234567);
    for (int layer = 0; layer < 6; ++layer) {
        float *t = out + (size_t)layer * W * W;
        std::memset(t, 0, sizeof(float) * (size_t)W * W);
        auto at = [&](int x, int y) -> float & { return t[x + y * W]; };
        const int bits = kEdgeBits[layer];
        auto edge_rng = [&](int bit) { return Lcg((bits & bit) ? 5647381u : 7654321u); };
        {  // bottom: row 2 (centre line of the band), then rows 3 and 4 mirrored onto 1 and 0
            Lcg r = edge_rng(1);
            for (int x = 5; x <= W / 2; ++x) { float v = r.signed_unit(); at(x, 2) = v; at(W - 1 - x, 2) = v; }
            for (int y = 3; y <= 4; ++y)
                for (int x = 5; x < W - 5; ++x) { float v = r.signed_unit(); at(x, y) = v; at(W - 1 - x, 4 - y) = v; }
        }
        {  // right: column W-3, then columns W-4 and W-5 mirrored onto W-2 and W-1
            Lcg r = edge_rng(2);
            for (int y = 5; y <= W / 2; ++y) { float v = r.signed_unit(); at(W - 3, y) = v; at(W - 3, W - 1 - y) = v; }
            for (int x = W - 4; x >= W - 5; --x)
                for (int y = 5; y < W - 5; ++y) { float v = r.signed_unit(); at(x, y) = v; at(2 * W - 6 - x, W - 1 - y) = v; }
        }
        {  // top: row W-3, then rows W-2 and W-1 mirrored onto W-4 and W-5
            Lcg r = edge_rng(4);
            for (int x = 5; x <= W / 2; ++x) { float v = r.signed_unit(); at(x, W - 3) = v; at(W - 1 - x, W - 3) = v; }
            for (int y = W - 2; y <= W - 1; ++y)
                for (int x = 5; x < W - 5; ++x) { float v = r.signed_unit(); at(x, y) = v; at(W - 1 - x, 2 * W - 6 - y) = v; }
        }
        {  // left: column 2, then columns 1 and 0 mirrored onto 3 and 4
            Lcg r = edge_rng(8);
            for (int y = 5; y <= W / 2; ++y) { float v = r.signed_unit(); at(2, y) = v; at(2, W - 1 - y) = v; }
            for (int x = 1; x >= 0; --x)
                for (int y = 5; y < W - 5; ++y) { float v = r.signed_unit(); at(x, y) = v; at(4 - x, W - 1 - y) = v; }
        }
        for (int y = 5; y < W - 5; ++y)
            for (int x = 5; x < W - 5; ++x) at(x, y) = interior.signed_unit();
        for (int k = 0; k < W * W; ++k) t[k] = __half2float(__float2half_rn(t[k]));
    }
}

const __half *device_noise_table(int W, int *err)
{
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_noise_mu);
    auto key = std::make_pair(dev, W);
    auto it = g_noise_tables.find(key);
    if (it != g_noise_tables.end()) return it->second;
    std::vector<float> base((size_t)6 * W * W);
    build_dem_noise(W, base.data());
    // pre-rotate: entry (rot, layer, j, i) is the texel the shader reads for sample
    // (i, j) under rotation rot, i.e. (uvs[rot], uvs[(rot+1)%4]) with
    // uvs = (u, v, 1-u, 1-v), u = (i+0.5)/W, at NEAREST filtering
    const int P = round_up(W, 8);
    std::vector<__half> rot((size_t)4 * 6 * W * P, __float2half_rn(0.0f));
    for (int r = 0; r < 4; ++r)
        for (int l = 0; l < 6; ++l)
            for (int j = 0; j < W; ++j)
                for (int i = 0; i < W; ++i) {
                    int x, y;
                    switch (r) {
                    case 0: x = i; y = j; break;
                    case 1: x = j; y = W - 1 - i; break;
                    case 2: x = W - 1 - i; y = W - 1 - j; break;
                    default: x = W - 1 - j; y = i; break;
                    }
                    rot[(((size_t)r * 6 + l) * W + j) * P + i] = __float2half_rn(base[(size_t)l * W * W + x + (size_t)y * W]);
                }
    __half *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(__half) * rot.size());
    if (e == cudaSuccess) e = cudaMemcpy(d, rot.data(), sizeof(__half) * rot.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        if (d) cudaFree(d);
        *err = cuda_fail("noise table upload", e);
        return nullptr;
    }
    g_noise_tables[key] = d;
    return d;
}

}  // namespace tp

extern "C" int tp_dem_noise(int tile_width, float *out)
{
    if (tile_width < 11 || !out) return tp::fail(TP_E_BAD_ARG, "tp_dem_noise: bad arguments");
    tp::build_dem_noise(tile_width, out);
    return TP_OK;
}

extern "C" float tp_cnoise(float x, float y) { return gradient_noise()(x, y); }

// Layer and rotation of a tile's noise (ElevationProducer.cpp:345-374): one bit per
// tile edge, set when the gradient noise at the edge midpoint is positive, in a
// parameterisation continuous across the six faces of a cube planet (face 1 is
// the top face, 6 the bottom, 2..5 the sides; face 0 is a flat terrain).
extern "C" int tp_noise_select(int face, int level, int tx, int ty, int *rot, int *layer)
{
    if (!rot || !layer || level < 0 || level > 30) return tp::fail(TP_E_BAD_ARG, "tp_noise_select: bad arguments");
    const GradientNoise2 &N = gradient_noise();
    auto pos = [&](double x, double y) { return N((float)x, (float)y) > 0.0f; };
    int bits = 0;
    if (face == 1) {
        const int o = 1 << level;
        bits |= pos(tx + 0.5, ty + o) ? 1 : 0;
        bits |= (tx == o - 1 ? pos(ty + o + 0.5, o) : pos(tx + 1, ty + o + 0.5)) ? 2 : 0;
        bits |= (ty == o - 1 ? pos((3 * o - 1 - tx) + 0.5, o) : pos(tx + 0.5, ty + o + 1)) ? 4 : 0;
        bits |= (tx == 0 ? pos((4 * o - 1 - ty) + 0.5, o) : pos(tx, ty + o + 0.5)) ? 8 : 0;
    } else if (face == 6) {
        const int o = 1 << level;
        bits |= (ty == 0 ? pos((3 * o - 1 - tx) + 0.5, 0) : pos(tx + 0.5, ty - o)) ? 1 : 0;
        bits |= (tx == o - 1 ? pos((2 * o - 1 - ty) + 0.5, 0) : pos(tx + 1, ty - o + 0.5)) ? 2 : 0;
        bits |= pos(tx + 0.5, ty - o + 1) ? 4 : 0;
        bits |= (tx == 0 ? pos(3 * o + ty + 0.5, 0) : pos(tx, ty - o + 0.5)) ? 8 : 0;
    } else {
        const int o = (1 << level) * (face - 2);
        bits |= pos(tx + o + 0.5, ty) ? 1 : 0;
        bits |= pos((tx + o + 1) % (4 << level), ty + 0.5) ? 2 : 0;
        bits |= pos(tx + o + 0.5, ty + 1) ? 4 : 0;
        bits |= pos(tx + o, ty + 0.5) ? 8 : 0;
    }
    // the 16 edge patterns onto (rotation, layer): layer ids {0,1,3,5,7,15}
    static const int kRot[16] = {0, 0, 1, 0, 2, 0, 1, 0, 3, 3, 1, 3, 2, 2, 1, 0};
    static const int kLayer[16] = {0, 1, 1, 2, 1, 3, 2, 4, 1, 2, 3, 4, 2, 4, 4, 5};
    *rot = kRot[bits];
    *layer = kLayer[bits];
    return TP_OK;
}
