// Elevation layers: the TileLayer draws over a produced elevation tile and the
// blend pass that folds them into zm, as ElevationProducer::doCreateTile runs them
// when the producer has layers (terrain/.../dem/ElevationProducer.cpp:383-399).
//
// The reference draws each layer's meshes with OpenGL into the tile's framebuffer,
// which holds (zf, zc, zm, 0) after the upsample quad (terrain1/upsampleShader.glsl:124).
// The road layer (graph/.../dem/RoadElevationLayer.cpp:388-437) clears the depth
// buffer, writes only the z and w channels under a LESS test and draws triangle
// meshes built on the host by ElevationGraphLayer::drawCurveAltitude
// (ElevationGraphLayer.cpp:82-380): vertices (x, y, altitude, u) in clip coordinates,
// u the signed road-width coordinate.  Its fragment program
// (graph1/roadLayerElevationShader.glsl) writes, at d = |u|,
//   z = altitude + 0.03 (1 - smoothstep(0.98, 1, d)),  w = smoothstep(1, 2, d),
//   depth = 0.1 d + 0.3.
// The water layer (graph/.../dem/WaterElevationLayer.cpp:240-350) draws a sequence
// of passes with their own depth tests (ALWAYS, NOTEQUAL, LESS), depth and colour
// masks: its areas with the constant fill program (river1/fillShader.glsl), then
// area boundaries, other curves and rivers with river1/waterLayerElevationShader.glsl
// (z = st.x or st.x - 1 + max(d - 1, 0), w = smoothstep(1, 2, d), depth 0.1 d + 0.3,
// 0.1 d + 0.15 or 1 for river = 0, 1, 2).
// The blend program then replaces z by zf min(w, 1) + z (1 - min(w, 1))
// (graph1/blendShader.glsl, edit3, river1), or by the 3x3 box filter of that blend
// (demo/shaders/elevation/blendShader.glsl).
//
// Here one CTA produces one tile: the CTA sets up all the tile's triangles (records
// in global scratch), then, per pass (a run of meshes with one state, a new one at
// each depth clear), its warps take triangles in turn and keep per texel, in shared
// memory, one key over the fragments that pass the depth test against the depth
// stored before the pass, and a resolve pass writes z, w and depth of the winning
// fragments as the masks allow; then the blend.  A pass is order-independent:
//  - LESS with depth writes leaves the first fragment of least depth: the least
//    (depth bits, triangle number) key (depth >= 0 orders its bits as the floats);
//  - every other supported state (LESS or ALWAYS without depth writes, ALWAYS with
//    them, NOTEQUAL without them) leaves the last fragment that passes, its test
//    reading only the depth stored before the pass: the largest triangle number.
// NOTEQUAL with depth writes would test against depths written during the pass and
// is refused.  Texel state (key, z, w, depth: 20 bytes) for the whole tile, or row
// bands of wide tiles.
// Rasterisation rules (the reference leaves them to the GL driver): vertex window
// coordinates snapped to 1/256 texel, coverage of the texel
// centre by exact integer edge functions with a top-left rule (y up, row 0 at the
// bottom), attributes interpolated at the texel centre in the plane form
// a0 + (a1 - a0) l1 + (a2 - a0) l2 of the barycentric weights l_k, fp32 depth.
// Every floating-point operation is rounded alone, so the oracle's restatement
// gives the same bits.
#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "tp_internal.h"

namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr int kSubpixel = 256;              // 8 sub-texel bits
constexpr float kMaxSnapped = 8388608.0f;   // |window coordinate| * 256 <= 2^23

// 24 bytes per mesh (copied to the device by every call)
struct DevMesh {
    int first_vertex, first_index, ntri, tri_base;
    int flags;  // bit 0 strip, bit 1 depth clear, bits 2-4 program (TP_LAYER_*), bits 5-9 pass state
    float fill_depth;
};
constexpr int kMeshStrip = 1, kMeshClear = 2;
__host__ __device__ __forceinline__ int mesh_program(const DevMesh &M) { return (M.flags >> 2) & 7; }
__host__ __device__ __forceinline__ int mesh_state(const DevMesh &M) { return (M.flags >> 5) & 31; }
struct DevJob {
    int slot, first_mesh, n_meshes, ntri;
    long long tri_offset;  // the tile's first triangle record in the call's scratch
};

// One triangle after set-up (counter-clockwise, snapped): edge q (from vertex q + 1
// to vertex q + 2, the weight of vertex q) is E_q = A_q px + B_q py + C_q at the
// sub-texel point (px, py), exact in 64 bits.
struct __align__(16) Tri {
    long long C[3];
    int A[3], B[3];
    float a0, da1, da2;      // altitude at vertex 0, and vertex 1, 2 minus vertex 0
    float u0, du1, du2;      // road-width coordinate likewise
    float area;              // twice the area, as float
    int ix0, ix1, jy0, jy1;  // texel bounding box, clipped to the tile
    int bits;                // bits 0-2: edge q is not top-left (ties not covered);
                             // bit 3 valid; bit 4 clear depth before this triangle
    uint32_t inv_cols;       // ceil(2^32 / box width) for box widths >= 2 (t / width = umulhi(t, inv))
    int prog;                // fragment program (TP_LAYER_*)
    float fill_depth;        // the fill program's depth, clamped to [0, 1]
    int pad;
};
constexpr int kValid = 8, kClear = 16;

__device__ __forceinline__ int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

// t / d by a multiply-high: m = ceil(2^32 / d) gives floor(t / d) == umulhi(t, m) for
// 2 <= d <= 4096 and every t below 2^20 (m d = 2^32 + e with 0 < e <= d, and t e < 2^32).
__device__ __forceinline__ uint32_t div_magic(int d) { return 0xFFFFFFFFu / (uint32_t)d + 1u; }
__device__ __forceinline__ int div_by(int t, uint32_t m) { return (int)__umulhi((uint32_t)t, m); }

__device__ __forceinline__ bool snap(float c, int W, int *out)
{
    const float w = __fmul_rn(__fmul_rn(__fadd_rn(c, 1.0f), 0.5f * (float)W), (float)kSubpixel);
    if (!(fabsf(w) <= kMaxSnapped)) return false;
    *out = __float2int_rn(w);
    return true;
}

__device__ __forceinline__ float smoothstep_rn(float e0, float e1, float x)
{
    float t = __fdiv_rn(__fsub_rn(x, e0), __fsub_rn(e1, e0));
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    return __fmul_rn(__fmul_rn(t, t), __fsub_rn(3.0f, __fmul_rn(2.0f, t)));
}

__device__ __forceinline__ long long edge_fn(int xa, int ya, int xb, int yb, int px, int py)
{
    return (long long)(xb - xa) * (long long)(py - ya) - (long long)(yb - ya) * (long long)(px - xa);
}

__device__ void setup(Tri &t, const DevJob &J, const DevMesh *meshes, const float4 *verts, const uint32_t *idx,
                      int nv, int g, int W)
{
    int m = J.first_mesh;
    const int mend = J.first_mesh + J.n_meshes;
    while (m + 1 < mend && meshes[m + 1].tri_base <= g) ++m;
    const DevMesh M = meshes[m];
    const int k = g - M.tri_base;
    int c[3];
    if (M.flags & kMeshStrip) {
        // GL's strip order keeps the winding of odd triangles: (k + 1, k, k + 2)
        c[0] = (k & 1) ? k + 1 : k;
        c[1] = (k & 1) ? k : k + 1;
        c[2] = k + 2;
    } else {
        c[0] = 3 * k;
        c[1] = 3 * k + 1;
        c[2] = 3 * k + 2;
    }
    t.bits = (k == 0 && (M.flags & kMeshClear)) ? kClear : 0;
    t.prog = mesh_program(M);
    t.fill_depth = M.fill_depth;
    float4 v[3];
    bool ok = true;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        // an index past the vertex array (device-built meshes are not checked on the
        // host) drops the triangle
        const uint32_t vi = M.first_index >= 0 ? idx[M.first_index + c[q]] : (uint32_t)c[q];
        ok = ok && (long long)M.first_vertex + vi < (long long)nv;
        v[q] = ok ? verts[M.first_vertex + vi] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    int X[3], Y[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        ok = ok && snap(v[q].x, W, &X[q]);
        ok = ok && snap(v[q].y, W, &Y[q]);
    }
    if (!ok) return;
    long long a2 = edge_fn(X[0], Y[0], X[1], Y[1], X[2], Y[2]);
    if (a2 == 0) return;
    if (a2 < 0) {  // no face culling: clockwise triangles are drawn as their mirror
        int s = X[1]; X[1] = X[2]; X[2] = s;
        s = Y[1]; Y[1] = Y[2]; Y[2] = s;
        const float4 f = v[1]; v[1] = v[2]; v[2] = f;
        a2 = -a2;
    }
    t.area = __ll2float_rn(a2);
    t.a0 = v[0].z;
    t.da1 = __fsub_rn(v[1].z, v[0].z);
    t.da2 = __fsub_rn(v[2].z, v[0].z);
    t.u0 = v[0].w;
    t.du1 = __fsub_rn(v[1].w, v[0].w);
    t.du2 = __fsub_rn(v[2].w, v[0].w);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int a = (q + 1) % 3, b = (q + 2) % 3;
        const int dx = X[b] - X[a], dy = Y[b] - Y[a];
        t.A[q] = -dy;
        t.B[q] = dx;
        t.C[q] = (long long)dy * X[a] - (long long)dx * Y[a];
        if (!(dy < 0 || (dy == 0 && dx < 0))) t.bits |= 1 << q;
    }
    const int xmin = min(X[0], min(X[1], X[2])), xmax = max(X[0], max(X[1], X[2]));
    const int ymin = min(Y[0], min(Y[1], Y[2])), ymax = max(Y[0], max(Y[1], Y[2]));
    const int h = kSubpixel / 2;
    t.ix0 = max(floor_div(xmin - h + kSubpixel - 1, kSubpixel), 0);
    t.ix1 = min(floor_div(xmax - h, kSubpixel), W - 1);
    t.jy0 = max(floor_div(ymin - h + kSubpixel - 1, kSubpixel), 0);
    t.jy1 = min(floor_div(ymax - h, kSubpixel), W - 1);
    if (t.ix0 > t.ix1 || t.jy0 > t.jy1) return;
    const uint32_t cols = (uint32_t)(t.ix1 - t.ix0 + 1);
    t.inv_cols = cols >= 2 ? 0xFFFFFFFFu / cols + 1u : 0u;
    t.bits |= kValid;
}

// smoothstep(0.98, 1, d) of the road fragment program, each operation rounded; the
// division only where the result is not clamped (the same bits as always dividing)
__device__ __forceinline__ float road_edge_step(float d)
{
    if (d <= 0.98f) return 0.0f;
    if (d >= 1.0f) return 1.0f;
    return smoothstep_rn(0.98f, 1.0f, d);
}

// smoothstep(1, 2, d): the division by 2 - 1 = 1 is exact
__device__ __forceinline__ float road_blend_step(float d)
{
    float t = fminf(fmaxf(__fsub_rn(d, 1.0f), 0.0f), 1.0f);
    return __fmul_rn(__fmul_rn(t, t), __fsub_rn(3.0f, __fmul_rn(2.0f, t)));
}

constexpr int kTriWords = (int)(sizeof(Tri) / 4);

// The triangle record whose 32-bit word k lane k holds (lanes 0 .. kTriWords - 1),
// as every lane's copy: the fields the rasteriser reads, by shuffles.
__device__ __forceinline__ Tri tri_from_lanes(uint32_t w)
{
    auto word = [&](int k) { return __shfl_sync(0xffffffffu, w, k); };
    auto wide = [&](int k) { return (long long)(((unsigned long long)word(k + 1) << 32) | word(k)); };
    Tri t;
    const int c0 = (int)(offsetof(Tri, C) / 4), a0 = (int)(offsetof(Tri, A) / 4), b0 = (int)(offsetof(Tri, B) / 4);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        t.C[q] = wide(c0 + 2 * q);
        t.A[q] = (int)word(a0 + q);
        t.B[q] = (int)word(b0 + q);
    }
    t.a0 = __uint_as_float(word(offsetof(Tri, a0) / 4));
    t.da1 = __uint_as_float(word(offsetof(Tri, da1) / 4));
    t.da2 = __uint_as_float(word(offsetof(Tri, da2) / 4));
    t.u0 = __uint_as_float(word(offsetof(Tri, u0) / 4));
    t.du1 = __uint_as_float(word(offsetof(Tri, du1) / 4));
    t.du2 = __uint_as_float(word(offsetof(Tri, du2) / 4));
    t.area = __uint_as_float(word(offsetof(Tri, area) / 4));
    t.ix0 = (int)word(offsetof(Tri, ix0) / 4);
    t.ix1 = (int)word(offsetof(Tri, ix1) / 4);
    t.jy0 = (int)word(offsetof(Tri, jy0) / 4);
    t.jy1 = (int)word(offsetof(Tri, jy1) / 4);
    t.bits = (int)word(offsetof(Tri, bits) / 4);
    t.inv_cols = word(offsetof(Tri, inv_cols) / 4);
    t.prog = (int)word(offsetof(Tri, prog) / 4);
    t.fill_depth = __uint_as_float(word(offsetof(Tri, fill_depth) / 4));
    return t;
}

__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }

// The fragment of triangle T at the centre of texel (i, r), if T covers it: the
// barycentric weights l1, l2 (plane form), the second attribute u and the depth of
// T's fragment program (the road program's when kRoad: every mesh of the launch has it).
template <bool kRoad>
__device__ __forceinline__ bool fragment(const Tri &T, int i, int r, float &l1, float &l2, float &u, float &depth)
{
    const int px = i * kSubpixel + kSubpixel / 2, py = r * kSubpixel + kSubpixel / 2;
    const long long e0 = T.C[0] + (long long)T.A[0] * px + (long long)T.B[0] * py;
    const long long e1 = T.C[1] + (long long)T.A[1] * px + (long long)T.B[1] * py;
    const long long e2 = T.C[2] + (long long)T.A[2] * px + (long long)T.B[2] * py;
    if (e0 < (T.bits & 1) || e1 < ((T.bits >> 1) & 1) || e2 < ((T.bits >> 2) & 1)) return false;
    // plane form a0 + (a1 - a0) l1 + (a2 - a0) l2: constant attributes stay exact
    l1 = __fdiv_rn(__ll2float_rn(e1), T.area);
    l2 = __fdiv_rn(__ll2float_rn(e2), T.area);
    u = __fadd_rn(__fadd_rn(T.u0, __fmul_rn(T.du1, l1)), __fmul_rn(T.du2, l2));
    const float d = fabsf(u);
    switch (kRoad ? TP_LAYER_ROAD : T.prog) {
    case TP_LAYER_WATER_RIVER: depth = clamp01(__fadd_rn(__fmul_rn(d, 0.1f), 0.15f)); break;
    case TP_LAYER_WATER_LARGE: depth = 1.0f; break;
    case TP_LAYER_FILL: depth = T.fill_depth; break;
    default: depth = clamp01(__fadd_rn(__fmul_rn(d, 0.1f), 0.3f)); break;  // road, water river = 0
    }
    return true;
}

// z and w of T's fragment program at weights (l1, l2) and second attribute u.
template <bool kRoad>
__device__ __forceinline__ void shade(const Tri &T, float l1, float l2, float u, float &z, float &w)
{
    const float a = __fadd_rn(__fadd_rn(T.a0, __fmul_rn(T.da1, l1)), __fmul_rn(T.da2, l2));
    const float d = fabsf(u);
    switch (kRoad ? TP_LAYER_ROAD : T.prog) {
    case TP_LAYER_ROAD:
        z = __fadd_rn(a, __fmul_rn(0.03f, __fsub_rn(1.0f, road_edge_step(d))));
        w = road_blend_step(d);
        break;
    case TP_LAYER_WATER:
        z = a;
        w = road_blend_step(d);
        break;
    case TP_LAYER_FILL:
        z = a;
        w = u;
        break;
    default:  // water, river = 1 or 2
        z = __fadd_rn(__fsub_rn(a, 1.0f), fmaxf(__fsub_rn(d, 1.0f), 0.0f));
        w = road_blend_step(d);
        break;
    }
}

// Pass kinds: the least (depth bits, triangle) key for LESS with depth writes, the
// largest triangle number for the other supported states, by depth test.
enum PassKind { kLeast = 0, kLastLess = 1, kLastAlways = 2, kLastNotEqual = 3 };

// The starting key of a texel in a least pass whose stored depth has bits `sb`: a
// fragment's key (depth bits, triangle) is below it exactly when depth < stored
// (depths >= 0 order their bits as the floats; triangle numbers stay below 2^31), so
// the LESS test needs no read of the stored depth.  Stored depth 0: nothing passes.
__device__ __forceinline__ unsigned long long least_start(float stored)
{
    const uint32_t sb = __float_as_uint(stored);
    return sb == 0u ? 0ull : (((unsigned long long)(sb - 1u) << 32) | 0xFFFFFFFFull);
}

// One warp per triangle of the pass, the texels of its box spread over the lanes; a
// triangle's record is read one word per lane, the next one a step ahead, and its
// fields broadcast by shuffles.
template <int kKind, bool kRoad>
__device__ __forceinline__ void raster_pass(const Tri *tt, int seg0, int seg1, int warp, int lane, int h0, int h1,
                                            int W, unsigned long long *key, const float *dep)
{
    const uint32_t *tw = reinterpret_cast<const uint32_t *>(tt);
    int g = seg0 + warp;
    uint32_t cur = (g < seg1 && lane < kTriWords) ? tw[(size_t)g * kTriWords + lane] : 0u;
    for (; g < seg1; g += kWarps) {
        const uint32_t nxt =
            (g + kWarps < seg1 && lane < kTriWords) ? tw[(size_t)(g + kWarps) * kTriWords + lane] : 0u;
        const Tri T = tri_from_lanes(cur);
        cur = nxt;
        if (!(T.bits & kValid)) continue;
        const int lo = max(T.jy0, h0), hi = min(T.jy1, h1 - 1);
        if (lo > hi) continue;
        const int cols = T.ix1 - T.ix0 + 1, count = (hi - lo + 1) * cols;
        const uint32_t tag = (uint32_t)(g - seg0);
        for (int t = lane; t < count; t += 32) {
            const int q = cols >= 2 ? (int)__umulhi((uint32_t)t, T.inv_cols) : t;
            const int r = lo + q, i = T.ix0 + (t - q * cols);
            float l1, l2, u, depth;
            if (!fragment<kRoad>(T, i, r, l1, l2, u, depth)) continue;
            const int p = (r - h0) * W + i;
            if (kKind == kLeast) {
                atomicMin(key + p, ((unsigned long long)__float_as_uint(depth) << 32) | tag);
            } else {
                if (kKind == kLastLess && !(depth < dep[p])) continue;
                if (kKind == kLastNotEqual && !(depth != dep[p])) continue;
                atomicMax(key + p, (unsigned long long)tag + 1ull);
            }
        }
    }
}

// The tile's passes, each over the texels of a band with a row of halo on each
// side: a key per texel (raster_pass) over the fragments that pass the depth test
// against the depth stored before the pass, then a resolve pass that writes z, w and
// depth of each texel's winning fragment as the masks allow.  kDepth false: every
// mesh of the launch has the road layer's state (LESS with depth writes), so passes
// split only at depth clears and each starts from depth 1: no stored depth (16 bytes
// of texel state instead of 20, which leaves more of the SM's L1 to the triangle
// records).  kRoad: every mesh of the launch has the road layer's program.
template <bool kDepth, bool kRoad>
__global__ void __launch_bounds__(kThreads)
layers_kernel(float *elev, int W, int pitch, long long plane_stride, long long slot_stride, const DevJob *jobs,
              const DevMesh *meshes, const float4 *verts, const uint32_t *idx, int nv, int blend_mode, int band_rows,
              Tri *scratch)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int span = (band_rows + 2) * W;
    unsigned long long *key = reinterpret_cast<unsigned long long *>(smem_raw);
    float *zl = reinterpret_cast<float *>(key + span);
    float *wv = zl + span;
    float *dep = kDepth ? wv + span : nullptr;
    float *bl = reinterpret_cast<float *>(key);  // the blend values, once the keys are done
    // the original zm of each band's last row, which the next band reads as its
    // lower halo after this band has written its output (two rows, alternating)
    float *saved = wv + (kDepth ? 2 : 1) * span;
    const DevJob J = jobs[blockIdx.x];
    float *zf_plane = elev + (long long)J.slot * slot_stride;
    float *zm_plane = zf_plane + 2 * plane_stride;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t wmag = div_magic(W);  // texel t of a band: row t / W
    Tri *tt = scratch + J.tri_offset;
    for (int g = threadIdx.x; g < J.ntri; g += kThreads) setup(tt[g], J, meshes, verts, idx, nv, g, W);
    __syncthreads();

    const int mend = J.first_mesh + J.n_meshes;
    for (int b0 = 0, band = 0; b0 < W; b0 += band_rows, ++band) {
        const int b1 = min(b0 + band_rows, W);
        const int h0 = max(b0 - 1, 0), h1 = min(b1 + 1, W);
        const int nt = (h1 - h0) * W;
        float *save_now = saved + (band & 1) * W;
        const float *save_prev = saved + ((band + 1) & 1) * W;
        // the framebuffer before the layers: z = zm, w = 0, depth 1
        for (int t = threadIdx.x; t < nt; t += kThreads) {
            const int tr = div_by(t, wmag), r = h0 + tr, cc = t - tr * W;
            const float z = (b0 > 0 && r == h0) ? save_prev[cc] : zm_plane[(long long)r * pitch + cc];
            if (r == b1 - 1) save_now[cc] = z;
            zl[t] = z;
            wv[t] = 0.0f;
            if (kDepth) dep[t] = 1.0f;
        }
        // passes: runs of meshes with one state, a new one at each mesh that clears
        // the depth buffer
        for (int m = J.first_mesh; m < mend;) {
            const int state = mesh_state(meshes[m]);
            const bool clear = (meshes[m].flags & kMeshClear) != 0;
            int m2 = m + 1;
            while (m2 < mend && !(meshes[m2].flags & kMeshClear) && mesh_state(meshes[m2]) == state) ++m2;
            const int seg0 = meshes[m].tri_base, seg1 = m2 < mend ? meshes[m2].tri_base : J.ntri;
            m = m2;
            if (seg0 == seg1) continue;
            const int test = state & 3;
            const bool write_depth = !(state & TP_NO_DEPTH_WRITE), write_z = !(state & TP_NO_Z_WRITE),
                       write_w = !(state & TP_NO_W_WRITE);
            const int kind = (!kDepth || (test == TP_DEPTH_LESS && write_depth)) ? kLeast
                             : test == TP_DEPTH_LESS                                 ? kLastLess
                             : test == TP_DEPTH_ALWAYS                               ? kLastAlways
                                                                                     : kLastNotEqual;
            for (int t = threadIdx.x; t < nt; t += kThreads) {
                if (kDepth && clear) dep[t] = 1.0f;
                key[t] = kind == kLeast ? least_start(kDepth ? dep[t] : 1.0f) : 0ull;
            }
            __syncthreads();
            if (!kDepth) {
                raster_pass<kLeast, kRoad>(tt, seg0, seg1, warp, lane, h0, h1, W, key, dep);
            } else switch (kind) {
            case kLeast: raster_pass<kLeast, kRoad>(tt, seg0, seg1, warp, lane, h0, h1, W, key, dep); break;
            case kLastLess: raster_pass<kLastLess, kRoad>(tt, seg0, seg1, warp, lane, h0, h1, W, key, dep); break;
            case kLastAlways: raster_pass<kLastAlways, kRoad>(tt, seg0, seg1, warp, lane, h0, h1, W, key, dep); break;
            default: raster_pass<kLastNotEqual, kRoad>(tt, seg0, seg1, warp, lane, h0, h1, W, key, dep); break;
            }
            __syncthreads();
            // resolve: z, w and depth of the winning fragment (the same operations, the
            // same bits)
            for (int t = threadIdx.x; t < nt; t += kThreads) {
                const unsigned long long k = key[t];
                if (k == (kind == kLeast ? least_start(kDepth ? dep[t] : 1.0f) : 0ull)) continue;
                const Tri &T = tt[seg0 + (int)(kind == kLeast ? (uint32_t)k : (uint32_t)(k - 1ull))];
                const int tr = div_by(t, wmag), r = h0 + tr, i = t - tr * W;
                float l1, l2, u, depth, z, w;
                fragment<kRoad>(T, i, r, l1, l2, u, depth);
                shade<kRoad>(T, l1, l2, u, z, w);
                if (write_z) zl[t] = z;
                if (write_w) wv[t] = w;
                if (kDepth && write_depth) dep[t] = depth;
            }
            __syncthreads();
        }
        // blend(v) = zf min(w, 1) + z (1 - min(w, 1))
        for (int t = threadIdx.x; t < nt; t += kThreads) {
            const int tr = div_by(t, wmag), r = h0 + tr, cc = t - tr * W;
            const float b = fminf(wv[t], 1.0f);
            bl[t] = __fadd_rn(__fmul_rn(zf_plane[(long long)r * pitch + cc], b), __fmul_rn(zl[t], __fsub_rn(1.0f, b)));
        }
        __syncthreads();
        for (int t = threadIdx.x; t < (b1 - b0) * W; t += kThreads) {
            const int tr = div_by(t, wmag), r = b0 + tr, cc = t - tr * W;
            float out;
            if (blend_mode == 0) {
                out = bl[(r - h0) * W + cc];
            } else {
                // texture reads clamped to the edge; sums in the shader's order
                auto at = [&](int dr, int dc) {
                    const int rr = min(max(r + dr, 0), W - 1), c2 = min(max(cc + dc, 0), W - 1);
                    return bl[(rr - h0) * W + c2];
                };
                const float sx = at(0, 0);
                const float sy = __fadd_rn(__fadd_rn(__fadd_rn(at(0, 1), at(0, -1)), at(1, 0)), at(-1, 0));
                const float sz = __fadd_rn(__fadd_rn(__fadd_rn(at(1, 1), at(-1, 1)), at(-1, -1)), at(1, -1));
                const float f = 1.0f / 9.0f;
                out = __fadd_rn(__fadd_rn(__fmul_rn(sx, f), __fmul_rn(sy, f)), __fmul_rn(sz, f));
            }
            zm_plane[(long long)r * pitch + cc] = out;
        }
        __syncthreads();
    }
}

// Rows per band: the band's keys, z, w and (with stored depths) depth, `texel_bytes`
// per texel with a row of halo on each side, in about 220 KB of shared memory (the
// 101-wide tile in one band), bands of equal height.
int band_rows_for(int W, int texel_bytes)
{
    const int max_rows = 220000 / (texel_bytes * W) - 2;
    if (max_rows < 1) return 0;
    if (max_rows >= W) return W;
    const int bands = (W + max_rows - 1) / max_rows;
    return (W + bands - 1) / bands;
}

// Validates and numbers the meshes, copies what is in host memory into a device
// buffer shared by all calls, launches, and waits for the launch (the buffer is
// reused by the next call).  Vertices / indices are read in place when `*_dev`.
int run_layers(tp_storage *elev, const tp_layer_job *jobs, int n, const tp_layer_mesh *meshes, int n_meshes,
               const float *vertices, bool vert_dev, int n_vertices, const uint32_t *indices, bool idx_dev,
               int n_indices, int blend_mode, void *stream)
{
    using tp::fail;
    if (!elev || n < 0 || (n > 0 && !jobs) || n_meshes < 0 || (n_meshes > 0 && !meshes) || n_vertices < 0 ||
        (n_vertices > 0 && !vertices) || n_indices < 0 || (n_indices > 0 && !indices) ||
        (blend_mode != 0 && blend_mode != 1))
        return fail(TP_E_BAD_ARG, "tp_elevation_layers: bad arguments");
    std::vector<DevMesh> dm(n_meshes);
    std::vector<uint8_t> mesh_used(n_meshes, 0);
    bool stored_depth = false, road = true;  // a mesh with another state / program than the road layer's
    for (int m = 0; m < n_meshes; ++m) {
        const tp_layer_mesh &M = meshes[m];
        if (M.count < 0 || (M.mode != TP_TRIANGLES && M.mode != TP_TRIANGLE_STRIP) || M.first_vertex < 0 ||
            M.first_vertex > n_vertices)
            return fail(TP_E_BAD_ARG, "tp_elevation_layers: bad mesh");
        if ((M.program | M.state) != 0 || !std::isfinite(M.fill_depth)) {
            const int rc = tp::check_layer_pass(M.program, M.state, M.fill_depth, "tp_elevation_layers");
            if (rc) return rc;
            stored_depth = stored_depth || M.state != 0;
            road = road && M.program == TP_LAYER_ROAD;
        }
        const int ntri = M.mode == TP_TRIANGLES ? M.count / 3 : (M.count >= 3 ? M.count - 2 : 0);
        const int used = M.mode == TP_TRIANGLES ? 3 * ntri : (ntri > 0 ? M.count : 0);
        if (M.first_index >= 0) {
            if ((long long)M.first_index + used > n_indices)
                return fail(TP_E_BAD_ARG, "tp_elevation_layers: mesh indices out of range");
            if (!idx_dev)
                for (int k = 0; k < used; ++k)
                    if ((long long)M.first_vertex + indices[M.first_index + k] >= n_vertices)
                        return fail(TP_E_BAD_ARG, "tp_elevation_layers: vertex index out of range");
        } else if ((long long)M.first_vertex + used > n_vertices) {
            return fail(TP_E_BAD_ARG, "tp_elevation_layers: mesh vertices out of range");
        }
        const int flags = (M.mode == TP_TRIANGLE_STRIP ? kMeshStrip : 0) | (M.clear_depth ? kMeshClear : 0) |
                          (M.program << 2) | (M.state << 5);
        dm[m] = DevMesh{M.first_vertex, M.first_index, ntri, 0, flags,
                        M.fill_depth <= 0.0f ? 0.0f : (M.fill_depth >= 1.0f ? 1.0f : M.fill_depth)};
    }
    if (elev->on_device != 1 || elev->channels < 3)
        return fail(TP_E_BAD_ARG, "tp_elevation_layers: needs a device elevation storage (zf, zc, zm)");
    if (n == 0) return TP_OK;
    const int W = elev->W;
    if (band_rows_for(W, 20) < 1) return fail(TP_E_BAD_ARG, "tp_elevation_layers: tile too wide");
    std::vector<DevJob> dj(n);
    long long total_tri = 0;
    for (int k = 0; k < n; ++k) {
        const tp_layer_job &j = jobs[k];
        if (j.slot < 0 || j.slot >= elev->capacity || j.first_mesh < 0 || j.n_meshes < 0 ||
            (long long)j.first_mesh + j.n_meshes > n_meshes)
            return fail(TP_E_BAD_ARG, "tp_elevation_layers: bad job");
        for (int m = j.first_mesh; m < j.first_mesh + j.n_meshes; ++m) {
            if (mesh_used[m]) return fail(TP_E_BAD_ARG, "tp_elevation_layers: a mesh belongs to two jobs");
            mesh_used[m] = 1;
        }
        // triangle numbers within the tile; a depth clear of a mesh without
        // triangles moves to the next mesh that has some
        int tri = 0, pending_clear = 0;
        for (int m = j.first_mesh; m < j.first_mesh + j.n_meshes; ++m) {
            dm[m].tri_base = tri;
            pending_clear |= dm[m].flags & kMeshClear;
            dm[m].flags = (dm[m].flags & ~kMeshClear) | (dm[m].ntri > 0 ? pending_clear : 0);
            if (dm[m].ntri > 0) pending_clear = 0;
            tri += dm[m].ntri;
        }
        dj[k] = DevJob{j.slot, j.first_mesh, j.n_meshes, tri, total_tri};
        total_tri += tri;
    }

    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t bj = al(sizeof(DevJob) * n), bm = al(sizeof(DevMesh) * (n_meshes ? n_meshes : 1));
    const size_t bv = vert_dev ? 0 : al(sizeof(float) * 4 * (size_t)(n_vertices ? n_vertices : 1));
    const size_t bi = idx_dev ? 0 : al(sizeof(uint32_t) * (size_t)(n_indices ? n_indices : 1));
    const size_t bt = al(sizeof(Tri) * (size_t)(total_tri ? total_tri : 1));  // triangle records
    const size_t need = bj + bm + bv + bi + bt;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    char *dbuf = nullptr;
    {
        int rc = tp::device_scratch(tp::kScratchLayers, need, stream, &dbuf);
        if (rc) return rc;
    }
    const float4 *dv = vert_dev ? reinterpret_cast<const float4 *>(vertices)
                                : reinterpret_cast<const float4 *>(dbuf + bj + bm);
    const uint32_t *di = idx_dev ? indices : reinterpret_cast<const uint32_t *>(dbuf + bj + bm + bv);
    cudaError_t e = cudaMemcpyAsync(dbuf, dj.data(), sizeof(DevJob) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && n_meshes)
        e = cudaMemcpyAsync(dbuf + bj, dm.data(), sizeof(DevMesh) * n_meshes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && n_vertices && !vert_dev)
        e = cudaMemcpyAsync(dbuf + bj + bm, vertices, sizeof(float) * 4 * (size_t)n_vertices, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && n_indices && !idx_dev)
        e = cudaMemcpyAsync(dbuf + bj + bm + bv, indices, sizeof(uint32_t) * (size_t)n_indices, cudaMemcpyHostToDevice,
                            s);
    if (e != cudaSuccess) return tp::cuda_fail("cudaMemcpyAsync (layer meshes)", e);
    const int texel_bytes = stored_depth ? 20 : 16;
    const int rows = band_rows_for(W, texel_bytes);
    const size_t smem = (size_t)texel_bytes * (rows + 2) * W + sizeof(float) * 2 * (size_t)W;
    auto kernel = stored_depth ? (road ? layers_kernel<true, true> : layers_kernel<true, false>)
                               : (road ? layers_kernel<false, true> : layers_kernel<false, false>);
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return tp::cuda_fail("cudaFuncSetAttribute (layers)", e);
    kernel<<<n, kThreads, smem, s>>>(elev->base, W, elev->pitch, elev->plane_stride, elev->slot_stride,
                                     reinterpret_cast<const DevJob *>(dbuf),
                                     reinterpret_cast<const DevMesh *>(dbuf + bj), dv, di, n_vertices, blend_mode,
                                     rows, reinterpret_cast<Tri *>(dbuf + bj + bm + bv + bi));
    e = cudaGetLastError();
    if (e != cudaSuccess) return tp::cuda_fail("layers kernel launch", e);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return tp::cuda_fail("cudaStreamSynchronize (layers)", e);
    return TP_OK;
}

}  // namespace

namespace tp {

int check_layer_pass(int program, int state, float fill_depth, const char *who)
{
    char msg[160];
    if (program < TP_LAYER_ROAD || program > TP_LAYER_FILL) {
        std::snprintf(msg, sizeof msg, "%s: unknown layer program %d", who, program);
        return fail(TP_E_BAD_ARG, msg);
    }
    const int test = state & 3;
    if ((state & ~(3 | TP_NO_DEPTH_WRITE | TP_NO_Z_WRITE | TP_NO_W_WRITE)) != 0 || test > TP_DEPTH_NOTEQUAL) {
        std::snprintf(msg, sizeof msg, "%s: unknown pass state %#x", who, state);
        return fail(TP_E_BAD_ARG, msg);
    }
    if (test == TP_DEPTH_NOTEQUAL && !(state & TP_NO_DEPTH_WRITE)) {
        std::snprintf(msg, sizeof msg, "%s: pass state NOTEQUAL with depth writes is not supported", who);
        return fail(TP_E_BAD_ARG, msg);
    }
    if (!std::isfinite(fill_depth)) {
        std::snprintf(msg, sizeof msg, "%s: fill depth is not finite", who);
        return fail(TP_E_BAD_ARG, msg);
    }
    return TP_OK;
}

}  // namespace tp

extern "C" int tp_elevation_layers(tp_storage *elev, const tp_layer_job *jobs, int n, const tp_layer_mesh *meshes,
                                   int n_meshes, const float *vertices, int n_vertices, const uint32_t *indices,
                                   int n_indices, int blend_mode, void *stream)
{
    return run_layers(elev, jobs, n, meshes, n_meshes, vertices, false, n_vertices, indices, false, n_indices,
                      blend_mode, stream);
}

extern "C" int tp_elevation_layers_device(tp_storage *elev, const tp_layer_job *jobs, int n,
                                          const tp_layer_mesh *meshes, int n_meshes, const float *vertices_dev,
                                          int n_vertices, const uint32_t *indices_dev, int n_indices, int blend_mode,
                                          void *stream)
{
    return run_layers(elev, jobs, n, meshes, n_meshes, vertices_dev, true, n_vertices, indices_dev, true, n_indices,
                      blend_mode, stream);
}
