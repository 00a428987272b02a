// Elevation layers: the TileLayer draws over a produced elevation tile and the
// blend pass that folds them into zm, as ElevationProducer::doCreateTile runs them
// when the producer has layers (terrain/.../dem/ElevationProducer.cpp:383-399).
//
// The reference draws each layer's meshes with OpenGL into the tile's framebuffer,
// which holds (zf, zc, zm, 0) after the upsample quad (terrain1/upsampleShader.glsl:124),
// under a LESS depth test.  The road layer (graph/.../dem/RoadElevationLayer.cpp:388-437)
// clears the depth buffer, writes only the z and w channels and draws triangle meshes
// built on the host by ElevationGraphLayer::drawCurveAltitude
// (ElevationGraphLayer.cpp:82-380): vertices (x, y, altitude, u) in clip coordinates,
// u the signed road-width coordinate.  Its fragment program
// (graph1/roadLayerElevationShader.glsl) writes, at d = |u|,
//   z = altitude + 0.03 (1 - smoothstep(0.98, 1, d)),  w = smoothstep(1, 2, d),
//   depth = 0.1 d + 0.3.
// The blend program then replaces z by zf min(w, 1) + z (1 - min(w, 1))
// (graph1/blendShader.glsl, edit3, river1), or by the 3x3 box filter of that blend
// (demo/shaders/elevation/blendShader.glsl).
//
// Here one CTA produces one tile: the tile's z, w and depth live in shared memory
// (row bands of at most ~140 KB for wide tiles), triangles are set up 256 at a time
// (one per thread) and rasterised in order, each pixel owned by one thread (rows by
// warp, columns by lane), so the per-pixel order of primitives is the draw order,
// as GL guarantees.  Rasterisation rules (the reference leaves them to the GL
// driver): vertex window coordinates snapped to 1/256 texel, coverage of the texel
// centre by exact integer edge functions with a top-left rule (y up, row 0 at the
// bottom), attributes interpolated at the texel centre in the plane form
// a0 + (a1 - a0) l1 + (a2 - a0) l2 of the barycentric weights l_k, fp32 depth.
// Every floating-point operation is rounded alone, so the oracle's restatement
// gives the same bits.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <vector>

#include "tp_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kSubpixel = 256;              // 8 sub-texel bits
constexpr float kMaxSnapped = 8388608.0f;   // |window coordinate| * 256 <= 2^23

struct DevMesh {
    int first_vertex, first_index, mode, ntri, tri_base, clear;
    int pad[2];
};
struct DevJob {
    int slot, first_mesh, n_meshes, ntri;
};

// One triangle after set-up (counter-clockwise, snapped).
struct Tri {
    int X[3], Y[3];
    float alt[3], u[3];
    int ix0, ix1, jy0, jy1;  // texel bounding box, clipped to the tile
    int bias[3];             // 0 for a top-left edge (ties covered), 1 otherwise
    float area;              // twice the signed area, as float
    int flags;               // bit 0 valid, bit 1 clear depth before this triangle
    int pad;
};

__device__ __forceinline__ int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

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
                      int g, int W)
{
    t.flags = 0;
    int m = J.first_mesh;
    const int mend = J.first_mesh + J.n_meshes;
    while (m + 1 < mend && meshes[m + 1].tri_base <= g) ++m;
    const DevMesh M = meshes[m];
    const int k = g - M.tri_base;
    int c[3];
    if (M.mode == TP_TRIANGLE_STRIP) {
        // GL's strip order keeps the winding of odd triangles: (k + 1, k, k + 2)
        c[0] = (k & 1) ? k + 1 : k;
        c[1] = (k & 1) ? k : k + 1;
        c[2] = k + 2;
    } else {
        c[0] = 3 * k;
        c[1] = 3 * k + 1;
        c[2] = 3 * k + 2;
    }
    float4 v[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int vi = M.first_index >= 0 ? (int)idx[M.first_index + c[q]] : c[q];
        v[q] = verts[M.first_vertex + vi];
    }
    const int clear = (k == 0 && M.clear) ? 2 : 0;
    t.flags = clear;
    bool ok = true;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        ok = ok && snap(v[q].x, W, &t.X[q]);
        ok = ok && snap(v[q].y, W, &t.Y[q]);
        t.alt[q] = v[q].z;
        t.u[q] = v[q].w;
    }
    if (!ok) return;
    long long a2 = edge_fn(t.X[0], t.Y[0], t.X[1], t.Y[1], t.X[2], t.Y[2]);
    if (a2 == 0) return;
    if (a2 < 0) {  // no face culling: clockwise triangles are drawn as their mirror
        int s = t.X[1]; t.X[1] = t.X[2]; t.X[2] = s;
        s = t.Y[1]; t.Y[1] = t.Y[2]; t.Y[2] = s;
        float f = t.alt[1]; t.alt[1] = t.alt[2]; t.alt[2] = f;
        f = t.u[1]; t.u[1] = t.u[2]; t.u[2] = f;
        a2 = -a2;
    }
    t.area = __ll2float_rn(a2);
    // edge q runs from vertex q + 1 to vertex q + 2 (the weight of vertex q)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int a = (q + 1) % 3, b = (q + 2) % 3;
        const int dx = t.X[b] - t.X[a], dy = t.Y[b] - t.Y[a];
        t.bias[q] = (dy < 0 || (dy == 0 && dx < 0)) ? 0 : 1;
    }
    const int xmin = min(t.X[0], min(t.X[1], t.X[2])), xmax = max(t.X[0], max(t.X[1], t.X[2]));
    const int ymin = min(t.Y[0], min(t.Y[1], t.Y[2])), ymax = max(t.Y[0], max(t.Y[1], t.Y[2]));
    const int h = kSubpixel / 2;
    t.ix0 = max(floor_div(xmin - h + kSubpixel - 1, kSubpixel), 0);
    t.ix1 = min(floor_div(xmax - h, kSubpixel), W - 1);
    t.jy0 = max(floor_div(ymin - h + kSubpixel - 1, kSubpixel), 0);
    t.jy1 = min(floor_div(ymax - h, kSubpixel), W - 1);
    if (t.ix0 > t.ix1 || t.jy0 > t.jy1) return;
    t.flags |= 1;
}

__global__ void __launch_bounds__(kThreads)
layers_kernel(float *elev, int W, int pitch, long long plane_stride, long long slot_stride, const DevJob *jobs,
              const DevMesh *meshes, const float4 *verts, const uint32_t *idx, int blend_mode, int band_rows)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Tri *tris = reinterpret_cast<Tri *>(smem_raw);
    const int span = (band_rows + 2) * W;
    float *zl = reinterpret_cast<float *>(tris + kThreads);
    float *wv = zl + span;
    float *dep = wv + span;
    // the original zm of each band's last row, which the next band reads as its
    // lower halo after this band has written its output (two rows, alternating)
    float *saved = dep + span;
    const DevJob J = jobs[blockIdx.x];
    float *zf_plane = elev + (long long)J.slot * slot_stride;
    float *zm_plane = zf_plane + 2 * plane_stride;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    for (int b0 = 0, band = 0; b0 < W; b0 += band_rows, ++band) {
        const int b1 = min(b0 + band_rows, W);
        const int h0 = max(b0 - 1, 0), h1 = min(b1 + 1, W);
        float *save_now = saved + (band & 1) * W;
        const float *save_prev = saved + ((band + 1) & 1) * W;
        // the framebuffer before the layers: z = zm, w = 0, depth cleared to 1
        for (int t = threadIdx.x; t < (h1 - h0) * W; t += kThreads) {
            const int r = h0 + t / W, cc = t - (t / W) * W;
            const float z = (b0 > 0 && r == h0) ? save_prev[cc] : zm_plane[(long long)r * pitch + cc];
            if (r == b1 - 1) save_now[cc] = z;
            zl[t] = z;
            wv[t] = 0.0f;
            dep[t] = 1.0f;
        }
        for (int base = 0; base < J.ntri; base += kThreads) {
            __syncthreads();
            if (base + (int)threadIdx.x < J.ntri) setup(tris[threadIdx.x], J, meshes, verts, idx, base + threadIdx.x, W);
            __syncthreads();
            const int cnt = min(kThreads, J.ntri - base);
            for (int k = 0; k < cnt; ++k) {
                const Tri &T = tris[k];
                const int flags = T.flags;
                if (flags & 2) {  // a new layer: its own pixels' depth back to 1
                    for (int r = h0 + ((warp - h0) & (kWarps - 1)); r < h1; r += kWarps)
                        for (int cc = lane; cc < W; cc += 32) dep[(r - h0) * W + cc] = 1.0f;
                }
                if (!(flags & 1)) continue;
                const int lo = max(T.jy0, h0), hi = min(T.jy1, h1 - 1);
                for (int r = lo + ((warp - lo) & (kWarps - 1)); r <= hi; r += kWarps) {
                    const int py = r * kSubpixel + kSubpixel / 2;
                    for (int i = T.ix0 + ((lane - T.ix0) & 31); i <= T.ix1; i += 32) {
                        const int px = i * kSubpixel + kSubpixel / 2;
                        const long long e0 = edge_fn(T.X[1], T.Y[1], T.X[2], T.Y[2], px, py);
                        const long long e1 = edge_fn(T.X[2], T.Y[2], T.X[0], T.Y[0], px, py);
                        const long long e2 = edge_fn(T.X[0], T.Y[0], T.X[1], T.Y[1], px, py);
                        if (e0 < T.bias[0] || e1 < T.bias[1] || e2 < T.bias[2]) continue;
                        // plane form a0 + (a1 - a0) l1 + (a2 - a0) l2: constant attributes stay exact
                        const float l1 = __fdiv_rn(__ll2float_rn(e1), T.area);
                        const float l2 = __fdiv_rn(__ll2float_rn(e2), T.area);
                        const float alt = __fadd_rn(__fadd_rn(T.alt[0], __fmul_rn(__fsub_rn(T.alt[1], T.alt[0]), l1)),
                                                    __fmul_rn(__fsub_rn(T.alt[2], T.alt[0]), l2));
                        const float u = __fadd_rn(__fadd_rn(T.u[0], __fmul_rn(__fsub_rn(T.u[1], T.u[0]), l1)),
                                                  __fmul_rn(__fsub_rn(T.u[2], T.u[0]), l2));
                        const float d = fabsf(u);
                        const float depth = fminf(fmaxf(__fadd_rn(__fmul_rn(d, 0.1f), 0.3f), 0.0f), 1.0f);
                        const int p = (r - h0) * W + i;
                        if (!(depth < dep[p])) continue;
                        dep[p] = depth;
                        zl[p] = __fadd_rn(alt, __fmul_rn(0.03f, __fsub_rn(1.0f, smoothstep_rn(0.98f, 1.0f, d))));
                        wv[p] = smoothstep_rn(1.0f, 2.0f, d);
                    }
                }
            }
        }
        __syncthreads();
        // blend(v) = zf min(w, 1) + z (1 - min(w, 1)), kept in the depth array
        for (int t = threadIdx.x; t < (h1 - h0) * W; t += kThreads) {
            const int r = h0 + t / W, cc = t - (t / W) * W;
            const float b = fminf(wv[t], 1.0f);
            dep[t] = __fadd_rn(__fmul_rn(zf_plane[(long long)r * pitch + cc], b), __fmul_rn(zl[t], __fsub_rn(1.0f, b)));
        }
        __syncthreads();
        for (int t = threadIdx.x; t < (b1 - b0) * W; t += kThreads) {
            const int r = b0 + t / W, cc = t - (t / W) * W;
            float out;
            if (blend_mode == 0) {
                out = dep[(r - h0) * W + cc];
            } else {
                // texture reads clamped to the edge; sums in the shader's order
                auto at = [&](int dr, int dc) {
                    const int rr = min(max(r + dr, 0), W - 1), c2 = min(max(cc + dc, 0), W - 1);
                    return dep[(rr - h0) * W + c2];
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

// Rows per band: the band's z, w and depth (with a row of halo on each side) in
// about 140 KB of shared memory.
int band_rows_for(int W)
{
    const int rows = 140000 / (12 * W) - 2;
    return rows >= W ? W : rows;
}

}  // namespace

extern "C" int tp_elevation_layers(tp_storage *elev, const tp_layer_job *jobs, int n, const tp_layer_mesh *meshes,
                                   int n_meshes, const float *vertices, int n_vertices, const uint32_t *indices,
                                   int n_indices, int blend_mode, void *stream)
{
    using tp::fail;
    if (!elev || n < 0 || (n > 0 && !jobs) || n_meshes < 0 || (n_meshes > 0 && !meshes) || n_vertices < 0 ||
        (n_vertices > 0 && !vertices) || n_indices < 0 || (n_indices > 0 && !indices) ||
        (blend_mode != 0 && blend_mode != 1))
        return fail(TP_E_BAD_ARG, "tp_elevation_layers: bad arguments");
    if (elev->on_device != 1 || elev->channels < 3)
        return fail(TP_E_BAD_ARG, "tp_elevation_layers: needs a device elevation storage (zf, zc, zm)");
    if (n == 0) return TP_OK;
    const int W = elev->W;
    if (band_rows_for(W) < 1) return fail(TP_E_BAD_ARG, "tp_elevation_layers: tile too wide");
    std::vector<DevMesh> dm(n_meshes);
    std::vector<uint8_t> mesh_used(n_meshes, 0);
    for (int m = 0; m < n_meshes; ++m) {
        const tp_layer_mesh &M = meshes[m];
        if (M.count < 0 || (M.mode != TP_TRIANGLES && M.mode != TP_TRIANGLE_STRIP) || M.first_vertex < 0 ||
            M.first_vertex > n_vertices)
            return fail(TP_E_BAD_ARG, "tp_elevation_layers: bad mesh");
        const int ntri = M.mode == TP_TRIANGLES ? M.count / 3 : (M.count >= 3 ? M.count - 2 : 0);
        const int used = M.mode == TP_TRIANGLES ? 3 * ntri : (ntri > 0 ? M.count : 0);
        if (M.first_index >= 0) {
            if ((long long)M.first_index + used > n_indices)
                return fail(TP_E_BAD_ARG, "tp_elevation_layers: mesh indices out of range");
            for (int k = 0; k < used; ++k)
                if ((long long)M.first_vertex + indices[M.first_index + k] >= n_vertices)
                    return fail(TP_E_BAD_ARG, "tp_elevation_layers: vertex index out of range");
        } else if ((long long)M.first_vertex + used > n_vertices) {
            return fail(TP_E_BAD_ARG, "tp_elevation_layers: mesh vertices out of range");
        }
        dm[m] = DevMesh{M.first_vertex, M.first_index, M.mode, ntri, 0, M.clear_depth ? 1 : 0, {0, 0}};
    }
    std::vector<DevJob> dj(n);
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
            pending_clear |= dm[m].clear;
            dm[m].clear = dm[m].ntri > 0 ? pending_clear : 0;
            if (dm[m].ntri > 0) pending_clear = 0;
            tri += dm[m].ntri;
        }
        dj[k] = DevJob{j.slot, j.first_mesh, j.n_meshes, tri};
    }

    static std::mutex mu;
    static char *dbuf = nullptr;
    static size_t dcap = 0;
    std::lock_guard<std::mutex> lk(mu);
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t bj = al(sizeof(DevJob) * n), bm = al(sizeof(DevMesh) * (n_meshes ? n_meshes : 1));
    const size_t bv = al(sizeof(float) * 4 * (size_t)(n_vertices ? n_vertices : 1));
    const size_t bi = al(sizeof(uint32_t) * (size_t)(n_indices ? n_indices : 1));
    const size_t need = bj + bm + bv + bi;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (dcap < need) {
        if (dbuf) {
            cudaStreamSynchronize(s);
            cudaFree(dbuf);
        }
        dbuf = nullptr;
        dcap = 0;
        cudaError_t e = cudaMalloc(&dbuf, need);
        if (e != cudaSuccess) return tp::cuda_fail("cudaMalloc (layer meshes)", e);
        dcap = need;
    }
    cudaError_t e = cudaMemcpyAsync(dbuf, dj.data(), sizeof(DevJob) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && n_meshes)
        e = cudaMemcpyAsync(dbuf + bj, dm.data(), sizeof(DevMesh) * n_meshes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && n_vertices)
        e = cudaMemcpyAsync(dbuf + bj + bm, vertices, sizeof(float) * 4 * (size_t)n_vertices, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && n_indices)
        e = cudaMemcpyAsync(dbuf + bj + bm + bv, indices, sizeof(uint32_t) * (size_t)n_indices, cudaMemcpyHostToDevice,
                            s);
    if (e != cudaSuccess) return tp::cuda_fail("cudaMemcpyAsync (layer meshes)", e);
    const int rows = band_rows_for(W);
    const size_t smem = sizeof(Tri) * kThreads + sizeof(float) * (3 * (size_t)(rows + 2) * W + 2 * (size_t)W);
    e = cudaFuncSetAttribute(layers_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return tp::cuda_fail("cudaFuncSetAttribute (layers)", e);
    layers_kernel<<<n, kThreads, smem, s>>>(elev->base, W, elev->pitch, elev->plane_stride, elev->slot_stride,
                                            reinterpret_cast<const DevJob *>(dbuf),
                                            reinterpret_cast<const DevMesh *>(dbuf + bj),
                                            reinterpret_cast<const float4 *>(dbuf + bj + bm),
                                            reinterpret_cast<const uint32_t *>(dbuf + bj + bm + bv), blend_mode, rows);
    e = cudaGetLastError();
    if (e != cudaSuccess) return tp::cuda_fail("layers kernel launch", e);
    // the mesh buffer is reused by the next call
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return tp::cuda_fail("cudaStreamSynchronize (layers)", e);
    return TP_OK;
}
