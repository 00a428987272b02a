/*
 * CPU oracle of the elevation layer pass -- TEST INFRASTRUCTURE ONLY.
 * Build with -O2 -ffp-contract=off (oracle/build.py): every float operation is
 * rounded on its own, in the order written here.
 *
 * Follows, relative to the reference project root:
 *  - the layer pass of ElevationProducer::doCreateTile:
 *    src/terrain/sources/proland/dem/ElevationProducer.cpp:378-399 (framebuffer
 *    cleared, upsample quad writing (zf, zc, zm, 0), layers drawn under a LESS depth
 *    test, then the blend quad);
 *  - the road elevation layer: src/graph/sources/proland/dem/RoadElevationLayer.cpp:388-437
 *    (depth cleared, colour mask z and w) with
 *    src/graph/examples/graph1/roadLayerElevationShader.glsl (fragment z, w, depth);
 *  - the water elevation layer: src/graph/sources/proland/dem/WaterElevationLayer.cpp:
 *    240-350 (its passes' depth tests, depth and colour masks) with
 *    src/river/examples/river1/waterLayerElevationShader.glsl (river = 0, 1, 2) and
 *    src/river/examples/river1/fillShader.glsl;
 *  - the blend programs: src/graph/examples/graph1/blendShader.glsl (mode 0) and
 *    src/demo/shaders/elevation/blendShader.glsl (mode 1, 3x3 box filter, texture
 *    reads clamped to the edge).
 *
 * Rasterisation, which the reference leaves to the GL driver, is fixed as: window
 * coordinates (x + 1) W / 2 snapped to 1/256 texel (round half to even), texel
 * (i, j) covered when its centre (i + 1/2, j + 1/2) is inside the triangle by exact
 * integer edge functions, centres on an edge covered for top and left edges only (y
 * up, counter-clockwise after reordering), attributes interpolated as
 * a0 + (a1 - a0) l1 + (a2 - a0) l2 with l_k = e_k / (2 area) in float (a constant
 * attribute stays exact), fp32 depth clamped to [0, 1], triangles and their fragments
 * in draw order (GL's strip order (k+1, k, k+2) for odd k), each fragment tested
 * against the depth stored at its texel and written through the masks.  The fragment
 * programs and both blends equal the reference's shaders compiled as C++
 * (tests/test_oracle_vs_reference_gpu.py); the rasterisation rule is this oracle's, as the
 * GL driver's is not source.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

static int snap(float c, int W, int *out)
{
    float w = (c + 1.0f) * (0.5f * (float)W);
    w = w * 256.0f;
    if (!(fabsf(w) <= 8388608.0f)) return 0;
    *out = (int)rintf(w);
    return 1;
}

static float smoothstep_f(float e0, float e1, float x)
{
    float t = (x - e0) / (e1 - e0);
    if (t < 0.0f) t = 0.0f;
    if (t > 1.0f) t = 1.0f;
    return t * t * (3.0f - 2.0f * t);
}

static long long edge(int xa, int ya, int xb, int yb, int px, int py)
{
    return (long long)(xb - xa) * (long long)(py - ya) - (long long)(yb - ya) * (long long)(px - xa);
}

static float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }

/* depth, z and w of a fragment of a mesh's program at attributes (a, u) */
static void fragment_program(const or_layer_mesh *M, float a, float u, float *dp, float *z, float *w)
{
    const float d = fabsf(u);
    switch (M->program) {
    case 0: /* roadLayerElevationShader */
        *z = a + 0.03f * (1.0f - smoothstep_f(0.98f, 1.0f, d));
        *w = smoothstep_f(1.0f, 2.0f, d);
        *dp = clamp01(d * 0.1f + 0.3f);
        break;
    case 4: /* fillShader: the colour's blue and alpha, the depth uniform */
        *z = a;
        *w = u;
        *dp = clamp01(M->fill_depth);
        break;
    default: { /* waterLayerElevationShader, river = program - 1 */
        const int river = M->program - 1;
        float zz = a;
        if (river != 0) {
            const float e = d - 1.0f;
            zz = (zz - 1.0f) + (e > 0.0f ? e : 0.0f);
        }
        *z = zz;
        *w = smoothstep_f(1.0f, 2.0f, d);
        *dp = river == 2 ? 1.0f : river == 1 ? clamp01(d * 0.1f + 0.15f) : clamp01(d * 0.1f + 0.3f);
        break;
    }
    }
}

static void draw_triangle(int W, const or_layer_mesh *M, const float *v0, const float *v1, const float *v2, float *z,
                          float *w, float *depth)
{    int X[3], Y[3];
    float alt[3], u[3];
    const float *v[3] = {v0, v1, v2};
    for (int q = 0; q < 3; ++q) {
        if (!snap(v[q][0], W, &X[q]) || !snap(v[q][1], W, &Y[q])) return;
        alt[q] = v[q][2];
        u[q] = v[q][3];
    }
    long long a2 = edge(X[0], Y[0], X[1], Y[1], X[2], Y[2]);
    if (a2 == 0) return;
    if (a2 < 0) {
        int t = X[1]; X[1] = X[2]; X[2] = t;
        t = Y[1]; Y[1] = Y[2]; Y[2] = t;
        float f = alt[1]; alt[1] = alt[2]; alt[2] = f;
        f = u[1]; u[1] = u[2]; u[2] = f;
        a2 = -a2;
    }
    const float area = (float)a2;
    int topleft[3];
    for (int q = 0; q < 3; ++q) {
        const int a = (q + 1) % 3, b = (q + 2) % 3;
        const int dx = X[b] - X[a], dy = Y[b] - Y[a];
        topleft[q] = dy < 0 || (dy == 0 && dx < 0);
    }
    int xmin = X[0], xmax = X[0], ymin = Y[0], ymax = Y[0];
    for (int q = 1; q < 3; ++q) {
        if (X[q] < xmin) xmin = X[q];
        if (X[q] > xmax) xmax = X[q];
        if (Y[q] < ymin) ymin = Y[q];
        if (Y[q] > ymax) ymax = Y[q];
    }
    int i0 = floor_div(xmin - 128 + 255, 256), i1 = floor_div(xmax - 128, 256);
    int j0 = floor_div(ymin - 128 + 255, 256), j1 = floor_div(ymax - 128, 256);
    if (i0 < 0) i0 = 0;
    if (j0 < 0) j0 = 0;
    if (i1 > W - 1) i1 = W - 1;
    if (j1 > W - 1) j1 = W - 1;
    for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
            const int px = 256 * i + 128, py = 256 * j + 128;
            const long long e[3] = {edge(X[1], Y[1], X[2], Y[2], px, py), edge(X[2], Y[2], X[0], Y[0], px, py),
                                    edge(X[0], Y[0], X[1], Y[1], px, py)};
            int in = 1;
            for (int q = 0; q < 3; ++q)
                if (e[q] < 0 || (e[q] == 0 && !topleft[q])) in = 0;
            if (!in) continue;
            const float l1 = (float)e[1] / area, l2 = (float)e[2] / area;
            const float a = alt[0] + (alt[1] - alt[0]) * l1 + (alt[2] - alt[0]) * l2;
            const float uu = u[0] + (u[1] - u[0]) * l1 + (u[2] - u[0]) * l2;
            float dp, fz, fw;
            fragment_program(M, a, uu, &dp, &fz, &fw);
            const int p = j * W + i;
            const int test = M->state & 3;
            if (test == 0 && !(dp < depth[p])) continue;   /* LESS */
            if (test == 2 && !(dp != depth[p])) continue;  /* NOTEQUAL */
            if (!(M->state & 4)) depth[p] = dp;
            if (!(M->state & 8)) z[p] = fz;
            if (!(M->state & 16)) w[p] = fw;
        }
}

void or_layer_tile(int W, const float *zf, const float *zm, const or_layer_mesh *meshes, int n_meshes,
                   const float *vertices, const uint32_t *indices, int blend_mode, float *zm_out)
{
    const size_t N = (size_t)W * W;
    float *z = (float *)malloc(N * sizeof(float));
    float *w = (float *)malloc(N * sizeof(float));
    float *depth = (float *)malloc(N * sizeof(float));
    for (size_t p = 0; p < N; ++p) {
        z[p] = zm[p];
        w[p] = 0.0f;
        depth[p] = 1.0f;
    }
    for (int m = 0; m < n_meshes; ++m) {
        const or_layer_mesh *M = &meshes[m];
        if (M->clear_depth)
            for (size_t p = 0; p < N; ++p) depth[p] = 1.0f;
        const int ntri = M->mode == 0 ? M->count / 3 : (M->count >= 3 ? M->count - 2 : 0);
        for (int k = 0; k < ntri; ++k) {
            int c[3];
            if (M->mode == 1) {
                c[0] = (k & 1) ? k + 1 : k;
                c[1] = (k & 1) ? k : k + 1;
                c[2] = k + 2;
            } else {
                c[0] = 3 * k;
                c[1] = 3 * k + 1;
                c[2] = 3 * k + 2;
            }
            const float *v[3];
            for (int q = 0; q < 3; ++q) {
                const int vi = M->first_index >= 0 ? (int)indices[M->first_index + c[q]] : c[q];
                v[q] = vertices + 4 * (size_t)(M->first_vertex + vi);
            }
            draw_triangle(W, M, v[0], v[1], v[2], z, w, depth);
        }
    }
    or_layer_blend(W, zf, z, w, blend_mode, zm_out);
    free(z);
    free(w);
    free(depth);
}

void or_layer_fragment(int program, float fill_depth, float a, float u, float *out)
{
    or_layer_mesh M;
    memset(&M, 0, sizeof(M));
    M.program = program;
    M.fill_depth = fill_depth;
    fragment_program(&M, a, u, &out[0], &out[1], &out[2]);
}

void or_layer_blend(int W, const float *zf, const float *z, const float *w, int blend_mode, float *zm_out)
{
    const size_t N = (size_t)W * W;
    float *bl = (float *)malloc(N * sizeof(float));
    for (size_t p = 0; p < N; ++p) {
        const float b = w[p] < 1.0f ? w[p] : 1.0f;
        bl[p] = zf[p] * b + z[p] * (1.0f - b);
    }
    for (int j = 0; j < W; ++j)
        for (int i = 0; i < W; ++i) {
            if (blend_mode == 0) {
                zm_out[j * W + i] = bl[j * W + i];
                continue;
            }
#define AT(dj, di) bl[(size_t)(j + (dj) < 0 ? 0 : j + (dj) > W - 1 ? W - 1 : j + (dj)) * W + \
                      (i + (di) < 0 ? 0 : i + (di) > W - 1 ? W - 1 : i + (di))]
            const float sx = AT(0, 0);
            const float sy = AT(0, 1) + AT(0, -1) + AT(1, 0) + AT(-1, 0);
            const float sz = AT(1, 1) + AT(-1, 1) + AT(-1, -1) + AT(1, -1);
#undef AT
            const float f = 1.0f / 9.0f;
            zm_out[j * W + i] = sx * f + sy * f + sz * f;
        }
    free(bl);
}
