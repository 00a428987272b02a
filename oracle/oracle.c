/*
 * CPU oracle for the terrain tile-production path -- TEST INFRASTRUCTURE ONLY.
 * See oracle.h for the contract.  Build with -O2 -ffp-contract=off (oracle/build.py).
 *
 * Reference paths are relative to the reference project root.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* LCG (src/core/sources/proland/math/noise.h:50-68).  The reference keeps the
 * seed in a C `long`; on both 32- and 64-bit longs the masked result is
 * (seed * 1103515245 + 12345) mod 2^31, which is what is computed here. */
long or_lrandom(long *seed)
{
    uint64_t s = (uint64_t)(*seed);
    s = (s * 1103515245ull + 12345ull) & 0x7FFFFFFFull;
    *seed = (long)s;
    return (long)s;
}

float or_frandom(long *seed)
{
    long r = or_lrandom(seed) >> 7;          /* top 24 of the 31 bits */
    return (float)r / (float)(1 << 24);
}

/* float -> binary16 with round-to-nearest-even, back to float.  The reference
 * uploads its noise table as an R16F texture (ElevationProducer.cpp:129). */
float or_half_round(float x)
{
    uint32_t u;
    memcpy(&u, &x, 4);
    uint32_t sign = u & 0x80000000u;
    uint32_t a = u & 0x7FFFFFFFu;
    float ax;
    memcpy(&ax, &a, 4);
    float r;
    if (a >= 0x7F800000u) {
        r = ax;                                  /* inf / nan passthrough */
    } else if (ax >= 65520.0f) {
        r = INFINITY;                            /* rounds past the largest half */
    } else if (ax < 6.103515625e-05f) {          /* half subnormal range: quantum 2^-24 */
        double q = (double)ax * 16777216.0;      /* exact */
        double f = floor(q);
        double d = q - f;
        if (d > 0.5 || (d == 0.5 && fmod(f, 2.0) != 0.0)) f += 1.0;
        r = (float)(f / 16777216.0);
    } else {
        /* normal half: keep 10 fraction bits (of float's 23), RNE on the dropped 13 */
        uint32_t drop = a & 0x1FFFu;
        uint32_t keep = a & ~0x1FFFu;
        if (drop > 0x1000u || (drop == 0x1000u && (keep & 0x2000u))) keep += 0x2000u;
        memcpy(&r, &keep, 4);
    }
    uint32_t ru;
    memcpy(&ru, &r, 4);
    ru |= sign;
    memcpy(&r, &ru, 4);
    return r;
}

/* Noise table of createDemNoise (ElevationProducer.cpp:50-133): six W x W layers
 * whose border bands are drawn from one of two fixed seeds, chosen per edge by the
 * layer's edge bits, and mirrored so that two tiles sharing an edge see the same
 * values; the centre comes from one seed that runs on across the layers. */
void or_dem_noise(int W, float *out)
{
    static const int edge_bits[6] = {0, 1, 3, 5, 7, 15};
    long centre_seed = 1234567;
    for (int layer = 0; layer < 6; ++layer) {
        float *t = out + (size_t)layer * W * W;
        int bits = edge_bits[layer];
        memset(t, 0, sizeof(float) * (size_t)W * W);
#define PUT(x, y, v) t[(x) + (y) * W] = (v)
        long s;
        float v;
        /* bottom edge */
        s = (bits & 1) ? 5647381 : 7654321;
        for (int h = 5; h <= W / 2; ++h) {
            v = or_frandom(&s) * 2.0f - 1.0f;
            PUT(h, 2, v); PUT(W - 1 - h, 2, v);
        }
        for (int y = 3; y < 5; ++y)
            for (int h = 5; h < W - 5; ++h) {
                v = or_frandom(&s) * 2.0f - 1.0f;
                PUT(h, y, v); PUT(W - 1 - h, 4 - y, v);
            }
        /* right edge */
        s = (bits & 2) ? 5647381 : 7654321;
        for (int y = 5; y <= W / 2; ++y) {
            v = or_frandom(&s) * 2.0f - 1.0f;
            PUT(W - 3, y, v); PUT(W - 3, W - 1 - y, v);
        }
        for (int x = W - 4; x >= W - 5; --x)
            for (int y = 5; y < W - 5; ++y) {
                v = or_frandom(&s) * 2.0f - 1.0f;
                PUT(x, y, v); PUT(2 * W - 6 - x, W - 1 - y, v);
            }
        /* top edge */
        s = (bits & 4) ? 5647381 : 7654321;
        for (int h = 5; h <= W / 2; ++h) {
            v = or_frandom(&s) * 2.0f - 1.0f;
            PUT(h, W - 3, v); PUT(W - 1 - h, W - 3, v);
        }
        for (int y = W - 2; y < W; ++y)
            for (int h = 5; h < W - 5; ++h) {
                v = or_frandom(&s) * 2.0f - 1.0f;
                PUT(h, y, v); PUT(W - 1 - h, 2 * W - 6 - y, v);
            }
        /* left edge */
        s = (bits & 8) ? 5647381 : 7654321;
        for (int y = 5; y <= W / 2; ++y) {
            v = or_frandom(&s) * 2.0f - 1.0f;
            PUT(2, y, v); PUT(2, W - 1 - y, v);
        }
        for (int x = 1; x >= 0; --x)
            for (int y = 5; y < W - 5; ++y) {
                v = or_frandom(&s) * 2.0f - 1.0f;
                PUT(x, y, v); PUT(4 - x, W - 1 - y, v);
            }
        /* centre */
        for (int y = 5; y < W - 5; ++y)
            for (int x = 5; x < W - 5; ++x)
                PUT(x, y, or_frandom(&centre_seed) * 2.0f - 1.0f);
#undef PUT
        for (int k = 0; k < W * W; ++k) t[k] = or_half_round(t[k]);
    }
}

/* ------------------------------------------------------------------------- */
/* 2D gradient noise of noise.cpp:60-165 (period 0).  Only its sign is used by
 * the elevation producer, to pick the noise layer of a tile. */
static int g_perm[2 * 256 + 2];
static float g_grad2[2 * 256 + 2][2];
static pthread_once_t g_perlin_once = PTHREAD_ONCE_INIT;

static void perlin_init(void)
{
    long seed = 12345;
    int i;
    for (i = 0; i < 256; ++i) {
        g_perm[i] = i;
        /* the reference draws a 1D gradient, then the 2D one, then a 3D one,
         * all from the same stream: keep the stream aligned */
        (void)or_lrandom(&seed);
        for (int k = 0; k < 2; ++k)
            g_grad2[i][k] = (float)((or_lrandom(&seed) % 512) - 256) / 256;
        float len = sqrtf(g_grad2[i][0] * g_grad2[i][0] + g_grad2[i][1] * g_grad2[i][1]);
        g_grad2[i][0] /= len;
        g_grad2[i][1] /= len;
        for (int k = 0; k < 3; ++k) (void)or_lrandom(&seed);
    }
    for (i = 255; i > 0; --i) {
        int j = (int)(or_lrandom(&seed) % 256);
        int tmp = g_perm[i];
        g_perm[i] = g_perm[j];
        g_perm[j] = tmp;
    }
    for (i = 0; i < 256 + 2; ++i) {
        g_perm[256 + i] = g_perm[i];
        g_grad2[256 + i][0] = g_grad2[i][0];
        g_grad2[256 + i][1] = g_grad2[i][1];
    }
}

float or_cnoise2(float x, float y)
{
    pthread_once(&g_perlin_once, perlin_init);
    float t;
    t = x + 0x1000;
    int bx0 = ((int)t) & 0xFF, bx1 = (bx0 + 1) & 0xFF;
    float rx0 = t - (int)floorf(t), rx1 = rx0 - 1.0f;
    t = y + 0x1000;
    int by0 = ((int)t) & 0xFF, by1 = (by0 + 1) & 0xFF;
    float ry0 = t - (int)floorf(t), ry1 = ry0 - 1.0f;
    int i = g_perm[bx0], j = g_perm[bx1];
    int b00 = g_perm[i + by0], b10 = g_perm[j + by0];
    int b01 = g_perm[i + by1], b11 = g_perm[j + by1];
    float sx = rx0 * rx0 * (3.0f - 2.0f * rx0);
    float sy = ry0 * ry0 * (3.0f - 2.0f * ry0);
    float u, v, a, b;
    u = rx0 * g_grad2[b00][0] + ry0 * g_grad2[b00][1];
    v = rx1 * g_grad2[b10][0] + ry0 * g_grad2[b10][1];
    a = u + sx * (v - u);
    u = rx0 * g_grad2[b01][0] + ry1 * g_grad2[b01][1];
    v = rx1 * g_grad2[b11][0] + ry1 * g_grad2[b11][1];
    b = u + sx * (v - u);
    return a + sy * (b - a);
}

/* Per-tile noise rotation and layer (ElevationProducer.cpp:345-374).  The four
 * edge bits say, for each tile edge, the sign of the noise at that edge midpoint
 * in a face-continuous parameterisation; the 16 patterns map onto the 6 layers
 * of or_dem_noise and a rotation. */
void or_noise_select(int face, int level, int tx, int ty, int *rot, int *layer)
{
    int e;
    if (face == 1) {
        int o = 1 << level;
        e  = or_cnoise2((float)(tx + 0.5), (float)(ty + o)) > 0.0f ? 1 : 0;
        e += (tx == o - 1 ? or_cnoise2((float)(ty + o + 0.5), (float)o)
                          : or_cnoise2((float)(tx + 1), (float)(ty + o + 0.5))) > 0.0f ? 2 : 0;
        e += (ty == o - 1 ? or_cnoise2((float)((3 * o - 1 - tx) + 0.5), (float)o)
                          : or_cnoise2((float)(tx + 0.5), (float)(ty + o + 1))) > 0.0f ? 4 : 0;
        e += (tx == 0 ? or_cnoise2((float)((4 * o - 1 - ty) + 0.5), (float)o)
                      : or_cnoise2((float)tx, (float)(ty + o + 0.5))) > 0.0f ? 8 : 0;
    } else if (face == 6) {
        int o = 1 << level;
        e  = (ty == 0 ? or_cnoise2((float)((3 * o - 1 - tx) + 0.5), 0.0f)
                      : or_cnoise2((float)(tx + 0.5), (float)(ty - o))) > 0.0f ? 1 : 0;
        e += (tx == o - 1 ? or_cnoise2((float)((2 * o - 1 - ty) + 0.5), 0.0f)
                          : or_cnoise2((float)(tx + 1), (float)(ty - o + 0.5))) > 0.0f ? 2 : 0;
        e += or_cnoise2((float)(tx + 0.5), (float)(ty - o + 1)) > 0.0f ? 4 : 0;
        e += (tx == 0 ? or_cnoise2((float)(3 * o + ty + 0.5), 0.0f)
                      : or_cnoise2((float)tx, (float)(ty - o + 0.5))) > 0.0f ? 8 : 0;
    } else {
        int o = (1 << level) * (face - 2);
        e  = or_cnoise2((float)(tx + o + 0.5), (float)ty) > 0.0f ? 1 : 0;
        e += or_cnoise2((float)((tx + o + 1) % (4 << level)), (float)(ty + 0.5)) > 0.0f ? 2 : 0;
        e += or_cnoise2((float)(tx + o + 0.5), (float)(ty + 1)) > 0.0f ? 4 : 0;
        e += or_cnoise2((float)(tx + o), (float)(ty + 0.5)) > 0.0f ? 8 : 0;
    }
    static const int rots[16]   = {0, 0, 1, 0, 2, 0, 1, 0, 3, 3, 1, 3, 2, 2, 1, 0};
    static const int layers[16] = {0, 1, 1, 2, 1, 3, 2, 4, 1, 2, 3, 4, 2, 4, 4, 5};
    *rot = rots[e];
    *layer = layers[e];
}

/* ------------------------------------------------------------------------- */
/* 2x interpolating upsample of one child sample (CPUElevationProducer.cpp:202-238;
 * identical loops in ResidualProducer.cpp:342-384 and HeightMipmap.cpp:449-497). */
static float upsample_sample(const float *P, int pitch, int i, int j, int px, int py)
{
    const float *c = P + (i / 2 + px) + (size_t)(j / 2 + py) * pitch;
    if ((j & 1) == 0) {
        if ((i & 1) == 0) return c[0];
        return ((c[0] + c[1]) * 9 - (c[-1] + c[2])) / 16;
    }
    if ((i & 1) == 0)
        return ((c[0] + c[pitch]) * 9 - (c[-pitch] + c[2 * pitch])) / 16;
    float z = 0;
    for (int dj = -1; dj <= 2; ++dj) {
        float f = (dj == -1 || dj == 2) ? -1 / 16.0f : 9 / 16.0f;
        for (int di = -1; di <= 2; ++di) {
            float g = (di == -1 || di == 2) ? -1 / 16.0f : 9 / 16.0f;
            z += f * g * c[di + (ptrdiff_t)dj * pitch];
        }
    }
    return z;
}

static double upsample_sample_f64(const float *P, int pitch, int i, int j, int px, int py)
{
    const float *c = P + (i / 2 + px) + (size_t)(j / 2 + py) * pitch;
    static const double w[4] = {-1.0 / 16, 9.0 / 16, 9.0 / 16, -1.0 / 16};
    if ((j & 1) == 0) {
        if ((i & 1) == 0) return c[0];
        double s = 0;
        for (int d = -1; d <= 2; ++d) s += w[d + 1] * c[d];
        return s;
    }
    if ((i & 1) == 0) {
        double s = 0;
        for (int d = -1; d <= 2; ++d) s += w[d + 1] * c[(ptrdiff_t)d * pitch];
        return s;
    }
    double s = 0;
    for (int dj = -1; dj <= 2; ++dj)
        for (int di = -1; di <= 2; ++di) s += w[dj + 1] * w[di + 1] * c[di + (ptrdiff_t)dj * pitch];
    return s;
}

void or_cpu_elevation_tile(int W, int level, int tx, int ty,
                           const float *parent, int parent_pitch,
                           const float *residual, int res_pitch, int rx, int ry,
                           float *out, int out_pitch)
{
    int n = W - 5;
    int px = 1 + (tx % 2) * n / 2;
    int py = 1 + (ty % 2) * n / 2;
    for (int j = 0; j < W; ++j)
        for (int i = 0; i < W; ++i) {
            float z = level == 0 ? 0.0f : upsample_sample(parent, parent_pitch, i, j, px, py);
            float r = residual ? residual[(i + rx) + (size_t)(j + ry) * res_pitch] : 0.0f;
            out[i + (size_t)j * out_pitch] = z + r;
        }
}

/* ---- shader-only parts ---------------------------------------------------- */
/* 4x4 operator matrices of demo/shaders/elevation/upsampleShader.glsl:60-115, in
 * the order their literals list them: entry k weighs parent sample
 * (x0 + k % 4, y0 + k / 4) of the 4x4 neighbourhood. */
static const float k_slopex[4][16] = {
    {0, 0, 0, 0, 1, 0, -1, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0.5f, 0.5f, -0.5f, -0.5f, 0, 0, 0, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0.5f, 0, -0.5f, 0, 0.5f, 0, -0.5f, 0, 0, 0, 0, 0},
    {0, 0, 0, 0, 0.25f, 0.25f, -0.25f, -0.25f, 0.25f, 0.25f, -0.25f, -0.25f, 0, 0, 0, 0}};
static const float k_slopey[4][16] = {
    {0, 1, 0, 0, 0, 0, 0, 0, 0, -1, 0, 0, 0, 0, 0, 0},
    {0, 0.5f, 0.5f, 0, 0, 0, 0, 0, 0, -0.5f, -0.5f, 0, 0, 0, 0, 0},
    {0, 0.5f, 0, 0, 0, 0.5f, 0, 0, 0, -0.5f, 0, 0, 0, -0.5f, 0, 0},
    {0, 0.25f, 0.25f, 0, 0, 0.25f, 0.25f, 0, 0, -0.25f, -0.25f, 0, 0, -0.25f, -0.25f, 0}};
static const float k_curv[4][16] = {
    {0, -1, 0, 0, -1, 4, -1, 0, 0, -1, 0, 0, 0, 0, 0, 0},
    {0, -0.5f, -0.5f, 0, -0.5f, 1.5f, 1.5f, -0.5f, 0, -0.5f, -0.5f, 0, 0, 0, 0, 0},
    {0, -0.5f, 0, 0, -0.5f, 1.5f, -0.5f, 0, -0.5f, 1.5f, -0.5f, 0, 0, -0.5f, 0, 0},
    {0, -0.25f, -0.25f, 0, -0.25f, 0.5f, 0.5f, -0.25f, -0.25f, 0.5f, 0.5f, -0.25f, 0, -0.25f, -0.25f, 0}};

/* mdot of the shader: sum over the four columns of 4-term dot products, each
 * evaluated left to right. */
static float mdot16(const float *cz, const float *M)
{
    float s = 0.0f;
    for (int c = 0; c < 4; ++c) {
        const float *a = cz + 4 * c, *b = M + 4 * c;
        float d = a[0] * b[0];
        d = d + a[1] * b[1];
        d = d + a[2] * b[2];
        d = d + a[3] * b[3];
        s = c == 0 ? d : s + d;
    }
    return s;
}

static inline int floordiv(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* Noise texel for sample (i, j) under rotation r: the shader reads
 * (uvs[r], uvs[(r+1)%4]) with uvs = (u, v, 1-u, 1-v), u = (i+0.5)/W. */
static inline int noise_index(int W, int rot, int i, int j)
{
    switch (rot & 3) {
    case 0: return i + j * W;
    case 1: return j + (W - 1 - i) * W;
    case 2: return (W - 1 - i) + (W - 1 - j) * W;
    default: return (W - 1 - j) + i * W;
    }
}

/* Demo-shader noise modulation m = max(clamp(4 curv, 0, 1.5), clamp(2 slope - 0.5, 0.1, 4))
 * (demo/shaders/elevation/upsampleShader.glsl:162-166). */
static float demo_modulation(const float *cz, int mi, float mps)
{
    float sx = mdot16(cz, k_slopex[mi]);
    float sy = mdot16(cz, k_slopey[mi]);
    float nz = 2.0f * mps;
    float slope = sqrtf(sx * sx + sy * sy) / nz;
    float curv = mdot16(cz, k_curv[mi]) / mps;
    float a = 4.0f * curv;
    a = a < 0.0f ? 0.0f : (a > 1.5f ? 1.5f : a);
    float b = 2.0f * slope - 0.5f;
    b = b < 0.1f ? 0.1f : (b > 4.0f ? 4.0f : b);
    return a > b ? a : b;
}

/* zc: mean of the parent zm at two coarse-mesh vertices, or the larger diagonal
 * at flipped cell centres (terrain1/upsampleShader.glsl:118-121,
 * terrain4/upsampleShader.glsl:118-127).  The shader's float floor() of ij/(2g)
 * (+0.5) equals the integer floor division used here for every integer ij.
 * Parent texels outside the tile clamp to its edge. */
static float coarse_z(const or_elev_tile *t, int i, int j, int dx, int dy)
{
    int g = t->grid_g, W = t->W, pp = t->parent_pitch;
    int cx = i - 2, cy = j - 2;
    int kxr = floordiv(cx + g, 2 * g), kxf = floordiv(cx, 2 * g);
    int kyr = floordiv(cy + g, 2 * g), kyf = floordiv(cy, 2 * g);
    int X_r = clampi(2 + dx + g * kxr, 0, W - 1), X_f = clampi(2 + dx + g * kxf, 0, W - 1);
    int Y_r = clampi(2 + dy + g * kyr, 0, W - 1), Y_f = clampi(2 + dy + g * kyf, 0, W - 1);
    const float *P = t->parent_zm;
    float zc1 = P[X_r + (size_t)Y_f * pp];
    float zc3 = P[X_f + (size_t)Y_r * pp];
    if (t->flip && ((cx % (2 * g)) + 2 * g) % (2 * g) == g && ((cy % (2 * g)) + 2 * g) % (2 * g) == g) {
        float zc0 = P[X_f + (size_t)Y_f * pp];
        float zc2 = P[X_r + (size_t)Y_r * pp];
        return (zc3 + zc1 >= zc0 + zc2 ? zc1 + zc3 : zc0 + zc2) * 0.5f;
    }
    return (zc1 + zc3) * 0.5f;
}

void or_elevation_tile(const or_elev_tile *t)
{
    int W = t->W, n = W - 5;
    int dx = (t->tx % 2) * (n / 2), dy = (t->ty % 2) * (n / 2);
    int px = 1 + dx, py = 1 + dy;
    for (int j = 0; j < W; ++j)
        for (int i = 0; i < W; ++i) {
            float zf = t->residual ? t->rscale * t->residual[(i + t->rx) + (size_t)(j + t->ry) * t->res_pitch] : 0.0f;
            if (t->noise) {
                float N = t->noise[noise_index(W, t->noise_rot, i, j)];
                float amp = t->noise_amp;
                if (t->noise_mode == 0) {
                    zf = zf + fabsf(amp) * N;
                } else if (amp < 0.0f) {
                    zf = zf - amp * N;
                } else {
                    float cz[16] = {0};
                    if (t->level > 0)
                        for (int k = 0; k < 16; ++k)
                            cz[k] = t->parent_zf[clampi(i / 2 + dx + k % 4, 0, W - 1) +
                                                 (size_t)clampi(j / 2 + dy + k / 4, 0, W - 1) * t->parent_pitch];
                    float m = demo_modulation(cz, (i & 1) + 2 * (j & 1), t->meters_per_sample);
                    zf = zf + m * amp * N;
                }
            }
            float zc = zf;
            if (t->level > 0) {
                zf = zf + upsample_sample(t->parent_zf, t->parent_pitch, i, j, px, py);
                zc = coarse_z(t, i, j, dx, dy);
            }
            float zm = t->no_clamp ? zf : (zf > 0.0f ? zf : 0.0f);
            size_t o = i + (size_t)j * t->out_pitch;
            t->out_zf[o] = zf;
            t->out_zc[o] = zc;
            t->out_zm[o] = zm;
        }
}

void or_elevation_tile_f64(const or_elev_tile *t, double *ozf, double *ozc, double *ozm)
{
    int W = t->W, n = W - 5;
    int dx = (t->tx % 2) * (n / 2), dy = (t->ty % 2) * (n / 2);
    int px = 1 + dx, py = 1 + dy;
    for (int j = 0; j < W; ++j)
        for (int i = 0; i < W; ++i) {
            double zf = t->residual ? (double)t->rscale * t->residual[(i + t->rx) + (size_t)(j + t->ry) * t->res_pitch] : 0.0;
            if (t->noise) {
                double N = t->noise[noise_index(W, t->noise_rot, i, j)];
                double amp = t->noise_amp;
                if (t->noise_mode == 0) {
                    zf += fabs(amp) * N;
                } else if (amp < 0.0) {
                    zf -= amp * N;
                } else {
                    float cz[16] = {0};
                    if (t->level > 0)
                        for (int k = 0; k < 16; ++k)
                            cz[k] = t->parent_zf[clampi(i / 2 + dx + k % 4, 0, W - 1) +
                                                 (size_t)clampi(j / 2 + dy + k / 4, 0, W - 1) * t->parent_pitch];
                    double m = demo_modulation(cz, (i & 1) + 2 * (j & 1), t->meters_per_sample);
                    zf += m * amp * N;
                }
            }
            double zc = zf;
            if (t->level > 0) {
                zf += upsample_sample_f64(t->parent_zf, t->parent_pitch, i, j, px, py);
                zc = coarse_z(t, i, j, dx, dy);
            }
            size_t o = i + (size_t)j * t->out_pitch;
            ozf[o] = zf;
            ozc[o] = zc;
            ozm[o] = t->no_clamp ? zf : (zf > 0.0 ? zf : 0.0);
        }
}

/* ---- normals -------------------------------------------------------------- */
/* Flat normal of terrain1/normalShader.glsl:57-74: the cross product of the
 * central differences (2h, 0, z1 - z0) x (0, 2h, z3 - z2), normalised, xy kept;
 * h = tile_meters / n is the sample spacing.  The zm channel at the texel of the
 * sample is read exactly (point sampling). */
void or_normals_flat(int W, const float *zm, int zm_pitch, float tile_meters,
                     int format, float *nx, float *ny, int out_pitch)
{
    int n = W - 5;
    float h2 = 2.0f * (tile_meters / (float)n);
    for (int q = 0; q <= n; ++q)
        for (int p = 0; p <= n; ++p) {
            const float *c = zm + (p + 2) + (size_t)(q + 2) * zm_pitch;
            float ax = -(c[1] - c[-1]);
            float ay = -(c[zm_pitch] - c[-zm_pitch]);
            float inv = 1.0f / sqrtf(ax * ax + ay * ay + h2 * h2);
            float vx = ax * inv, vy = ay * inv;
            size_t o = p + (size_t)q * out_pitch;
            if (format == 3) {
                float ux = vx * 0.5f + 0.5f, uy = vy * 0.5f + 0.5f;
                nx[o] = floorf(fminf(fmaxf(ux, 0.0f), 1.0f) * 255.0f + 0.5f);
                ny[o] = floorf(fminf(fmaxf(uy, 0.0f), 1.0f) * 255.0f + 0.5f);
            } else {
                nx[o] = vx;
                ny[o] = vy;
            }
        }
}

/* The same normals as the reference's GL path samples zm: terrain1/normalShader.glsl
 * fetches texel X at (X + 0.25) / width (NormalProducer.cpp:210-213) from a LINEAR
 * storage (terrain1/helloworld.xml:30-32), so each fetch is the bilinear blend of
 * texels X - 1 and X with weights 0.25 / 0.75 in each direction.  For reporting how
 * far that sampling is from the texel-exact finite differences the product
 * computes; nothing is compared against it. */
static float gl_linear_fetch(const float *zm, int pitch, int X, int Y)
{
    const float *r0 = zm + (size_t)(Y - 1) * pitch, *r1 = zm + (size_t)Y * pitch;
    return 0.0625f * r0[X - 1] + 0.1875f * r0[X] + 0.1875f * r1[X - 1] + 0.5625f * r1[X];
}

void or_normals_flat_gl_linear(int W, const float *zm, int zm_pitch, float tile_meters, float *nx, float *ny,
                               int out_pitch)
{
    int n = W - 5;
    float h2 = 2.0f * (tile_meters / (float)n);
    for (int q = 0; q <= n; ++q)
        for (int p = 0; p <= n; ++p) {
            const int X = p + 2, Y = q + 2;
            float ax = -(gl_linear_fetch(zm, zm_pitch, X + 1, Y) - gl_linear_fetch(zm, zm_pitch, X - 1, Y));
            float ay = -(gl_linear_fetch(zm, zm_pitch, X, Y + 1) - gl_linear_fetch(zm, zm_pitch, X, Y - 1));
            float inv = 1.0f / sqrtf(ax * ax + ay * ay + h2 * h2);
            nx[p + (size_t)q * out_pitch] = ax * inv;
            ny[p + (size_t)q * out_pitch] = ay * inv;
        }
}

void or_normals_flat_f64(int W, const double *zm, int zm_pitch, double tile_meters,
                         double *nx, double *ny, int out_pitch)
{
    int n = W - 5;
    double h2 = 2.0 * tile_meters / n;
    for (int q = 0; q <= n; ++q)
        for (int p = 0; p <= n; ++p) {
            const double *c = zm + (p + 2) + (size_t)(q + 2) * zm_pitch;
            double ax = -(c[1] - c[-1]), ay = -(c[zm_pitch] - c[-zm_pitch]);
            double inv = 1.0 / sqrt(ax * ax + ay * ay + h2 * h2);
            nx[p + (size_t)q * out_pitch] = ax * inv;
            ny[p + (size_t)q * out_pitch] = ay * inv;
        }
}

/* ---- spherical deformation ------------------------------------------------ */
static void v3_norm(const double *v, double *o, double *len)
{
    double l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    o[0] = v[0] / l; o[1] = v[1] / l; o[2] = v[2] / l;
    if (len) *len = l;
}

/* NormalProducer.cpp:215-273: corners of the tile on the sphere of radius
 * R = D/2 relative to their mean, their unit verticals and distances, and the
 * world-to-tangent frame at the tile centre. */
void or_sphere_frame_make(double D, int level, int tx, int ty, or_sphere_frame *f)
{
    double R = D / 2.0;
    double s = (double)(1 << level);
    double x0 = (double)tx / s * D - R, x1 = (double)(tx + 1) / s * D - R;
    double y0 = (double)ty / s * D - R, y1 = (double)(ty + 1) / s * D - R;
    double p[4][3] = {{x0, y0, R}, {x1, y0, R}, {x0, y1, R}, {x1, y1, R}};
    double v[4][3], l[4], vc[3] = {0, 0, 0};
    for (int k = 0; k < 4; ++k) {
        v3_norm(p[k], v[k], &l[k]);
        for (int c = 0; c < 3; ++c) vc[c] += v[k][c];
    }
    for (int c = 0; c < 3; ++c) vc[c] *= 0.25;
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 4; ++k) {
            f->C[r * 4 + k] = (float)(v[k][r] * R - vc[r] * R);
            f->N[r * 4 + k] = (float)v[k][r];
        }
    for (int k = 0; k < 4; ++k) {
        f->C[12 + k] = 1.0f;
        f->N[12 + k] = 0.0f;
        f->L[k] = (float)l[k];
    }
    double pc[3] = {(x0 + x1) * 0.5, (y0 + y1) * 0.5, R}, uz[3], ux[3], uy[3];
    v3_norm(pc, uz, NULL);
    double t[3] = {uz[2], 0.0, -uz[0]};   /* (0,1,0) x uz */
    v3_norm(t, ux, NULL);
    uy[0] = uz[1] * ux[2] - uz[2] * ux[1];
    uy[1] = uz[2] * ux[0] - uz[0] * ux[2];
    uy[2] = uz[0] * ux[1] - uz[1] * ux[0];
    for (int c = 0; c < 3; ++c) {
        f->W2T[0 + c] = (float)ux[c];
        f->W2T[3 + c] = (float)uy[c];
        f->W2T[6 + c] = (float)uz[c];
    }
    f->R = (float)R;
    f->size = (float)(D / s);
}

/* getWorldPosition of terrain2/normalShader.glsl:56-73 */
static void sphere_pos(const or_sphere_frame *f, float n, float u, float v, float h, float *out)
{
    u = u / n;
    v = v / n;
    float U = 1.0f - u, V = 1.0f - v;
    float al[4] = {U * V, u * V, U * v, u * v};
    float d = al[0] * f->L[0] + al[1] * f->L[1] + al[2] * f->L[2] + al[3] * f->L[3];
    float ap[4];
    for (int k = 0; k < 4; ++k) ap[k] = al[k] * f->L[k] / d;
    float up[3], cp[3];
    for (int r = 0; r < 3; ++r) {
        up[r] = f->N[r * 4 + 0] * ap[0] + f->N[r * 4 + 1] * ap[1] + f->N[r * 4 + 2] * ap[2] + f->N[r * 4 + 3] * ap[3];
        cp[r] = f->C[r * 4 + 0] * ap[0] + f->C[r * 4 + 1] * ap[1] + f->C[r * 4 + 2] * ap[2] + f->C[r * 4 + 3] * ap[3];
    }
    float R = f->R;
    float e0 = R / 32.0f, e1 = R / 64.0f;
    float s = (f->size - e0) / (e1 - e0);
    s = s < 0.0f ? 0.0f : (s > 1.0f ? 1.0f : s);
    s = s * s * (3.0f - 2.0f * s);
    float len = sqrtf(up[0] * up[0] + up[1] * up[1] + up[2] * up[2]);
    float k = len * (1.0f - s) + 1.0f * s;
    float hp = (h + R * (1.0f - k)) / k;
    for (int r = 0; r < 3; ++r) out[r] = cp[r] + hp * up[r];
}

void or_normals_sphere(int W, const float *zm, int zm_pitch, const or_sphere_frame *f,
                       float *nx, float *ny, int out_pitch)
{
    int n = W - 5;
    for (int q = 0; q <= n; ++q)
        for (int p = 0; p <= n; ++p) {
            const float *c = zm + (p + 2) + (size_t)(q + 2) * zm_pitch;
            float p0[3], p1[3], p2[3], p3[3];
            sphere_pos(f, (float)n, (float)(p - 1), (float)q, c[-1], p0);
            sphere_pos(f, (float)n, (float)(p + 1), (float)q, c[1], p1);
            sphere_pos(f, (float)n, (float)p, (float)(q - 1), c[-zm_pitch], p2);
            sphere_pos(f, (float)n, (float)p, (float)(q + 1), c[zm_pitch], p3);
            float a[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
            float b[3] = {p3[0] - p2[0], p3[1] - p2[1], p3[2] - p2[2]};
            float cr[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
            float inv = 1.0f / sqrtf(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
            for (int k = 0; k < 3; ++k) cr[k] *= inv;
            size_t o = p + (size_t)q * out_pitch;
            nx[o] = f->W2T[0] * cr[0] + f->W2T[1] * cr[1] + f->W2T[2] * cr[2];
            ny[o] = f->W2T[3] * cr[0] + f->W2T[4] * cr[1] + f->W2T[5] * cr[2];
        }
}

/* parentToTangentFrame (NormalProducer.cpp:256-270): the child's world-to-tangent
 * frame times the parent tile centre's tangent-to-world frame, row-major. */
void or_parent_to_tangent(double D, int level, int tx, int ty, float *p2t)
{
    double R = D / 2.0, sc = (double)(1 << level);
    double x0 = (double)tx / sc * D - R, x1 = (double)(tx + 1) / sc * D - R;
    double y0 = (double)ty / sc * D - R, y1 = (double)(ty + 1) / sc * D - R;
    double pc[3] = {(x0 + x1) * 0.5, (y0 + y1) * 0.5, R}, w[3][3], t[3][3];
    double uz[3], ux[3], uy[3];
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) {
            double ps = (double)(1 << (level - 1));
            pc[0] = ((double)(tx / 2) + 0.5) / ps * D - R;
            pc[1] = ((double)(ty / 2) + 0.5) / ps * D - R;
            pc[2] = R;
        }
        v3_norm(pc, uz, NULL);
        double a[3] = {uz[2], 0.0, -uz[0]};
        v3_norm(a, ux, NULL);
        uy[0] = uz[1] * ux[2] - uz[2] * ux[1];
        uy[1] = uz[2] * ux[0] - uz[0] * ux[2];
        uy[2] = uz[0] * ux[1] - uz[1] * ux[0];
        for (int c = 0; c < 3; ++c) {
            if (pass == 0) { w[0][c] = ux[c]; w[1][c] = uy[c]; w[2][c] = uz[c]; }
            else { t[c][0] = ux[c]; t[c][1] = uy[c]; t[c][2] = uz[c]; }
        }
    }
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) p2t[r * 3 + c] = (float)(w[r][0] * t[0][c] + w[r][1] * t[1][c] + w[r][2] * t[2][c]);
}

static float unorm8(float v)
{
    v = v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v);
    return floorf(v * 255.0f + 0.5f) / 255.0f;
}

/* NormalProducer::doCreateTile in its four output formats (demo
 * normalShader.glsl:93-124): nf from the finite differences of zm (flat, or on the
 * sphere frame f); nc, for formats 0 and 1 above level 0, the mean of the parent
 * normal tile's nf at the two nearest coarse-mesh vertices
 * g floor(ij / 2g + (1/2, 0)) and g floor(ij / 2g + (0, 1/2)), g = (Wn - 1) / gridMeshSize,
 * in the parent's quadrant (tx % 2, ty % 2) x (Wn - 1) / 2 (point sampled),
 * decoded from unsigned for format 1 and rotated by parentToTangentFrame (p2t)
 * on a sphere; otherwise nc = nf.  Formats 1 and 3 are 8-bit unsigned textures:
 * their values are stored as k / 255.  pnx/pny: the parent's first two planes. */
void or_normals_full(int W, const float *zm, int zm_pitch, float tile_meters, const or_sphere_frame *f,
                     const float *p2t, int format, int grid_mesh, int tx, int ty, const float *pnx, const float *pny,
                     int ppitch, float *o0, float *o1, float *o2, float *o3, int out_pitch)
{
    const int Wn = W - 4, n = W - 5;
    float *nfx = (float *)malloc(sizeof(float) * Wn * Wn), *nfy = (float *)malloc(sizeof(float) * Wn * Wn);
    if (f)
        or_normals_sphere(W, zm, zm_pitch, f, nfx, nfy, Wn);
    else
        or_normals_flat(W, zm, zm_pitch, tile_meters, 2, nfx, nfy, Wn);
    const int g = (Wn - 1) / grid_mesh;
    const int dxi = (tx % 2) * ((Wn - 1) / 2), dyi = (ty % 2) * ((Wn - 1) / 2);
    const int coarse = (format == 0 || format == 1) && pnx && pny;
    for (int q = 0; q <= n; ++q)
        for (int p = 0; p <= n; ++p) {
            const size_t k = p + (size_t)q * Wn, o = p + (size_t)q * out_pitch;
            float vx = nfx[k], vy = nfy[k], cx = vx, cy = vy;
            if (coarse) {
                const int ax = g * ((p + g) / (2 * g)) + dxi, ay = g * (q / (2 * g)) + dyi;
                const int bx = g * (p / (2 * g)) + dxi, by = g * ((q + g) / (2 * g)) + dyi;
                cx = (pnx[ax + (size_t)ay * ppitch] + pnx[bx + (size_t)by * ppitch]) * 0.5f;
                cy = (pny[ax + (size_t)ay * ppitch] + pny[bx + (size_t)by * ppitch]) * 0.5f;
                if (format == 1) {
                    cx = cx * 2.0f - 1.0f;
                    cy = cy * 2.0f - 1.0f;
                }
                if (f && p2t) {
                    float cz2 = 1.0f - (cx * cx + cy * cy);
                    const float cz = sqrtf(cz2 > 0.0f ? cz2 : 0.0f);
                    const float rx = p2t[0] * cx + p2t[1] * cy + p2t[2] * cz;
                    const float ry = p2t[3] * cx + p2t[4] * cy + p2t[5] * cz;
                    cx = rx;
                    cy = ry;
                }
            }
            if (format == 0) {
                o0[o] = vx; o1[o] = vy; o2[o] = cx; o3[o] = cy;
            } else if (format == 1) {
                o0[o] = unorm8(vx * 0.5f + 0.5f); o1[o] = unorm8(vy * 0.5f + 0.5f);
                o2[o] = unorm8(cx * 0.5f + 0.5f); o3[o] = unorm8(cy * 0.5f + 0.5f);
            } else if (format == 2) {
                o0[o] = vx; o1[o] = vy;
            } else {
                o0[o] = unorm8(vx * 0.5f + 0.5f); o1[o] = unorm8(vy * 0.5f + 0.5f);
            }
        }
    free(nfx);
    free(nfy);
}

/* FP64 twin of or_sphere_frame_make + or_normals_sphere: the frame and the
 * positions in double, from double heights (the FP64 evaluation the errors of
 * the float path are stated against). */
void or_normals_sphere_f64(int W, const double *zm, int zm_pitch, double D, int level, int tx, int ty,
                           double *nx, double *ny, int out_pitch)
{
    double R = D / 2.0, sc = (double)(1 << level);
    double x0 = (double)tx / sc * D - R, x1 = (double)(tx + 1) / sc * D - R;
    double y0 = (double)ty / sc * D - R, y1 = (double)(ty + 1) / sc * D - R;
    double p[4][3] = {{x0, y0, R}, {x1, y0, R}, {x0, y1, R}, {x1, y1, R}};
    double v[4][3], L[4], vc[3] = {0, 0, 0}, C[3][4], N[3][4];
    for (int k = 0; k < 4; ++k) {
        v3_norm(p[k], v[k], &L[k]);
        for (int c = 0; c < 3; ++c) vc[c] += v[k][c];
    }
    for (int c = 0; c < 3; ++c) vc[c] *= 0.25;
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 4; ++k) {
            C[r][k] = v[k][r] * R - vc[r] * R;
            N[r][k] = v[k][r];
        }
    double pc[3] = {(x0 + x1) * 0.5, (y0 + y1) * 0.5, R}, uz[3], ux[3], uy[3];
    v3_norm(pc, uz, NULL);
    double t[3] = {uz[2], 0.0, -uz[0]};
    v3_norm(t, ux, NULL);
    uy[0] = uz[1] * ux[2] - uz[2] * ux[1];
    uy[1] = uz[2] * ux[0] - uz[0] * ux[2];
    uy[2] = uz[0] * ux[1] - uz[1] * ux[0];
    double size = D / sc, e0 = R / 32.0, e1 = R / 64.0;
    double sm = (size - e0) / (e1 - e0);
    sm = sm < 0.0 ? 0.0 : (sm > 1.0 ? 1.0 : sm);
    sm = sm * sm * (3.0 - 2.0 * sm);
    int n = W - 5;
    for (int q = 0; q <= n; ++q)
        for (int pp = 0; pp <= n; ++pp) {
            double P[4][3];
            const int du[4] = {-1, 1, 0, 0}, dv[4] = {0, 0, -1, 1};
            for (int m = 0; m < 4; ++m) {
                double u = (double)(pp + du[m]) / n, vv = (double)(q + dv[m]) / n;
                double al[4] = {(1 - u) * (1 - vv), u * (1 - vv), (1 - u) * vv, u * vv};
                double d = 0.0, ap[4], up[3], cp[3];
                for (int k = 0; k < 4; ++k) d += al[k] * L[k];
                for (int k = 0; k < 4; ++k) ap[k] = al[k] * L[k] / d;
                for (int r = 0; r < 3; ++r) {
                    up[r] = cp[r] = 0.0;
                    for (int k = 0; k < 4; ++k) {
                        up[r] += N[r][k] * ap[k];
                        cp[r] += C[r][k] * ap[k];
                    }
                }
                double len = sqrt(up[0] * up[0] + up[1] * up[1] + up[2] * up[2]);
                double kk = len * (1.0 - sm) + sm;
                double h = zm[(pp + 2 + du[m]) + (size_t)(q + 2 + dv[m]) * zm_pitch];
                double hp = (h + R * (1.0 - kk)) / kk;
                for (int r = 0; r < 3; ++r) P[m][r] = cp[r] + hp * up[r];
            }
            double a[3], b[3], cr[3];
            for (int r = 0; r < 3; ++r) {
                a[r] = P[1][r] - P[0][r];
                b[r] = P[3][r] - P[2][r];
            }
            cr[0] = a[1] * b[2] - a[2] * b[1];
            cr[1] = a[2] * b[0] - a[0] * b[2];
            cr[2] = a[0] * b[1] - a[1] * b[0];
            double inv = 1.0 / sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
            size_t o = pp + (size_t)q * out_pitch;
            nx[o] = (ux[0] * cr[0] + ux[1] * cr[1] + ux[2] * cr[2]) * inv;
            ny[o] = (uy[0] * cr[0] + uy[1] * cr[1] + uy[2] * cr[2]) * inv;
        }
}

/* ---- batch runner for the timed CPU baseline ------------------------------ */
typedef struct {
    const or_job *jobs;
    int begin, end;
    atomic_int *next;  /* shared job counter: threads take jobs one at a time */
} or_span;

static void run_one(const or_job *b)
{
    or_elev_tile t;
    memset(&t, 0, sizeof t);
    t.W = b->W; t.level = b->level; t.tx = b->tx; t.ty = b->ty;
    t.parent_zf = b->parent_zf; t.parent_zm = b->parent_zm; t.parent_pitch = b->parent_pitch;
    t.residual = b->residual; t.res_pitch = b->res_pitch; t.rx = b->rx; t.ry = b->ry; t.rscale = b->rscale;
    t.noise = b->noise; t.noise_rot = b->noise_rot; t.noise_amp = b->noise_amp;
    t.grid_g = (b->W - 5) / 24;
    t.out_zf = b->out_zf; t.out_zc = b->out_zc; t.out_zm = b->out_zm; t.out_pitch = b->out_pitch;
    or_elevation_tile(&t);
    or_normals_flat(b->W, b->out_zm, b->out_pitch, b->tile_meters, 2, b->out_nx, b->out_ny, b->nrm_pitch);
}

static void *run_span(void *arg)
{
    or_span *s = (or_span *)arg;
    if (!s->next) {
        for (int k = s->begin; k < s->end; ++k) run_one(&s->jobs[k]);
        return NULL;
    }
    /* jobs of different tile widths differ ~4x in work: taking them one at a time
     * keeps every thread busy until the batch is done */
    for (;;) {
        const int k = atomic_fetch_add(s->next, 1);
        if (k >= s->end) break;
        run_one(&s->jobs[k]);
    }
    return NULL;
}

void or_run_jobs(const or_job *jobs, int n, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (nthreads == 1) {
        or_span s = {jobs, 0, n, NULL};
        run_span(&s);
        return;
    }
    pthread_t th[256];
    or_span sp[256];
    atomic_int next;
    atomic_init(&next, 0);
    for (int k = 0; k < nthreads; ++k) {
        sp[k].jobs = jobs;
        sp[k].begin = 0;
        sp[k].end = n;
        sp[k].next = &next;
        pthread_create(&th[k], NULL, run_span, &sp[k]);
    }
    for (int k = 0; k < nthreads; ++k) pthread_join(th[k], NULL);
}

/* ---- preprocess ------------------------------------------------------------ */
/* HeightMipmap::computeResidual / encodeResidual / computeApproxTile
 * (HeightMipmap.cpp:449-559) for one tile of width W (pitch W). */
void or_compute_residual(int W, int tx, int ty, const float *parent_approx,
                         const float *fine, float *residual_q, int16_t *encoded, float *approx)
{
    int n = W - 5;
    int px = 1 + (tx % 2) * n / 2, py = 1 + (ty % 2) * n / 2;
    for (int j = 0; j < W; ++j)
        for (int i = 0; i < W; ++i) {
            float z = upsample_sample(parent_approx, W, i, j, px, py);
            int o = i + j * W;
            float diff = fine[o] - z;
            short q = (short)roundf(diff);
            if (encoded) encoded[o] = q;
            if (residual_q) residual_q[o] = (float)q;
            if (approx) approx[o] = z + (float)q;
        }
}

/* ResidualProducer::upsample (ResidualProducer.cpp:342-384): child of a tile of
 * `tilesize` intervals at quadrant (tx % 2, ty % 2); both arrays have pitch n. */
void or_residual_upsample(int n, int tilesize, int tx, int ty, const float *parent, float *out)
{
    int px = 1 + (tx % 2) * tilesize / 2, py = 1 + (ty % 2) * tilesize / 2;
    for (int j = 0; j <= tilesize + 4; ++j)
        for (int i = 0; i <= tilesize + 4; ++i)
            out[i + (size_t)j * n] = upsample_sample(parent, n, i, j, px, py);
}

/* ---------------------------------------------------------------- synthetic residuals
 * The product's synthetic residual source (tp_residual_producer_set_synthetic):
 * per tile key h(seed ^ h(level ^ h(tx ^ h(ty)))), per sample s = i + j W the
 * twelve 16-bit halves of h(key + 6 s + m), m = 0..5, as (k + 0.5) / 65536; their
 * sum minus 6 (exact in float) times sigma. */
static uint32_t syn_hash(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

void or_synthetic_residual(uint32_t seed, int level, int tx, int ty, float sigma, int W, float *out)
{
    const uint32_t key = syn_hash(seed ^ syn_hash((uint32_t)level ^ syn_hash((uint32_t)tx ^ syn_hash((uint32_t)ty))));
    for (int j = 0; j < W; ++j)
        for (int i = 0; i < W; ++i) {
            const uint32_t s = (uint32_t)(i + j * W);
            float acc = 0.0f;
            for (uint32_t m = 0; m < 6; ++m) {
                const uint32_t h = syn_hash(key + 6u * s + m);
                acc += ((float)(h >> 16) + 0.5f) / 65536.0f;
                acc += ((float)(h & 0xffffu) + 0.5f) / 65536.0f;
            }
            out[i + j * W] = (acc - 6.0f) * sigma;
        }
}

/* ---------------------------------------------------------------- deep-level pairs
 * The product's tp_fbm_pairs for one tile: the field (or_fbm_f64) on the parent's
 * and the child's windows, up = the stencil of the (fp32) parent, res = child - up
 * formed in double and rounded once. */
void or_fbm_pair(int octaves, int base_cells, float amplitude, uint32_t seed, int ts, int level, int tx, int ty,
                 float *up, float *res, float *fine)
{
    const int W = ts + 5;
    const double norm = (double)amplitude / (2.0 - ldexp(1.0, 1 - octaves));
    const double ps = 1.0 / ((double)ts * (double)(1u << (level - 1))), cs = 1.0 / ((double)ts * (double)(1u << level));
    float *parent = (float *)malloc(sizeof(float) * W * W);
    for (int j = 0; j < W; ++j)
        for (int i = 0; i < W; ++i)
            parent[i + j * W] = (float)or_fbm_f64((double)(i + ts * (tx / 2) - 2) * ps, (double)(j + ts * (ty / 2) - 2) * ps,
                                                  octaves, base_cells, norm, seed);
    const int px = 1 + (tx % 2) * ts / 2, py = 1 + (ty % 2) * ts / 2;
    for (int j = 0; j < W; ++j)
        for (int i = 0; i < W; ++i) {
            const double f = or_fbm_f64((double)(i + ts * tx - 2) * cs, (double)(j + ts * ty - 2) * cs, octaves,
                                        base_cells, norm, seed);
            const float z = upsample_sample(parent, W, i, j, px, py);
            up[i + j * W] = z;
            res[i + j * W] = (float)(f - (double)z);
            if (fine) fine[i + j * W] = (float)f;
        }
    free(parent);
}
