/*
 * CPU oracle of the ortho (colour) tile producer -- TEST INFRASTRUCTURE ONLY.
 * Build with -O2 -ffp-contract=off (oracle/build.py): every float operation is
 * rounded on its own, in the order written here.
 *
 * Follows, relative to the reference project root:
 *  - createOrthoNoise: src/terrain/sources/proland/ortho/OrthoProducer.cpp:26-122
 *  - the uniforms doCreateTile sets: OrthoProducer.cpp:292-382
 *  - the upsample fragment shader: src/terrain/examples/terrain3/upsampleOrthoShader.glsl
 *    (the demo copy, src/demo/shaders/ortho/upsampleOrthoShader.glsl, is the same
 *    arithmetic)
 *  - tile ids of the ortho .dat pyramids: OrthoCPUProducer.cpp:250-253
 *
 * Texel values are exact integers 0..255 (an 8-bit texel read as k / 255 and
 * scaled by 255 is taken to be k), and the framebuffer write of result / 255 is
 * clamp to [0, 1], times 255, rounded to the nearest integer with ties to even.
 */
#include "oracle.h"

#include <math.h>
#include <string.h>

void or_ortho_noise(int W, uint8_t *out)
{
    static const int layer_bits[6] = {0, 1, 3, 5, 7, 15};
    long centre = 1234567;   /* one sequence through the centres of all six layers */
    for (int nl = 0; nl < 6; ++nl) {
        uint8_t *n = out + (size_t)nl * W * W * 4;
        const int l = layer_bits[nl];
        long s;
        memset(n, 128, (size_t)W * W * 4);
#define PX(x, y, c) n[4 * ((size_t)(x) + (size_t)(y) * W) + (c)]
        /* bottom rows 2..3, mirrored into rows 1..0 */
        s = (l & 1) == 0 ? 7654321 : 5647381;
        for (int y = 2; y < 4; ++y)
            for (int x = 4; x < W - 4; ++x)
                for (int c = 0; c < 4; ++c) {
                    const int v = (int)(or_frandom(&s) * 255.0f);
                    PX(x, y, c) = (uint8_t)v;
                    PX(W - 1 - x, 3 - y, c) = (uint8_t)v;
                }
        /* right columns W-3, W-4, mirrored into W-2, W-1 */
        s = (l & 2) == 0 ? 7654321 : 5647381;
        for (int x = W - 3; x >= W - 4; --x)
            for (int y = 4; y < W - 4; ++y)
                for (int c = 0; c < 4; ++c) {
                    const int v = (int)(or_frandom(&s) * 255.0f);
                    PX(x, y, c) = (uint8_t)v;
                    PX(2 * W - 5 - x, W - 1 - y, c) = (uint8_t)v;
                }
        /* top rows W-2, W-1, mirrored into W-3, W-4 */
        s = (l & 4) == 0 ? 7654321 : 5647381;
        for (int y = W - 2; y < W; ++y)
            for (int x = 4; x < W - 4; ++x)
                for (int c = 0; c < 4; ++c) {
                    const int v = (int)(or_frandom(&s) * 255.0f);
                    PX(x, y, c) = (uint8_t)v;
                    PX(W - 1 - x, 2 * W - 5 - y, c) = (uint8_t)v;
                }
        /* left columns 1, 0, mirrored into 2, 3 */
        s = (l & 8) == 0 ? 7654321 : 5647381;
        for (int x = 1; x >= 0; --x)
            for (int y = 4; y < W - 4; ++y)
                for (int c = 0; c < 4; ++c) {
                    const int v = (int)(or_frandom(&s) * 255.0f);
                    PX(x, y, c) = (uint8_t)v;
                    PX(3 - x, W - 1 - y, c) = (uint8_t)v;
                }
        for (int y = 4; y < W - 4; ++y)
            for (int x = 4; x < W - 4; ++x)
                for (int c = 0; c < 4; ++c) PX(x, y, c) = (uint8_t)(int)(or_frandom(&centre) * 255.0f);
#undef PX
    }
}

int or_ortho_tile_id(int level, int tx, int ty)
{
    return tx + ty * (1 << level) + ((1 << (2 * level)) - 1) / 3;
}

static float smoothstep_f(float e0, float e1, float x)
{
    float t = (x - e0) / (e1 - e0);
    t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
    return t * t * (3.0f - 2.0f * t);
}

/* rgb_to_hsv of the shader, component by component */
static void rgb_to_hsv(const float *rgb, float *hsv)
{
    const float mn = fminf(rgb[0], fminf(rgb[1], rgb[2]));
    const float mx = fmaxf(rgb[0], fmaxf(rgb[1], rgb[2]));
    const float delta = mx - mn;
    hsv[0] = 0.0f;
    hsv[1] = 0.0f;
    hsv[2] = mx;
    if (delta != 0.0f) {
        hsv[1] = delta / mx;
        float d[3];
        for (int c = 0; c < 3; ++c) d[c] = ((mx - rgb[c]) / 6.0f + delta / 2.0f) / delta;
        if (rgb[0] == mx) hsv[0] = d[2] - d[1];
        else if (rgb[1] == mx) hsv[0] = (1.0f / 3.0f) + d[0] - d[2];
        else if (rgb[2] == mx) hsv[0] = (2.0f / 3.0f) + d[1] - d[0];
        if (hsv[0] < 0.0f) hsv[0] += 1.0f;
        if (hsv[0] > 1.0f) hsv[0] -= 1.0f;
    }
}

static void hsv_to_rgb(const float *hsv, float *rgb)
{
    rgb[0] = rgb[1] = rgb[2] = hsv[2];
    if (hsv[1] != 0.0f) {
        const float h = hsv[0] * 6.0f;
        const float i = floorf(h);
        const float v1 = hsv[2] * (1.0f - hsv[1]);
        const float v2 = hsv[2] * (1.0f - hsv[1] * (h - i));
        const float v3 = hsv[2] * (1.0f - hsv[1] * (1.0f - (h - i)));
        if (i == 0.0f) { rgb[0] = hsv[2]; rgb[1] = v3; rgb[2] = v1; }
        else if (i == 1.0f) { rgb[0] = v2; rgb[1] = hsv[2]; rgb[2] = v1; }
        else if (i == 2.0f) { rgb[0] = v1; rgb[1] = hsv[2]; rgb[2] = v3; }
        else if (i == 3.0f) { rgb[0] = v1; rgb[1] = v2; rgb[2] = hsv[2]; }
        else if (i == 4.0f) { rgb[0] = v3; rgb[1] = v1; rgb[2] = hsv[2]; }
        else { rgb[0] = hsv[2]; rgb[1] = v1; rgb[2] = v2; }
    }
}

static uint8_t to_unorm8(float result)
{
    float f = result / 255.0f;
    f = f < 0.0f ? 0.0f : (f > 1.0f ? 1.0f : f);
    return (uint8_t)(int)rintf(f * 255.0f);
}

void or_ortho_tile(const or_ortho_job *t)
{
    const int W = t->W, n = W - 4;
    /* noiseColor uniform (OrthoProducer.cpp:376-380): hsv mode scales alpha by scale */
    float nc[4];
    for (int c = 0; c < 4; ++c) {
        if (t->hsv) {
            const float m = c < 3 ? t->noise_amp : t->scale * t->noise_amp;
            nc[c] = t->noise_color[c] * m / 255.0f;
        } else {
            nc[c] = t->noise_color[c] * t->scale * t->noise_amp / 255.0f;
        }
    }
    const int has_parent = t->level > 0 && t->parent != NULL;
    const float rscale = t->residual ? t->scale : -1.0f;   /* residualOSH.w */
    const int dx = (t->tx % 2) * (n / 2), dy = (t->ty % 2) * (n / 2);
    static const float masks[4][4] = {{1, 3, 3, 9}, {3, 1, 9, 3}, {3, 9, 1, 3}, {9, 3, 3, 1}};
    for (int j = 0; j < W; ++j)
        for (int i = 0; i < W; ++i) {
            float r[4];
            for (int c = 0; c < 4; ++c) {
                if (t->residual) r[c] = (float)t->residual[4 * ((size_t)j * W + i) + c];
                else if (!has_parent) r[c] = t->root_color[c] * 255.0f;
                else r[c] = 128.0f;
            }
            if (has_parent) {
                const float *m = masks[(i % 2) + 2 * (j % 2)];
                const int px = (i + 1) / 2 + dx, py = (j + 1) / 2 + dy;
                const uint8_t *p0 = t->parent + 4 * ((size_t)py * W + px);
                const uint8_t *p2 = p0 + 4 * (size_t)W;
                for (int c = 0; c < 4; ++c) {
                    const float s = m[0] * (float)p0[c] + m[1] * (float)p0[4 + c] + m[2] * (float)p2[c] +
                                    m[3] * (float)p2[4 + c];
                    const float cc = floorf(s / 16.0f);
                    r[c] = (r[c] - 128.0f) * rscale + cc;
                }
            }
            /* noise texel of the rotated layer (NEAREST at texel centres) */
            int x, y;
            switch (t->noise_rot) {
            case 0: x = i; y = j; break;
            case 1: x = j; y = W - 1 - i; break;
            case 2: x = W - 1 - i; y = W - 1 - j; break;
            default: x = W - 1 - j; y = i; break;
            }
            const uint8_t *nz = t->noise + 4 * ((size_t)y * W + x);
            float nv[4];
            for (int c = 0; c < 4; ++c) nv[c] = (float)nz[c];
            float out[4];
            if (t->hsv) {
                float rgb[3], hsv[3];
                for (int c = 0; c < 3; ++c) rgb[c] = r[c] / 255.0f;
                rgb_to_hsv(rgb, hsv);
                const float k = 1.0f - smoothstep_f(0.4f, 0.8f, hsv[2]);
                for (int c = 0; c < 3; ++c) hsv[c] *= 1.0f + k * nc[c] * (nv[c] - 128.0f) / 255.0f;
                hsv[0] = hsv[0] - floorf(hsv[0]);
                hsv[1] = hsv[1] < 0.0f ? 0.0f : (hsv[1] > 1.0f ? 1.0f : hsv[1]);
                hsv[2] = hsv[2] < 0.0f ? 0.0f : (hsv[2] > 1.0f ? 1.0f : hsv[2]);
                hsv_to_rgb(hsv, rgb);
                for (int c = 0; c < 3; ++c) out[c] = rgb[c] * 255.0f;
                out[3] = nc[3] * (nv[3] - 128.0f) + r[3];
            } else {
                for (int c = 0; c < 4; ++c) out[c] = nc[c] * (nv[c] - 128.0f) + r[c];
            }
            uint8_t *o = t->out + 4 * ((size_t)j * W + i);
            for (int c = 0; c < 4; ++c) o[c] = to_unorm8(out[c]);
        }
}
