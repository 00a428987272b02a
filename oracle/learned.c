/* Test infrastructure: CPU restatement of (1) the device preprocess's procedural
 * height field and level tiles, and (2) the learned residual predictor's forward
 * and backward passes.  The product's CUDA kernels are checked against these;
 * nothing here is linked into the product.
 *
 * (1) follows HeightMipmap::getTile / AbstractTileCache::getTileHeight
 * (HeightMipmap.cpp:399-407, AbstractTileCache.cpp:73-92): level samples are base
 * samples at stride 2^(max_level - level), coordinates clamped to the level.
 *
 * (2) has no reference counterpart (the reference stores residuals).  Two modes:
 * emulate = 1 rounds to bf16 where the GPU stores bf16 (inputs, weights, saved
 * pre-activations, activations, pre-activation gradients) and evaluates the
 * element-wise math in float, accumulating sums in double; emulate = 0 computes
 * everything in double with no rounding, for finite-difference checks of the
 * backward formulas. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* ------------------------------------------------------------ height field */
static float lattice(uint32_t x, uint32_t y, uint32_t z)
{
    uint32_t h = x * 0x8da6b343u ^ y * 0xd8163841u ^ z * 0xcb1ab31fu;
    h ^= h >> 16;
    h *= 0x7feb352du;
    h ^= h >> 15;
    h *= 0x846ca68bu;
    h ^= h >> 16;
    return (float)(h >> 8) * (1.0f / 8388608.0f) - 1.0f;
}

/* The same field in double precision at domain point (u, v), in metres (the
 * product's windowed sampler for deep levels; each operation rounded alone). */
double or_fbm_f64(double u, double v, int octaves, int base_cells, double norm, uint32_t seed)
{
    double sum = 0.0, amp = 1.0;
    for (int o = 0; o < octaves; ++o) {
        const double cells = (double)(base_cells << o);
        const double gx = u * cells, gy = v * cells;
        const double fx0 = floor(gx), fy0 = floor(gy);
        const uint32_t ix = (uint32_t)(long long)fx0, iy = (uint32_t)(long long)fy0, oz = seed * 977u + (uint32_t)o;
        double fx = gx - fx0, fy = gy - fy0;
        fx = (fx * fx) * (3.0 - 2.0 * fx);
        fy = (fy * fy) * (3.0 - 2.0 * fy);
        const double v00 = lattice(ix, iy, oz), v10 = lattice(ix + 1, iy, oz);
        const double v01 = lattice(ix, iy + 1, oz), v11 = lattice(ix + 1, iy + 1, oz);
        const double a0 = v00 + (v10 - v00) * fx;
        const double a1 = v01 + (v11 - v01) * fx;
        sum = sum + amp * (a0 + (a1 - a0) * fy);
        amp *= 0.5;
    }
    return sum * norm;
}

void or_fbm_heights(int size, int octaves, int base_cells, float amplitude, float quantum, uint32_t seed, int16_t *out)
{
    const float norm = (float)((double)amplitude / (2.0 - ldexp(1.0, 1 - octaves)));
    for (int y = 0; y < size; ++y)
        for (int x = 0; x < size; ++x) {
            const float u = (float)x / (float)(size - 1), v = (float)y / (float)(size - 1);
            float sum = 0.0f, amp = 1.0f;
            for (int o = 0; o < octaves; ++o) {
                const float cells = (float)(base_cells << o);
                const float gx = u * cells, gy = v * cells;
                const float fx0 = floorf(gx), fy0 = floorf(gy);
                const uint32_t ix = (uint32_t)(int)fx0, iy = (uint32_t)(int)fy0, oz = seed * 977u + (uint32_t)o;
                float fx = gx - fx0, fy = gy - fy0;
                fx = (fx * fx) * (3.0f - 2.0f * fx);
                fy = (fy * fy) * (3.0f - 2.0f * fy);
                const float v00 = lattice(ix, iy, oz), v10 = lattice(ix + 1, iy, oz);
                const float v01 = lattice(ix, iy + 1, oz), v11 = lattice(ix + 1, iy + 1, oz);
                const float a0 = v00 + (v10 - v00) * fx;
                const float a1 = v01 + (v11 - v01) * fx;
                sum = sum + amp * (a0 + (a1 - a0) * fy);
                amp *= 0.5f;
            }
            float q = rintf((sum * norm) / quantum);
            q = fminf(fmaxf(q, -32767.0f), 32767.0f);
            out[(size_t)y * size + x] = (int16_t)q;
        }
}

void or_level_tile(const int16_t *base, int ts, int max_level, int level, int tx, int ty, float scale, float *out)
{
    const int W = ts + 5, width = ts << level, shift = max_level - level, base_size = (ts << max_level) + 1;
    for (int j = 0; j < W; ++j)
        for (int i = 0; i < W; ++i) {
            int x = i + ts * tx - 2, y = j + ts * ty - 2;
            x = x < 0 ? 0 : (x > width ? width : x);
            y = y < 0 ? 0 : (y > width ? width : y);
            out[j * W + i] = (float)base[((size_t)y << shift) * base_size + ((size_t)x << shift)] / scale;
        }
}

/* ------------------------------------------------------------ learned net */
#define NL 5
#define NLEV 24
static const int CIN[NL] = {16, 32, 32, 32, 32};
static const int COUT[NL] = {32, 32, 32, 32, 16};

static void offsets(int *woff, int *boff, int *emb, int *total)
{
    int off = 0;
    for (int l = 0; l < NL; ++l) {
        woff[l] = off;
        off += COUT[l] * 9 * CIN[l];
        boff[l] = off;
        off += COUT[l];
    }
    *emb = off;
    off += NLEV * COUT[0];
    *total = off;
}

int or_learned_param_count(void)
{
    int w[NL], b[NL], e, t;
    offsets(w, b, &e, &t);
    return t;
}

static float bf16r(float x)
{
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;
    u += 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
    memcpy(&x, &u, 4);
    return x;
}

/* GELU in its tanh form: 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))) */
static double gelu_d(double z)
{
    return 0.5 * z * (1.0 + tanh(0.7978845608028654 * (z + 0.044715 * z * z * z)));
}
static double gelu_grad_d(double z)
{
    const double t = tanh(0.7978845608028654 * (z + 0.044715 * z * z * z));
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * 0.7978845608028654 * (1.0 + 0.134145 * z * z);
}
static float gelu_f(float z)
{
    const float t = tanhf(0.7978845608028654f * (z + 0.044715f * z * z * z));
    return 0.5f * z * (1.0f + t);
}
static float gelu_grad_f(float z)
{
    const float t = tanhf(0.7978845608028654f * (z + 0.044715f * z * z * z));
    return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * 0.7978845608028654f * (1.0f + 0.134145f * z * z);
}

/* Z[img][p][co] = sum_{tap, ci} X[img][p + tap][ci] w[co][tap][ci], zero outside the image */
static void conv_fwd(int W, int n, const double *X, int cin, const double *w, int cout, double *Z)
{
    for (int img = 0; img < n; ++img)
        for (int y = 0; y < W; ++y)
            for (int x = 0; x < W; ++x) {
                double *z = Z + (((size_t)img * W + y) * W + x) * cout;
                for (int co = 0; co < cout; ++co) z[co] = 0.0;
                for (int t = 0; t < 9; ++t) {
                    const int yy = y + t / 3 - 1, xx = x + t % 3 - 1;
                    if (yy < 0 || yy >= W || xx < 0 || xx >= W) continue;
                    const double *xi = X + (((size_t)img * W + yy) * W + xx) * cin;
                    for (int co = 0; co < cout; ++co) {
                        const double *wr = w + ((size_t)co * 9 + t) * cin;
                        double s = 0.0;
                        for (int ci = 0; ci < cin; ++ci) s += xi[ci] * wr[ci];
                        z[co] += s;
                    }
                }
            }
}

/* dX[img][p][ci] = sum_{tap, co} dZ[img][p - tap][co] w[co][tap][ci] */
static void conv_bwd_data(int W, int n, const double *dZ, int cout, const double *w, int cin, double *dX)
{
    memset(dX, 0, sizeof(double) * (size_t)n * W * W * cin);
    for (int img = 0; img < n; ++img)
        for (int y = 0; y < W; ++y)
            for (int x = 0; x < W; ++x) {
                const double *dz = dZ + (((size_t)img * W + y) * W + x) * cout;
                for (int t = 0; t < 9; ++t) {
                    const int yy = y + t / 3 - 1, xx = x + t % 3 - 1;
                    if (yy < 0 || yy >= W || xx < 0 || xx >= W) continue;
                    double *dx = dX + (((size_t)img * W + yy) * W + xx) * cin;
                    for (int co = 0; co < cout; ++co) {
                        if (dz[co] == 0.0) continue;
                        const double *wr = w + ((size_t)co * 9 + t) * cin;
                        for (int ci = 0; ci < cin; ++ci) dx[ci] += dz[co] * wr[ci];
                    }
                }
            }
}

/* gw[co][tap][ci] += sum_p dZ[p][co] X[p + tap][ci]; gb[co] += sum_p dZ[p][co];
 * gemb[level(img)][co] += the same per image (when gemb) */
static void conv_bwd_weight(int W, int n, const double *X, int cin, const double *dZ, int cout, const int *levels,
                            double *gw, double *gb, double *gemb)
{
    for (int img = 0; img < n; ++img)
        for (int y = 0; y < W; ++y)
            for (int x = 0; x < W; ++x) {
                const double *dz = dZ + (((size_t)img * W + y) * W + x) * cout;
                for (int co = 0; co < cout; ++co) {
                    gb[co] += dz[co];
                    if (gemb) gemb[(size_t)levels[img] * cout + co] += dz[co];
                }
                for (int t = 0; t < 9; ++t) {
                    const int yy = y + t / 3 - 1, xx = x + t % 3 - 1;
                    if (yy < 0 || yy >= W || xx < 0 || xx >= W) continue;
                    const double *xi = X + (((size_t)img * W + yy) * W + xx) * cin;
                    for (int co = 0; co < cout; ++co) {
                        if (dz[co] == 0.0) continue;
                        double *g = gw + ((size_t)co * 9 + t) * cin;
                        for (int ci = 0; ci < cin; ++ci) g[ci] += dz[co] * xi[ci];
                    }
                }
            }
}

double or_learned_loss_grad(int W, int n, const float *params, const float *up, const float *target, const int *levels,
                            const float *sigma_in, const float *sigma_out, int emulate, float *pred_out, double *grad)
{
    int woff[NL], boff[NL], emb, total;
    offsets(woff, boff, &emb, &total);
    const size_t np = (size_t)W * W, P = np * n;
    double *w[NL];
    for (int l = 0; l < NL; ++l) {
        const size_t cnt = (size_t)COUT[l] * 9 * CIN[l];
        w[l] = (double *)malloc(sizeof(double) * cnt);
        for (size_t i = 0; i < cnt; ++i) w[l][i] = emulate ? (double)bf16r(params[woff[l] + i]) : (double)params[woff[l] + i];
    }
    double *X[NL], *Zs[NL - 1];
    for (int l = 0; l < NL; ++l) X[l] = (double *)calloc(P * CIN[l], sizeof(double));
    for (int l = 0; l < NL - 1; ++l) Zs[l] = (double *)calloc(P * COUT[l], sizeof(double));
    double *Zt = (double *)malloc(sizeof(double) * P * 32);
    double *pred = (double *)malloc(sizeof(double) * P);
    /* input channels: height (minus the tile mean, over sigma_in), x parity, y parity, 1,
     * the second differences u[x-1] + u[x+1] - 2 u[x] along x and y (0 on the edge
     * columns / rows) over sigma_out, in float before the bf16 rounding */
    for (int img = 0; img < n; ++img) {
        const float *u = up + img * np;
        double s = 0.0;
        for (size_t i = 0; i < np; ++i) s += u[i];
        const int lev = levels[img];
        for (size_t i = 0; i < np; ++i) {
            const int y = (int)(i / W), x = (int)(i % W);
            const int ex = x > 0 && x < W - 1, ey = y > 0 && y < W - 1;
            double *xi = X[0] + (img * np + i) * 16;
            if (emulate) {
                const float mean = (float)(s / (double)np), inv = 1.0f / sigma_in[lev], inv2 = 1.0f / sigma_out[lev];
                xi[0] = bf16r((u[i] - mean) * inv);
                const float d2x = ex ? (u[i - 1] + u[i + 1]) - 2.0f * u[i] : 0.0f;
                const float d2y = ey ? (u[i - W] + u[i + W]) - 2.0f * u[i] : 0.0f;
                xi[4] = bf16r(d2x * inv2);
                xi[5] = bf16r(d2y * inv2);
            } else {
                xi[0] = ((double)u[i] - s / (double)np) / (double)sigma_in[lev];
                xi[4] = ex ? ((double)u[i - 1] + u[i + 1] - 2.0 * u[i]) / (double)sigma_out[lev] : 0.0;
                xi[5] = ey ? ((double)u[i - W] + u[i + W] - 2.0 * u[i]) / (double)sigma_out[lev] : 0.0;
            }
            xi[1] = x & 1;
            xi[2] = y & 1;
            xi[3] = 1.0;
        }
    }
    for (int l = 0; l < NL; ++l) {
        const int cout = COUT[l];
        conv_fwd(W, n, X[l], CIN[l], w[l], cout, Zt);
        for (int img = 0; img < n; ++img)
            for (size_t i = 0; i < np; ++i) {
                double *z = Zt + (img * np + i) * cout;
                for (int co = 0; co < cout; ++co) {
                    const double add = (double)params[boff[l] + co] +
                                       (l == 0 ? (double)params[emb + (size_t)levels[img] * cout + co] : 0.0);
                    if (emulate) {
                        const float addf = params[boff[l] + co] + (l == 0 ? params[emb + (size_t)levels[img] * cout + co] : 0.0f);
                        const float zf = (float)z[co] + addf;
                        if (l < NL - 1) {
                            Zs[l][(img * np + i) * cout + co] = bf16r(zf);
                            X[l + 1][(img * np + i) * cout + co] = bf16r(gelu_f(zf));
                        } else if (co == 0) {
                            pred[img * np + i] = zf;
                        }
                    } else {
                        const double zd = z[co] + add;
                        if (l < NL - 1) {
                            Zs[l][(img * np + i) * cout + co] = zd;
                            X[l + 1][(img * np + i) * cout + co] = gelu_d(zd);
                        } else if (co == 0) {
                            pred[img * np + i] = zd;
                        }
                    }
                }
            }
    }
    if (pred_out)
        for (size_t i = 0; i < P; ++i) pred_out[i] = (float)pred[i];
    double loss = 0.0;
    double *dZ = (double *)calloc(P * 32, sizeof(double));
    double *dX = (double *)calloc(P * 32, sizeof(double));
    for (int img = 0; img < n; ++img)
        for (size_t i = 0; i < np; ++i) {
            const size_t k = img * np + i;
            double d;
            if (emulate) {
                const float t = target[k] / sigma_out[levels[img]];
                const float df = (float)pred[k] - t;
                d = df;
                dZ[k * 16] = bf16r(2.0f * df * (1.0f / (float)P));
            } else {
                d = pred[k] - (double)target[k] / (double)sigma_out[levels[img]];
                dZ[k * 16] = 2.0 * d / (double)P;
            }
            loss += d * d;
        }
    if (grad) {
        memset(grad, 0, sizeof(double) * total);
        for (int l = NL - 1; l >= 0; --l) {
            conv_bwd_weight(W, n, X[l], CIN[l], dZ, COUT[l], levels, grad + woff[l], grad + boff[l],
                            l == 0 ? grad + emb : NULL);
            if (l == 0) break;
            const int c = CIN[l];
            conv_bwd_data(W, n, dZ, COUT[l], w[l], c, dX);
            for (size_t k = 0; k < P * c; ++k) {
                const double z = Zs[l - 1][k];
                dZ[k] = emulate ? (double)bf16r((float)dX[k] * gelu_grad_f((float)z)) : dX[k] * gelu_grad_d(z);
            }
        }
    }
    for (int l = 0; l < NL; ++l) {
        free(w[l]);
        free(X[l]);
    }
    for (int l = 0; l < NL - 1; ++l) free(Zs[l]);
    free(Zt);
    free(pred);
    free(dZ);
    free(dX);
    return loss / (double)P;
}
