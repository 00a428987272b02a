// Learned residual predictor: a 5-layer 3x3 convolutional net (32 features, GELU)
// that maps an upsampled parent tile (plus a per-level embedding) to the residual
// tile the stencil leaves out.  BF16 activations and weights, FP32 accumulation in
// tensor memory, trained by the library's own forward/backward kernels.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace tp {
namespace learned {

constexpr int kLayers = 5;
constexpr int kCin[kLayers] = {16, 32, 32, 32, 32};    // layer 0 input: 6 used channels, padded to 16
constexpr int kCout[kLayers] = {32, 32, 32, 32, 16};   // last layer: 1 used channel, padded to 16
constexpr int kLevels = 24;                            // rows of the level embedding / sigma tables
// height, x parity, y parity, ones, and the second differences of the upsampled
// tile along x and y over the level's output sigma (computed in fp32 before the bf16
// rounding: they keep the curvature that a bf16 height loses at deep levels)
constexpr int kInputChannels = 6;

// Pixel blocks of the convolutions: 8 columns x 16 rows = one 128-row MMA tile.
constexpr int kBlockX = 8, kBlockY = 16;

// One convolution launch.  Activations are NHWC bf16 images of (W+2)^2 pixels with
// a zero border of one pixel, read through a TMA tensor map.
struct ConvLaunch {
    int W, nimg, tiles_x, tiles_y;
    const uint8_t *wpack;        // packed B operand (weights), 9 * Cin * Cout bf16
    const float *bias;           // [Cout]
    const float *emb;            // [kLevels][Cout] level embedding (layer 0) or null
    const int *level;            // [nimg] level of each image (device)
    __nv_bfloat16 *out;          // mode 0: activation; mode 2: gradient of the previous pre-activation
    __nv_bfloat16 *zsave;        // mode 0: pre-activation (for the backward pass) or null
    const __nv_bfloat16 *zprev;  // mode 2: the previous layer's saved pre-activation
    float *out_f32;              // mode 1: [nimg][W][W] output channel 0
    int *status;
    // mode 3 (first layer of an inference pass): the input channels made from the
    // upsampled parent tiles instead of read from an activation image
    const float *up;             // [nimg][W][W]
    const float *mean;           // [nimg] tile means
    const float *sigma_in;       // [kLevels]
    const float *sigma_out;      // [kLevels] (scale of the second-difference channels)
};

// Two consecutive convolutions of an inference pass in one launch (the first 16 -> 32
// with its input made from the upsampled tiles, or a hidden 32 -> 32 reading an
// activation image, then a hidden 32 -> 32): the first layer's outputs on the block's
// 10 x 18 halo stay in shared memory as the second layer's operand.
struct FusedLaunch {
    int W, nimg, tiles_x, tiles_y;
    const uint8_t *wpack_a, *wpack_b;  // packed B operands of the two layers
    const float *bias_a, *bias_b;      // [32] each
    const float *emb;                  // [kLevels][32] level embedding of the first layer, or null
    const int *level;                  // [nimg]
    __nv_bfloat16 *out;                // the second layer's activation image
    int *status;
    const float *up, *mean, *sigma_in, *sigma_out;  // first-layer input (first pair only)
};

// Weight gradient of one layer over a batch: dW[co][tap][ci] += sum_p dZ[p][co] X[p + tap][ci].
struct WgradLaunch {
    int W, nimg, tiles_x, tiles_y;
    float *gw;        // [Cout][9][Cin]
    float *gb;        // [Cout]
    float *gemb;      // [kLevels][Cout] or null
    const int *level; // [nimg]
    int *status;
};

enum ConvMode { kHidden = 0, kLast = 1, kBackData = 2, kFirst = 3 };

int launch_conv(int cin, int cout, int mode, const ConvLaunch &a, const CUtensorMap *halo, cudaStream_t s);
int launch_wgrad(int cin, int cout, const WgradLaunch &a, const CUtensorMap *xbox, const CUtensorMap *zbox,
                 cudaStream_t s);
int encode_act_map(void *base, int W, int channels, int nimg, int box_x, int box_y, CUtensorMap *out);
// first: the pair starting at layer 0 (input from the upsampled tiles); else a pair of
// hidden layers whose input is read through `wide` (12 x 20 pixel boxes of 32 channels)
int launch_fused(bool first, const FusedLaunch &a, const CUtensorMap *wide, cudaStream_t s);
// A fused pair's output block is 8 x 14 pixels (its second layer's MMA tile keeps the 8 x 16
// shape, two rows unused), so that the first layer's 10 x 16 region is covered exactly by two
// 8 x 16 MMA tiles at columns 0 and 2; its input halo is 12 x 18.
constexpr int kFusedBlockY = kBlockY - 2;
constexpr int kWideX = kBlockX + 4, kWideY = kFusedBlockY + 4;

// small kernels
void launch_pack(const float *w, int cin, int cout, uint8_t *fwd, uint8_t *bwd, cudaStream_t s);
void launch_prep(const float *up, const int *level, const float *sigma_in, const float *sigma_out, int W, int nimg,
                 __nv_bfloat16 *x0, cudaStream_t s);
// Per-tile means of the upsampled parents (the same sums as launch_prep's).
void launch_means(const float *up, int W, int nimg, float *mean, cudaStream_t s);
void launch_loss(const float *pred, const float *target, const int *level, const float *sigma_out, int W, int nimg,
                 __nv_bfloat16 *dz, float *loss, cudaStream_t s);
void launch_adam(float *p, const float *g, float *m, float *v, const float *mask, int n, float lr, float b1, float b2,
                 float eps, int step, cudaStream_t s);
void launch_scale_out(const float *pred, const int *level, const float *sigma_out, int W, int nimg, float *out,
                      cudaStream_t s);
void launch_gather(const float *up, const float *res, const int *src, const int *dihedral, int W, int n, float *up_out,
                   float *res_out, cudaStream_t s);
void launch_upsample(const float *elev, int pitch, long long plane_stride, long long slot_stride, const int *parent_slot,
                     const int *tx, const int *ty, int W, int n, float *up, cudaStream_t s);
void launch_store_residuals(const float *pred, const int *level, const float *sigma_out, int W, int n, float *res,
                            int pitch, long long slot_stride, const int *slots, cudaStream_t s);

}  // namespace learned
}  // namespace tp
