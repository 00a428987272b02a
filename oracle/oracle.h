/*
 * CPU oracle for the terrain tile-production path -- TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the arithmetic of Proland 4.0's elevation,
 * residual and normal producers.  It is what the CUDA product is compared
 * against; the product never links, loads or calls it.  Only the test-suite,
 * the smoke check and the CPU-baseline leg of the benchmark use it.
 *
 * Each function cites the reference file:line it follows (paths relative to the
 * reference project root).  Compile with -ffp-contract=off so that every float
 * operation is rounded on its own, exactly as written: the CUDA kernels follow
 * the same operation order with explicitly rounded intrinsics, which makes the
 * elevation outputs bit-identical on both sides.
 *
 * Parity pins: the stencil, residual addressing, int16 residual decode and tile
 * ids are pinned by the reference's DEM.dat fixtures and by mathematical known
 * answers (tests/test_oracle_*.py).  Noise-layer selection, zc/flip and normals
 * have no reference fixture: for those the oracle is a restatement only.
 */
#ifndef PROLAND_ORACLE_H
#define PROLAND_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- LCG, noise table, Perlin noise sign (math/noise.h:50-68, noise.cpp:68-165) ---- */
long  or_lrandom(long *seed);
float or_frandom(long *seed);
float or_half_round(float x);                 /* float -> IEEE half (RNE) -> float */
void  or_dem_noise(int W, float *out);        /* 6*W*W fp16-rounded values (ElevationProducer.cpp:50-133) */
float or_cnoise2(float x, float y);           /* noise.cpp:118-165 with period 0 */
void  or_noise_select(int face, int level, int tx, int ty, int *rot, int *layer); /* ElevationProducer.cpp:347-374 */

/* ---- per-tile parameters of one elevation tile ---- */
typedef struct {
    int W;               /* tile width incl. 2-sample borders on each side: n + 5 */
    int level;           /* 0: no parent */
    int tx, ty;          /* quadtree coordinates */
    const float *parent_zf;  /* parent zf plane (W x W, pitch parent_pitch); unused at level 0 */
    const float *parent_zm;  /* parent zm plane */
    int parent_pitch;
    const float *residual;   /* residual tile (Wr x Wr, pitch res_pitch) or NULL */
    int res_pitch;
    int rx, ry;              /* residual sub-window origin: (tx % mod) * n, (ty % mod) * n */
    float rscale;            /* residualOSH.w */
    const float *noise;      /* one noise layer (W x W, fp16-rounded) or NULL */
    int noise_rot;           /* 0..3 */
    float noise_amp;         /* noiseAmp[level] */
    int noise_mode;          /* 0: |amp| N (terrain1 shader), 1: slope/curvature modulated (demo shader) */
    float meters_per_sample; /* tileWSDF.y, demo noise mode only */
    int grid_g;              /* tileWSDF.z = n / gridSize */
    int flip;                /* tileWSDF.w */
    int no_clamp;            /* NO_CLAMP: zm = zf */
    float *out_zf, *out_zc, *out_zm;
    int out_pitch;
} or_elev_tile;

/* Full elevation tile (zf, zc, zm): upsampleShader.glsl main() semantics with the
 * stencil evaluated in CPUElevationProducer.cpp:202-245 order. */
void or_elevation_tile(const or_elev_tile *t);
/* FP64 evaluation of the same definition (outputs as double, pitch out_pitch). */
void or_elevation_tile_f64(const or_elev_tile *t, double *zf, double *zc, double *zm);
/* CPUElevationProducer::doCreateTile (CPUElevationProducer.cpp:156-248): zf = z + r only. */
void or_cpu_elevation_tile(int W, int level, int tx, int ty,
                           const float *parent, int parent_pitch,
                           const float *residual, int res_pitch, int rx, int ry,
                           float *out, int out_pitch);

/* ---- normals ---- */
/* Flat normals, (W-4)^2 samples from the zm plane (terrain1/normalShader.glsl:52-74,
 * NormalProducer.cpp:274-283).  tile_meters = rootQuadSize / 2^level.
 * format 2: two signed fp32 planes; format 3: RG8 unsigned (values written as floats 0..255). */
void or_normals_flat(int W, const float *zm, int zm_pitch, float tile_meters,
                     int format, float *nx, float *ny, int out_pitch);
/* Reporting only: the normals with the GL path's LINEAR fetches at +0.25-texel
 * offsets (NormalProducer.cpp:210-213; see oracle.c). */
void or_normals_flat_gl_linear(int W, const float *zm, int zm_pitch, float tile_meters, float *nx, float *ny,
                               int out_pitch);
void or_normals_flat_f64(int W, const double *zm, int zm_pitch, double tile_meters,
                         double *nx, double *ny, int out_pitch);

/* Spherical-deformation frames of one tile (NormalProducer.cpp:215-273), FP64 on the
 * host and cast to float as the reference uploads them.  Layout of the 44 floats:
 * C[16] (row-major 4x4), N[16] (row-major), L[4], W2T[9] (row-major 3x3), R, tileMeters... */
typedef struct {
    float C[16];
    float N[16];
    float L[4];
    float W2T[9];
    float R;          /* deform.w */
    float size;       /* deform.z = D / 2^level */
} or_sphere_frame;
void or_sphere_frame_make(double rootQuadSize, int level, int tx, int ty, or_sphere_frame *f);
/* Sphere normals (terrain2/normalShader.glsl:56-89). */
void or_normals_sphere(int W, const float *zm, int zm_pitch, const or_sphere_frame *f,
                       float *nx, float *ny, int out_pitch);

/* ---- batch helpers for the timed CPU baseline ---- */
typedef struct {
    int W, level, tx, ty;
    const float *parent_zf, *parent_zm; int parent_pitch;
    const float *residual; int res_pitch; int rx, ry; float rscale;
    const float *noise; int noise_rot; float noise_amp;
    float tile_meters;
    float *out_zf, *out_zc, *out_zm; int out_pitch;
    float *out_nx, *out_ny; int nrm_pitch;
} or_job;
/* Elevation + flat normals for n jobs on nthreads host threads (grid g = n/24). */
void or_run_jobs(const or_job *jobs, int n, int nthreads);

/* ---- preprocess (HeightMipmap.cpp:449-559) ---- */
/* residual = fine - upsample(parentApprox); encoded = short(roundf(residual));
 * approx = upsample + encoded.  Tile is W x W with pitch W. */
void or_compute_residual(int W, int tx, int ty, const float *parent_approx,
                         const float *fine, float *residual_q, int16_t *encoded, float *approx);

/* ResidualProducer::upsample for the small tiles below the pyramid's minLevel. */
void or_residual_upsample(int n, int tilesize, int tx, int ty, const float *parent, float *out);

void or_normals_sphere_f64(int W, const double *zm, int zm_pitch, double D, int level, int tx, int ty,
                           double *nx, double *ny, int out_pitch);

void or_parent_to_tangent(double D, int level, int tx, int ty, float *p2t);
void or_normals_full(int W, const float *zm, int zm_pitch, float tile_meters, const or_sphere_frame *f,
                     const float *p2t, int format, int grid_mesh, int tx, int ty, const float *pnx, const float *pny,
                     int ppitch, float *o0, float *o1, float *o2, float *o3, int out_pitch);

/* ---- learned.c: device preprocess height field, level tiles, learned net ---- */
/* the product's synthetic residual tile (sum of twelve 16-bit uniforms - 6) x sigma */
void or_synthetic_residual(uint32_t seed, int level, int tx, int ty, float sigma, int W, float *out);
/* the fBm in double precision at (u, v), metres; norm = amplitude / (2 - 2^(1 - octaves)) */
double or_fbm_f64(double u, double v, int octaves, int base_cells, double norm, uint32_t seed);
/* one (upsampled parent, residual) pair of the field at any level (tp_fbm_pairs) */
void or_fbm_pair(int octaves, int base_cells, float amplitude, uint32_t seed, int ts, int level, int tx, int ty,
                 float *up, float *res, float *fine);
void or_fbm_heights(int size, int octaves, int base_cells, float amplitude, float quantum, uint32_t seed, int16_t *out);
void or_level_tile(const int16_t *base, int ts, int max_level, int level, int tx, int ty, float scale, float *out);
int or_learned_param_count(void);
double or_learned_loss_grad(int W, int n, const float *params, const float *up, const float *target, const int *levels,
                            const float *sigma_in, const float *sigma_out, int emulate, float *pred_out, double *grad);

/* ---- ortho (colour) tiles: ortho.c --------------------------------------
 * or_ortho_noise: createOrthoNoise (OrthoProducer.cpp:26-122), 6 layers of
 * W x W RGBA8.  or_ortho_tile: one OrthoProducer::doCreateTile
 * (OrthoProducer.cpp:292-382) with terrain3/upsampleOrthoShader.glsl; tiles are
 * dense W x W RGBA8 (4 bytes per texel, R first), W = tileSize + 4. */
typedef struct {
    int W, level, tx, ty;
    const uint8_t *parent;    /* parent tile, NULL at level 0 */
    const uint8_t *residual;  /* residual tile, NULL when the residual producer has none */
    const uint8_t *noise;     /* the selected noise layer (W x W RGBA8) */
    int noise_rot;            /* 0..3 */
    float noise_amp;          /* noiseAmp[level] (rs) */
    float root_color[4];      /* rnoise / 255 */
    float noise_color[4];     /* cnoise / 255 */
    float scale;              /* residual scale */
    int hsv;
    uint8_t *out;             /* W x W RGBA8 */
} or_ortho_job;
void or_ortho_noise(int W, uint8_t *out);
void or_ortho_tile(const or_ortho_job *t);
int  or_ortho_tile_id(int level, int tx, int ty);   /* OrthoCPUProducer.cpp:250-253 */

/* ---- elevation layers (layers.c): road and water layer meshes drawn into one
 * tile and blended into zm (ElevationProducer.cpp:378-399, RoadElevationLayer.cpp:
 * 388-437, WaterElevationLayer.cpp:240-350, graph1/roadLayerElevationShader.glsl,
 * river1/waterLayerElevationShader.glsl and fillShader.glsl, graph1 and demo
 * blendShader.glsl).  Vertices are (x, y, a, u) in clip coordinates; indices count
 * from the mesh's first vertex; mode 0 triangles, 1 triangle strip; program 0 road,
 * 1-3 water with river = 0-2, 4 fill; state: depth test in bits 0-1 (0 LESS, 1
 * ALWAYS, 2 NOTEQUAL), 4 no depth write, 8 no z write, 16 no w write.  zf, zm,
 * zm_out are dense W x W. ---- */
typedef struct {
    int first_vertex, count, first_index, mode, clear_depth, program, state;
    float fill_depth;
} or_layer_mesh;
void or_layer_tile(int W, const float *zf, const float *zm, const or_layer_mesh *meshes, int n_meshes,
                   const float *vertices, const uint32_t *indices, int blend_mode, float *zm_out);
/* one fragment of `program` at the interpolated attributes (a, u): out = (depth
 * clamped to [0, 1], z, w) */
void or_layer_fragment(int program, float fill_depth, float a, float u, float *out);
/* the blend pass alone, from the layers' z and w planes (dense W x W) */
void or_layer_blend(int W, const float *zf, const float *z, const float *w, int blend_mode, float *zm_out);

#ifdef __cplusplus
}
#endif

#endif
