/* A plain C client of the library's C ABI, as a Proland build or a cgo / JNI shim
 * would bind it: only the header, plain pointers and return codes.  It runs the
 * host-side parts (no GPU needed): noise tables, residual and ortho pyramid
 * readers, and the TileCache / TileProducer protocol on bookkeeping storages.
 * Prints one line per check; exits non-zero on the first failure. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "proland_gb300.h"

#define CHECK(cond, what)                                                   \
    do {                                                                    \
        if (!(cond)) {                                                      \
            printf("FAIL %s: %s\n", what, tp_last_error());                 \
            return 1;                                                       \
        }                                                                   \
        printf("ok %s\n", what);                                            \
    } while (0)

/* A layer callback: one triangle strip (never called here: nothing is produced without a GPU). */
static int road_layer(void *user, int level, int tx, int ty, tp_layer_builder *b)
{
    static const float v[16] = {-1, -0.1f, 10, -3, -1, 0.1f, 10, 3, 1, -0.1f, 10, -3, 1, 0.1f, 10, 3};
    (void)user; (void)level; (void)tx; (void)ty;
    return tp_layer_builder_add_mesh(b, v, 4, NULL, 0, TP_TRIANGLE_STRIP);
}

int main(int argc, char **argv)
{
    if (argc < 3) {
        printf("usage: %s DEM.dat RGB.dat\n", argv[0]);
        return 2;
    }
    CHECK(tp_version() > 0, "version");
    CHECK(tp_layer_builder_set_pass(NULL, TP_LAYER_FILL, TP_DEPTH_ALWAYS | TP_NO_Z_WRITE, 0.02f) == TP_E_BAD_ARG,
          "layer pass state needs a builder");

    /* createDemNoise and createOrthoNoise tables */
    float *dem = malloc(sizeof(float) * 6 * 101 * 101);
    CHECK(tp_dem_noise(101, dem) == TP_OK && dem[2 * 101 + 50] >= -1.0f && dem[2 * 101 + 50] <= 1.0f, "dem noise");
    unsigned char *on = malloc(6 * 196 * 196 * 4);
    CHECK(tp_ortho_noise(196, on) == TP_OK && on[0] == 128, "ortho noise");
    int rot = -1, layer = -1;
    CHECK(tp_noise_select(1, 5, 7, 9, &rot, &layer) == TP_OK && rot >= 0 && rot < 4 && layer >= 0 && layer < 6,
          "noise select");

    /* ResidualProducer's .dat pyramid */
    tp_dat *d = NULL;
    CHECK(tp_dat_open(argv[1], &d) == TP_OK, "dat open");
    int info[7];
    float scale = 0.0f;
    CHECK(tp_dat_info(d, info, &scale) == TP_OK && info[2] > 0, "dat info");
    int16_t *tile = malloc(sizeof(int16_t) * 512 * 512);
    int w = 0;
    /* tiles above minLevel (info[0]) are tileSize >> (minLevel - level) wide (ResidualProducer.cpp:253-256) */
    CHECK(tp_dat_read_tile(d, 0, 0, 0, tile, 512 * 512, &w) == TP_OK && w == (info[2] >> info[0]) + 5, "dat tile");
    CHECK(tp_dat_read_tile(d, 40, 0, 0, tile, 512 * 512, &w) == TP_E_BAD_ARG, "dat tile outside the pyramid");
    tp_dat_close(d);

    /* OrthoCPUProducer's .dat pyramid */
    tp_ortho_dat *od = NULL;
    CHECK(tp_ortho_dat_open(argv[2], &od) == TP_OK, "ortho dat open");
    int oinfo[8];
    CHECK(tp_ortho_dat_info(od, oinfo) == TP_OK && oinfo[1] == 192 && oinfo[2] == 4, "ortho dat info");
    uint32_t *texels = malloc(sizeof(uint32_t) * 196 * 196);
    CHECK(tp_ortho_dat_read_rgba(od, 0, 0, 0, texels, 196 * 196, &w) == TP_OK && w == 196, "ortho tile");
    tp_ortho_dat_close(od);

    /* TileCache / TileProducer protocol on bookkeeping storages (no device memory) */
    tp_storage *es = NULL, *ns = NULL, *rs = NULL;
    CHECK(tp_storage_create(101, 3, 8, 2, &es) == TP_OK && tp_storage_create(97, 2, 8, 2, &ns) == TP_OK &&
              tp_storage_create(101, 1, 8, 2, &rs) == TP_OK,
          "storages");
    tp_cache *ec = NULL, *nc = NULL, *rc = NULL;
    CHECK(tp_cache_create(es, "elev", &ec) == TP_OK && tp_cache_create(ns, "nrm", &nc) == TP_OK &&
              tp_cache_create(rs, "res", &rc) == TP_OK,
          "caches");
    tp_producer *res = NULL, *elev = NULL, *nrm = NULL;
    const float amps[3] = {-140.0f, -100.0f, -15.0f};
    tp_elev_params p;
    memset(&p, 0, sizeof p);
    p.grid_size = 24;
    p.normal_format = 2;
    CHECK(tp_residual_producer_create(rc, "", 0, 1.0f, &res) == TP_OK &&
              tp_elevation_producer_create(ec, res, amps, 3, &p, 1, &elev) == TP_OK &&
              tp_normal_producer_create(nc, elev, 0, &nrm) == TP_OK,
          "producers");
    CHECK(tp_producer_border(elev) == 2 && tp_producer_border(nrm) == 0, "borders");
    /* a road layer on the elevation producer (TileProducer::addLayer); only elevation
     * producers take layers, and the blend program is 0 or 1 */
    CHECK(tp_elevation_producer_add_layer(elev, road_layer, NULL) == TP_OK &&
              tp_elevation_producer_add_layer(nrm, road_layer, NULL) == TP_E_BAD_ARG &&
              tp_elevation_producer_set_blend(elev, 1) == TP_OK && tp_elevation_producer_set_blend(elev, 2) == TP_E_BAD_ARG,
          "layers");
    tp_tile *t = tp_producer_get_tile(nrm, 2, 1, 3);
    int level, tx, ty, slot, users, done;
    CHECK(t != NULL && tp_tile_info(t, &level, &tx, &ty, &slot, &users, &done) == TP_OK && level == 2 && users == 1 &&
              !done,
          "getTile queues the tile");
    /* the normal tile holds its elevation tile and its parent normal tile (for the coarse
     * normals); each elevation tile holds its parent and its residual: levels 0..2 of all three */
    printf("queued: normals %d, elevations %d, residuals %d\n", tp_producer_queued(nrm), tp_producer_queued(elev),
           tp_producer_queued(res));
    CHECK(tp_producer_queued(nrm) == 3 && tp_producer_queued(elev) == 3 && tp_producer_queued(res) == 3,
          "dependencies queued");
    CHECK(tp_producer_put_tile(nrm, t) == 0 && tp_cache_unused_tiles(nc) == 1, "putTile keeps the tile unused");
    /* a full cache answers NULL with TP_E_CACHE_FULL, as TileCache::getTile answers NULL */
    tp_storage *tiny = NULL;
    tp_cache *tc = NULL;
    tp_producer *te = NULL;
    CHECK(tp_storage_create(101, 3, 2, 2, &tiny) == TP_OK && tp_cache_create(tiny, "tiny", &tc) == TP_OK &&
              tp_elevation_producer_create(tc, NULL, amps, 3, &p, 1, &te) == TP_OK,
          "small cache");
    CHECK(tp_producer_get_tile(te, 4, 3, 3) == NULL, "full cache gives NULL");
    tp_producer_destroy(te);
    tp_cache_destroy(tc);
    tp_storage_destroy(tiny);
    tp_producer_destroy(nrm);
    tp_producer_destroy(elev);
    tp_producer_destroy(res);
    tp_cache_destroy(ec);
    tp_cache_destroy(nc);
    tp_cache_destroy(rc);
    tp_storage_destroy(es);
    tp_storage_destroy(ns);
    tp_storage_destroy(rs);
    free(dem);
    free(on);
    free(tile);
    free(texels);
    printf("all ok\n");
    return 0;
}
