// Multi-threaded client of the TileCache / TileProducer protocol on bookkeeping-only
// storages (no GPU): threads acquire, look up, prefetch and release tiles of shared
// residual, elevation and normal producers (an elevation tile acquires its parent and
// residual tile, a normal tile its elevation and parent tiles), one thread
// invalidates the elevation producer now and then, and one thread runs a sampler
// over an independent residual producer.  Built by tests/test_host_sanitizers.py
// with the library's host sources under AddressSanitizer + UndefinedBehaviorSanitizer
// and under ThreadSanitizer; the run must end with no report, every call answered
// as the protocol allows, and the sampler's tiles all released.  (Elevation and normal
// tiles stay queued -- nothing produces them without a GPU -- and keep the tiles they
// are made from acquired, as a producer's task does until it has run.)
#include <atomic>
#include <cstdio>
#include <random>
#include <thread>
#include <vector>

#include "proland_gb300.h"

#define CHECK(cond, what)                                                      \
    do {                                                                       \
        if (!(cond)) {                                                         \
            std::printf("FAIL %s: %s\n", what, tp_last_error());               \
            return 1;                                                          \
        }                                                                      \
    } while (0)

namespace {

constexpr int kBook = 2;  // bookkeeping-only storage: slots without device memory

struct Held {
    tp_producer *p;
    tp_tile *t;
};

std::atomic<int> g_fail{0};

void worker(unsigned seed, tp_producer *const *prods, int nprod, int ops)
{
    std::mt19937 rng(seed);
    std::vector<Held> held;
    for (int k = 0; k < ops && !g_fail.load(); ++k) {
        tp_producer *p = prods[rng() % nprod];
        const int level = (int)(rng() % 6);
        const int tx = (int)(rng() % (1u << level)), ty = (int)(rng() % (1u << level));
        const unsigned op = rng() % 10;
        if (op < 4 || held.empty()) {
            tp_tile *t = tp_producer_get_tile(p, level, tx, ty);
            if (t) held.push_back(Held{p, t});  // NULL: the cache is full, a normal answer
        } else if (op < 8) {
            const size_t i = rng() % held.size();
            if (tp_producer_put_tile(held[i].p, held[i].t) < 0) g_fail = 1;
            held[i] = held.back();
            held.pop_back();
        } else if (op < 9) {
            tp_tile *t = tp_producer_find_tile(p, level, tx, ty, 1, 0);
            (void)t;
            if (tp_producer_queued(p) < 0) g_fail = 1;
        } else {
            if (tp_producer_prefetch_tile(p, level, tx, ty) < 0) g_fail = 1;
        }
        if (held.size() > 12) {
            if (tp_producer_put_tile(held.front().p, held.front().t) < 0) g_fail = 1;
            held.erase(held.begin());
        }
    }
    for (const Held &h : held)
        if (tp_producer_put_tile(h.p, h.t) < 0) g_fail = 1;
}

void invalidator(tp_producer *e, int rounds)
{
    for (int k = 0; k < rounds && !g_fail.load(); ++k) {
        if (tp_producer_invalidate_tiles(e) != TP_OK) g_fail = 1;
        std::this_thread::yield();
    }
}

void sampling(tp_sampler *s, int frames)
{
    std::mt19937 rng(99);
    for (int f = 0; f < frames && !g_fail.load(); ++f) {
        std::vector<tp_tile_req> req;
        for (int q = 0; q < 12; ++q) {
            int level = (int)(rng() % 5), tx = (int)(rng() % (1u << level)), ty = (int)(rng() % (1u << level));
            for (; level >= 0; --level, tx /= 2, ty /= 2) req.push_back(tp_tile_req{level, tx, ty});
        }
        int fresh = 0;
        if (tp_sampler_update(s, req.data(), (int)req.size(), nullptr, &fresh) != TP_OK) g_fail = 1;
    }
}

}  // namespace

int main()
{
    tp_storage *rs = nullptr, *es = nullptr, *ns = nullptr, *ss = nullptr;
    CHECK(tp_storage_create(101, 1, 48, kBook, &rs) == TP_OK, "residual storage");
    CHECK(tp_storage_create(101, 3, 64, kBook, &es) == TP_OK, "elevation storage");
    CHECK(tp_storage_create(97, 2, 40, kBook, &ns) == TP_OK, "normal storage");
    CHECK(tp_storage_create(101, 1, 512, kBook, &ss) == TP_OK, "sampler storage");
    tp_cache *rc = nullptr, *ec = nullptr, *nc = nullptr, *sc = nullptr;
    CHECK(tp_cache_create(rs, "residuals", &rc) == TP_OK && tp_cache_create(es, "elevations", &ec) == TP_OK &&
              tp_cache_create(ns, "normals", &nc) == TP_OK && tp_cache_create(ss, "sampled", &sc) == TP_OK,
          "caches");
    tp_producer *r = nullptr, *e = nullptr, *n = nullptr, *sr = nullptr;
    const float amps[2] = {-140.0f, -100.0f};
    tp_elev_params params = {24, 0, 0, 0, 2, 0, 0, 0};
    CHECK(tp_residual_producer_create(rc, nullptr, 0, 1.0f, &r) == TP_OK, "residual producer");
    CHECK(tp_elevation_producer_create(ec, r, amps, 2, &params, 0, &e) == TP_OK, "elevation producer");
    CHECK(tp_normal_producer_create(nc, e, 0, &n) == TP_OK, "normal producer");
    CHECK(tp_residual_producer_create(sc, nullptr, 0, 1.0f, &sr) == TP_OK, "sampled producer");
    CHECK(tp_producer_set_root_quad_size(e, 50000.0f) == TP_OK && tp_producer_set_root_quad_size(n, 50000.0f) == TP_OK,
          "root quad size");
    tp_sampler *sampler = nullptr;
    CHECK(tp_sampler_create(&sr, 1, &sampler) == TP_OK, "sampler");

    tp_producer *const prods[3] = {r, e, n};
    std::vector<std::thread> threads;
    for (unsigned k = 0; k < 4; ++k) threads.emplace_back(worker, 1234u + k, prods, 3, 6000);
    threads.emplace_back(invalidator, e, 200);
    threads.emplace_back(sampling, sampler, 300);
    for (std::thread &t : threads) t.join();
    CHECK(!g_fail.load(), "operations");

    CHECK(tp_sampler_destroy(sampler) == TP_OK, "sampler destroy");
    CHECK(tp_cache_used_tiles(sc) == 0, "every sampled tile released");
    CHECK(tp_cache_used_tiles(ec) >= 0 && tp_cache_used_tiles(ec) <= 64 && tp_cache_used_tiles(nc) <= 40 &&
              tp_cache_used_tiles(rc) <= 48,
          "tile counts within the capacities");
    for (tp_producer *p : {n, e, r, sr}) tp_producer_destroy(p);
    for (tp_cache *c : {nc, ec, rc, sc}) tp_cache_destroy(c);
    for (tp_storage *s : {ns, es, rs, ss}) tp_storage_destroy(s);
    std::printf("cache stress ok\n");
    return 0;
}
