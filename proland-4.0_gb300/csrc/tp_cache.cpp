// TileCache and TileProducer over device slot pools.
//
// The cache follows TileCache.cpp:150-377: tiles are keyed by
// (producer id, level, tx, ty); a tile with users is "used", a tile without is
// kept in an LRU list of "unused" tiles whose slots are recycled, oldest first,
// when the storage has no free slot; getTile returns NULL when nothing can be
// recycled (a full cache).  A tile whose content is not produced yet is queued
// on its producer together with the tiles it is made from (TileProducer's
// startCreateTile, e.g. ElevationProducer.cpp:246-271, NormalProducer.cpp:139-156),
// which are acquired with getTile and released with putTile once it is produced
// (stopCreateTile).  tp_scheduler_run produces every queued tile of a set of
// producers: residual tiles on the host (file decode) and one upload, then each
// elevation producer's queue as one frame launch ordered parents-first, with
// the normal tiles of the same (level, tx, ty) produced by the same launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <list>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "tp_internal.h"
#include "tp_trace.h"

namespace {

enum Kind { kResidual = 0, kElevation = 1, kNormal = 2, kOrthoResidual = 3, kOrtho = 4 };
// tile id (producer id, level, tx, ty), TileCache.h:80-86
struct TKey {
    uint64_t a = 0, b = 0;  // (producer id, level), (tx, ty)
    TKey() = default;
    TKey(int producer, int level, int tx, int ty)
        : a(((uint64_t)(uint32_t)producer << 32) | (uint32_t)level), b(((uint64_t)(uint32_t)tx << 32) | (uint32_t)ty)
    {
    }
    bool operator==(const TKey &o) const { return a == o.a && b == o.b; }
};
struct TKeyHash {
    size_t operator()(const TKey &k) const
    {
        uint64_t x = k.a * 0x9e3779b97f4a7c15ull ^ (k.b + 0x632be59bd9b4e019ull + (k.a << 6) + (k.a >> 2));
        x ^= x >> 31;
        x *= 0xbf58476d1ce4e5b9ull;
        x ^= x >> 29;
        return (size_t)x;
    }
};

// Key -> value tables of the caches (tile key -> tile) and samplers (quad key ->
// position): open addressing with linear probing, the keys held in the table itself
// (one cache line touched per lookup in the common case instead of a bucket array and
// a list node), a power-of-two capacity of at least twice the entries, deletion by
// backward shift (no tombstones).  A slot is empty when its value equals `empty`.
template <class K, class V, class Hash>
class FlatTable {
public:
    explicit FlatTable(V empty) : empty_(empty) {}
    void reserve(size_t n)
    {
        size_t cap = 16;
        while (cap < 2 * n) cap <<= 1;
        if (cap > slots_.size()) rehash(cap);
    }
    size_t size() const { return size_; }
    // the value's slot, or null
    V *find(const K &k)
    {
        if (slots_.empty()) return nullptr;
        for (size_t i = Hash()(k) & mask_;; i = (i + 1) & mask_) {
            Slot &e = slots_[i];
            if (e.v == empty_) return nullptr;
            if (e.k == k) return &e.v;
        }
    }
    const V *find(const K &k) const { return const_cast<FlatTable *>(this)->find(k); }
    void insert(const K &k, V v)  // k is not in the table
    {
        if (2 * (size_ + 1) > slots_.size()) rehash(slots_.empty() ? 16 : 2 * slots_.size());
        size_t i = Hash()(k) & mask_;
        while (slots_[i].v != empty_) i = (i + 1) & mask_;
        slots_[i] = Slot{k, v};
        ++size_;
    }
    void erase(const K &k)
    {
        if (slots_.empty()) return;
        size_t i = Hash()(k) & mask_;
        for (;; i = (i + 1) & mask_) {
            if (slots_[i].v == empty_) return;
            if (slots_[i].k == k) break;
        }
        // backward shift: move later entries of the probe run into the hole when their
        // home position does not lie cyclically in (hole, their position]
        size_t hole = i;
        for (size_t j = (i + 1) & mask_; slots_[j].v != empty_; j = (j + 1) & mask_) {
            const size_t home = Hash()(slots_[j].k) & mask_;
            const bool stays = hole <= j ? (home > hole && home <= j) : (home > hole || home <= j);
            if (stays) continue;
            slots_[hole] = slots_[j];
            hole = j;
        }
        slots_[hole] = Slot{K{}, empty_};
        --size_;
    }
    template <class F>
    void for_each(F f) const
    {
        for (const Slot &e : slots_)
            if (e.v != empty_) f(e.v);
    }

private:
    struct Slot {
        K k;
        V v;
    };
    void rehash(size_t cap)
    {
        std::vector<Slot> old(cap, Slot{K{}, empty_});
        old.swap(slots_);
        mask_ = cap - 1;
        size_ = 0;
        for (const Slot &e : old)
            if (e.v != empty_) insert(e.k, e.v);
    }
    std::vector<Slot> slots_;
    size_t mask_ = 0, size_ = 0;
    V empty_;
};

int next_producer_id()
{
    static std::mutex mu;
    static int next = 1;
    std::lock_guard<std::mutex> lk(mu);
    return next++;
}

}  // namespace

struct tp_tile {
    int producer_id = 0, level = 0, tx = 0, ty = 0;
    int slot = -1;
    int users = 0;
    bool done = false;    // content produced
    bool queued = false;  // waiting in its producer's queue
    // tiles acquired to produce this one, released once it is produced
    tp_tile *dep_parent = nullptr;
    tp_producer *dep_parent_owner = nullptr;
    tp_tile *dep_input = nullptr;  // residual tile (elevation) or elevation tile (normal)
    tp_producer *dep_input_owner = nullptr;
    // the cache's list of unused tiles (users == 0), least recently used first
    tp_tile *lru_prev = nullptr, *lru_next = nullptr;
    // while an elevation launch is being built: the tile's job index in it (-1 when it
    // is not in the launch) and the normal tile whose normals the launch fuses in
    int job = -1;
    tp_tile *fused_normal = nullptr;
};

struct tp_cache {
    tp_storage *storage = nullptr;
    std::string name;
    std::recursive_mutex mu;
    // every tile holding a slot: used (users > 0) or unused (users == 0, in the LRU list)
    FlatTable<TKey, tp_tile *, TKeyHash> tiles{nullptr};
    tp_tile *lru_head = nullptr, *lru_tail = nullptr;
    int n_unused = 0;
    long long queries = 0, misses = 0;

    void lru_push_back(tp_tile *t)
    {
        t->lru_prev = lru_tail;
        t->lru_next = nullptr;
        if (lru_tail) lru_tail->lru_next = t;
        else lru_head = t;
        lru_tail = t;
        ++n_unused;
    }
    void lru_unlink(tp_tile *t)
    {
        if (t->lru_prev) t->lru_prev->lru_next = t->lru_next;
        else lru_head = t->lru_next;
        if (t->lru_next) t->lru_next->lru_prev = t->lru_prev;
        else lru_tail = t->lru_prev;
        t->lru_prev = t->lru_next = nullptr;
        --n_unused;
    }
};

struct tp_producer {
    Kind kind = kElevation;
    int id = 0;
    tp_cache *cache = nullptr;
    float root_quad_size = 0.0f;
    std::vector<tp_tile *> queue;
    // residual producer
    tp_dat *dat = nullptr;
    bool own_dat = false;
    int delta = 0;
    float zscale = 1.0f;
    tp_residual_source source = nullptr;
    void *source_user = nullptr;
    // elevation producer
    tp_producer *residuals = nullptr;
    std::vector<float> noise_amp;
    tp_elev_params params{};
    int face = 0;
    tp_frame *frame = nullptr;
    // normal producer
    tp_producer *elevations = nullptr;
    int deform = 0;
    int normal_format = 2;  // 0..3 (NormalProducer.cpp:195); 0/1 add coarse normals
    int device_decode = 0;  // residual producer over a .dat file: decode tiles on the device
    // residual producer with synthetic tiles: sigma0 * ratio^level, generator seed
    bool synthetic = false;
    double syn_sigma0 = 0.0, syn_ratio = 1.0;
    uint32_t syn_seed = 0;
    int grid_mesh = 24;
    // ortho residual producer (OrthoCPUProducer): tiles of an ortho .dat file, or zeros
    tp_ortho_dat *odat = nullptr;
    int ortho_max_level = 1;
    int ortho_border = 2;
    // ortho producer (OrthoProducer); residuals, noise_amp and face as above
    tp_ortho_params oparams{};
    int max_level = -1;
    // elevation producer layers (TileProducer::addLayer) and the blend program
    std::vector<std::pair<tp_layer_fn, void *>> layers;
    int blend_mode = 0;
};

// Meshes that a producer's layers draw for one level's tiles.
struct tp_layer_builder {
    std::vector<tp_layer_mesh> meshes;
    std::vector<float> vertices;
    std::vector<uint32_t> indices;
    bool layer_start = false;  // the next mesh is the first of a layer: it clears the depth buffer
    int program = TP_LAYER_ROAD, state = 0;  // the next meshes' fragment program and pass state
    float fill_depth = 0.0f;
};

namespace {

TKey key_of(const tp_producer *p, int level, int tx, int ty) { return TKey(p->id, level, tx, ty); }

void release_deps(tp_tile *t);

// Drops a tile that is being recycled: its queued production is cancelled.
// A recycled tile that was still queued (acquired, then released before its
// production ran) leaves its producer's queue and releases what it had acquired.
void unqueue_tile(tp_tile *t, tp_producer *owner)
{
    if (t->queued && owner) {
        auto &q = owner->queue;
        q.erase(std::remove(q.begin(), q.end(), t), q.end());
        t->queued = false;
        release_deps(t);
    }
}

}  // namespace

namespace tp {

// Registry of producers by id, to find a recycled tile's owner.
static std::mutex g_prod_mu;
static std::map<int, tp_producer *> g_producers;

static tp_producer *producer_by_id(int id)
{
    std::lock_guard<std::mutex> lk(g_prod_mu);
    auto it = g_producers.find(id);
    return it == g_producers.end() ? nullptr : it->second;
}

}  // namespace tp

namespace {

int schedule(tp_producer *p, tp_tile *t);
int put_tile(tp_producer *p, tp_tile *t);

// TileCache::getTile (TileCache.cpp:174-252).
tp_tile *get_tile(tp_producer *p, int level, int tx, int ty, int *users_before, int *err)
{
    tp_cache *c = p->cache;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    const TKey k = key_of(p, level, tx, ty);
    tp_tile *t = nullptr;
    if (tp_tile **found = c->tiles.find(k)) {
        t = *found;
        if (t->users == 0) {
            ++c->queries;
            c->lru_unlink(t);  // an unused tile in the cache: used again
        }
    } else {
        ++c->queries;
        int slot = tp_storage_new_slot(c->storage);
        if (slot < 0 && c->lru_head) {
            // recycle the least recently used unused tile: its slot and its record (no
            // allocation per new tile)
            tp_tile *old = c->lru_head;
            c->lru_unlink(old);
            c->tiles.erase(TKey(old->producer_id, old->level, old->tx, old->ty));
            slot = old->slot;
            if (old->queued) unqueue_tile(old, tp::producer_by_id(old->producer_id));
            *old = tp_tile{};
            t = old;
            c->tiles.insert(k, t);
        }
        if (slot < 0) {
            if (err) *err = tp::fail(TP_E_CACHE_FULL, "Insufficient tile cache size (" + c->name + ")");
            return nullptr;
        }
        ++c->misses;
        if (!t) {
            t = new tp_tile;
            c->tiles.insert(k, t);
        }
        t->producer_id = p->id;
        t->level = level;
        t->tx = tx;
        t->ty = ty;
        t->slot = slot;
    }
    if (users_before) *users_before = t->users;
    t->users += 1;
    if (!t->done && !t->queued) {
        int rc = schedule(p, t);
        if (rc) {
            // the tiles it is made from cannot be had: hand it back, unproduced
            if (err) *err = rc;
            put_tile(p, t);
            return nullptr;
        }
    }
    return t;
}

// TileCache::putTile (TileCache.cpp:312-336).
int put_tile(tp_producer *p, tp_tile *t)
{
    tp_cache *c = p->cache;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    t->users -= 1;
    if (t->users == 0) c->lru_push_back(t);  // kept in the cache, unused
    return t->users;
}

void release_deps(tp_tile *t)
{
    if (t->dep_parent) put_tile(t->dep_parent_owner, t->dep_parent);
    if (t->dep_input) put_tile(t->dep_input_owner, t->dep_input);
    t->dep_parent = t->dep_input = nullptr;
    t->dep_parent_owner = t->dep_input_owner = nullptr;
}

bool residual_has_tile(const tp_producer *r, int level, int tx, int ty);

// startCreateTile: acquire the tiles this tile is made from, then queue it.
int schedule(tp_producer *p, tp_tile *t)
{
    int err = TP_OK;
    if (p->kind == kElevation) {
        if (t->level > 0) {
            t->dep_parent = get_tile(p, t->level - 1, t->tx / 2, t->ty / 2, nullptr, &err);
            if (!t->dep_parent) return err ? err : tp::fail(TP_E_CACHE_FULL, "cache full (parent)");
            t->dep_parent_owner = p;
        }
        if (p->residuals) {
            const int n = p->cache->storage->W - 5;
            const int mod = (p->residuals->cache->storage->W - 5) / n;
            if (residual_has_tile(p->residuals, t->level, t->tx / mod, t->ty / mod)) {
                t->dep_input = get_tile(p->residuals, t->level, t->tx / mod, t->ty / mod, nullptr, &err);
                if (!t->dep_input) {
                    release_deps(t);
                    return err ? err : tp::fail(TP_E_CACHE_FULL, "cache full (residual)");
                }
                t->dep_input_owner = p->residuals;
            }
        }
    } else if (p->kind == kOrtho) {
        // OrthoProducer::startCreateTile (OrthoProducer.cpp:245-264): the parent tile and the
        // residual tile of the same (level, tx, ty)
        if (t->level > 0) {
            t->dep_parent = get_tile(p, t->level - 1, t->tx / 2, t->ty / 2, nullptr, &err);
            if (!t->dep_parent) return err ? err : tp::fail(TP_E_CACHE_FULL, "cache full (ortho parent)");
            t->dep_parent_owner = p;
        }
        if (p->residuals && tp_producer_has_tile(p->residuals, t->level, t->tx, t->ty) == 1) {
            t->dep_input = get_tile(p->residuals, t->level, t->tx, t->ty, nullptr, &err);
            if (!t->dep_input) {
                release_deps(t);
                return err ? err : tp::fail(TP_E_CACHE_FULL, "cache full (ortho residual)");
            }
            t->dep_input_owner = p->residuals;
        }
    } else if (p->kind == kNormal) {
        t->dep_input = get_tile(p->elevations, t->level, t->tx, t->ty, nullptr, &err);
        if (!t->dep_input) return err ? err : tp::fail(TP_E_CACHE_FULL, "cache full (elevation)");
        t->dep_input_owner = p->elevations;
        if (t->level > 0) {
            t->dep_parent = get_tile(p, t->level - 1, t->tx / 2, t->ty / 2, nullptr, &err);
            if (!t->dep_parent) {
                release_deps(t);
                return err ? err : tp::fail(TP_E_CACHE_FULL, "cache full (parent normals)");
            }
            t->dep_parent_owner = p;
        }
    }
    t->queued = true;
    p->queue.push_back(t);
    return TP_OK;
}

// ResidualProducer::hasTile (ResidualProducer.cpp:161-175).
bool residual_has_tile(const tp_producer *r, int level, int tx, int ty)
{
    if (r->synthetic || !r->dat) return true;  // synthetic source or zero residuals: every tile exists
    const int l = level + r->delta - r->dat->root_level;
    return l >= 0 && (tx >> l) == r->dat->root_tx && (ty >> l) == r->dat->root_ty && l <= r->dat->max_level;
}

// ResidualProducer::upsample (ResidualProducer.cpp:342-384): 2x interpolation of
// a tile of `tilesize` intervals into its child at (tx % 2, ty % 2); n is the
// pitch of both arrays.  Used only to chain the pyramid's levels up to the
// root when the producer starts `delta` levels below the file's first level.
void upsample_small(int level_tilesize, int tx, int ty, const float *parent, float *out, int pitch)
{
    const int ts = level_tilesize;
    const int px = 1 + (tx % 2) * ts / 2, py = 1 + (ty % 2) * ts / 2;
    for (int j = 0; j <= ts + 4; ++j)
        for (int i = 0; i <= ts + 4; ++i) {
            const float *cc = parent + (i / 2 + px) + (size_t)(j / 2 + py) * pitch;
            float z;
            if ((j & 1) == 0) {
                z = (i & 1) == 0 ? cc[0] : ((cc[0] + cc[1]) * 9 - (cc[-1] + cc[2])) / 16;
            } else if ((i & 1) == 0) {
                z = ((cc[0] + cc[pitch]) * 9 - (cc[-pitch] + cc[2 * pitch])) / 16;
            } else {
                z = 0;
                for (int dj = -1; dj <= 2; ++dj) {
                    const float f = (dj == -1 || dj == 2) ? -1 / 16.0f : 9 / 16.0f;
                    for (int di = -1; di <= 2; ++di) {
                        const float g = (di == -1 || di == 2) ? -1 / 16.0f : 9 / 16.0f;
                        z += f * g * cc[di + (ptrdiff_t)dj * pitch];
                    }
                }
            }
            out[i + (size_t)j * pitch] = z;
        }
}

// ResidualProducer::doCreateTile + readTile (ResidualProducer.cpp:177-232,
// 268-340) into a dense Wr x Wr host tile.
float synthetic_sigma(const tp_producer *r, int level)
{
    return (float)(r->syn_sigma0 * std::pow(r->syn_ratio, (double)level));
}

int produce_residual(tp_producer *r, const tp_tile *t, float *out)
{
    const int Wr = r->cache->storage->W;
    std::fill(out, out + (size_t)Wr * Wr, 0.0f);
    if (r->synthetic) {
        tp::synthetic_residual_host(r->syn_seed, t->level, t->tx, t->ty, synthetic_sigma(r, t->level), Wr, out, Wr);
        return TP_OK;
    }
    if (r->source) {
        int rc = r->source(r->source_user, t->level, t->tx, t->ty, out, Wr);
        return rc ? tp::fail(TP_E_IO, "residual source callback failed") : TP_OK;
    }
    if (!r->dat) return TP_OK;  // zero residuals
    const tp_dat *d = r->dat;
    int level = t->level + r->delta - d->root_level;
    if (level < 0 || (t->tx >> level) != d->root_tx || (t->ty >> level) != d->root_ty) return TP_OK;
    const int tx = t->tx - (d->root_tx << level), ty = t->ty - (d->root_ty << level);
    const float scale = d->scale * r->zscale;
    if (d->tile_size + 5 != Wr) return tp::fail(TP_E_BAD_ARG, "residual storage width does not match the file");
    auto read = [&](int lv, int x, int y, const float *base) -> int {
        std::vector<int16_t> v;
        int w = 0;
        int rc = tp::dat_tile_int16(d, lv, x, y, v, &w);
        if (rc) return rc;
        for (int j = 0; j < w; ++j)
            for (int i = 0; i < w; ++i) {
                const size_t o = i + (size_t)j * Wr;
                out[o] = base ? base[o] + v[i + (size_t)j * w] * scale : v[i + (size_t)j * w] * scale;
            }
        return TP_OK;
    };
    if (r->delta > 0 && level == r->delta) {
        // the root of a producer started delta levels down: chain levels 0..delta
        std::vector<float> tmp((size_t)Wr * Wr);
        int rc = read(0, 0, 0, nullptr);
        for (int i = 1; i <= r->delta && !rc; ++i) {
            const int ts = (i < d->min_level ? d->tile_size >> (d->min_level - i) : d->tile_size);
            upsample_small(ts, 0, 0, out, tmp.data(), Wr);
            rc = read(i, 0, 0, tmp.data());
        }
        return rc;
    }
    return read(level, tx, ty, nullptr);
}

}  // namespace

// ---------------------------------------------------------------- C ABI: cache
extern "C" int tp_cache_create(tp_storage *storage, const char *name, tp_cache **out)
{
    if (!storage || !out) return tp::fail(TP_E_BAD_ARG, "tp_cache_create: bad arguments");
    auto *c = new tp_cache;
    c->storage = storage;
    c->name = name ? name : "";
    c->tiles.reserve((size_t)storage->capacity);  // one entry per slot at most: no rehash
    *out = c;
    return TP_OK;
}

extern "C" int tp_cache_destroy(tp_cache *c)
{
    if (!c) return TP_OK;
    c->tiles.for_each([](tp_tile *t) { delete t; });
    delete c;
    return TP_OK;
}

extern "C" int tp_cache_used_tiles(tp_cache *c)
{
    if (!c) return TP_E_BAD_ARG;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    return (int)c->tiles.size() - c->n_unused;
}

extern "C" int tp_cache_unused_tiles(tp_cache *c)
{
    if (!c) return TP_E_BAD_ARG;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    return c->n_unused;
}

extern "C" int tp_cache_stats(tp_cache *c, long long *queries, long long *misses)
{
    if (!c) return TP_E_BAD_ARG;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    if (queries) *queries = c->queries;
    if (misses) *misses = c->misses;
    return TP_OK;
}

// ---------------------------------------------------------------- C ABI: producers
static tp_producer *new_producer(Kind kind, tp_cache *cache)
{
    auto *p = new tp_producer;
    p->kind = kind;
    p->id = next_producer_id();
    p->cache = cache;
    std::lock_guard<std::mutex> lk(tp::g_prod_mu);
    tp::g_producers[p->id] = p;
    return p;
}

extern "C" int tp_residual_producer_create(tp_cache *cache, const char *file, int delta, float zscale,
                                           tp_producer **out)
{
    if (!cache || !out) return tp::fail(TP_E_BAD_ARG, "tp_residual_producer_create: bad arguments");
    *out = nullptr;
    tp_dat *d = nullptr;
    if (file && file[0]) {
        int rc = tp_dat_open(file, &d);
        if (rc) return rc;
        if (delta < 0 || delta > d->min_level) {
            tp_dat_close(d);
            return tp::fail(TP_E_BAD_ARG, "tp_residual_producer_create: delta must be in [0, minLevel]");
        }
        if (d->tile_size + 5 != cache->storage->W) {
            tp_dat_close(d);
            return tp::fail(TP_E_BAD_ARG, "residual cache tile width does not match the file's tileSize + 5");
        }
    }
    tp_producer *p = new_producer(kResidual, cache);
    p->dat = d;
    p->own_dat = d != nullptr;
    p->delta = d && d->root_level == 0 ? delta : 0;
    p->zscale = zscale;
    *out = p;
    return TP_OK;
}

extern "C" int tp_residual_producer_set_source(tp_producer *p, tp_residual_source fn, void *user)
{
    if (!p || p->kind != kResidual) return tp::fail(TP_E_BAD_ARG, "tp_residual_producer_set_source: not a residual producer");
    p->source = fn;
    p->source_user = user;
    return TP_OK;
}

extern "C" int tp_elevation_producer_create(tp_cache *cache, tp_producer *residuals, const float *noise_amp, int n_noise,
                                            const tp_elev_params *params, int face, tp_producer **out)
{
    if (!cache || !params || !out || n_noise < 0 || (n_noise > 0 && !noise_amp))
        return tp::fail(TP_E_BAD_ARG, "tp_elevation_producer_create: bad arguments");
    if (cache->storage->channels != 3) return tp::fail(TP_E_BAD_ARG, "elevation cache must have 3-channel slots");
    if (residuals && residuals->kind != kResidual) return tp::fail(TP_E_BAD_ARG, "residuals must be a residual producer");
    tp_producer *p = new_producer(kElevation, cache);
    p->residuals = residuals;
    p->noise_amp.assign(noise_amp, noise_amp + n_noise);
    p->params = *params;
    p->face = face;
    *out = p;
    return TP_OK;
}

extern "C" int tp_normal_producer_create(tp_cache *cache, tp_producer *elevations, int deform, tp_producer **out)
{
    if (!cache || !elevations || !out || elevations->kind != kElevation)
        return tp::fail(TP_E_BAD_ARG, "tp_normal_producer_create: bad arguments");
    if ((cache->storage->channels != 2 && cache->storage->channels != 4) ||
        cache->storage->W != elevations->cache->storage->W - 4)
        return tp::fail(TP_E_BAD_ARG, "normal cache must have 2- or 4-channel slots of width W - 4");
    tp_producer *p = new_producer(kNormal, cache);
    p->elevations = elevations;
    p->deform = deform;
    // as the reference picks the format from the storage (NormalProducer.cpp:195): 4 signed
    // components carry the coarse normals too
    p->normal_format = cache->storage->channels == 4 ? 0 : 2;
    *out = p;
    return TP_OK;
}

extern "C" int tp_ortho_residual_producer_create(tp_cache *cache, const char *file, tp_producer **out)
{
    if (!cache || !out) return tp::fail(TP_E_BAD_ARG, "tp_ortho_residual_producer_create: bad arguments");
    *out = nullptr;
    if (cache->storage->channels != 1) return tp::fail(TP_E_BAD_ARG, "ortho residual cache must hold RGBA8 texels (1 channel)");
    tp_ortho_dat *d = nullptr;
    int max_level = 1, border = 2;  // OrthoCPUProducer.cpp:73-78: no file, zero tiles at levels 0 and 1
    if (file && file[0]) {
        int rc = tp_ortho_dat_open(file, &d);
        if (rc) return rc;
        int info[8];
        tp_ortho_dat_info(d, info);
        max_level = info[0];
        border = (info[6] & 2) ? 0 : 2;
        if ((info[6] & 1) || info[1] + 2 * border != cache->storage->W) {
            tp_ortho_dat_close(d);
            return tp::fail(TP_E_BAD_ARG, "ortho residual cache width must be the file's tileSize + 2 border (no DXT)");
        }
    }
    tp_producer *p = new_producer(kOrthoResidual, cache);
    p->odat = d;
    p->own_dat = d != nullptr;
    p->ortho_max_level = max_level;
    p->ortho_border = border;
    *out = p;
    return TP_OK;
}

extern "C" int tp_ortho_producer_create(tp_cache *cache, tp_producer *residuals, const tp_ortho_params *params,
                                        const float *noise_amp, int n_noise, int face, int max_level,
                                        tp_producer **out)
{
    if (!cache || !params || !out || n_noise < 0 || (n_noise > 0 && !noise_amp) || max_level < -1)
        return tp::fail(TP_E_BAD_ARG, "tp_ortho_producer_create: bad arguments");
    *out = nullptr;
    const tp_storage *s = cache->storage;
    if (s->channels != 1 || s->W % 4 != 0)
        return tp::fail(TP_E_BAD_ARG, "ortho cache must hold RGBA8 texels (1 channel) of a width that is a multiple of 4");
    if (residuals && (residuals->kind != kOrthoResidual || residuals->cache->storage->W != s->W ||
                      residuals->ortho_border != 2))
        return tp::fail(TP_E_BAD_ARG, "ortho residuals must be an ortho residual producer of the same width, border 2");
    tp_producer *p = new_producer(kOrtho, cache);
    p->residuals = residuals;
    p->oparams = *params;
    p->noise_amp.assign(noise_amp, noise_amp + n_noise);
    p->face = face;
    p->max_level = max_level;
    *out = p;
    return TP_OK;
}

extern "C" int tp_residual_producer_set_synthetic(tp_producer *p, double sigma0, double ratio, unsigned seed)
{
    if (!p || p->kind != kResidual) return tp::fail(TP_E_BAD_ARG, "tp_residual_producer_set_synthetic: not a residual producer");
    if (!(sigma0 >= 0.0) || !(ratio > 0.0)) return tp::fail(TP_E_BAD_ARG, "tp_residual_producer_set_synthetic: bad sigma");
    std::lock_guard<std::recursive_mutex> lk(p->cache->mu);
    p->synthetic = true;
    p->syn_sigma0 = sigma0;
    p->syn_ratio = ratio;
    p->syn_seed = seed;
    return TP_OK;
}

extern "C" int tp_residual_producer_set_device_decode(tp_producer *p, int on)
{
    if (!p || p->kind != kResidual) return tp::fail(TP_E_BAD_ARG, "tp_residual_producer_set_device_decode: not a residual producer");
    p->device_decode = on ? 1 : 0;
    return TP_OK;
}

extern "C" int tp_normal_producer_set_format(tp_producer *p, int format, int grid_mesh)
{
    if (!p || p->kind != kNormal || format < 0 || format > 3 || grid_mesh < 1)
        return tp::fail(TP_E_BAD_ARG, "tp_normal_producer_set_format: bad arguments");
    if (p->cache->storage->channels < (format <= 1 ? 4 : 2))
        return tp::fail(TP_E_BAD_ARG, "tp_normal_producer_set_format: formats 0 and 1 need a 4-channel storage");
    p->normal_format = format;
    p->grid_mesh = grid_mesh;
    return TP_OK;
}

extern "C" int tp_layer_builder_add_mesh(tp_layer_builder *b, const float *vertices, int n_vertices,
                                         const uint32_t *indices, int n_indices, int mode)
{
    if (!b || n_vertices < 0 || (n_vertices > 0 && !vertices) || n_indices < 0 || (n_indices > 0 && !indices) ||
        (mode != TP_TRIANGLES && mode != TP_TRIANGLE_STRIP))
        return tp::fail(TP_E_BAD_ARG, "tp_layer_builder_add_mesh: bad arguments");
    for (int k = 0; k < n_indices; ++k)
        if (indices[k] >= (uint32_t)n_vertices) return tp::fail(TP_E_BAD_ARG, "tp_layer_builder_add_mesh: index out of range");
    tp_layer_mesh m;
    std::memset(&m, 0, sizeof m);
    m.first_vertex = (int32_t)(b->vertices.size() / 4);
    m.count = n_indices > 0 ? n_indices : n_vertices;
    m.first_index = n_indices > 0 ? (int32_t)b->indices.size() : -1;
    m.mode = mode;
    m.clear_depth = b->layer_start ? 1 : 0;
    m.program = b->program;
    m.state = b->state;
    m.fill_depth = b->fill_depth;
    b->layer_start = false;
    b->vertices.insert(b->vertices.end(), vertices, vertices + 4 * (size_t)n_vertices);
    b->indices.insert(b->indices.end(), indices, indices + n_indices);
    b->meshes.push_back(m);
    return TP_OK;
}

extern "C" int tp_layer_builder_set_pass(tp_layer_builder *b, int program, int state, float fill_depth)
{
    if (!b) return tp::fail(TP_E_BAD_ARG, "tp_layer_builder_set_pass: bad arguments");
    const int rc = tp::check_layer_pass(program, state, fill_depth, "tp_layer_builder_set_pass");
    if (rc) return rc;
    b->program = program;
    b->state = state;
    b->fill_depth = fill_depth;
    return TP_OK;
}

extern "C" int tp_elevation_producer_add_layer(tp_producer *p, tp_layer_fn fn, void *user)
{
    if (!p || p->kind != kElevation || !fn) return tp::fail(TP_E_BAD_ARG, "tp_elevation_producer_add_layer: bad arguments");
    if (p->cache->storage->channels < 3)
        return tp::fail(TP_E_BAD_ARG, "tp_elevation_producer_add_layer: layers need (zf, zc, zm) slots");
    std::lock_guard<std::recursive_mutex> lk(p->cache->mu);
    p->layers.emplace_back(fn, user);
    return TP_OK;
}

extern "C" int tp_elevation_producer_set_blend(tp_producer *p, int blend_mode)
{
    if (!p || p->kind != kElevation || (blend_mode != 0 && blend_mode != 1))
        return tp::fail(TP_E_BAD_ARG, "tp_elevation_producer_set_blend: bad arguments");
    p->blend_mode = blend_mode;
    return TP_OK;
}

extern "C" int tp_producer_destroy(tp_producer *p)
{
    if (!p) return TP_OK;
    {
        std::lock_guard<std::mutex> lk(tp::g_prod_mu);
        tp::g_producers.erase(p->id);
    }
    if (p->frame) tp_frame_destroy(p->frame);
    if (p->own_dat && p->dat) tp_dat_close(p->dat);
    if (p->own_dat && p->odat) tp_ortho_dat_close(p->odat);
    delete p;
    return TP_OK;
}

extern "C" int tp_producer_id(const tp_producer *p) { return p ? p->id : TP_E_BAD_ARG; }

extern "C" int tp_producer_border(const tp_producer *p)
{
    if (!p) return TP_E_BAD_ARG;
    if (p->kind == kOrthoResidual) return p->ortho_border;  // OrthoCPUProducer.cpp:98, 145-148
    return p->kind == kNormal ? 0 : 2;  // ElevationProducer.cpp:235-239, NormalProducer.cpp:124-127, OrthoProducer.cpp:217-221
}

extern "C" int tp_producer_set_root_quad_size(tp_producer *p, float size)
{
    if (!p || !(size > 0.0f)) return tp::fail(TP_E_BAD_ARG, "tp_producer_set_root_quad_size: bad arguments");
    p->root_quad_size = size;
    if ((p->kind == kElevation || p->kind == kOrtho) && p->residuals) p->residuals->root_quad_size = size;
    if (p->kind == kNormal) tp_producer_set_root_quad_size(p->elevations, size);
    return TP_OK;
}

extern "C" int tp_producer_has_tile(const tp_producer *p, int level, int tx, int ty)
{
    if (!p) return TP_E_BAD_ARG;
    if (p->kind == kResidual) return residual_has_tile(p, level, tx, ty) ? 1 : 0;
    if (level < 0 || tx < 0 || ty < 0 || level > 30 || (tx >> level) != 0 || (ty >> level) != 0) return 0;
    if (p->kind == kOrthoResidual) return level <= p->ortho_max_level ? 1 : 0;  // OrthoCPUProducer.cpp:151-154
    if (p->kind == kOrtho) return p->max_level == -1 || level <= p->max_level ? 1 : 0;  // OrthoProducer.cpp:223-226
    if (p->kind == kNormal) return tp_producer_has_tile(p->elevations, level, tx, ty);
    return level >= 0 && tx >= 0 && ty >= 0 && (tx >> level) == 0 && (ty >> level) == 0 ? 1 : 0;
}

extern "C" tp_tile *tp_producer_get_tile(tp_producer *p, int level, int tx, int ty)
{
    if (!p || level < 0 || level > 30 || tx < 0 || ty < 0 || (tx >> level) != 0 || (ty >> level) != 0) {
        tp::fail(TP_E_BAD_ARG, "tp_producer_get_tile: bad arguments");
        return nullptr;
    }
    int err = TP_OK;
    return get_tile(p, level, tx, ty, nullptr, &err);
}

extern "C" tp_tile *tp_producer_find_tile(tp_producer *p, int level, int tx, int ty, int include_cache, int done)
{
    if (!p) return nullptr;
    tp_cache *c = p->cache;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    const TKey k = key_of(p, level, tx, ty);
    tp_tile *const *found = c->tiles.find(k);
    tp_tile *t = found ? *found : nullptr;
    if (t && !(t->users > 0 || include_cache)) t = nullptr;
    if (t && done && !t->done) t = nullptr;
    return t;
}

extern "C" int tp_producer_put_tile(tp_producer *p, tp_tile *t)
{
    if (!p || !t) return tp::fail(TP_E_BAD_ARG, "tp_producer_put_tile: tile not held");
    // the tile's owner and users are read under its cache's lock: other threads change
    // them (a queued tile releasing what it acquired, a recycled record)
    std::lock_guard<std::recursive_mutex> lk(p->cache->mu);
    if (t->producer_id != p->id || t->users <= 0) return tp::fail(TP_E_BAD_ARG, "tp_producer_put_tile: tile not held");
    return put_tile(p, t);
}

// TileCache::prefetchTile (TileCache.cpp:254-310): create the tile (queued for
// production) among the unused tiles; 1 if a tile was created, 0 if it exists
// or the cache is full.
extern "C" int tp_producer_prefetch_tile(tp_producer *p, int level, int tx, int ty)
{
    if (!p || level < 0 || level > 30 || tx < 0 || ty < 0 || (tx >> level) != 0 || (ty >> level) != 0)
        return tp::fail(TP_E_BAD_ARG, "tp_producer_prefetch_tile: bad arguments");
    tp_cache *c = p->cache;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    const TKey k = key_of(p, level, tx, ty);
    if (c->tiles.find(k)) return 0;
    int err = TP_OK;
    tp_tile *t = get_tile(p, level, tx, ty, nullptr, &err);
    if (!t) return err == TP_E_CACHE_FULL ? 0 : err;
    put_tile(p, t);  // keep it, unused, at the back of the LRU list
    return 1;
}

// TileCache::invalidateTiles (TileCache.cpp:338-377): every tile of the
// producer is produced again before its next use.
extern "C" int tp_producer_invalidate_tiles(tp_producer *p)
{
    if (!p) return tp::fail(TP_E_BAD_ARG, "tp_producer_invalidate_tiles: bad arguments");
    tp_cache *c = p->cache;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    // collected first: scheduling acquires tiles, which changes the table
    std::vector<tp_tile *> mine;
    c->tiles.for_each([&](tp_tile *t) {
        if (t->producer_id == p->id && t->users > 0) mine.push_back(t);
    });
    std::sort(mine.begin(), mine.end(), [](const tp_tile *x, const tp_tile *y) {
        return std::make_tuple(x->level, x->ty, x->tx) < std::make_tuple(y->level, y->ty, y->tx);
    });
    for (tp_tile *t : mine) {
        t->done = false;
        if (!t->queued) {
            int rc = schedule(p, t);
            if (rc) return rc;
        }
    }
    for (tp_tile *t = c->lru_head; t; t = t->lru_next)
        if (t->producer_id == p->id) t->done = false;
    return TP_OK;
}

extern "C" int tp_producer_queued(const tp_producer *p)
{
    if (!p) return TP_E_BAD_ARG;
    std::lock_guard<std::recursive_mutex> lk(p->cache->mu);  // queues change under the cache's lock
    return (int)p->queue.size();
}

// ResidualProducer::doCreateTile on a host tile: the residual tile (level, tx, ty)
// as the producer would upload it (width = the residual cache's tile width).
extern "C" int tp_residual_tile(tp_producer *p, int level, int tx, int ty, float *out, int width)
{
    if (!p || p->kind != kResidual || !out || width != p->cache->storage->W || level < 0 || level > 30 || tx < 0 ||
        ty < 0 || (tx >> level) != 0 || (ty >> level) != 0)
        return tp::fail(TP_E_BAD_ARG, "tp_residual_tile: bad arguments");
    tp_tile t;
    t.level = level;
    t.tx = tx;
    t.ty = ty;
    return produce_residual(p, &t, out);
}

extern "C" int tp_tile_info(const tp_tile *t, int *level, int *tx, int *ty, int *slot, int *users, int *done)
{
    if (!t) return tp::fail(TP_E_BAD_ARG, "tp_tile_info: tile is NULL");
    if (level) *level = t->level;
    if (tx) *tx = t->tx;
    if (ty) *ty = t->ty;
    if (slot) *slot = t->slot;
    if (users) *users = t->users;
    if (done) *done = t->done ? 1 : 0;
    return TP_OK;
}

// ---------------------------------------------------------------- scheduler
namespace {

// Residual tiles of a .dat file decoded on the device; the root of a delta chain
// (upsampled through the levels above the file's root) stays on the host.
int run_residuals_device(tp_producer *r, void *stream)
{
    tp_dat *d = r->dat;
    std::vector<int> lv, txs, tys, slots;
    std::vector<tp_tile *> host;
    for (tp_tile *t : r->queue) {
        const int level = t->level + r->delta - d->root_level;
        if (r->delta > 0 && level == r->delta) {
            host.push_back(t);
            continue;
        }
        const bool inside = level >= 0 && (t->tx >> level) == d->root_tx && (t->ty >> level) == d->root_ty &&
                            level <= d->max_level;
        lv.push_back(inside ? level : -1);
        txs.push_back(inside ? t->tx - (d->root_tx << level) : 0);
        tys.push_back(inside ? t->ty - (d->root_ty << level) : 0);
        slots.push_back(t->slot);
    }
    int rc = tp_dat_decode_device(d, lv.data(), txs.data(), tys.data(), (int)lv.size(), d->scale * r->zscale,
                                  r->cache->storage, slots.data(), stream);
    if (rc) return rc;
    if (!host.empty()) {
        tp_storage *s = r->cache->storage;
        const size_t per = (size_t)s->W * s->W;
        std::vector<float> buf(per * host.size());
        std::vector<int> hs;
        for (size_t k = 0; k < host.size(); ++k) {
            rc = produce_residual(r, host[k], buf.data() + k * per);
            if (rc) return rc;
            hs.push_back(host[k]->slot);
        }
        rc = tp::staged_copy_slots(s, hs.data(), (int)hs.size(), 0, buf.data(), stream);
        if (rc) return rc;
        cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
        if (e != cudaSuccess) return tp::cuda_fail("cudaStreamSynchronize (residual upload)", e);
    }
    for (tp_tile *t : r->queue) {
        t->done = true;
        t->queued = false;
    }
    r->queue.clear();
    return TP_OK;
}

int run_residuals_synthetic(tp_producer *r, void *stream)
{
    std::vector<int> slots, lv, txs, tys;
    std::vector<float> sig;
    for (tp_tile *t : r->queue) {
        slots.push_back(t->slot);
        lv.push_back(t->level);
        txs.push_back(t->tx);
        tys.push_back(t->ty);
        sig.push_back(synthetic_sigma(r, t->level));
    }
    int rc = tp::synthetic_residuals_device(r->cache->storage, r->syn_seed, slots.data(), lv.data(), txs.data(),
                                            tys.data(), sig.data(), (int)slots.size(), stream);
    if (rc) return rc;
    for (tp_tile *t : r->queue) {
        t->done = true;
        t->queued = false;
    }
    r->queue.clear();
    return TP_OK;
}

int run_residuals(tp_producer *r, void *stream)
{
    if (r->queue.empty()) return TP_OK;
    tp::TraceScope ts("residuals", tp::kPhResiduals);
    if (r->synthetic && r->cache->storage->on_device == 1) return run_residuals_synthetic(r, stream);
    if (r->dat && r->device_decode && r->cache->storage->on_device == 1) return run_residuals_device(r, stream);
    tp_storage *s = r->cache->storage;
    const int Wr = s->W;
    const size_t per = (size_t)Wr * Wr;
    std::vector<float> host(per * r->queue.size());
    std::vector<int> slots;
    for (size_t k = 0; k < r->queue.size(); ++k) {
        int rc = produce_residual(r, r->queue[k], host.data() + k * per);
        if (rc) return rc;
        slots.push_back(r->queue[k]->slot);
    }
    if (s->on_device == 1) {
        int rc = tp::staged_copy_slots(s, slots.data(), (int)slots.size(), 0, host.data(), stream);
        if (rc) return rc;
        // the host buffer must live until the copy has read it
        cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
        if (e != cudaSuccess) return tp::cuda_fail("cudaStreamSynchronize (residual upload)", e);
    }
    for (tp_tile *t : r->queue) {
        t->done = true;
        t->queued = false;
    }
    r->queue.clear();
    return TP_OK;
}

// The tp_tile_job of an elevation tile; `index` maps tiles of the same launch to
// their job numbers (a parent found there is named in parent_job).
// The job of tile t; a parent in the same launch (its `job` set) becomes the job's
// parent_job, any other parent must be produced already.
int elevation_job(const tp_producer *e, const tp_tile *t, int normal_slot, tp_tile_job &j)
{
    const int n = e->cache->storage->W - 5;
    const int mod = e->residuals ? (e->residuals->cache->storage->W - 5) / n : 1;
    std::memset(&j, 0, sizeof j);
    j.level = t->level;
    j.tx = t->tx;
    j.ty = t->ty;
    j.out_slot = t->slot;
    j.parent_slot = t->dep_parent ? t->dep_parent->slot : -1;
    j.parent_job = -1;
    if (t->dep_parent) {
        if (t->dep_parent->job >= 0) j.parent_job = t->dep_parent->job;
        else if (!t->dep_parent->done) return tp::fail(TP_E_MISSING_PARENT, "elevation parent tile is not produced");
    }
    j.residual_slot = t->dep_input ? t->dep_input->slot : -1;
    j.rx = (t->tx % mod) * n;
    j.ry = (t->ty % mod) * n;
    j.rscale = 1.0f;
    j.normal_slot = normal_slot;
    int rot = 0, layer = 0;
    tp_noise_select(e->face, t->level, t->tx, t->ty, &rot, &layer);
    j.noise_rot = rot;
    j.noise_layer = layer;
    j.noise_amp = t->level < (int)e->noise_amp.size() ? e->noise_amp[t->level] : 0.0f;
    j.tile_meters = e->root_quad_size / (float)(1u << t->level);
    return TP_OK;
}

// The layer pass of tiles just produced: each layer's meshes for each tile, drawn
// and blended into zm (ElevationProducer.cpp:383-399).
int run_layers(tp_producer *e, const std::vector<tp_tile *> &tiles, void *stream)
{
    tp::TraceScope ts("layers", tp::kPhLayers);
    tp_layer_builder b;
    std::vector<tp_layer_job> jobs(tiles.size());
    for (size_t k = 0; k < tiles.size(); ++k) {
        const tp_tile *t = tiles[k];
        jobs[k] = tp_layer_job{t->slot, (int32_t)b.meshes.size(), 0, 0};
        for (const auto &l : e->layers) {
            b.layer_start = true;
            b.program = TP_LAYER_ROAD;
            b.state = 0;
            b.fill_depth = 0.0f;
            if (l.first(l.second, t->level, t->tx, t->ty, &b) != 0)
                return tp::fail(TP_E_BAD_ARG, "elevation layer callback failed");
        }
        jobs[k].n_meshes = (int32_t)b.meshes.size() - jobs[k].first_mesh;
    }
    return tp_elevation_layers(e->cache->storage, jobs.data(), (int)jobs.size(), b.meshes.data(), (int)b.meshes.size(),
                               b.vertices.data(), (int)(b.vertices.size() / 4), b.indices.data(),
                               (int)b.indices.size(), e->blend_mode, stream);
}

void finish_tiles(const std::vector<tp_tile *> &tiles)
{
    for (tp_tile *t : tiles) {
        t->done = true;
        t->queued = false;
        release_deps(t);
    }
}

int run_elevations(tp_producer *e, tp_producer *normals, void *stream)
{
    // normal tiles whose elevation tile is produced by this same launch are fused in
    // (flat deformation; spherical normals run in their own kernel afterwards; a
    // producer with layers changes zm after its launch, so its normals come later)
    const bool layered = !e->layers.empty();
    // marks on the tiles (elevation tile -> its fused normal tile, tile -> job index),
    // cleared on every way out
    std::vector<tp_tile *> fused;  // elevation tiles with a fused normal tile
    std::vector<tp_tile *> q;
    struct Clear {
        std::vector<tp_tile *> &f, &q;
        ~Clear()
        {
            for (tp_tile *t : f) t->fused_normal = nullptr;
            for (tp_tile *t : q) t->job = -1;
        }
    } clear_marks{fused, q};
    if (!layered && normals && !normals->deform && normals->normal_format == 2)
        for (tp_tile *nt : normals->queue)
            if (nt->dep_input && nt->dep_input->queued && !nt->dep_input->fused_normal) {
                nt->dep_input->fused_normal = nt;
                fused.push_back(nt->dep_input);
            }
    if (e->queue.empty()) return TP_OK;
    if (!(e->root_quad_size > 0.0f)) return tp::fail(TP_E_BAD_ARG, "elevation producer: root quad size not set");
    q = e->queue;
    std::stable_sort(q.begin(), q.end(), [](const tp_tile *a, const tp_tile *b) { return a->level < b->level; });
    if (!e->frame) tp_frame_create(&e->frame);
    if (layered) {
        // level by level: a level's launch, then its layer pass, then the next level
        size_t k = 0;
        int rc = TP_OK;
        while (k < q.size() && rc == TP_OK) {
            size_t k1 = k;
            while (k1 < q.size() && q[k1]->level == q[k]->level) ++k1;
            std::vector<tp_tile *> lvl(q.begin() + k, q.begin() + k1);
            std::vector<tp_tile_job> jobs(lvl.size());
            for (size_t i = 0; i < lvl.size() && rc == TP_OK; ++i) rc = elevation_job(e, lvl[i], -1, jobs[i]);
            if (rc == TP_OK) {
                tp_frame_clear(e->frame);
                rc = tp_frame_add(e->frame, e->cache->storage,
                                  e->residuals ? e->residuals->cache->storage : nullptr, nullptr, &e->params,
                                  jobs.data(), (int)jobs.size());
            }
            if (rc == TP_OK) rc = tp_frame_launch(e->frame, stream);
            if (rc == TP_OK) rc = run_layers(e, lvl, stream);
            if (rc == TP_OK) finish_tiles(lvl);
            k = k1;
        }
        std::vector<tp_tile *> rest;
        for (tp_tile *t : e->queue)
            if (!t->done) rest.push_back(t);
        e->queue.swap(rest);
        return rc;
    }
    std::vector<tp_tile_job> jobs(q.size());
    {
        tp::TraceScope ts("elevation jobs", tp::kPhElevJobs);
        for (size_t k = 0; k < q.size(); ++k) q[k]->job = (int)k;
        for (size_t k = 0; k < q.size(); ++k) {
            int rc = elevation_job(e, q[k], q[k]->fused_normal ? q[k]->fused_normal->slot : -1, jobs[k]);
            if (rc) return rc;
        }
    }
    {
        tp::TraceScope ts("frame setup", tp::kPhFrameSetup);
        tp_frame_clear(e->frame);
        int rc = tp_frame_add(e->frame, e->cache->storage, e->residuals ? e->residuals->cache->storage : nullptr,
                              normals && !fused.empty() ? normals->cache->storage : nullptr, &e->params, jobs.data(),
                              (int)jobs.size());
        if (rc) return rc;
    }
    {
        tp::TraceScope ts("elevation launch", tp::kPhFrameLaunch);
        int rc = tp_frame_launch(e->frame, stream);
        if (rc) return rc;
    }
    tp::TraceScope ts("finish", tp::kPhFinish);
    finish_tiles(q);
    e->queue.clear();
    if (normals) {
        std::vector<tp_tile *> rest;
        for (tp_tile *nt : normals->queue) {
            if (nt->dep_input && nt->dep_input->fused_normal == nt) {
                nt->done = true;
                nt->queued = false;
                release_deps(nt);
            } else {
                rest.push_back(nt);
            }
        }
        normals->queue.swap(rest);
    }
    return TP_OK;
}

// Normal tiles in a format other than 2 (coarse normals from the parent normal
// tile): one launch per level, parents first.
int run_normals_format(tp_producer *np, void *stream)
{
    tp_producer *e = np->elevations;
    std::vector<tp_tile *> q = np->queue;
    std::stable_sort(q.begin(), q.end(), [](const tp_tile *a, const tp_tile *b) { return a->level < b->level; });
    size_t k = 0;
    while (k < q.size()) {
        const int level = q[k]->level;
        std::vector<int> eslot, nslot, pslot, txs, tys;
        std::vector<float> meters, p2t;
        std::vector<tp::SphereFrame> frames;
        for (; k < q.size() && q[k]->level == level; ++k) {
            tp_tile *t = q[k];
            if (!t->dep_input || !t->dep_input->done)
                return tp::fail(TP_E_MISSING_PARENT, "normal tile's elevation is not produced");
            eslot.push_back(t->dep_input->slot);
            nslot.push_back(t->slot);
            pslot.push_back(t->dep_parent ? t->dep_parent->slot : -1);
            txs.push_back(t->tx);
            tys.push_back(t->ty);
            meters.push_back(e->root_quad_size / (float)(1u << t->level));
            if (np->deform) {
                frames.emplace_back();
                tp::sphere_frame(e->root_quad_size, t->level, t->tx, t->ty, &frames.back());
                p2t.resize(p2t.size() + 9, 0.0f);
                if (t->level > 0) tp::parent_to_tangent(e->root_quad_size, t->level, t->tx, t->ty, &p2t[p2t.size() - 9]);
            }
        }
        int rc = tp::launch_normals_format(e->cache->storage, np->cache->storage, eslot.data(), nslot.data(),
                                           meters.data(), pslot.data(), txs.data(), tys.data(), (int)eslot.size(),
                                           np->normal_format, np->grid_mesh, stream,
                                           np->deform ? frames.data() : nullptr, np->deform ? p2t.data() : nullptr);
        if (rc) return rc;
    }
    for (tp_tile *t : np->queue) {
        t->done = true;
        t->queued = false;
        release_deps(t);
    }
    np->queue.clear();
    return TP_OK;
}

int run_normals(tp_producer *np, void *stream)
{
    tp::TraceScope ts("normals", tp::kPhNormals);
    if (np->queue.empty()) return TP_OK;
    tp_producer *e = np->elevations;
    if (!(e->root_quad_size > 0.0f)) return tp::fail(TP_E_BAD_ARG, "normal producer: root quad size not set");
    if (np->normal_format != 2) return run_normals_format(np, stream);
    std::vector<int> eslot, nslot;
    std::vector<float> meters;
    std::vector<tp::SphereFrame> frames;
    for (tp_tile *t : np->queue) {
        if (!t->dep_input || !t->dep_input->done) return tp::fail(TP_E_MISSING_PARENT, "normal tile's elevation is not produced");
        eslot.push_back(t->dep_input->slot);
        nslot.push_back(t->slot);
        meters.push_back(e->root_quad_size / (float)(1u << t->level));
        if (np->deform) {
            frames.emplace_back();
            tp::sphere_frame(e->root_quad_size, t->level, t->tx, t->ty, &frames.back());
        }
    }
    int rc = tp::launch_normals(e->cache->storage, np->cache->storage, eslot.data(), nslot.data(), meters.data(),
                                (int)eslot.size(), stream, np->deform ? frames.data() : nullptr);
    if (rc) return rc;
    for (tp_tile *t : np->queue) {
        t->done = true;
        t->queued = false;
        release_deps(t);
    }
    np->queue.clear();
    return TP_OK;
}

// OrthoCPUProducer::doCreateTile (OrthoCPUProducer.cpp:170-236): decoded tiles (or zeros
// without a file) as RGBA8 texels, uploaded to their slots in one copy.
int run_ortho_residuals(tp_producer *r, void *stream)
{
    if (r->queue.empty()) return TP_OK;
    tp_storage *s = r->cache->storage;
    const size_t per = (size_t)s->W * s->W;
    std::vector<uint32_t> host(per * r->queue.size(), 0u);
    std::vector<int> slots;
    for (size_t k = 0; k < r->queue.size(); ++k) {
        const tp_tile *t = r->queue[k];
        if (r->odat) {
            int w = 0;
            int rc = tp_ortho_dat_read_rgba(r->odat, t->level, t->tx, t->ty, host.data() + k * per, (int)per, &w);
            if (rc) return rc;
        }
        slots.push_back(t->slot);
    }
    if (s->on_device == 1) {
        int rc = tp::staged_copy_slots(s, slots.data(), (int)slots.size(), 0,
                                       reinterpret_cast<const float *>(host.data()), stream);
        if (rc) return rc;
        cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
        if (e != cudaSuccess) return tp::cuda_fail("cudaStreamSynchronize (ortho residual upload)", e);
    }
    for (tp_tile *t : r->queue) {
        t->done = true;
        t->queued = false;
    }
    r->queue.clear();
    return TP_OK;
}

// OrthoProducer::doCreateTile (OrthoProducer.cpp:292-382) of every queued tile: one
// persistent ortho launch, parents before children.
int run_orthos(tp_producer *o, void *stream)
{
    if (o->queue.empty()) return TP_OK;
    std::vector<tp_tile *> q = o->queue;
    std::stable_sort(q.begin(), q.end(), [](const tp_tile *a, const tp_tile *b) { return a->level < b->level; });
    std::map<const tp_tile *, int> index;
    for (size_t k = 0; k < q.size(); ++k) index[q[k]] = (int)k;
    std::vector<tp_ortho_job> jobs(q.size());
    for (size_t k = 0; k < q.size(); ++k) {
        const tp_tile *t = q[k];
        tp_ortho_job &j = jobs[k];
        std::memset(&j, 0, sizeof j);
        j.level = t->level;
        j.tx = t->tx;
        j.ty = t->ty;
        j.out_slot = t->slot;
        j.parent_slot = t->dep_parent ? t->dep_parent->slot : -1;
        j.parent_job = -1;
        if (t->dep_parent) {
            auto it = index.find(t->dep_parent);
            if (it != index.end()) j.parent_job = it->second;
            else if (!t->dep_parent->done) return tp::fail(TP_E_MISSING_PARENT, "ortho parent tile is not produced");
        }
        j.residual_slot = t->dep_input ? t->dep_input->slot : -1;
        tp_noise_select(o->face, t->level, t->tx, t->ty, &j.noise_rot, &j.noise_layer);
        j.noise_amp = t->level < (int)o->noise_amp.size() ? o->noise_amp[t->level] : 0.0f;
    }
    int rc = tp_ortho_batch(o->cache->storage, o->residuals ? o->residuals->cache->storage : nullptr, &o->oparams,
                            jobs.data(), (int)jobs.size(), stream);
    if (rc) return rc;
    for (tp_tile *t : q) {
        t->done = true;
        t->queued = false;
        release_deps(t);
    }
    o->queue.clear();
    return TP_OK;
}

}  // namespace

// Produces every queued tile of the given producers (and of the producers they
// use): residuals, then elevations (with fused normals), then other normals.
extern "C" int tp_scheduler_run(tp_producer *const *producers, int n, void *stream)
{
    if (n < 0 || (n > 0 && !producers)) return tp::fail(TP_E_BAD_ARG, "tp_scheduler_run: bad arguments");
    std::vector<tp_producer *> res, elev, nrm, ores, orth;
    auto add = [](std::vector<tp_producer *> &v, tp_producer *p) {
        if (p && std::find(v.begin(), v.end(), p) == v.end()) v.push_back(p);
    };
    for (int k = 0; k < n; ++k) {
        tp_producer *p = producers[k];
        if (!p) continue;
        if (p->kind == kOrtho) {
            add(orth, p);
            if (p->residuals) add(ores, p->residuals);
            continue;
        }
        if (p->kind == kOrthoResidual) {
            add(ores, p);
            continue;
        }
        if (p->kind == kNormal) {
            add(nrm, p);
            p = p->elevations;
        }
        if (p->kind == kElevation) {
            add(elev, p);
            p = p->residuals;
        }
        if (p && p->kind == kResidual) add(res, p);
    }
    for (tp_producer *r : res) {
        int rc = run_residuals(r, stream);
        if (rc) return rc;
    }
    for (tp_producer *e : elev) {
        tp_producer *fuse = nullptr;
        for (tp_producer *np : nrm)
            if (np->elevations == e) {
                fuse = np;
                break;
            }
        int rc = run_elevations(e, fuse, stream);
        if (rc) return rc;
    }
    for (tp_producer *np : nrm) {
        int rc = run_normals(np, stream);
        if (rc) return rc;
    }
    for (tp_producer *r : ores) {
        int rc = run_ortho_residuals(r, stream);
        if (rc) return rc;
    }
    for (tp_producer *o : orth) {
        int rc = run_orthos(o, stream);
        if (rc) return rc;
    }
    return TP_OK;
}

namespace tp {

// parentToTangentFrame (NormalProducer.cpp:256-270): the tile's world-to-tangent frame
// times the tangent-to-world frame at its parent's centre, in FP64, row-major floats.
void parent_to_tangent(double D, int level, int tx, int ty, float *p2t)
{
    auto frame = [&](double cx, double cy, double m[3][3]) {
        const double R = D / 2.0;
        const double l = std::sqrt(cx * cx + cy * cy + R * R);
        const double uz[3] = {cx / l, cy / l, R / l};
        const double a[3] = {uz[2], 0.0, -uz[0]};  // (0, 1, 0) x uz
        const double la = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        const double ux[3] = {a[0] / la, a[1] / la, a[2] / la};
        const double uy[3] = {uz[1] * ux[2] - uz[2] * ux[1], uz[2] * ux[0] - uz[0] * ux[2], uz[0] * ux[1] - uz[1] * ux[0]};
        for (int c = 0; c < 3; ++c) {
            m[0][c] = ux[c];
            m[1][c] = uy[c];
            m[2][c] = uz[c];
        }
    };
    const double R = D / 2.0, s = (double)(1u << level), ps = (double)(1u << (level > 0 ? level - 1 : 0));
    double w[3][3], t[3][3];
    frame(((double)tx + 0.5) / s * D - R, ((double)ty + 0.5) / s * D - R, w);
    frame(((double)(tx / 2) + 0.5) / ps * D - R, ((double)(ty / 2) + 0.5) / ps * D - R, t);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)  // w * t^T: t's rows are the parent's tangent axes
            p2t[r * 3 + c] = (float)(w[r][0] * t[c][0] + w[r][1] * t[c][1] + w[r][2] * t[c][2]);
}

// NormalProducer.cpp:215-273: the tile's corners on the sphere of radius
// R = D / 2 (D the root quad size) centred below the face, their unit verticals and
// distances, and the rotation into the tangent frame at the tile centre.
void sphere_frame(double D, int level, int tx, int ty, SphereFrame *f)
{
    const double R = D / 2.0, s = (double)(1u << level);
    const double x0 = (double)tx / s * D - R, x1 = (double)(tx + 1) / s * D - R;
    const double y0 = (double)ty / s * D - R, y1 = (double)(ty + 1) / s * D - R;
    const double P[4][3] = {{x0, y0, R}, {x1, y0, R}, {x0, y1, R}, {x1, y1, R}};
    double v[4][3], l[4], vc[3] = {0, 0, 0};
    for (int k = 0; k < 4; ++k) {
        l[k] = std::sqrt(P[k][0] * P[k][0] + P[k][1] * P[k][1] + P[k][2] * P[k][2]);
        for (int c = 0; c < 3; ++c) {
            v[k][c] = P[k][c] / l[k];
            vc[c] += v[k][c];
        }
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
    const double pc[3] = {(x0 + x1) * 0.5, (y0 + y1) * 0.5, R};
    const double lc = std::sqrt(pc[0] * pc[0] + pc[1] * pc[1] + pc[2] * pc[2]);
    const double uz[3] = {pc[0] / lc, pc[1] / lc, pc[2] / lc};
    const double t[3] = {uz[2], 0.0, -uz[0]};  // (0, 1, 0) x uz
    const double lt = std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    const double ux[3] = {t[0] / lt, t[1] / lt, t[2] / lt};
    const double uy[3] = {uz[1] * ux[2] - uz[2] * ux[1], uz[2] * ux[0] - uz[0] * ux[2], uz[0] * ux[1] - uz[1] * ux[0]};
    for (int c = 0; c < 3; ++c) {
        f->W2T[c] = (float)ux[c];
        f->W2T[3 + c] = (float)uy[c];
        f->W2T[6 + c] = (float)uz[c];
    }
    f->R = (float)R;
    f->size = (float)(D / s);
}

}  // namespace tp

// A queued, unproduced tile that nobody uses any more: its task is dropped and the
// tiles it was to be made from are released (and dropped in turn when orphaned).
static void cancel_orphan(tp_producer *p, tp_tile *t)
{
    if (!p || !t || t->users != 0 || t->done || !t->queued) return;
    auto &q = p->queue;
    q.erase(std::remove(q.begin(), q.end(), t), q.end());
    t->queued = false;
    tp_tile *deps[2] = {t->dep_parent, t->dep_input};
    tp_producer *owners[2] = {t->dep_parent_owner, t->dep_input_owner};
    release_deps(t);
    for (int k = 0; k < 2; ++k) cancel_orphan(owners[k], deps[k]);
}

// The frame form of TileProducer's per-tile protocol (TileProducer.h:331-378: one
// CreateTile task per getTile, each running doCreateTile): every requested tile is
// acquired as getTile does, then all queued tiles of the producer (with their
// inputs) are produced in one scheduler run.  Each returned tile holds one user,
// released with tp_producer_put_tile.  On failure the tiles acquired by this call
// are released and none is returned.
extern "C" int tp_create_tiles(tp_producer *p, const tp_tile_req *reqs, int n, tp_tile **tiles_out, void *stream)
{
    if (!p || n < 0 || (n > 0 && (!reqs || !tiles_out))) return tp::fail(TP_E_BAD_ARG, "tp_create_tiles: bad arguments");
    for (int i = 0; i < n; ++i) {
        const tp_tile_req &r = reqs[i];
        if (r.level < 0 || r.level > 30 || r.tx < 0 || r.ty < 0 || (r.tx >> r.level) != 0 || (r.ty >> r.level) != 0)
            return tp::fail(TP_E_BAD_ARG, "tp_create_tiles: bad quadtree coordinates");
    }
    int rc = TP_OK;
    int got = 0;
    for (; got < n; ++got) {
        tiles_out[got] = get_tile(p, reqs[got].level, reqs[got].tx, reqs[got].ty, nullptr, &rc);
        if (!tiles_out[got]) break;
    }
    if (got == n) {
        tp_producer *all[1] = {p};
        rc = tp_scheduler_run(all, 1, stream);
        if (rc == TP_OK) return TP_OK;
    }
    if (rc == TP_OK) rc = TP_E_CACHE_FULL;
    const std::string msg = tp_last_error();
    for (int i = 0; i < got; ++i) {
        put_tile(p, tiles_out[i]);
        cancel_orphan(p, tiles_out[i]);
        tiles_out[i] = nullptr;
    }
    return tp::fail(rc, msg);
}

// doCreateTile of one tile (level, tx, ty): tp_create_tiles with one request.
extern "C" int tp_create_tile(tp_producer *p, int level, int tx, int ty, tp_tile **tile_out, void *stream)
{
    const tp_tile_req r = {level, tx, ty};
    return tp_create_tiles(p, &r, 1, tile_out, stream);
}

// ---------------------------------------------------------------- sampler
// The TileSamplers of one terrain node (TileSampler::getTiles, TileSampler.cpp:416-461):
// one user held on each producer's tile of every quad of the current quadtree; per
// update, the tiles of quads that disappeared are released (to the caches' LRUs), the
// new quads' tiles acquired (getTile, in request order: parents first; producers in
// the order given) and all produced by one scheduler run, so that normal tiles of
// new elevation tiles are fused into the elevation launch.
// A quad key's hash (splitmix64's finaliser).
struct QuadHash {
    size_t operator()(uint64_t x) const
    {
        x ^= x >> 31;
        x *= 0xbf58476d1ce4e5b9ull;
        x ^= x >> 29;
        x *= 0x94d049bb133111ebull;
        x ^= x >> 32;
        return (size_t)x;
    }
};

struct tp_sampler {
    static constexpr int kMaxProducers = 8;
    struct Quad {
        uint64_t key;
        uint64_t walk;   // its place in TileSampler's walk of the quadtree (walk_order)
        uint32_t stamp;  // the last update whose quadtree held it
        tp_tile *tiles[kMaxProducers];
    };
    std::vector<tp_producer *> producers;
    std::vector<Quad> held;                        // dense: released quads swap with the last one
    FlatTable<uint64_t, uint32_t, QuadHash> index{0xFFFFFFFFu};  // quad key -> position in `held`
    uint32_t frame = 0;
    std::vector<tp_tile_req> fresh;  // the last update's new quads
};

namespace {
uint64_t req_key(int level, int tx, int ty)
{
    return ((uint64_t)level << 58) | ((uint64_t)(uint32_t)tx << 29) | (uint64_t)(uint32_t)ty;
}

// The place of a quad in the walk TileSampler::putTiles / getTiles make over a quadtree
// (TileSampler.cpp:385-461): the root, then each child's subtree in index order
// (tx & 1) + 2 (ty & 1), a parent before its children.  Sorting by this key orders
// releases and acquisitions as the reference does, so that its caches' LRU lists
// receive the tiles in the same order and evict the same tiles.
// The key: the child indices from the root, 2 bits per level left-aligned (the bits of
// tx and ty interleaved, tx in the low bit of each pair), then the level.
uint64_t spread_bits(uint32_t v)   // bit i of v -> bit 2i
{
    uint64_t x = v;
    x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
    x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
    x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}

uint64_t walk_order(uint64_t key)
{
    const int level = (int)(key >> 58);
    const uint32_t tx = (uint32_t)(key >> 29) & 0x1FFFFFFFu, ty = (uint32_t)key & 0x1FFFFFFFu;
    const uint64_t path = (spread_bits(tx) | (spread_bits(ty) << 1)) << (2 * (29 - level));
    return (path << 5) | (uint64_t)level;
}

void sampler_drop(tp_sampler *s, size_t pos, bool cancel)
{
    tp_sampler::Quad &q = s->held[pos];
    for (size_t p = 0; p < s->producers.size(); ++p) {
        put_tile(s->producers[p], q.tiles[p]);
        if (cancel) cancel_orphan(s->producers[p], q.tiles[p]);
    }
    s->index.erase(q.key);
    if (pos + 1 != s->held.size()) {
        q = s->held.back();
        *s->index.find(q.key) = (uint32_t)pos;
    }
    s->held.pop_back();
}
}  // namespace

extern "C" int tp_sampler_create(tp_producer *const *producers, int n, tp_sampler **out)
{
    if (!producers || n < 1 || n > tp_sampler::kMaxProducers || !out)
        return tp::fail(TP_E_BAD_ARG, "tp_sampler_create: bad arguments");
    for (int i = 0; i < n; ++i)
        if (!producers[i]) return tp::fail(TP_E_BAD_ARG, "tp_sampler_create: a producer is NULL");
    *out = new tp_sampler;
    (*out)->producers.assign(producers, producers + n);
    (*out)->index.reserve(16384);
    return TP_OK;
}

extern "C" int tp_sampler_destroy(tp_sampler *s)
{
    if (!s) return TP_OK;
    for (auto &q : s->held)
        for (size_t i = 0; i < s->producers.size(); ++i) put_tile(s->producers[i], q.tiles[i]);
    delete s;
    return TP_OK;
}

extern "C" int tp_sampler_update(tp_sampler *s, const tp_tile_req *reqs, int n, void *stream, int *new_count)
{
    if (!s || n < 0 || (n > 0 && !reqs)) return tp::fail(TP_E_BAD_ARG, "tp_sampler_update: bad arguments");
    for (int i = 0; i < n; ++i) {
        const tp_tile_req &r = reqs[i];
        if (r.level < 0 || r.level > 29 || r.tx < 0 || r.ty < 0 || (r.tx >> r.level) != 0 || (r.ty >> r.level) != 0)
            return tp::fail(TP_E_BAD_ARG, "tp_sampler_update: bad quadtree coordinates");
    }
    const size_t np = s->producers.size();
    const uint32_t frame = ++s->frame;
    std::vector<int> fresh_idx;
    {
        // quads kept: stamped; quads that disappeared: their tiles go back to the caches
        // first, so that their slots can take the new tiles, in the walk order of
        // TileSampler::putTiles
        tp::TraceScope ts("sampler release", tp::kPhSamplerRelease);
        for (int i = 0; i < n; ++i) {
            const uint32_t *at = s->index.find(req_key(reqs[i].level, reqs[i].tx, reqs[i].ty));
            if (at) s->held[*at].stamp = frame;
            else fresh_idx.push_back(i);
        }
        std::vector<std::pair<uint64_t, uint64_t> > gone;   // (walk order, quad key)
        for (const tp_sampler::Quad &q : s->held)
            if (q.stamp != frame) gone.emplace_back(q.walk, q.key);
        std::sort(gone.begin(), gone.end());
        for (const auto &g : gone) sampler_drop(s, *s->index.find(g.second), false);
    }
    // the new quads acquired in the same walk order (a request list lists children near
    // to far); reported in request order
    std::vector<std::pair<uint64_t, int> > walk;   // (walk order, request index)
    walk.reserve(fresh_idx.size());
    for (int i : fresh_idx) walk.emplace_back(walk_order(req_key(reqs[i].level, reqs[i].tx, reqs[i].ty)), i);
    std::sort(walk.begin(), walk.end());
    s->fresh.clear();
    const size_t kept = s->held.size();
    int rc = TP_OK;
    {
        tp::TraceScope ts("sampler acquire", tp::kPhSamplerAcquire);
        for (const auto &w : walk) {
            const tp_tile_req &r = reqs[w.second];
            const uint64_t k = req_key(r.level, r.tx, r.ty);
            if (s->index.find(k)) continue;  // requested twice
            tp_sampler::Quad q;
            q.key = k;
            q.walk = w.first;
            q.stamp = frame;
            size_t got = 0;
            for (; got < np; ++got) {
                q.tiles[got] = get_tile(s->producers[got], r.level, r.tx, r.ty, nullptr, &rc);
                if (!q.tiles[got]) break;
            }
            if (got < np) {
                if (rc == TP_OK) rc = tp::fail(TP_E_CACHE_FULL, "tp_sampler_update: tile cache full");
                for (size_t p = 0; p < got; ++p) {
                    put_tile(s->producers[p], q.tiles[p]);
                    cancel_orphan(s->producers[p], q.tiles[p]);
                }
                break;
            }
            s->index.insert(k, (uint32_t)s->held.size());
            s->held.push_back(q);
        }
    }
    if (rc == TP_OK) {
        std::vector<char> reported(s->held.size() - kept, 0);   // each new quad once, in request order
        for (int i : fresh_idx) {
            const uint32_t *at = s->index.find(req_key(reqs[i].level, reqs[i].tx, reqs[i].ty));
            if (at && *at >= kept && !reported[*at - kept]) {
                reported[*at - kept] = 1;
                s->fresh.push_back(reqs[i]);
            }
        }
    }
    if (rc == TP_OK) rc = tp_scheduler_run(s->producers.data(), (int)np, stream);
    if (rc != TP_OK) {
        // no tile of this update stays acquired (the new quads sit after `kept`)
        const std::string msg = tp_last_error();
        while (s->held.size() > kept) sampler_drop(s, s->held.size() - 1, true);
        s->fresh.clear();
        return tp::fail(rc, msg);
    }
    if (new_count) *new_count = (int)s->fresh.size();
    return TP_OK;
}

extern "C" int tp_sampler_new_tiles(const tp_sampler *s, tp_tile_req *out, int capacity)
{
    if (!s || capacity < 0 || (capacity > 0 && !out)) return tp::fail(TP_E_BAD_ARG, "tp_sampler_new_tiles: bad arguments");
    const int n = (int)s->fresh.size();
    std::copy(s->fresh.begin(), s->fresh.begin() + std::min(n, capacity), out);
    return n;
}

extern "C" int tp_sampler_held(const tp_sampler *s) { return s ? (int)s->held.size() : TP_E_BAD_ARG; }

extern "C" tp_tile *tp_sampler_find(const tp_sampler *s, int producer, int level, int tx, int ty)
{
    if (!s || producer < 0 || producer >= (int)s->producers.size() || level < 0 || level > 29 || tx < 0 || ty < 0)
        return nullptr;
    const uint32_t *at = s->index.find(req_key(level, tx, ty));
    return at ? s->held[*at].tiles[producer] : nullptr;
}

extern "C" int tp_sphere_frame(double root_quad_size, int level, int tx, int ty, float *out47)
{
    if (!out47 || !(root_quad_size > 0.0) || level < 0 || level > 30) return tp::fail(TP_E_BAD_ARG, "tp_sphere_frame: bad arguments");
    tp::SphereFrame f;
    tp::sphere_frame(root_quad_size, level, tx, ty, &f);
    static_assert(sizeof(f) == 47 * sizeof(float), "frame layout");
    std::memcpy(out47, &f, sizeof f);
    return TP_OK;
}
