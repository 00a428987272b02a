"""The product's TileCache against the reference's own, compiled here by
oracle/ref_build.py: TileCache.cpp's getTile, putTile, findTile, prefetchTile and
TileStorage.cpp's slot list as written (TileCache.cpp:150-336,
TileStorage.cpp:36-122), over a storage whose slots are created in index order,
driven step by step beside the product's cache (tp_producer_get_tile / put_tile /
find_tile / prefetch_tile on bookkeeping-only storages) by random sequences: two
producers sharing one cache, a few tile keys reused often, capacities 3-8 so that
the cache fills and evicts.  After every step both agree on:

* whether getTile answered NULL (the cache full, no unused tile to evict), and the
  tile's users before the call;
* the slot each tile holds, up to one fixed renaming of slots (so the same least
  recently used tile is evicted each time);
* findTile with and without the unused tiles, prefetchTile's effect, putTile's
  users left, the used / unused tile counts and the storage's free slots.

Runs where the reference tree is present; skipped elsewhere."""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref(oracle_lib):
    L = oracle_lib.ref_lib()
    if L is None or not hasattr(L, "ref_cache_create"):
        pytest.skip("the reference sources are not on this machine")
    return L


@pytest.mark.parametrize("seed", range(12))
def test_cache_steps_match_reference(ref, product, seed):
    tp = product
    rng = np.random.default_rng(seed)
    capacity = 3 + seed % 6
    ref.ref_cache_create(capacity, 2)
    storage = tp.TileStorage(101, 1, capacity, on_device=tp.TileStorage.BOOKKEEPING)
    cache = tp.TileCache(storage, "tiles")
    prods = [tp.ResidualProducer(cache), tp.ResidualProducer(cache)]
    keys = [(lv, x, y) for lv in range(3) for x in range(1 << lv) for y in range(1 << lv)]
    held, pairing, fulls = [], {}, 0
    for step in range(800):
        op = int(rng.integers(0, 10))
        pid = int(rng.integers(0, 2))
        lv, x, y = keys[int(rng.integers(0, len(keys)))]
        where = (seed, step, op, pid, lv, x, y)
        if op < 4 or not held:
            users = C.c_int()
            rs = ref.ref_cache_get(pid, lv, x, y, C.byref(users))
            t = prods[pid].get_tile(lv, x, y)
            assert (rs < 0) == (t is None), where
            if t is None:
                fulls += 1
                continue
            info = t.info()
            assert info["users"] == users.value + 1, where
            assert pairing.setdefault(rs, info["slot"]) == info["slot"], where
            held.append((pid, lv, x, y, t))
        elif op < 7:
            pid, lv, x, y, t = held.pop(int(rng.integers(0, len(held))))
            assert ref.ref_cache_put(pid, lv, x, y) == prods[pid].put_tile(t), where
        elif op < 9:
            inc = bool(rng.integers(0, 2))
            rs = ref.ref_cache_find(pid, lv, x, y, int(inc))
            t = prods[pid].find_tile(lv, x, y, include_cache=inc)
            assert (rs < 0) == (t is None), where
            assert t is None or pairing.get(rs) == t.slot, where
        else:
            created = ref.ref_cache_prefetch(pid, lv, x, y)
            assert created == prods[pid].prefetch_tile(lv, x, y), where
            if created:
                rs = ref.ref_cache_find(pid, lv, x, y, 1)
                ps = prods[pid].find_tile(lv, x, y, include_cache=True).slot
                assert pairing.setdefault(rs, ps) == ps, where
        used, unused, free = C.c_int(), C.c_int(), C.c_int()
        ref.ref_cache_counts(C.byref(used), C.byref(unused), C.byref(free))
        assert (used.value, unused.value) == (cache.get_used_tiles(), cache.get_unused_tiles()), where
        assert free.value == storage.get_free_slots(), where
    for pid, lv, x, y, t in held:
        prods[pid].put_tile(t)
    assert len(pairing) == capacity      # every slot was handed out
    assert fulls > 0 or capacity > 6     # small caches filled up


@pytest.mark.parametrize("seed", range(6))
def test_tile_dependencies_match_reference(ref, product, seed):
    """The tiles a tile's task holds while it waits: ElevationProducer::startCreateTile
    (the parent elevation tile and the residual tile (level, tx / mod, ty / mod), mod the
    residual / elevation size ratio) and NormalProducer::startCreateTile (the parent
    normal tile and the elevation tile), as written, run by the reference's TileCache
    when it creates a tile (TileProducer::createTile calls startCreateTile) -- against
    the product's producers on bookkeeping-only storages: after every getTile of an
    elevation or normal tile, the used and unused counts of the residual, elevation and
    normal caches agree, and at the end the users of every requested tile, its parent
    and the residual and elevation tiles of its place."""
    tp = product
    rng = np.random.default_rng(seed)
    W, RW, cap = 101, (101, 197)[seed % 2], 400
    ref.ref_deps_create(W, RW, cap)
    rc = tp.TileCache(tp.TileStorage(RW, 1, cap, on_device=tp.TileStorage.BOOKKEEPING), "residuals")
    ec = tp.TileCache(tp.TileStorage(W, 3, cap, on_device=tp.TileStorage.BOOKKEEPING), "elevations")
    nc = tp.TileCache(tp.TileStorage(W - 4, 2, cap, on_device=tp.TileStorage.BOOKKEEPING), "normals")
    r = tp.ResidualProducer(rc)
    e = tp.ElevationProducer(ec, r, params=tp.make_params())
    n = tp.NormalProducer(nc, e)
    prods, caches, asked = [r, e, n], [rc, ec, nc], set()
    for step in range(150):
        k = int(rng.choice([1, 2, 2]))
        lv = int(rng.integers(0, 6))
        x, y = int(rng.integers(0, 1 << lv)), int(rng.integers(0, 1 << lv))
        assert ref.ref_deps_get(k, lv, x, y) == 0 and prods[k].get_tile(lv, x, y) is not None
        asked.add((k, lv, x, y))
        for c in range(3):
            used, unused = C.c_int(), C.c_int()
            ref.ref_deps_counts(c, C.byref(used), C.byref(unused))
            assert (used.value, unused.value) == (caches[c].get_used_tiles(), caches[c].get_unused_tiles()), \
                (seed, step, c)
    mod = (RW - 5) // (W - 5)
    for k, lv, x, y in sorted(asked):
        for c, (l2, x2, y2) in ((k, (lv, x, y)), (k, (lv - 1, x // 2, y // 2)), (0, (lv, x // mod, y // mod)),
                                (1, (lv, x, y))):
            if l2 < 0:
                continue
            f = prods[c].find_tile(l2, x2, y2, include_cache=True)
            assert ref.ref_deps_users(c, l2, x2, y2) == (f.info()["users"] if f is not None else -1), \
                (k, lv, x, y, c, l2, x2, y2)
