"""TileCache / TileProducer protocol on bookkeeping-only storages (no GPU):
users counts, the LRU of unused tiles and slot recycling, a full cache, the
tiles a producer's task acquires, prefetch.  Semantics of TileCache.cpp:150-377
and TileProducer.cpp:454-464, ElevationProducer.cpp:246-271,
NormalProducer.cpp:139-156."""
import pytest

BOOK = 2  # TileStorage.BOOKKEEPING


def elev_setup(tp, capacity=8, residual_capacity=8, Wr=101):
    es = tp.TileStorage(101, 3, capacity, on_device=BOOK)
    ec = tp.TileCache(es, "elevations")
    rs = tp.TileStorage(Wr, 1, residual_capacity, on_device=BOOK)
    rc = tp.TileCache(rs, "residuals")
    r = tp.ResidualProducer(rc)
    e = tp.ElevationProducer(ec, r, noise_amp=[-140.0, -100.0], params=tp.make_params())
    return es, ec, rs, rc, r, e


def test_users_and_unused_list(product):
    tp = product
    es, ec, rs, rc, r, e = elev_setup(tp)
    t = e.get_tile(0, 0, 0)
    assert t.info()["users"] == 1 and t.info()["done"] == 0
    assert e.get_tile(0, 0, 0).handle == t.handle
    assert t.info()["users"] == 2
    assert e.put_tile(t) == 1
    assert ec.get_used_tiles() == 1 and ec.get_unused_tiles() == 0
    assert e.put_tile(t) == 0
    assert ec.get_used_tiles() == 0 and ec.get_unused_tiles() == 1
    # still cached: findTile sees it only with includeCache
    assert e.find_tile(0, 0, 0) is None
    assert e.find_tile(0, 0, 0, include_cache=True).handle == t.handle
    # not produced yet: findTile(..., done=True) does not return it
    assert e.find_tile(0, 0, 0, include_cache=True, done=True) is None
    assert e.get_border() == 2 and r.get_border() == 2


def test_task_acquires_parent_and_residual(product):
    tp = product
    es, ec, rs, rc, r, e = elev_setup(tp)
    t = e.get_tile(2, 3, 1)
    # the tile, its parent (1, 1, 0) and grandparent (0, 0, 0) are used and queued
    assert ec.get_used_tiles() == 3
    assert e.queued() == 3
    for lvl, x, y, users in [(2, 3, 1, 1), (1, 1, 0, 1), (0, 0, 0, 1)]:
        f = e.find_tile(lvl, x, y)
        assert f is not None and f.info()["users"] == users
    # each queued elevation tile holds its residual tile (mod 1: same coordinates)
    assert rc.get_used_tiles() == 3 and r.queued() == 3
    # a sibling shares the parent: one more user on it
    e.get_tile(2, 2, 1)
    assert e.find_tile(1, 1, 0).info()["users"] == 2
    assert t.info()["users"] == 1


def test_residual_window_uses_the_residual_quadtree(product):
    tp = product
    es, ec, rs, rc, r, e = elev_setup(tp, Wr=197)  # mod 2: one residual tile per 2x2 elevation tiles
    for x, y in [(2, 2), (3, 2), (2, 3), (3, 3)]:
        e.get_tile(2, x, y)
    f = r.find_tile(2, 1, 1)
    assert f is not None and f.info()["users"] == 4


def test_lru_recycles_oldest_unused_slot(product):
    tp = product
    es = tp.TileStorage(101, 3, 3, on_device=BOOK)
    ec = tp.TileCache(es, "elevations")
    e = tp.ElevationProducer(ec, None, params=tp.make_params())
    a = e.get_tile(0, 0, 0)
    slot_a = a.slot
    e.put_tile(a)
    b = e.get_tile(1, 0, 0)          # holds (0, 0, 0) as its parent again
    assert e.find_tile(0, 0, 0).info()["users"] == 1
    c = e.get_tile(1, 1, 0)
    assert es.get_free_slots() == 0
    for t in (b, c):
        e.put_tile(t)
    # (1,0,0) and (1,1,0) are unused (in that order); (0,0,0) stays used by nobody?
    # no: their tasks still hold the parent until produced
    assert e.find_tile(0, 0, 0).info()["users"] == 2
    q0, m0 = ec.stats()
    d = e.get_tile(1, 0, 1)          # no free slot: recycles (1, 0, 0), the oldest unused
    assert d is not None
    assert e.find_tile(1, 0, 0, include_cache=True) is None
    assert e.find_tile(1, 1, 0, include_cache=True) is not None
    q1, m1 = ec.stats()
    assert q1 == q0 + 1 and m1 == m0 + 1
    assert slot_a in range(3)


def test_full_cache_returns_null(product):
    tp = product
    es = tp.TileStorage(101, 3, 2, on_device=BOOK)
    ec = tp.TileCache(es, "elevations")
    e = tp.ElevationProducer(ec, None, params=tp.make_params())
    a = e.get_tile(1, 0, 0)           # takes both slots: (1,0,0) and its parent
    assert a is not None
    assert e.get_tile(1, 1, 1) is None
    assert product.lib().tp_last_error().decode().startswith("Insufficient tile cache size")


def test_prefetch_and_normals(product):
    tp = product
    es, ec, rs, rc, r, e = elev_setup(tp)
    ns = tp.TileStorage(97, 2, 8, on_device=BOOK)
    nc = tp.TileCache(ns, "normals")
    n = tp.NormalProducer(nc, e)
    assert n.get_border() == 0
    assert n.has_tile(3, 5, 1)
    assert e.prefetch_tile(0, 0, 0) == 1
    assert e.prefetch_tile(0, 0, 0) == 0
    assert ec.get_unused_tiles() == 1 and e.queued() == 1
    t = n.get_tile(1, 1, 1)
    # a normal tile holds its elevation tile and its parent normal tile
    assert nc.get_used_tiles() == 2 and n.queued() == 2
    assert e.find_tile(1, 1, 1).info()["users"] == 1
    assert e.find_tile(0, 0, 0).info()["users"] >= 1   # revived from the unused list
    assert t.info()["level"] == 1


def test_bad_arguments(product):
    tp = product
    es, ec, rs, rc, r, e = elev_setup(tp)
    assert e.get_tile(2, 4, 0) is None   # tx outside level 2
    with pytest.raises(tp.TPError):
        e.prefetch_tile(-1, 0, 0)
    with pytest.raises(tp.TPError):
        tp.NormalProducer(ec, e)         # 3-channel cache: not a normal cache


def test_random_operations_match_a_model(product):
    """A long random sequence of getTile / putTile on a small cache (many evictions,
    re-used keys, tiles evicted while still queued) against a model of TileCache's
    semantics: users counts, the LRU order of unused tiles, recycling the oldest
    unused tile when no slot is free, NULL when every tile is used."""
    import random
    tp = product
    cap = 24
    rs = tp.TileStorage(101, 1, cap, on_device=BOOK)
    rc = tp.TileCache(rs, "residuals")
    r = tp.ResidualProducer(rc)
    rng = random.Random(7)
    keys = [(l, x, y) for l in (3, 4) for x in range(6) for y in range(6)]
    users, lru, held = {}, [], []      # model: key -> users; unused keys, oldest first
    for step in range(4000):
        if held and (rng.random() < 0.45 or len(held) >= cap):
            t, key = held.pop(rng.randrange(len(held)))
            left = r.put_tile(t)
            users[key] -= 1
            assert left == users[key]
            if users[key] == 0:
                lru.append(key)
        else:
            key = rng.choice(keys)
            t = r.get_tile(*key)
            if key in users:
                if users[key] == 0:
                    lru.remove(key)
                users[key] += 1
            elif len(users) < cap:
                users[key] = 1
            elif lru:
                del users[lru.pop(0)]          # the oldest unused tile gives its slot
                users[key] = 1
            else:
                assert t is None
                continue
            assert t is not None and t.info()["users"] == users[key], (step, key)
            held.append((t, key))
        if step % 97 == 0:
            assert rc.get_used_tiles() == sum(1 for u in users.values() if u > 0)
            assert rc.get_unused_tiles() == len(lru)
            for k in keys:
                f = r.find_tile(*k, include_cache=True)
                assert (f is not None) == (k in users), (step, k)
                if f is not None:
                    assert f.info()["users"] == users[k]
    for t, _ in held:
        r.put_tile(t)
    assert rc.get_used_tiles() == 0
