"""The TileSampler bookkeeping (tp_sampler_*) and the synthetic residual source on
bookkeeping-only storages (no GPU): a frame's new tiles are acquired, vanished
quads' tiles released to the LRU, a full cache leaves no tile of the failed update
acquired; synthetic tiles made on the host equal the oracle's restatement and have
the stated mean and deviation."""
import numpy as np
import pytest

import oracle

BOOK = 2


def residual_setup(tp, capacity):
    rs = tp.TileStorage(101, 1, capacity, on_device=BOOK)
    rc = tp.TileCache(rs, "residuals")
    r = tp.ResidualProducer(rc, synthetic=(2000.0, 0.5, 17))
    return rs, rc, r


def quad(level_max, cx, cy):
    """A small quadtree refined towards tile (level_max, cx, cy): parents first."""
    out = [(0, 0, 0)]
    for l in range(1, level_max + 1):
        px, py = cx >> (level_max - l + 1), cy >> (level_max - l + 1)
        for dy in range(2):
            for dx in range(2):
                out.append((l, 2 * px + dx, 2 * py + dy))
    return out


def test_sampler_acquires_new_and_releases_vanished(product):
    tp = product
    rs, rc, r = residual_setup(tp, 64)
    s = tp.TileSampler(r)
    a = quad(4, 3, 5)
    new = s.update(a)
    assert new == a and s.held() == len(a) and rc.get_used_tiles() == len(a)
    b = quad(4, 12, 9)
    new = s.update(b)
    assert new == [t for t in b if t not in set(a)]
    assert s.held() == len(b) and rc.get_used_tiles() == len(b)
    # the vanished tiles are in the LRU, still cached
    assert rc.get_unused_tiles() == len(set(a) - set(b))
    assert s.find(*b[-1]) is not None and s.find(*a[-1]) is None
    # the same quadtree again: nothing new
    assert s.update(b) == []
    s.close()
    assert rc.get_used_tiles() == 0


def test_sampler_full_cache_keeps_nothing_of_the_update(product):
    tp = product
    rs, rc, r = residual_setup(tp, 20)
    s = tp.TileSampler(r)
    a = quad(3, 1, 2)                       # 13 tiles
    s.update(a)
    big = quad(5, 30, 7)                    # 21 tiles, 5 shared with a
    with pytest.raises(tp.TPError) as e:
        s.update(big)
    assert e.value.code == tp.TP_E_CACHE_FULL
    kept = [t for t in a if t in set(big)]
    assert s.held() == len(kept) and rc.get_used_tiles() == len(kept)
    s.close()


def test_synthetic_residuals_host_match_oracle(product):
    tp = product
    rs, rc, r = residual_setup(tp, 4)
    for level, tx, ty in ((0, 0, 0), (3, 5, 2), (11, 2047, 1), (14, 9000, 16000)):
        sigma = np.float32(2000.0 * 0.5 ** level)
        got = r.tile(level, tx, ty)
        want = oracle.synthetic_residual(17, level, tx, ty, float(sigma), 101)
        assert np.array_equal(got, want), (level, tx, ty)
        z = want.astype(np.float64) / float(sigma)
        assert abs(z.mean()) < 0.05 and abs(z.std() - 1.0) < 0.03 and np.abs(z).max() <= 6.0
    # different tiles and seeds give different samples
    assert not np.array_equal(r.tile(3, 5, 2), r.tile(3, 5, 3))
    assert not np.array_equal(oracle.synthetic_residual(17, 3, 5, 2, 1.0, 101),
                              oracle.synthetic_residual(18, 3, 5, 2, 1.0, 101))


def test_sampler_random_updates(product):
    """Random quadtrees, one update each: the new quads are exactly those not held
    before (in request order), every requested quad is found afterwards and no other."""
    import random
    tp = product
    rs, rc, r = residual_setup(tp, 512)
    s = tp.TileSampler(r)
    rng = random.Random(3)
    universe = [(l, x, y) for l in range(5) for x in range(1 << l) for y in range(1 << l)]
    before = set()
    for step in range(60):
        req = []
        for _ in range(rng.randrange(1, 40)):
            l, x, y = rng.choice(universe)
            while l >= 0:
                req.append((l, x, y))
                l, x, y = l - 1, x // 2, y // 2
        want_new, seen = [], set()
        for t in req:
            if t not in before and t not in seen:
                want_new.append(t)
            seen.add(t)
        assert s.update(req) == want_new, step
        assert s.held() == len(seen) and rc.get_used_tiles() == len(seen)
        for t in universe:
            assert (s.find(*t) is not None) == (t in seen), (step, t)
        before = seen
    s.close()
    assert rc.get_used_tiles() == 0
