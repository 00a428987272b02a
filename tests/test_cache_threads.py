"""The host API from several threads at once (one mutex per cache, TileCache.cpp's
lock): 8 threads acquire and release tiles of a shared elevation producer on a cache
too small for the quadtree, so that recycling and full-cache answers happen under
contention.  Bookkeeping-only storages: no GPU.  Checks that nothing fails or
crashes, that every held tile stays valid while held, and that the slot accounting
adds up afterwards."""
import random
import threading

BOOK = 2


def test_concurrent_get_and_put(product):
    tp = product
    cap = 48
    es = tp.TileStorage(101, 3, cap, on_device=BOOK)
    ec = tp.TileCache(es, "elevations")
    rs = tp.TileStorage(101, 1, cap, on_device=BOOK)
    rc = tp.TileCache(rs, "residuals")
    r = tp.ResidualProducer(rc)
    e = tp.ElevationProducer(ec, r, noise_amp=[-140.0, -100.0], params=tp.make_params())
    errors = []
    stats = {"got": 0, "full": 0}
    lock = threading.Lock()

    def worker(seed):
        rnd = random.Random(seed)
        held = []
        try:
            for _ in range(1500):
                if held and (len(held) > 6 or rnd.random() < 0.45):
                    t, key = held.pop(rnd.randrange(len(held)))
                    info = t.info()
                    if (info["level"], info["tx"], info["ty"]) != key or info["users"] < 1:
                        errors.append("held tile changed: %s vs %s" % (info, key))
                    e.put_tile(t)
                    continue
                level = rnd.randrange(0, 4)
                key = (level, rnd.randrange(1 << level), rnd.randrange(1 << level))
                t = e.get_tile(*key)
                with lock:
                    if t is None:
                        stats["full"] += 1
                    else:
                        stats["got"] += 1
                if t is not None:
                    held.append((t, key))
            for t, _ in held:
                e.put_tile(t)
        except Exception as ex:  # noqa: BLE001
            errors.append(repr(ex))

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(8)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors[:5]
    assert stats["got"] > 1000
    used, unused = ec.get_used_tiles(), ec.get_unused_tiles()
    assert used + unused + es.get_free_slots() == cap
    assert rc.get_used_tiles() + rc.get_unused_tiles() + rs.get_free_slots() == cap
    # whatever is still used is held by queued tiles' tasks: cancelling the queue
    # (invalidateTiles) leaves nothing used
    e.invalidate_tiles()
    assert ec.get_used_tiles() + ec.get_unused_tiles() + es.get_free_slots() == cap
