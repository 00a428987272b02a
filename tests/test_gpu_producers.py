"""The TileCache / TileProducer path end to end on the GPU: tiles requested
with getTile, produced by tp_scheduler_run (residuals on the host, elevations
and fused normals in one launch, parents first), compared with the oracle run
tile by tile.  Includes the reference's DEM.dat residual pyramid with delta."""
import os

import numpy as np
import pytest

from tilecase import assert_normals_close

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ROOT = 100000.0


def download(storage, slot, channel):
    return storage.download(slot, 1, channel)[0]


def synthetic_residual(level, tx, ty, width):
    rng = np.random.default_rng(1000003 * level + 1009 * tx + ty)
    return (rng.standard_normal((width, width)) * 2000.0 * 0.5 ** level).astype(np.float32)


def oracle_tree(orc, tiles, W, noise_amp, face, residual_of, mod=1):
    """Oracle elevations of `tiles` (parents first), as {tile: (zf, zc, zm)}."""
    table = orc.dem_noise(W)
    n = W - 5
    out = {}
    for (l, x, y) in sorted(tiles):
        p = out.get((l - 1, x // 2, y // 2))
        rot, layer = orc.noise_select(face, l, x, y)
        amp = noise_amp[l] if l < len(noise_amp) else 0.0
        res = residual_of(l, x // mod, y // mod)
        out[(l, x, y)] = orc.elevation_tile(W, l, x, y, p[0] if p else None, p[2] if p else None, res,
                                            rx=(x % mod) * n, ry=(y % mod) * n, noise=table[layer],
                                            noise_rot=rot, noise_amp=amp)
    return out


def test_quadtree_through_producers(gpu, oracle_lib):
    tp, orc = gpu, oracle_lib
    W = 101
    es = tp.TileStorage(W, 3, 128)
    rs = tp.TileStorage(W, 1, 128)
    ns = tp.TileStorage(W - 4, 2, 128)
    ec, rc, nc = tp.TileCache(es, "e"), tp.TileCache(rs, "r"), tp.TileCache(ns, "n")
    r = tp.ResidualProducer(rc, source=synthetic_residual)
    amps = [-140.0, -100.0, -15.0, -8.0, 5.0]
    e = tp.ElevationProducer(ec, r, noise_amp=amps, params=tp.make_params(), face=1)
    nrm = tp.NormalProducer(nc, e)
    nrm.set_root_quad_size(ROOT)
    wanted = [(3, x, y) for x in range(8) for y in range(8) if (x + y) % 3 == 0]
    held = [nrm.get_tile(*t) for t in wanted]
    assert all(h is not None for h in held)
    tp.scheduler_run([nrm])
    tp.stream_check()
    assert e.queued() == 0 and nrm.queued() == 0 and r.queued() == 0
    tree = set()
    for (l, x, y) in wanted:
        while l >= 0:
            tree.add((l, x, y))
            l, x, y = l - 1, x // 2, y // 2
    want = oracle_tree(orc, tree, W, amps, 1, lambda l, x, y: synthetic_residual(l, x, y, W))
    for t in sorted(tree):
        et = e.find_tile(*t, include_cache=True, done=True)
        assert et is not None, t
        zf = download(es, et.slot, tp.ZF)
        zc = download(es, et.slot, tp.ZC)
        assert np.array_equal(zf, want[t][0]), t
        assert np.array_equal(zc, want[t][1]), t
    for h, t in zip(held, wanted):
        enx, eny = orc.normals_flat(W, want[t][2], ROOT / (1 << t[0]))
        assert_normals_close(download(ns, h.slot, tp.NX), enx, "nx %s" % (t,))
        assert_normals_close(download(ns, h.slot, tp.NY), eny, "ny %s" % (t,))
    # a normal tile requested after its elevation tile was produced (normals-only kernel)
    late = nrm.get_tile(2, 1, 1)
    tp.scheduler_run([nrm])
    tp.stream_check()
    enx, _ = orc.normals_flat(W, want[(2, 1, 1)][2], ROOT / 4)
    assert_normals_close(download(ns, late.slot, tp.NX), enx, "late nx")


def test_eviction_and_reproduction(gpu, oracle_lib):
    """A cache too small for the frame recycles unused tiles; asking again for an
    evicted tile produces it again, with the same bits."""
    tp, orc = gpu, oracle_lib
    W = 101
    es = tp.TileStorage(W, 3, 6)
    rs = tp.TileStorage(W, 1, 6)
    ec, rc = tp.TileCache(es, "e"), tp.TileCache(rs, "r")
    r = tp.ResidualProducer(rc, source=synthetic_residual)
    e = tp.ElevationProducer(ec, r, params=tp.make_params())
    e.set_root_quad_size(ROOT)
    first = e.get_tile(2, 0, 0)
    tp.scheduler_run([e])
    zf0 = download(es, first.slot, tp.ZF)
    e.put_tile(first)
    for x in range(1, 4):            # push (2,0,0) out of the cache
        t = e.get_tile(2, x, 3)
        tp.scheduler_run([e])
        e.put_tile(t)
    again = e.get_tile(2, 0, 0)
    assert again.info()["done"] in (0, 1)
    tp.scheduler_run([e])
    tp.stream_check()
    assert np.array_equal(download(es, again.slot, tp.ZF), zf0)
    want = oracle_tree(orc, {(0, 0, 0), (1, 0, 0), (2, 0, 0)}, W, [], 0,
                       lambda l, x, y: synthetic_residual(l, x, y, W))
    assert np.array_equal(zf0, want[(2, 0, 0)][0])


@pytest.mark.parametrize("device_decode", [False, True])
def test_dem_dat_residuals_terrain4_layout(gpu, oracle_lib, device_decode):
    """101-wide elevations over the reference's 197-wide residual pyramid with
    delta 2 (terrain/examples/terrain4/helloworld.xml): mod 2 residual windows;
    residual tiles decoded on the host or on the device."""
    tp, orc = gpu, oracle_lib
    path = os.path.join(GOLDEN, "dem_edit3_mini.dat")
    es = tp.TileStorage(101, 3, 32)
    rs = tp.TileStorage(197, 1, 8)
    ec, rc = tp.TileCache(es, "e"), tp.TileCache(rs, "r")
    r = tp.ResidualProducer(rc, path, delta=2, zscale=0.1, device_decode=device_decode)
    e = tp.ElevationProducer(ec, r, params=tp.make_params(), face=0)
    e.set_root_quad_size(ROOT)
    assert r.has_tile(0, 0, 0) and r.has_tile(1, 0, 0) and r.has_tile(2, 1, 1)
    tiles = [(1, x, y) for x in range(2) for y in range(2)]
    held = [e.get_tile(*t) for t in tiles]
    tp.scheduler_run([e])
    tp.stream_check()
    # the residual tiles as the producer computes them on the host (pinned to the
    # reference decode by test_dat_and_inflate)
    res = {}
    for (l, x, y) in [(0, 0, 0), (1, 0, 0)]:
        res[(l, x, y)] = r.tile(l, x, y)
    want = oracle_tree(orc, {(0, 0, 0)} | set(tiles), 101, [], 0, lambda l, x, y: res[(l, x, y)], mod=2)
    for h, t in zip(held, tiles):
        assert np.array_equal(download(es, h.slot, tp.ZF), want[t][0]), t


@pytest.mark.parametrize("face", [1, 3])
def test_planet_face_sphere_normals(gpu, oracle_lib, face):
    """Normals of a spherically deformed face (NormalProducer deform, terrain2
    normal shader) against the oracle's sphere normals, from the same elevations."""
    tp, orc = gpu, oracle_lib
    W = 197
    D = 2.0 * 6360000.0
    es = tp.TileStorage(W, 3, 64)
    rs = tp.TileStorage(W, 1, 64)
    ns = tp.TileStorage(W - 4, 2, 64)
    ec, rc, nc = tp.TileCache(es, "e"), tp.TileCache(rs, "r"), tp.TileCache(ns, "n")
    r = tp.ResidualProducer(rc, source=synthetic_residual)
    amps = [300.0 * 0.55 ** l for l in range(12)]
    e = tp.ElevationProducer(ec, r, noise_amp=amps, params=tp.make_params(), face=face)
    n = tp.NormalProducer(nc, e, deform=True)
    n.set_root_quad_size(D)
    wanted = [(0, 0, 0), (3, 5, 2), (6, 40, 17)]
    held = [n.get_tile(*t) for t in wanted]
    tp.scheduler_run([n])
    tp.stream_check()
    for h, t in zip(held, wanted):
        et = e.find_tile(*t, include_cache=True, done=True)
        zm = download(es, et.slot, tp.ZM)
        f = orc.sphere_frame(D, *t)
        enx, eny = orc.normals_sphere(W, zm, f)
        assert_normals_close(download(ns, h.slot, tp.NX), enx, "sphere nx %s" % (t,))
        assert_normals_close(download(ns, h.slot, tp.NY), eny, "sphere ny %s" % (t,))


def test_create_tiles_frame_form_and_cache_full(gpu, oracle_lib):
    """tp_create_tiles / tp_create_tile (the batched doCreateTile): produced tiles
    equal the oracle's; a request that overflows the cache fails with
    TP_E_CACHE_FULL and leaves none of its tiles acquired."""
    tp, orc = gpu, oracle_lib
    W = 101
    es, rs = tp.TileStorage(W, 3, 64), tp.TileStorage(W, 1, 64)
    ec, rc = tp.TileCache(es, "e"), tp.TileCache(rs, "r")
    r = tp.ResidualProducer(rc, source=synthetic_residual)
    amps = [-140.0, -100.0, -15.0]
    e = tp.ElevationProducer(ec, r, noise_amp=amps, params=tp.make_params(), face=0)
    e.set_root_quad_size(ROOT)
    reqs = [(2, 1, 3), (2, 2, 3), (1, 0, 1)]
    tiles = e.create_tiles(reqs)
    one = e.create_tile(2, 3, 0)
    tree = set()
    for (l, x, y) in reqs + [(2, 3, 0)]:
        while l >= 0:
            tree.add((l, x, y))
            l, x, y = l - 1, x // 2, y // 2
    want = oracle_tree(orc, tree, W, amps, 0, lambda l, x, y: synthetic_residual(l, x, y, W))
    for t, h in zip(reqs + [(2, 3, 0)], tiles + [one]):
        info = h.info()
        assert info["done"] == 1 and info["users"] >= 1 and (info["level"], info["tx"], info["ty"]) == t
        assert np.array_equal(download(es, h.slot, tp.ZF), want[t][0]), t
    for h in tiles + [one]:
        e.put_tile(h)
    # a 4-slot cache cannot hold six level-2 tiles and their parents
    small = tp.TileStorage(W, 3, 4)
    sc = tp.TileCache(small, "small")
    e2 = tp.ElevationProducer(sc, r, noise_amp=amps, params=tp.make_params(), face=0)
    e2.set_root_quad_size(ROOT)
    with pytest.raises(tp.TPError) as err:
        e2.create_tiles([(2, x, y) for x in range(3) for y in range(2)])
    assert err.value.code == tp.TP_E_CACHE_FULL
    assert sc.get_used_tiles() == 0
