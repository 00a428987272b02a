"""Elevation layers on the GPU: road meshes drawn into produced elevation tiles and
blended into zm (tp_elevation_layers), bit for bit against the oracle, for 101- and
197-wide tiles (the wide ones in several row bands) and both blend programs; then a
layered elevation producer, whose tiles are made level by level so that children
read their parents' blended zm, against the oracle chained over the levels."""
import numpy as np
import pytest

from tilecase import assert_normals_close

pytestmark = pytest.mark.gpu
ROOT = 100000.0


def tile_meshes(rng, W, k):
    """A mix of the mesh forms a layer draws: road strips, indexed triangle lists,
    plain strips, a depth clear on an empty mesh."""
    from proland_gb300 import layers
    meshes = []
    if k % 4 == 3:
        return meshes
    size = 1000.0
    for r in range(1 + k % 3):
        a = rng.uniform(-200, 1200, 2)
        b = rng.uniform(-200, 1200, 2)
        mid = (a + b) / 2 + rng.uniform(-150, 150, 2)
        v = layers.road_strip([a, mid, b], rng.uniform(-50, 300, 3), float(rng.uniform(5, 40)), (0.0, 0.0), size, W)
        meshes.append((v, None, 1, r == 0))
    nv = 12
    v = np.column_stack([rng.uniform(-1.1, 1.1, nv), rng.uniform(-1.1, 1.1, nv), rng.uniform(0, 400, nv),
                         rng.uniform(-3, 3, nv)]).astype(np.float32)
    meshes.append((v, rng.integers(0, nv, 18).astype(np.uint32), 0, False))
    meshes.append((np.zeros((0, 4), np.float32), None, 0, True))     # a layer that draws nothing
    meshes.append((v[:7], None, 1, False))
    return meshes


@pytest.mark.parametrize("W", [101, 197])
@pytest.mark.parametrize("blend_mode", [0, 1])
def test_layers_match_oracle(gpu, oracle_lib, W, blend_mode):
    tp = gpu
    rng = np.random.default_rng(W * 10 + blend_mode)
    n = 8
    zf = (rng.standard_normal((n, W, W)) * 200.0).astype(np.float32)
    zc = (rng.standard_normal((n, W, W)) * 200.0).astype(np.float32)
    zm = np.maximum(zf, np.float32(0.0))
    elev = tp.TileStorage(W, 3, n + 2)
    slots = [(3 * k + 1) % (n + 2) for k in range(n)]
    for k, s in enumerate(slots):
        elev.upload(s, tp.ZF, zf[k:k + 1])
        elev.upload(s, tp.ZC, zc[k:k + 1])
        elev.upload(s, tp.ZM, zm[k:k + 1])
    meshes = [tile_meshes(rng, W, k) for k in range(n)]
    tp.elevation_layers(elev, list(zip(slots, meshes)), blend_mode)
    tp.stream_check()
    changed = 0
    for k, s in enumerate(slots):
        want = oracle_lib.layer_tile(W, zf[k], zm[k], meshes[k], blend_mode)
        got = elev.download(s, 1, tp.ZM)[0]
        assert np.array_equal(got, want), "tile %d (W %d, blend %d)" % (k, W, blend_mode)
        assert np.array_equal(elev.download(s, 1, tp.ZF)[0], zf[k])
        assert np.array_equal(elev.download(s, 1, tp.ZC)[0], zc[k])
        changed += int(not np.array_equal(got, zm[k]))
    assert changed >= n // 2


def test_layers_reject_bad_meshes(gpu):
    tp = gpu
    elev = tp.TileStorage(101, 3, 2)
    v = np.zeros((3, 4), np.float32)
    with pytest.raises(tp.TPError):
        tp.elevation_layers(elev, [(0, [(v, np.array([0, 1, 3], np.uint32), 0, True)])])
    with pytest.raises(tp.TPError):
        tp.elevation_layers(elev, [(5, [(v, None, 0, True)])])
    with pytest.raises(tp.TPError):
        tp.elevation_layers(elev, [(0, [(v, None, 7, True)])])


ROAD = np.array([[-30000.0, -12000.0], [-5000.0, 2000.0], [8000.0, 1000.0], [30000.0, 15000.0]])
ROAD_Z = np.array([120.0, 80.0, 40.0, 200.0])


def road_layer(level, tx, ty, W):
    from proland_gb300 import layers
    size = ROOT / (1 << level)
    origin = (ROOT * (tx / (1 << level) - 0.5), ROOT * (ty / (1 << level) - 0.5))
    return [(layers.road_strip(ROAD, ROAD_Z, 300.0, origin, size, W), None, 1)]


@pytest.mark.parametrize("blend_mode", [0, 1])
def test_layered_producer_levels(gpu, oracle_lib, blend_mode):
    tp, orc = gpu, oracle_lib
    W = 101
    es = tp.TileStorage(W, 3, 64)
    rs = tp.TileStorage(W, 1, 64)
    ns = tp.TileStorage(W - 4, 2, 64)
    ec, rc, nc = tp.TileCache(es, "e"), tp.TileCache(rs, "r"), tp.TileCache(ns, "n")

    def residual(level, tx, ty, width):
        g = np.random.default_rng(7919 * level + 31 * tx + ty)
        return (g.standard_normal((width, width)) * 900.0 * 0.5 ** level).astype(np.float32)
    r = tp.ResidualProducer(rc, source=residual)
    amps = [-60.0, -30.0, 12.0, -6.0]
    e = tp.ElevationProducer(ec, r, noise_amp=amps, params=tp.make_params(), face=1)
    e.add_layer(lambda l, x, y: road_layer(l, x, y, W))
    e.set_blend(blend_mode)
    nrm = tp.NormalProducer(nc, e)
    nrm.set_root_quad_size(ROOT)
    wanted = [(3, x, y) for x in range(2, 6) for y in range(3, 6)]
    held = [nrm.get_tile(*t) for t in wanted]
    assert all(h is not None for h in held)
    tp.scheduler_run([nrm])
    tp.stream_check()
    assert e.queued() == 0 and nrm.queued() == 0
    tree = set()
    for (l, x, y) in wanted:
        while l >= 0:
            tree.add((l, x, y))
            l, x, y = l - 1, x // 2, y // 2
    table = orc.dem_noise(W)
    want = {}
    for (l, x, y) in sorted(tree):
        p = want.get((l - 1, x // 2, y // 2))
        rot, layer = orc.noise_select(1, l, x, y)
        zf, zc, zm = orc.elevation_tile(W, l, x, y, p[0] if p else None, p[2] if p else None, residual(l, x, y, W),
                                        noise=table[layer], noise_rot=rot, noise_amp=amps[l])
        meshes = [(v, ix, mode, True) for v, ix, mode in road_layer(l, x, y, W)]
        want[(l, x, y)] = (zf, zc, orc.layer_tile(W, zf, zm, meshes, blend_mode))
    roads = 0
    for t in sorted(tree):
        et = e.find_tile(*t, include_cache=True, done=True)
        assert et is not None, t
        for ch, name in ((tp.ZF, "zf"), (tp.ZC, "zc"), (tp.ZM, "zm")):
            got = es.download(et.slot, 1, ch)[0]
            assert np.array_equal(got, want[t][ch]), "%s of %s" % (name, t)
        zf, _, zm = want[t]
        roads += int(not np.array_equal(zm, np.maximum(zf, 0)))
    assert roads >= 4
    for h, t in zip(held, wanted):
        enx, eny = orc.normals_flat(W, want[t][2], ROOT / (1 << t[0]))
        assert_normals_close(ns.download(h.slot, 1, tp.NX)[0], enx, "nx %s" % (t,))
        assert_normals_close(ns.download(h.slot, 1, tp.NY)[0], eny, "ny %s" % (t,))


def test_device_meshes_same_as_host(gpu, oracle_lib):
    """tp_elevation_layers_device reads the meshes from device memory: the same tiles;
    an index past the vertex array drops its triangle there."""
    import torch
    tp = gpu
    W, n = 101, 4
    rng = np.random.default_rng(11)
    zf = (rng.standard_normal((n, W, W)) * 200.0).astype(np.float32)
    zm = np.maximum(zf, np.float32(0.0))
    elev = tp.TileStorage(W, 3, n)
    meshes = [tile_meshes(rng, W, k) for k in range(n)]
    batch = tp.LayerBatch(list(zip(range(n), meshes)))
    outs = []
    for run in (lambda: batch.run(elev), lambda: batch.to_device(torch).run_device(elev)):
        elev.upload(0, tp.ZF, zf)
        elev.upload(0, tp.ZM, zm)
        run()
        tp.stream_check()
        outs.append(elev.download(0, n, tp.ZM))
    assert np.array_equal(outs[0], outs[1])
    for k in range(n):
        assert np.array_equal(outs[0][k], oracle_lib.layer_tile(W, zf[k], zm[k], meshes[k], 0))
    # one triangle whose third index is out of range, next to a valid one
    v = np.array([[-0.5, -0.5, 50, 0], [0.5, -0.5, 50, 0], [0.0, 0.5, 50, 0]], np.float32)
    bad = tp.LayerBatch([(0, [(v, np.array([0, 1, 2, 0, 1, 3], np.uint32), tp.TRIANGLES, True)])])
    bad.to_device(torch)
    elev.upload(0, tp.ZF, zf[:1])
    elev.upload(0, tp.ZM, zm[:1])
    bad.run_device(elev)
    tp.stream_check()
    want = oracle_lib.layer_tile(W, zf[0], zm[0], [(v, np.array([0, 1, 2], np.uint32), 0, True)], 0)
    assert np.array_equal(elev.download(0, 1, tp.ZM)[0], want)
