"""The water elevation layer on the GPU (tp_elevation_layers with fragment programs
and pass states), bit for bit against the oracle's in-order restatement:

* tiles drawn with the pass sequence of WaterElevationLayer::doCreateTile
  (proland_gb300.layers.water_layer: lake fill, boundaries, other curves under
  NOTEQUAL, rivers with caps under LESS), 101- and 197-wide (several row bands),
  both blend programs;
* adversarial passes: many overlapping triangles of equal depth under every
  supported state (ALWAYS and LESS without depth writes keep the last fragment,
  LESS with depth writes the first of least depth, NOTEQUAL against depths written
  by earlier passes), programs mixed within a pass, z / w masks, clears between
  passes, road and water meshes in one tile;
* the same meshes from device memory;
* a layered elevation producer whose callback draws the water layer (with
  tp_layer_builder_set_pass), chained over the levels."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LESS, ALWAYS, NOTEQUAL = 0, 1, 2
NO_DEPTH, NO_Z, NO_W = 4, 8, 16
STATES = [LESS, LESS | NO_DEPTH, LESS | NO_W, ALWAYS, ALWAYS | NO_Z, ALWAYS | NO_DEPTH, NOTEQUAL | NO_DEPTH,
          NOTEQUAL | NO_DEPTH | NO_W, LESS | NO_DEPTH | NO_Z]
ROOT = 100000.0


def lake(rng, cx, cy, r, n=9):
    ang = np.sort(rng.uniform(0, 2 * np.pi, n))
    rad = r * rng.uniform(0.6, 1.0, n)
    return np.column_stack([cx + rad * np.cos(ang), cy + rad * np.sin(ang)])


def water_tile(rng, W, origin=(0.0, 0.0), size=1000.0, k=0):
    from proland_gb300 import layers
    ox, oy = origin
    areas, boundaries = [], []
    if k % 3 != 2:
        outer = lake(rng, ox + size * rng.uniform(0.2, 0.8), oy + size * rng.uniform(0.2, 0.8), size * 0.3)
        island = lake(rng, outer[:, 0].mean(), outer[:, 1].mean(), size * 0.06, 6)
        areas.append([outer, island])
        boundaries.append((np.vstack([outer, outer[:1]]), 1))
        boundaries.append((np.vstack([island, island[:1]]), 0))
    curves = [([(ox - 100, oy + size * rng.uniform(0, 1)), (ox + size + 100, oy + size * rng.uniform(0, 1))],
               rng.uniform(0, 50, 2), float(rng.uniform(10, 60)))]
    rivers = []
    for _ in range(1 + k % 2):
        a = (ox + size * rng.uniform(-0.1, 1.1), oy - 50)
        m = (ox + size * rng.uniform(0.2, 0.8), oy + size * rng.uniform(0.3, 0.7))
        b = (ox + size * rng.uniform(-0.1, 1.1), oy + size + 50)
        rivers.append(([a, m, b], rng.uniform(-20, 80, 3), float(rng.uniform(8, 40)), bool(k & 1), True))
    return layers.water_layer(origin, size, W, areas=areas, boundaries=boundaries, curves=curves, rivers=rivers)


def as_batch(ms):
    """Producer-callback tuples -> LayerBatch tuples, the first mesh clearing depth."""
    return [(v, ix, mode, i == 0, prog, state, fd) for i, (v, ix, mode, prog, state, fd) in enumerate(ms)]


def adversarial(rng, W, k):
    """Random passes of overlapping triangles: equal depths (constant u, fill depths)
    so that order decides, programs mixed within a pass, clears between passes."""
    out = []
    for p in range(6):
        state = STATES[int(rng.integers(0, len(STATES)))]
        clear = p == 0 or rng.uniform() < 0.15
        for m in range(int(rng.integers(1, 4))):
            prog = int(rng.integers(0, 5))
            nv = int(rng.integers(3, 25))
            u = rng.choice([0.0, 0.5, 1.5, -1.25, 2.5]) if rng.uniform() < 0.6 else None
            v = np.column_stack([rng.uniform(-1.2, 1.2, nv), rng.uniform(-1.2, 1.2, nv), rng.uniform(-50, 400, nv),
                                 np.full(nv, u) if u is not None else rng.uniform(-3, 3, nv)]).astype(np.float32)
            mode = int(rng.integers(0, 2))
            ix = rng.integers(0, nv, 3 * int(rng.integers(1, 12))).astype(np.uint32) if rng.uniform() < 0.4 else None
            fd = float(rng.choice([0.02, 0.3, 0.5, 1.0, -0.5]))
            out.append((v, ix, mode if ix is None else 0, clear and m == 0, prog, state, fd))
    return out


def run_tiles(tp, oracle_lib, W, meshes, blend_mode, seed, device=False):
    import torch
    n = len(meshes)
    rng = np.random.default_rng(seed)
    zf = (rng.standard_normal((n, W, W)) * 60.0).astype(np.float32)
    zc = (rng.standard_normal((n, W, W)) * 60.0).astype(np.float32)
    zm = np.maximum(zf, np.float32(0.0))
    elev = tp.TileStorage(W, 3, n + 1)
    slots = [int(s) for s in rng.permutation(n + 1)[:n]]   # distinct slots, not in tile order
    for k, s in enumerate(slots):
        elev.upload(s, tp.ZF, zf[k:k + 1])
        elev.upload(s, tp.ZC, zc[k:k + 1])
        elev.upload(s, tp.ZM, zm[k:k + 1])
    batch = tp.LayerBatch(list(zip(slots, meshes)))
    if device:
        batch.to_device(torch).run_device(elev, blend_mode)
    else:
        batch.run(elev, blend_mode)
    tp.stream_check()
    changed = 0
    for k, s in enumerate(slots):
        want = oracle_lib.layer_tile(W, zf[k], zm[k], meshes[k], blend_mode)
        got = elev.download(s, 1, tp.ZM)[0]
        assert np.array_equal(got, want), "tile %d (W %d, blend %d)" % (k, W, blend_mode)
        assert np.array_equal(elev.download(s, 1, tp.ZF)[0], zf[k])
        assert np.array_equal(elev.download(s, 1, tp.ZC)[0], zc[k])
        changed += int(not np.array_equal(got, zm[k]))
    return changed


@pytest.mark.parametrize("W", [101, 197])
@pytest.mark.parametrize("blend_mode", [0, 1])
def test_water_layer_tiles_match_oracle(gpu, oracle_lib, W, blend_mode):
    rng = np.random.default_rng(W + 7 * blend_mode)
    meshes = [as_batch(water_tile(rng, W, k=k)) for k in range(6)]
    assert run_tiles(gpu, oracle_lib, W, meshes, blend_mode, W) >= 5


@pytest.mark.parametrize("W", [101, 197])
def test_adversarial_passes_match_oracle(gpu, oracle_lib, W):
    from proland_gb300 import layers
    rng = np.random.default_rng(100 + W)
    meshes = [adversarial(rng, W, k) for k in range(12)]
    # road and water layers in one tile: a road layer, then the water layer
    road = layers.road_strip([(-100.0, 300.0), (1100.0, 700.0)], [10.0, 40.0], 20.0, (0.0, 0.0), 1000.0, W)
    meshes.append([(road, None, 1, True)] + as_batch(water_tile(rng, W, k=1)))
    assert run_tiles(gpu, oracle_lib, W, meshes, 0, 3 * W) >= 10


def test_device_meshes_with_pass_states(gpu, oracle_lib):
    rng = np.random.default_rng(77)
    meshes = [adversarial(rng, 101, k) for k in range(4)] + [as_batch(water_tile(rng, 101, k=0))]
    run_tiles(gpu, oracle_lib, 101, meshes, 1, 5, device=True)


def water_callback(level, tx, ty, W):
    size = ROOT / (1 << level)
    origin = (ROOT * (tx / (1 << level) - 0.5), ROOT * (ty / (1 << level) - 0.5))
    g = np.random.default_rng(0)      # the same graph on every tile, in world coordinates
    from proland_gb300 import layers
    outer = lake(g, -8000.0, 6000.0, 9000.0)
    rivers = [([(-30000.0, -20000.0), (-9000.0, 2000.0), (20000.0, 30000.0)], [300.0, 120.0, 40.0], 400.0, True, True)]
    curves = [([(-30000.0, 8000.0), (30000.0, 4000.0)], [90.0, 60.0], 600.0)]
    return layers.water_layer(origin, size, W, areas=[[outer]], boundaries=[(np.vstack([outer, outer[:1]]), 1)],
                              curves=curves, rivers=rivers)


def test_water_layered_producer_levels(gpu, oracle_lib):
    tp, orc = gpu, oracle_lib
    W = 101
    es, rs = tp.TileStorage(W, 3, 64), tp.TileStorage(W, 1, 64)
    ec, rc = tp.TileCache(es, "e"), tp.TileCache(rs, "r")

    def residual(level, tx, ty, width):
        g = np.random.default_rng(104729 * level + 31 * tx + ty)
        return (g.standard_normal((width, width)) * 700.0 * 0.5 ** level).astype(np.float32)
    r = tp.ResidualProducer(rc, source=residual)
    amps = [-40.0, -20.0, 10.0, -5.0]
    e = tp.ElevationProducer(ec, r, noise_amp=amps, params=tp.make_params(), face=0)
    e.add_layer(lambda l, x, y: water_callback(l, x, y, W))
    e.set_root_quad_size(ROOT)
    wanted = [(3, x, y) for x in range(2, 6) for y in range(2, 5)]
    held = [e.get_tile(*t) for t in wanted]
    assert all(h is not None for h in held)
    tp.scheduler_run([e])
    tp.stream_check()
    tree = set()
    for (l, x, y) in wanted:
        while l >= 0:
            tree.add((l, x, y))
            l, x, y = l - 1, x // 2, y // 2
    table = orc.dem_noise(W)
    want = {}
    for (l, x, y) in sorted(tree):
        p = want.get((l - 1, x // 2, y // 2))
        rot, layer = orc.noise_select(0, l, x, y)
        zf, zc, zm = orc.elevation_tile(W, l, x, y, p[0] if p else None, p[2] if p else None, residual(l, x, y, W),
                                        noise=table[layer], noise_rot=rot, noise_amp=amps[l])
        want[(l, x, y)] = (zf, zc, orc.layer_tile(W, zf, zm, as_batch(water_callback(l, x, y, W)), 0))
    touched = 0
    for t in sorted(tree):
        et = e.find_tile(*t, include_cache=True, done=True)
        assert et is not None, t
        for ch, name in ((tp.ZF, "zf"), (tp.ZC, "zc"), (tp.ZM, "zm")):
            assert np.array_equal(es.download(et.slot, 1, ch)[0], want[t][ch]), "%s of %s" % (name, t)
        touched += int(not np.array_equal(want[t][2], np.maximum(want[t][0], 0)))
    assert touched >= 4


def test_each_kernel_variant(gpu, oracle_lib):
    """The launch picks a kernel by what its meshes use: stored depths (a state other
    than LESS with depth writes) or not, the road program only or any program.  One
    batch for each of the four."""
    from proland_gb300 import layers
    rng = np.random.default_rng(31)
    W = 101

    def roads(k):
        out = []
        for r in range(2):
            a, b = rng.uniform(-200, 1200, 2), rng.uniform(-200, 1200, 2)
            v = layers.road_strip([a, (a + b) / 2, b], rng.uniform(0, 300, 3), float(rng.uniform(5, 40)), (0.0, 0.0),
                                  1000.0, W)
            out.append((v, None, 1, r == 0))
        return out
    batches = {
        "no stored depth, road program": [roads(k) for k in range(4)],
        "no stored depth, any program": [as_batch(water_tile(rng, W, k=2)) for _ in range(4)],   # rivers only
        "stored depth, road program": [[(v, ix, mode, clear, 0, STATES[(k + j) % len(STATES)], 0.0)
                                        for j, (v, ix, mode, clear, *_r) in enumerate(adversarial(rng, W, k))]
                                       for k in range(4)],
        "stored depth, any program": [adversarial(rng, W, k) for k in range(4)],
    }
    for name, meshes in batches.items():
        assert run_tiles(gpu, oracle_lib, W, meshes, 0, 9) >= 3, name


@pytest.mark.parametrize("W", [101, 197])
def test_road_layer_tiles_match_oracle(gpu, oracle_lib, W):
    """layers.road_layer's meshes (strips with start and end caps, narrow roads left out)
    drawn by the layer kernel, bit for bit against the oracle, both blend programs."""
    from proland_gb300 import layers
    rng = np.random.default_rng(5 + W)
    meshes = []
    for k in range(6):
        roads = []
        for r in range(3):
            pts = np.column_stack([rng.uniform(-150, 1150, 4), rng.uniform(-150, 1150, 4)])
            roads.append((pts, rng.uniform(-30, 250, 4), float(rng.uniform(4, 45)), bool((k + r) & 1),
                          bool((k + r) & 2)))
        roads.append((np.array([[0.0, 500.0], [1000.0, 520.0]]), [10.0, 20.0], 0.5))   # too narrow to draw
        meshes.append(as_batch(layers.road_layer((0.0, 0.0), 1000.0, W, roads=roads)))
    for blend_mode in (0, 1):
        assert run_tiles(gpu, oracle_lib, W, meshes, blend_mode, W + blend_mode) >= 5
