"""The water elevation layer on the CPU: the oracle's fragment programs (water shader
with river = 0, 1, 2, the fill shader) and pass states (ALWAYS, NOTEQUAL, LESS with
and without depth writes, z / w masks) on known answers; the order semantics the
GPU's order-independent passes rely on; the mesh builders of proland_gb300.layers
(odd-winding fill, drawCurve part strips, altitude strips with caps, the pass
sequence of WaterElevationLayer::doCreateTile); and the host-side checks of program
and state."""
import numpy as np
import pytest

W = 101
LESS, ALWAYS, NOTEQUAL = 0, 1, 2
NO_DEPTH, NO_Z, NO_W = 4, 8, 16
ROAD, WATER, RIVER, LARGE, FILL = 0, 1, 2, 3, 4


def f32(x):
    return np.float32(x)


def clip(xw):
    return np.float32(2.0 * xw / W - 1.0)


def quad(x0, y0, x1, y1, a, u):
    """Two triangles covering texels x0..x1-1, y0..y1-1 (window coordinates)."""
    p = [(x0, y0), (x1, y0), (x1, y1), (x0, y0), (x1, y1), (x0, y1)]
    return np.array([[clip(x), clip(y), a, u] for x, y in p], np.float32)


def full(a, u):
    return quad(-1, -1, W + 1, W + 1, a, u)


def tile_inputs(seed=1):
    rng = np.random.default_rng(seed)
    zf = (rng.standard_normal((W, W)) * 50.0).astype(np.float32)
    return zf, np.maximum(zf, f32(0.0))


def smooth12(d):
    t = np.clip(f32(d) - f32(1.0), f32(0.0), f32(1.0)).astype(np.float32)
    return t * t * (f32(3.0) - f32(2.0) * t)


def blend(zf, z, w):
    b = np.minimum(f32(w), f32(1.0))
    return zf * b + f32(z) * (f32(1.0) - b)


def mesh(v, program, state, fill_depth=0.0, clear=False, mode=0):
    return (v, None, mode, clear, program, state, fill_depth)


def test_water_programs_known_answers(oracle_lib):
    zf, zm = tile_inputs()
    # river = 0: z = st.x, w = smoothstep(1, 2, |st.y|)
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(full(10.0, 1.25), WATER, LESS, clear=True)])
    assert np.array_equal(out, blend(zf, 10.0, smooth12(1.25)))
    # river = 1: z = st.x - 1 + max(|st.y| - 1, 0)
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(full(10.0, -1.5), RIVER, LESS, clear=True)])
    assert np.array_equal(out, blend(zf, f32(9.0) + f32(0.5), smooth12(1.5)))
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(full(10.0, 0.5), RIVER, LESS, clear=True)])
    assert np.array_equal(out, blend(zf, 9.0, 0.0))
    # river = 2 writes depth 1: a LESS test against the cleared 1 never passes
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(full(10.0, 0.5), LARGE, LESS, clear=True)])
    assert np.array_equal(out, zm)
    # fill: z and w are the colour's blue and alpha (vertex attributes here)
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(full(7.0, 0.25), FILL, ALWAYS, 0.02, clear=True)])
    assert np.array_equal(out, blend(zf, 7.0, 0.25))


def test_depth_tests_and_masks(oracle_lib):
    zf, zm = tile_inputs(2)
    # LESS with depth writes: the nearer fragment wins whatever the order
    near, far = full(5.0, 0.0), full(9.0, 0.5)   # road depths 0.3 and 0.35
    for order in ((near, far), (far, near)):
        out = oracle_lib.layer_tile(W, zf, zm, [mesh(v, ROAD, LESS, clear=k == 0) for k, v in enumerate(order)])
        assert np.array_equal(out, blend(zf, f32(5.0) + f32(0.03) * (f32(1.0) - f32(0.0)), 0.0))
    # LESS without depth writes, ALWAYS with them: the last fragment wins
    for state in (LESS | NO_DEPTH, ALWAYS):
        out = oracle_lib.layer_tile(W, zf, zm, [mesh(near, WATER, state, clear=True), mesh(far, WATER, state)])
        assert np.array_equal(out, blend(zf, 9.0, 0.0))
    # masks: z only keeps w = 0 from before; w only keeps z = zm
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(full(3.0, 1.5), WATER, ALWAYS | NO_W, clear=True)])
    assert np.array_equal(out, blend(zf, 3.0, 0.0))
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(full(3.0, 1.5), WATER, ALWAYS | NO_Z, clear=True)])
    assert np.array_equal(out, blend(zf, zm, smooth12(1.5)))


def test_fill_then_notequal_touches_only_the_filled_texels(oracle_lib):
    """The water layer's area pass: a fill at depth 0.02 (w only), then river = 2 under
    NOTEQUAL (depth 1 differs from the stored depth only where the fill drew), z only;
    a later clear forgets the fill."""
    zf, zm = tile_inputs(3)
    fill = quad(20, 30, 60, 70, 0.0, 0.0)
    large = full(100.0, 0.0)
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(fill, FILL, ALWAYS | NO_Z, 0.02, clear=True),
                                            mesh(large, LARGE, NOTEQUAL | NO_DEPTH | NO_W)])
    inside = np.zeros((W, W), bool)
    inside[30:70, 20:60] = True
    assert np.array_equal(out[inside], np.full(inside.sum(), 99.0, np.float32))
    assert np.array_equal(out[~inside], zm[~inside])
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(fill, FILL, ALWAYS | NO_Z, 0.02, clear=True),
                                            mesh(large, LARGE, NOTEQUAL | NO_DEPTH | NO_W, clear=True)])
    assert np.array_equal(out, zm)


def test_boundary_depth_then_less(oracle_lib):
    """A river = 1 boundary written under ALWAYS at depth 0.1 d + 0.15 hides a later
    river = 1 fragment of larger depth under LESS, and not one of smaller depth."""
    zf, zm = tile_inputs(4)
    boundary = full(0.0, 1.5)   # depth 0.3, w = 0.5
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(boundary, RIVER, ALWAYS | NO_Z, clear=True),
                                            mesh(full(50.0, 1.9), RIVER, LESS)])   # depth 0.34: hidden
    assert np.array_equal(out, blend(zf, zm, smooth12(1.5)))
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(boundary, RIVER, ALWAYS | NO_Z, clear=True),
                                            mesh(full(50.0, 0.2), RIVER, LESS)])   # depth 0.17: drawn
    assert np.array_equal(out, blend(zf, 49.0, 0.0))


def test_fill_triangles_odd_winding(product, oracle_lib):
    from proland_gb300 import layers
    tr = (0.5 * W, 0.5 * W, 2.0 / W, 1.0)       # world = window coordinates
    outer = [(10, 10), (90, 10), (90, 90), (10, 90)]
    hole = [(40, 40), (60, 40), (60, 60), (40, 60)]
    zf, zm = tile_inputs(5)
    v = layers.fill_triangles([outer, hole], tr, 0.0, 1.0)
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(v, FILL, ALWAYS, 0.02, clear=True)])
    ring = np.zeros((W, W), bool)
    ring[10:90, 10:90] = True
    ring[40:60, 40:60] = False
    assert np.array_equal(out[ring], zf[ring]) and np.array_equal(out[~ring], zm[~ring])
    # a bow tie: the two triangles of a self-crossing contour, each once
    bow = [(10, 10), (90, 90), (90, 10), (10, 90)]
    v = layers.fill_triangles([bow], tr, 0.0, 1.0)
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(v, FILL, ALWAYS, 0.02, clear=True)])
    j, i = np.mgrid[0:W, 0:W] + 0.5
    # the left and right triangles, between the diagonals and the vertical sides
    inside = (np.abs(j - 50) < np.abs(i - 50)) & (np.abs(i - 50) < 40)
    edge = (np.abs(np.abs(i - 50) - np.abs(j - 50)) < 0.02) | (np.abs(np.abs(i - 50) - 40) < 0.02)
    assert inside.sum() > 2000
    assert np.array_equal(out[inside & ~edge], zf[inside & ~edge])
    assert np.array_equal(out[~inside & ~edge], zm[~inside & ~edge])


def test_curve_part_strip(product):
    """A straight boundary along +x with part (0, 12, 1, 2): the curve side at u = 1,
    the other 12 world units towards -y at u = 2 (drawCurve's (dy, -dx) offset)."""
    from proland_gb300 import layers
    tr = (0.0, 0.0, 0.01, 1.0)
    v = layers.curve_part_strip([(0.0, 0.0), (50.0, 0.0), (100.0, 0.0)], (0.0, 12.0, 1.0, 2.0), tr)
    assert v.shape == (6, 4)
    assert np.allclose(v[0::2, :2], [[0, 0], [0.5, 0], [1.0, 0]])
    assert np.allclose(v[1::2, :2], [[0, -0.12], [0.5, -0.12], [1.0, -0.12]])
    assert np.array_equal(v[:, 3], np.float32([1, 2, 1, 2, 1, 2])) and not v[:, 2].any()


def test_altitude_strip_caps(product):
    from proland_gb300 import layers
    tr = (0.0, 0.0, 0.01, 1.0)
    ms = layers.curve_altitude_meshes([(0.0, 0.0), (40.0, 0.0)], [5.0, 9.0], 6.0, 3.0, 10.0, tr, True, True)
    assert [m[2] for m in ms] == [0, 1, 0]
    cap0, strip, cap1 = ms
    assert cap0[0].shape == (8, 4) and cap0[1].size == 18 and cap1[0].shape == (8, 4)
    # the strip: 2 vertices per point plus 2 per subdivision (40 / 10 - 1 = 3)
    assert strip[0].shape == (10, 4) and np.array_equal(strip[0][:, 3], np.float32([-3, 3] * 5))
    assert np.allclose(strip[0][:, 2], [5, 5, 6, 6, 7, 7, 8, 8, 9, 9])
    # caps: the start one behind the first point (x < 0), the end one beyond the last
    assert cap0[0][:, 0].min() < 0 and cap1[0][:, 0].max() > 0.4
    assert np.array_equal(np.sort(np.unique(cap0[0][:, 3])), np.float32([1, 3]))


def test_water_layer_pass_sequence(product):
    from proland_gb300 import layers
    lake = [[(100.0, 100.0), (600.0, 120.0), (500.0, 700.0)]]
    ms = layers.water_layer((0.0, 0.0), 1000.0, W, areas=[lake],
                            boundaries=[(np.array(lake[0] + [lake[0][0]]), 1)],
                            curves=[([(0.0, 500.0), (1000.0, 500.0)], [10.0, 12.0], 30.0),
                                    ([(0.0, 0.0), (10.0, 10.0)], [0.0, 0.0], 0.5)],   # too narrow: skipped
                            rivers=[([(500.0, 0.0), (500.0, 1000.0)], [20.0, 4.0], 25.0, True, False)])
    got = [(m[3], m[4], m[5]) for m in ms]
    assert got == [(FILL, ALWAYS | NO_Z, 0.02), (RIVER, ALWAYS | NO_Z, 0.0), (LARGE, NOTEQUAL | NO_DEPTH | NO_W, 0.0),
                   (RIVER, LESS, 0.0), (RIVER, LESS, 0.0)]
    assert ms[3][2] == 0 and ms[3][1] is not None        # the river's start cap, then its strip
    # no areas: the river pass alone
    ms = layers.water_layer((0.0, 0.0), 1000.0, W, curves=[([(0.0, 500.0), (1000.0, 500.0)], [10.0, 12.0], 30.0)],
                            rivers=[([(500.0, 0.0), (500.0, 1000.0)], [20.0, 4.0], 25.0)])
    assert [(m[3], m[4]) for m in ms] == [(RIVER, LESS)]


def test_road_strip_widths(product):
    """road_strip is the TOTALWIDTH strip: u = -/+ TOTALWIDTH / BASEWIDTH in float."""
    from proland_gb300 import layers
    v = layers.road_strip([(0.0, 500.0), (1000.0, 500.0)], [3.0, 3.0], 20.0, (0.0, 0.0), 1000.0, W)
    scale = layers.tile_transform((0.0, 0.0), 1000.0, W)[3]
    base = layers.base_width(20.0, scale)
    assert np.array_equal(np.abs(v[:, 3]), np.full(len(v), f32(f32(base * f32(3.0)) / base)))


def test_host_rejects_bad_pass_states(product):
    """tp_elevation_layers and tp_layer_builder_set_pass refuse an unknown program or
    state, NOTEQUAL with depth writes (order-dependent) and a non-finite fill depth,
    before looking at the storage."""
    tp = product
    elev = tp.TileStorage(W, 3, 2, on_device=2)
    v = full(1.0, 0.0)
    for program, state, fd, what in ((9, 0, 0.0, "program"), (0, 3, 0.0, "state"), (0, 64, 0.0, "state"),
                                     (1, NOTEQUAL, 0.0, "NOTEQUAL"), (4, ALWAYS, float("nan"), "fill depth")):
        with pytest.raises(tp.TPError) as e:
            tp.elevation_layers(elev, [(0, [(v, None, 0, True, program, state, fd)])])
        assert e.value.code == tp.TP_E_BAD_ARG and what in tp.lib().tp_last_error().decode(), what
    # a supported state gets past the checks to the storage check
    with pytest.raises(tp.TPError) as e:
        tp.elevation_layers(elev, [(0, [(v, None, 0, True, LARGE, NOTEQUAL | NO_DEPTH | NO_W, 0.0)])])
    assert "device elevation storage" in tp.lib().tp_last_error().decode()
    assert tp.lib().tp_layer_builder_set_pass(None, 0, 0, 0.0) == tp.TP_E_BAD_ARG


def _odd_winding(px, py, contours):
    """Crossing-number parity of the points (px, py) against the contours (x, y up)."""
    inside = np.zeros(px.shape, bool)
    for c in contours:
        c = np.asarray(c, np.float64)
        x0, y0 = c[:, 0], c[:, 1]
        x1, y1 = np.roll(x0, -1), np.roll(y0, -1)
        for a, b, c2, d in zip(x0, y0, x1, y1):
            if b == d:
                continue
            cond = (py >= min(b, d)) & (py < max(b, d))
            xc = a + (py - b) * (c2 - a) / (d - b)
            inside ^= cond & (px < xc)
    return inside


def _edge_distance(px, py, contours):
    dist = np.full(px.shape, np.inf)
    for c in contours:
        c = np.asarray(c, np.float64)
        for (a, b), (c2, d) in zip(c, np.roll(c, -1, axis=0)):
            vx, vy = c2 - a, d - b
            t = np.clip(((px - a) * vx + (py - b) * vy) / max(vx * vx + vy * vy, 1e-30), 0.0, 1.0)
            dist = np.minimum(dist, np.hypot(px - (a + t * vx), py - (b + t * vy)))
    return dist


@pytest.mark.parametrize("seed", range(6))
def test_fill_triangles_cover_the_odd_winding_region(product, oracle_lib, seed):
    """Random star-shaped and self-crossing contours (one to three, nested or
    overlapping): every texel centre further than 0.05 texel from all edges is filled
    exactly when its crossing count is odd."""
    from proland_gb300 import layers
    rng = np.random.default_rng(seed)
    tr = (0.5 * W, 0.5 * W, 2.0 / W, 1.0)       # world = window coordinates
    contours = []
    for _ in range(int(rng.integers(1, 4))):
        cx, cy, r = rng.uniform(25, 76, 2).tolist() + [float(rng.uniform(10, 40))]
        n = int(rng.integers(3, 12))
        ang = rng.uniform(0, 2 * np.pi, n)
        if rng.uniform() < 0.6:
            ang = np.sort(ang)                   # star-shaped; unsorted angles cross themselves
        rad = r * rng.uniform(0.3, 1.0, n)
        contours.append(np.column_stack([cx + rad * np.cos(ang), cy + rad * np.sin(ang)]))
    zf, zm = tile_inputs(20 + seed)
    v = layers.fill_triangles(contours, tr, 0.0, 1.0)
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(v, FILL, ALWAYS, 0.02, clear=True)])
    j, i = np.mgrid[0:W, 0:W] + 0.5
    inside = _odd_winding(i, j, contours)
    clear = _edge_distance(i, j, contours) > 0.05
    covered = out == zf                          # w = 1: zm became zf
    same_value = zf == zm                         # texels where zf == zm cannot tell
    check = clear & ~same_value
    assert check.sum() > 5000
    assert np.array_equal(covered[check], inside[check])


@pytest.mark.parametrize("seed", range(4))
def test_road_strip_covers_its_total_width(product, oracle_lib, seed):
    """A straight road of constant altitude at a random angle: the texels within half of
    TOTALWIDTH of its axis (0.05 texel margin) change, those beyond do not.  The tile is
    96 world units across (W = 101, border 2), so world units are texels."""
    from proland_gb300 import layers
    rng = np.random.default_rng(40 + seed)
    size = 96.0
    ang = float(rng.uniform(0, np.pi))
    c = np.array([48.0, 48.0]) + rng.uniform(-15, 15, 2)
    d = np.array([np.cos(ang), np.sin(ang)])
    pts = [c - 150 * d, c, c + 150 * d]
    width = float(rng.uniform(3, 12))
    v = layers.road_strip(pts, [5000.0] * 3, width, (0.0, 0.0), size, W)
    scale = layers.tile_transform((0.0, 0.0), size, W)[3]
    half = float(layers.base_width(width, scale)) * 3.0 / 2.0
    zf, _ = tile_inputs(60 + seed)
    zm = zf + np.float32(1000.0)   # zm apart from zf: the strip's outer third blends to zf exactly
    out = oracle_lib.layer_tile(W, zf, zm, [(v, None, 1, True)])
    j, i = np.mgrid[0:W, 0:W] + 0.5
    # window = world + 2.5: the tile's origin sits at the 2-texel border plus the half texel
    px, py = i - 2.5 - c[0], j - 2.5 - c[1]
    dist = np.abs(px * d[1] - py * d[0])
    assert (dist < half - 0.05).sum() > 200
    changed = out != zm
    assert changed[dist < half - 0.05].all()
    assert not changed[dist > half + 0.05].any()


@pytest.mark.parametrize("seed", range(4))
def test_boundary_strip_covers_twelve_units_on_its_right(product, oracle_lib, seed):
    """drawCurve with part (0, 12, 1, 2) along a straight curve at a random angle: the
    strip spans the 12 world units on the curve's right (u from 1 on the curve to 2),
    so under river = 1 (w = smoothstep(1, 2, u), alpha only) the texels strictly inside
    that band change and the texels elsewhere do not.  World units are texels here."""
    from proland_gb300 import layers
    rng = np.random.default_rng(80 + seed)
    tr = layers.tile_transform((0.0, 0.0), 96.0, W)
    ang = float(rng.uniform(0, 2 * np.pi))
    c = np.array([48.0, 48.0]) + rng.uniform(-10, 10, 2)
    d = np.array([np.cos(ang), np.sin(ang)])
    pts = [c - 150 * d, c, c + 150 * d]
    v = layers.curve_part_strip(pts, (0.0, 12.0, 1.0, 2.0), tr)
    zf, _ = tile_inputs(90 + seed)
    zm = zf + np.float32(1000.0)
    out = oracle_lib.layer_tile(W, zf, zm, [mesh(v, RIVER, ALWAYS | NO_Z, clear=True, mode=1)])
    j, i = np.mgrid[0:W, 0:W] + 0.5
    px, py = i - 2.5 - c[0], j - 2.5 - c[1]
    right = px * d[1] - py * d[0]        # offset along (dy, -dx): the strip's side
    changed = out != zm
    inside = (right > 0.3) & (right < 11.95)
    assert inside.sum() > 500
    assert changed[inside].all()
    assert not changed[(right < -0.05) | (right > 12.05)].any()
