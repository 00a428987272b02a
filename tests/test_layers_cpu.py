"""The elevation-layer oracle (road meshes drawn into a tile, then the blend) on
known answers: coverage of texel centres by the top-left rule, depth order and
depth clears, the fragment program's z / w, both blend programs, strip and index
forms of the same triangles, and the road-strip builder.  CPU only."""
import numpy as np
import pytest

W = 101


def clip(xw):
    """Clip coordinate of window coordinate xw (texels) on a W-wide tile."""
    return np.float32(2.0 * xw / W - 1.0)


def tri(p0, p1, p2, alt=0.0, u=0.0):
    return np.array([[clip(p[0]), clip(p[1]), alt, u] for p in (p0, p1, p2)], np.float32)


def tile_inputs(seed=1):
    rng = np.random.default_rng(seed)
    zf = (rng.standard_normal((W, W)) * 50.0).astype(np.float32)
    return zf, np.maximum(zf, np.float32(0.0))


def f32(x):
    return np.float32(x)


def smoothstep(e0, e1, x):
    t = (f32(x) - f32(e0)) / (f32(e1) - f32(e0))
    t = np.clip(t, f32(0.0), f32(1.0)).astype(np.float32)
    return t * t * (f32(3.0) - f32(2.0) * t)


def test_no_meshes_keeps_zm(oracle_lib):
    zf, zm = tile_inputs()
    out = oracle_lib.layer_tile(W, zf, zm, [])
    assert np.array_equal(out, zm)


def test_right_triangle_coverage(oracle_lib):
    """Window corners (0,0), (10,0), (0,10): centres with i + j <= 8 are inside; the
    hypotenuse (i + j = 9 has its centre on it) is a right edge, so not covered."""
    zf, zm = tile_inputs()
    for order in ((0, 1, 2), (0, 2, 1)):
        pts = [(0, 0), (10, 0), (0, 10)]
        v = tri(*[pts[k] for k in order], alt=500.0)
        out = oracle_lib.layer_tile(W, zf, zm, [(v, None, 0, True)])
        j, i = np.mgrid[0:W, 0:W]
        inside = (i + j) <= 8
        assert np.array_equal(out[inside], np.full(inside.sum(), f32(500.0) + f32(0.03), np.float32))
        assert np.array_equal(out[~inside], zm[~inside])
        assert inside.sum() == 45


def test_shared_diagonal_goes_to_one_triangle(oracle_lib):
    """A square split on its diagonal (texel centres on it): the diagonal is the left
    edge of the lower triangle and the right edge of the upper one."""
    zf, zm = tile_inputs()
    lower = tri((0, 0), (8, 0), (8, 8), alt=100.0)
    upper = tri((0, 0), (8, 8), (0, 8), alt=200.0)
    out = oracle_lib.layer_tile(W, zf, zm, [(np.concatenate([lower, upper]), None, 0, True)])
    j, i = np.mgrid[0:W, 0:W]
    sq = (i < 8) & (j < 8)
    assert np.array_equal(out[sq & (i >= j)], np.full((sq & (i >= j)).sum(), f32(100.0) + f32(0.03), np.float32))
    assert np.array_equal(out[sq & (i < j)], np.full((sq & (i < j)).sum(), f32(200.0) + f32(0.03), np.float32))
    assert np.array_equal(out[~sq], zm[~sq])


def full_quad(alt, u):
    a = np.array([[-2, -2, alt, u], [2, -2, alt, u], [2, 2, alt, u]], np.float32)
    b = np.array([[-2, -2, alt, u], [2, 2, alt, u], [-2, 2, alt, u]], np.float32)
    return np.concatenate([a, b])


def test_depth_test_and_clear(oracle_lib):
    zf, zm = tile_inputs()
    near = full_quad(10.0, 0.0)    # depth 0.3
    far = full_quad(20.0, 0.5)     # depth 0.35: fails LESS against the near quad
    out = oracle_lib.layer_tile(W, zf, zm, [(near, None, 0, True), (far, None, 0, False)])
    z_near = f32(10.0) + f32(0.03) * (f32(1.0) - smoothstep(0.98, 1.0, 0.0))
    assert np.array_equal(out, np.full((W, W), z_near, np.float32))
    # a second layer clears the depth buffer first: its quad wins
    out = oracle_lib.layer_tile(W, zf, zm, [(near, None, 0, True), (far, None, 0, True)])
    assert np.array_equal(out, np.full((W, W), f32(20.0) + f32(0.03), np.float32))
    # the same depth does not pass LESS: the first quad stays
    out = oracle_lib.layer_tile(W, zf, zm, [(near, None, 0, True), (full_quad(30.0, 0.0), None, 0, False)])
    assert np.array_equal(out, np.full((W, W), z_near, np.float32))


@pytest.mark.parametrize("u", [0.5, 0.99, 1.25, 1.5, 1.9, 2.5, -1.5])
def test_fragment_and_blend0(oracle_lib, u):
    zf, zm = tile_inputs(3)
    out = oracle_lib.layer_tile(W, zf, zm, [(full_quad(40.0, u), None, 0, True)])
    d = abs(f32(u))
    z = f32(40.0) + f32(0.03) * (f32(1.0) - smoothstep(0.98, 1.0, d))
    b = min(smoothstep(1.0, 2.0, d), f32(1.0))
    want = (zf * b + z * (f32(1.0) - b)).astype(np.float32)
    assert np.array_equal(out, want)


def test_blend1_box_filter(oracle_lib):
    """The demo blend without any draw is the 3x3 box filter of zm, edges clamped,
    summed centre, edge neighbours, diagonal neighbours, each times 1/9."""
    zf, zm = tile_inputs(4)
    out = oracle_lib.layer_tile(W, zf, zm, [], blend_mode=1)
    p = np.pad(zm, 1, mode="edge")

    def at(dj, di):
        return p[1 + dj:1 + dj + W, 1 + di:1 + di + W]
    sy = ((at(0, 1) + at(0, -1)) + at(1, 0)) + at(-1, 0)
    sz = ((at(1, 1) + at(-1, 1)) + at(-1, -1)) + at(1, -1)
    f = f32(1.0) / f32(9.0)
    want = ((zm * f + sy * f) + sz * f).astype(np.float32)
    assert np.array_equal(out, want)


def test_strip_list_and_index_forms_agree(oracle_lib):
    rng = np.random.default_rng(5)
    zf, zm = tile_inputs(5)
    strip = np.column_stack([rng.uniform(-1.2, 1.2, 8), rng.uniform(-1.2, 1.2, 8),
                             rng.uniform(0, 100, 8), rng.uniform(-3, 3, 8)]).astype(np.float32)
    # the strip's triangles in GL order: (k, k+1, k+2) for even k, (k+1, k, k+2) for odd k
    order = []
    for k in range(len(strip) - 2):
        order += [k + 1, k, k + 2] if k & 1 else [k, k + 1, k + 2]
    as_list = strip[order]
    a = oracle_lib.layer_tile(W, zf, zm, [(strip, None, 1, True)])
    b = oracle_lib.layer_tile(W, zf, zm, [(as_list, None, 0, True)])
    c = oracle_lib.layer_tile(W, zf, zm, [(strip, np.array(order, np.uint32), 0, True)])
    d = oracle_lib.layer_tile(W, zf, zm, [(strip, np.arange(len(strip), dtype=np.uint32), 1, True)])
    assert np.array_equal(a, b) and np.array_equal(a, c) and np.array_equal(a, d)
    assert not np.array_equal(a, zm)


def test_far_vertex_drops_its_triangle(oracle_lib):
    zf, zm = tile_inputs()
    v = np.array([[-1, -1, 5, 0], [1e6, -1, 5, 0], [-1, 1, 5, 0]], np.float32)
    assert np.array_equal(oracle_lib.layer_tile(W, zf, zm, [(v, None, 0, True)]), zm)


def test_road_strip_builder(product, oracle_lib):
    """A straight road across the middle of a tile: the core (|u| < 1) takes the
    road altitude, texels beyond the total width keep zm."""
    from proland_gb300 import layers
    size = 1000.0
    v = layers.road_strip([(-100.0, 500.0), (1100.0, 500.0)], [30.0, 30.0], 20.0, (0.0, 0.0), size, W)
    assert v.shape[1] == 4 and v.shape[0] % 2 == 0
    assert np.allclose(np.abs(v[:, 3]), 3.0)
    zf, zm = tile_inputs(6)
    out = oracle_lib.layer_tile(W, zf, zm, [(v, None, 1, True)])
    # texel row of world y = 500 (the tile's centre row) is on the road's axis
    row = (W - 1) // 2
    assert np.allclose(out[row, 2:W - 2], 30.0 + 0.03, atol=1e-3)
    far = np.abs(np.arange(W) - row) > 10
    assert np.array_equal(out[far], zm[far])
