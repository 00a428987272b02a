"""The oracle's restatement of the shader path against the reference's own GPU path,
compiled here by oracle/ref_build.py: ElevationProducer::doCreateTile,
NormalProducer::doCreateTile and OrthoProducer::doCreateTile as written (their uniform set-up, the noise-layer
choice, the residual window, the FP64 sphere patch frames) drawing the reference's
upsample and normal shaders, rewritten mechanically as C++ (oracle/ref_glsl.py)
against the GLSL stand-in oracle/ref_stubs/glsl.h.

What is compared, and how tightly:

* elevation tiles, every upsample shader (terrain1, terrain2, terrain4 with
  flipped diagonals, the demo's modulated noise with and without NO_CLAMP):
  zc bit for bit always; zf and zm bit for bit when the parent tile holds
  integers, where both the shader's 4x4 matrix dot product and the CPU producer's
  stencil order (CPUElevationProducer.cpp:202-238, which the oracle and the
  product follow) are exact; with arbitrary floats zf within a few units in the
  last place -- the two summation orders;
* normal tiles on the sphere (terrain2 and demo shaders, NormalProducer's FP64
  patch frames): float tiles within 2 units in the last place (GLSL's
  normalize divides by the length, the oracle multiplies by its reciprocal),
  8-bit tiles the same but for an odd texel one step apart; coarse normals bit
  for bit;
* flat normal tiles: the shader forms absolute world positions in float
  (normalShader.glsl getWorldPosition) and differences them, the oracle uses the
  exact sample spacing 2h; float normals agree within that position rounding
  (the bound below), 8-bit normals within one step; coarse normals (nc) bit for
  bit;
* the layers' fragment programs (road, water with river = 0, 1, 2, fill) bit for
  bit, and a producer with layers: the blend programs of graph1 and the demo
  drawn by ElevationProducer::doCreateTile after given layer planes, bit for bit;
* the ortho producer: createOrthoNoise byte for byte, and OrthoProducer::doCreateTile
  with the terrain3 and demo ortho shaders byte for byte after the 8-bit store;
* the layers' meshes: ElevationGraphLayer::drawCurveAltitude, GraphLayer::drawCurve
  of a part and RoadElevationLayer's placement of a road, against the product's mesh
  builder (proland_gb300.layers), vertex and index for index.

Texture sampling is the oracle's documented choice (the nearest texel) on both
sides.  Runs where the reference tree is present; skipped elsewhere."""
import numpy as np
import pytest

UPSAMPLE = {"terrain1": 0, "terrain2": 1, "terrain4": 2, "demo": 3, "demo_noclamp": 4}
NOISE_MODE = {"terrain1": 0, "terrain4": 0, "terrain2": 1, "demo": 1, "demo_noclamp": 1}
FLIPS = {"terrain4", "demo", "demo_noclamp"}            # shaders that read tileWSDF.w
NORMAL = {"terrain1": 0, "terrain2": 1, "demo": 2}
# the reference's example amplitudes (terrain2/helloworld.xml), both signs
AMPS = np.array([-3250, -1590, -1125, -795, -561, -397, -140, -100, 15, 8, 5, 2.5], np.float32)


@pytest.fixture(scope="module")
def ref(oracle_lib):
    L = oracle_lib.ref_lib()
    if L is None or not hasattr(L, "ref_gl_elevation_tile"):
        pytest.skip("the reference sources are not on this machine")
    return L


def _p(a):
    import ctypes as C
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


@pytest.fixture(scope="module")
def noise_tables(ref):
    """createDemNoise's table as the R16F texture holds it, per tile width."""
    out = {}
    for W in (37, 101, 197):
        raw = np.empty((6, W, W), np.float32)
        ref.ref_dem_noise(W, _p(raw))
        out[W] = raw.astype(np.float16).astype(np.float32)
    return out


def gl_elevation(ref, variant, W, level, tx, ty, face, parent, residual, rw, noise, root, grid, flip):
    prgba = None
    if parent is not None:
        prgba = np.ascontiguousarray(np.stack(list(parent) + [np.zeros_like(parent[0])], -1), np.float32)
    res = None if residual is None else np.ascontiguousarray(residual, np.float32)
    out = np.empty((W, W, 4), np.float32)
    rc = ref.ref_gl_elevation_tile(UPSAMPLE[variant], W, level, tx, ty, face, _p(prgba), _p(res), rw, _p(noise),
                                   _p(AMPS), len(AMPS), root, grid, int(flip), _p(out))
    assert rc == 0
    return out[..., 0], out[..., 1], out[..., 2], out[..., 3]


def oracle_elevation(orc, variant, W, level, tx, ty, face, parent, residual, rw, noise, root, grid, flip):
    rot, layer = orc.noise_select(face, level, tx, ty)
    amp = float(AMPS[level]) if level < len(AMPS) else 0.0
    mps = np.float32(np.float32(root / (1 << level)) / np.float32(W - 5))   # tileWSDF.y
    rx = ry = 0
    if residual is not None:
        mod = (rw - 5) // (W - 5)
        rx, ry = (tx % mod) * (W - 5), (ty % mod) * (W - 5)
    return orc.elevation_tile(W, level, tx, ty, parent[0] if parent else None, parent[2] if parent else None,
                              residual, rx=rx, ry=ry, noise=noise[layer], noise_rot=rot, noise_amp=amp,
                              noise_mode=NOISE_MODE[variant], meters_per_sample=float(mps),
                              grid_g=(W - 5) // grid, flip=flip, no_clamp=variant == "demo_noclamp")


TILES = [(0, 0, 0), (1, 1, 0), (2, 3, 1), (5, 17, 30), (9, 300, 511), (11, 2047, 6), (14, 9001, 16383)]


def _case(rng, W, level, integer, noclamp, rw_kind):
    parent = None
    if level > 0:
        zf = (rng.integers(-300, 300, (W, W)) if integer else rng.standard_normal((W, W)) * 150.0).astype(np.float32)
        zc = (rng.standard_normal((W, W)) * 150.0).astype(np.float32)
        zm = zf.copy() if noclamp else np.maximum(zf, np.float32(0.0))
        parent = (zf, zc, zm)
    rw = {"same": W, "double": 2 * W - 5, "missing": W, "none": 0}[rw_kind]
    residual = None
    if rw_kind in ("same", "double"):
        residual = (rng.standard_normal((rw, rw)) * 40.0).astype(np.float32)
    return parent, residual, rw


@pytest.mark.parametrize("variant", sorted(UPSAMPLE))
@pytest.mark.parametrize("W,grid", [(101, 24), (197, 24), (37, 8)])
def test_elevation_tiles_bit_exact_on_integer_parents(ref, oracle_lib, noise_tables, variant, W, grid):
    rng = np.random.default_rng(W + 7 * UPSAMPLE[variant])
    faces = range(1, 7) if variant == "terrain2" else [0]
    for k, (level, tx, ty) in enumerate(TILES):
        for rw_kind in ("same", "double", "missing", "none"):
            face = list(faces)[k % len(faces)]
            flip = variant in FLIPS and (k + len(rw_kind)) % 2 == 0
            parent, residual, rw = _case(rng, W, level, True, variant == "demo_noclamp", rw_kind)
            args = (variant, W, level, tx, ty, face, parent, residual, rw, noise_tables[W], 60000.0, grid, flip)
            got = gl_elevation(ref, *args)
            want = oracle_elevation(oracle_lib, *args)
            for name, g, w in zip(("zf", "zc", "zm"), got, want):
                assert np.array_equal(g, w), (name, variant, W, level, tx, ty, rw_kind, flip)
            assert not np.any(got[3]), "the fourth channel is written 0"


@pytest.mark.parametrize("variant", sorted(UPSAMPLE))
def test_elevation_tiles_on_float_parents(ref, oracle_lib, noise_tables, variant):
    """Arbitrary float parents: zc bit for bit, zf within a few ulps of the window's
    magnitude (the shader sums the 16 weighted samples column by column, the CPU
    producer rows of (a + b) * 9 - (c + d), / 16), zm = max(zf, 0) of its own zf."""
    rng = np.random.default_rng(11 + UPSAMPLE[variant])
    W, grid = 101, 24
    identical = total = 0
    for k, (level, tx, ty) in enumerate(TILES[1:]):
        flip = variant in FLIPS and k % 2 == 0
        parent, residual, rw = _case(rng, W, level, False, variant == "demo_noclamp", "same")
        args = (variant, W, level, tx, ty, 0, parent, residual, rw, noise_tables[W], 60000.0, grid, flip)
        zf, zc, zm, _ = gl_elevation(ref, *args)
        wf, wc, wm = oracle_elevation(oracle_lib, *args)
        assert np.array_equal(zc, wc), (variant, level)
        scale = np.float32(2.0 * np.abs(parent[0]).max() + np.abs(wf).max())
        assert np.abs(zf - wf).max() <= 8 * np.spacing(scale), (variant, level, np.abs(zf - wf).max())
        assert np.array_equal(zm, zf if variant == "demo_noclamp" else np.maximum(zf, np.float32(0.0)))
        identical += int(np.sum(zf == wf))
        total += zf.size
    # the even-even samples copy a parent sample and the odd rows or columns of a
    # 1D stencil often round the same way: most samples agree exactly
    assert identical >= 0.5 * total


def gl_normals(ref, variant, W, level, tx, ty, zm, fmt, parent, root, grid, deform):
    Wn, comps = W - 4, (4 if fmt < 2 else 2)
    erg = np.ascontiguousarray(np.stack([zm, zm, zm, np.zeros_like(zm)], -1), np.float32)
    par = None if parent is None else np.ascontiguousarray(np.stack(parent, -1), np.float32)
    out = np.empty((Wn, Wn, comps), np.float32)
    rc = ref.ref_gl_normal_tile(NORMAL[variant], W, level, tx, ty, _p(erg), fmt, _p(par), root, grid, int(deform),
                                _p(out))
    assert rc == 0
    return [out[..., k] for k in range(comps)]


def _normal_case(rng, W, level, fmt, amp=30.0):
    Wn = W - 4
    zm = (rng.standard_normal((W, W)) * amp).astype(np.float32)
    parent = None
    if level > 0 and fmt < 2:
        parent = [np.clip(rng.standard_normal((Wn, Wn)) * 0.3, -0.7, 0.7).astype(np.float32) for _ in range(4)]
        if fmt == 1:   # an RGBA8 parent holds k / 255
            parent = [(np.floor(np.clip(v * 0.5 + 0.5, 0, 1) * 255 + 0.5) / 255).astype(np.float32) for v in parent]
    return zm, parent


NORMAL_TILES = [(0, 0, 0, 1000.0), (1, 1, 0, 1000.0), (3, 5, 2, 10000.0), (6, 33, 60, 50000.0),
                (10, 700, 300, 6.4e6), (14, 9000, 5000, 6.4e6)]


@pytest.mark.parametrize("variant,fmt", [("terrain2", 3), ("demo", 3), ("demo", 1), ("demo", 0)])
def test_sphere_normal_tiles(ref, oracle_lib, variant, fmt):
    rng = np.random.default_rng(40 + fmt)
    W, grid = 101, 24
    for level, tx, ty, root in NORMAL_TILES:
        zm, parent = _normal_case(rng, W, level, fmt)
        got = gl_normals(ref, variant, W, level, tx, ty, zm, fmt, parent, root, grid, True)
        want = oracle_lib.normals_full(W, zm, root / (1 << level), fmt, tx, ty,
                                       parent=None if parent is None else parent[:2], root_quad_size=root,
                                       level=level, grid_mesh=grid)
        for k, (g, w) in enumerate(zip(got, want)):
            d = np.abs(g - w)
            if k >= 2 and level > 0:
                assert np.array_equal(g, w), (variant, fmt, level, k)   # the coarse normals
            elif fmt in (1, 3):
                # the float normals below differ by an ulp or two (GLSL's normalize is
                # v / length(v), the oracle's v * (1 / length(v))), which moves a value
                # across an 8-bit rounding boundary now and then
                assert d.max() <= 1.0 / 255 + 1e-6 and np.mean(d > 0) <= 0.001, (variant, fmt, level, k)
            else:
                assert d.max() <= 2 * np.spacing(np.float32(1.0)), (variant, fmt, level, k)


def flat_position_bound(root, level, tx, ty, W):
    """How far the shader's normals can be from the exact-spacing ones: each world
    position x0 + D u rounds to half an ulp of its magnitude, so a central difference
    of 2h carries a relative error up to ulp(|x0| + D) / 2h, and the unit normal's
    components move by about twice that."""
    D = root / (1 << level)
    x0 = tx / (1 << level) * root - root / 2
    y0 = ty / (1 << level) * root - root / 2
    h = D / (W - 5)
    mag = np.float32(max(abs(x0), abs(y0)) + D)
    return float(4 * np.spacing(mag) / (2 * h) + 4 * np.spacing(np.float32(1.0)))


@pytest.mark.parametrize("variant,fmt", [("terrain1", 3), ("demo", 0), ("demo", 1), ("demo", 2), ("demo", 3)])
def test_flat_normal_tiles(ref, oracle_lib, variant, fmt):
    rng = np.random.default_rng(60 + fmt + 7 * NORMAL[variant])
    W, grid = 101, 24
    for level, tx, ty, root in NORMAL_TILES:
        zm, parent = _normal_case(rng, W, level, fmt)
        got = gl_normals(ref, variant, W, level, tx, ty, zm, fmt, parent, root, grid, False)
        want = oracle_lib.normals_full(W, zm, root / (1 << level), fmt, tx, ty,
                                       parent=None if parent is None else parent[:2], level=level, grid_mesh=grid)
        bound = flat_position_bound(root, level, tx, ty, W)
        for k, (g, w) in enumerate(zip(got, want)):
            d = np.abs(g - w)
            if k >= 2 and level > 0:
                assert np.array_equal(g, w), ("nc", variant, fmt, level, k)   # the coarse normals
            elif fmt in (1, 3):
                assert d.max() <= 1.0 / 255 + 1e-6, (variant, fmt, level, k)
                if root <= 50000.0:
                    assert np.mean(d > 0) <= 0.005, (variant, fmt, level, k, np.mean(d > 0))
            else:
                assert d.max() <= bound, (variant, fmt, level, k, d.max(), bound)


LAYER = {"road_graph1": 0, "road_demo": 1, "water_river1": 2, "water_demo": 3, "fill": 4}
BLEND = {"graph1": 0, "demo": 1}


def gl_fragment(ref, shader, st, river=0, depth=0.0, color=(0.0, 0.0, 0.0, 0.0)):
    import ctypes as C
    data = np.empty(4, np.float32)
    fd = C.c_float()
    col = np.asarray(color, np.float32)
    assert ref.ref_gl_layer_fragment(LAYER[shader], river, depth, _p(col), float(st[0]), float(st[1]), _p(data),
                                     C.byref(fd)) == 0
    return data, fd.value


def _attributes(rng, n):
    """Interpolated (altitude, signed width coordinate) pairs, the smoothstep edges included."""
    a = rng.uniform(-500.0, 3000.0, n).astype(np.float32)
    u = rng.uniform(-3.0, 3.0, n).astype(np.float32)
    edges = np.float32([0.0, 0.98, 0.99, 1.0, 1.5, 2.0, 2.5])
    u[:2 * len(edges)] = np.concatenate([edges, -edges])
    return a, u


@pytest.mark.parametrize("shader", ["road_graph1", "road_demo", "water_river1", "water_demo"])
def test_layer_fragment_programs(ref, oracle_lib, shader):
    """The road and water layers' fragment shaders at random interpolated attributes
    against the oracle's programs: z and w bit for bit, the written depth once the
    depth buffer clamps it to [0, 1]; x and y written 0 (masked off by the layers)."""
    a, u = _attributes(np.random.default_rng(LAYER[shader]), 3000)
    rivers = [0] if shader.startswith("road") else [0, 1, 2]
    for river in rivers:
        program = 0 if shader.startswith("road") else 1 + river
        for ai, ui in zip(a, u):
            data, fd = gl_fragment(ref, shader, (ai, ui), river=river)
            dp, z, w = oracle_lib.layer_fragment(program, ai, ui)
            assert (np.float32(data[2]), np.float32(data[3])) == (np.float32(z), np.float32(w)), (shader, river, ai, ui)
            assert np.float32(min(max(fd, 0.0), 1.0)) == np.float32(dp), (shader, river, ai, ui, fd, dp)
            assert data[0] == 0.0 and data[1] == 0.0


def test_fill_fragment_program(ref, oracle_lib):
    """fillShader writes its colour uniform and depth uniform; the oracle's fill program
    carries the colour's z and w as the mesh's attributes and the depth as its
    fill depth (WaterElevationLayer.cpp:273-276 sets colour 0 and depth 0.02)."""
    rng = np.random.default_rng(5)
    cases = [((0.0, 0.0, 0.0, 0.0), 0.02)] + [(tuple(rng.uniform(-100, 100, 4)), float(d))
                                             for d in rng.uniform(-0.5, 1.5, 40)]
    for color, depth in cases:
        data, fd = gl_fragment(ref, "fill", (0.0, 0.0), depth=depth, color=color)
        col = np.float32(color)
        dp, z, w = oracle_lib.layer_fragment(4, col[2], col[3], fill_depth=depth)
        assert np.array_equal(data, col)
        assert (np.float32(z), np.float32(w)) == (col[2], col[3])
        assert np.float32(min(max(fd, 0.0), 1.0)) == np.float32(dp)


@pytest.mark.parametrize("blend", sorted(BLEND))
@pytest.mark.parametrize("variant", ["terrain1", "demo"])
def test_layered_tiles_blend(ref, oracle_lib, noise_tables, variant, blend):
    """A producer with layers: ElevationProducer::doCreateTile draws the upsample quad,
    the layers (here: given z and w planes written into the z and w channels), then the
    blend program into COLOR1, and copies COLOR1 into the slot.  zf and zc pass
    through, the layers' w is kept in the fourth channel, and zm is the oracle's blend
    of the oracle's zf with the layers' planes -- bit for bit on integer parents."""
    import ctypes as C
    rng = np.random.default_rng(3 + BLEND[blend] + 5 * UPSAMPLE[variant])
    W, grid = 101, 24
    for k, (level, tx, ty) in enumerate(TILES[:5]):
        parent, residual, rw = _case(rng, W, level, True, False, "same")
        z = (rng.standard_normal((W, W)) * 200.0).astype(np.float32)
        w = rng.choice(np.float32([0.0, 0.0, 0.25, 0.5, 1.0, 1.0, 1.7]), (W, W)).astype(np.float32)
        w[rng.uniform(size=(W, W)) < 0.3] = np.float32(rng.uniform())
        prgba = None
        if parent is not None:
            prgba = np.ascontiguousarray(np.stack(list(parent) + [np.zeros_like(parent[0])], -1), np.float32)
        out = np.empty((W, W, 4), np.float32)
        rc = ref.ref_gl_elevation_tile_layers(UPSAMPLE[variant], BLEND[blend], W, level, tx, ty, 0, _p(prgba),
                                              _p(residual), rw, _p(noise_tables[W]), _p(AMPS), len(AMPS),
                                              C.c_float(60000.0), grid, 0, _p(z), _p(w), _p(out))
        assert rc == 0
        wf, wc, _ = oracle_elevation(oracle_lib, variant, W, level, tx, ty, 0, parent, residual, rw,
                                     noise_tables[W], 60000.0, grid, False)
        assert np.array_equal(out[..., 0], wf) and np.array_equal(out[..., 1], wc), (variant, level)
        assert np.array_equal(out[..., 2], oracle_lib.layer_blend(W, wf, z, w, BLEND[blend])), (variant, blend, level)
        assert np.array_equal(out[..., 3], w)


ORTHO = {"terrain3": 0, "demo": 1}


@pytest.mark.parametrize("W", [20, 196, 260])
def test_ortho_noise_table(ref, oracle_lib, product, W):
    """createOrthoNoise (OrthoProducer.cpp:26-122), compiled as written: its RGBA8
    table is the oracle's and the product's byte for byte."""
    want = np.empty((6, W, W, 4), np.uint8)
    ref.ref_ortho_noise(W, want.ctypes.data)
    assert np.array_equal(oracle_lib.ortho_noise(W), want)
    assert np.array_equal(np.asarray(product.ortho_noise(W)).reshape(want.shape), want)


def _unorm8_even(data):
    """The RGBA8 framebuffer's store of the shader's output, rounding ties to even
    (the oracle's choice; GL leaves the rounding of ties to the implementation)."""
    return np.rint(np.clip(data, 0.0, 1.0).astype(np.float32) * np.float32(255.0)).astype(np.uint8)


@pytest.mark.parametrize("variant", sorted(ORTHO))
@pytest.mark.parametrize("hsv", [False, True])
def test_ortho_tiles(ref, oracle_lib, variant, hsv):
    """OrthoProducer::doCreateTile (its uniforms: the parent window, the residual
    scale, the noise layer and rotation, the noise colour in RGB or HSV form) drawing
    the upsample ortho shader of terrain3 or the demo: after the framebuffer's 8-bit
    store, every tile byte for byte the oracle's -- levels 0-9, faces 0-6, with and
    without a residual tile, parents and residuals random bytes."""
    import ctypes as C
    W = 196
    noise = np.empty((6, W, W, 4), np.uint8)
    ref.ref_ortho_noise(W, noise.ctypes.data)
    amps = np.float32([-1.0, 30.0, 20.0, 12.0, 8.0, 5.0, 3.0, 2.0, 1.0, 0.5])
    rng = np.random.default_rng(17 + 2 * ORTHO[variant] + int(hsv))
    for k, (level, tx, ty) in enumerate([(0, 0, 0), (1, 1, 0), (2, 3, 1), (4, 9, 14), (7, 100, 33), (9, 511, 2)]):
        for has_res in (True, False):
            face = k % 7
            parent = rng.integers(0, 256, (W, W, 4)).astype(np.uint8) if level > 0 else None
            res = rng.integers(0, 256, (W, W, 4)).astype(np.uint8) if has_res else None
            root_color = rng.uniform(0, 1, 4).astype(np.float32)
            noise_color = rng.uniform(0.2, 1.5, 4).astype(np.float32)
            scale = float(rng.choice([1.0, 2.0, 3.5]))
            out = np.empty((W, W, 4), np.float32)
            rc = ref.ref_gl_ortho_tile(ORTHO[variant], W, level, tx, ty, face,
                                       None if parent is None else parent.ctypes.data,
                                       None if res is None else res.ctypes.data, noise.ctypes.data, _p(amps),
                                       len(amps), _p(root_color), _p(noise_color), int(hsv), C.c_float(scale), _p(out))
            assert rc == 0
            rot, layer = oracle_lib.noise_select(face, level, tx, ty)
            amp = float(amps[level]) if level < len(amps) else 0.0
            want = oracle_lib.ortho_tile(W, level, tx, ty, parent, res, noise[layer], rot, amp, root_color=root_color,
                                         noise_color=noise_color, scale=scale, hsv=hsv)
            assert np.array_equal(_unorm8_even(out), want), (variant, hsv, level, tx, ty, face, has_res)


def _drawn(ref, n):
    import ctypes as C
    out = []
    for k in range(n):
        m, nv, ni = C.c_int(), C.c_int(), C.c_int()
        assert ref.ref_drawn_mesh(k, C.byref(m), C.byref(nv), C.byref(ni), None, None) == 0
        v = np.empty((nv.value, 4), np.float32)
        ix = np.empty(ni.value, np.uint32)
        ref.ref_drawn_mesh(k, C.byref(m), C.byref(nv), C.byref(ni), v.ctypes.data, ix.ctypes.data)
        out.append((v, ix if ni.value else None, m.value))
    return out


def _same_meshes(got, want):
    assert len(got) == len(want)
    for (gv, gi, gm), (wv, wi, wm) in zip(got, want):
        assert gm == wm
        assert np.array_equal(gv, np.asarray(wv, np.float32)), np.abs(gv - wv).max()
        assert (gi is None and wi is None) or np.array_equal(gi, wi)


def _polyline(rng, origin, size, n):
    pts = np.column_stack([origin[0] + rng.uniform(-100, size + 100, n), origin[1] + rng.uniform(-100, size + 100, n)])
    s = np.float32(np.concatenate([[0.0], np.cumsum(np.sqrt((np.diff(pts, axis=0) ** 2).sum(1)))]))
    return pts, s


def test_road_layer_meshes(ref, product):
    """RoadElevationLayer::doCreateTile's placement of a road (scale, tile offset,
    BASEWIDTH / TOTALWIDTH, the drawCurveAltitude call) and
    ElevationGraphLayer::drawCurveAltitude itself, against the product's mesh builder
    (proland_gb300.layers: tile_transform, base_width, curve_altitude_meshes,
    road_strip): every mesh -- start cap, strip, end cap -- vertex and index for index.
    The altitude profile is the identity (getAltitude(s) = s) and the builder gets the
    points' s as their altitudes, so that z shows where each vertex sampled the curve."""
    import ctypes as C
    from proland_gb300 import layers
    rng = np.random.default_rng(8)
    for trial in range(24):
        W = (101, 197)[trial % 2]
        size = 4000.0 / (1 << (trial % 5))
        origin = (float(rng.uniform(-8000, 8000)), float(rng.uniform(-8000, 8000)))
        pts, s = _polyline(rng, origin, size, 2 + trial % 5)
        width = float(rng.uniform(3.0, 40.0))
        cs, ce = trial % 2, (trial // 2) % 2
        sc = C.c_float()
        n = ref.ref_road_meshes(origin[0], origin[1], size, W, 2, np.ascontiguousarray(pts).ctypes.data,
                                s.ctypes.data, len(pts), width, cs, ce, C.byref(sc))
        tr = layers.tile_transform(origin, size, W)
        assert np.float32(sc.value) == np.float32(tr[3])
        base = layers.base_width(width, tr[3])
        total = np.float32(base * np.float32(3.0))
        step = max(np.float32(1.0), np.float32(np.float32(1.0) / tr[3]))
        want = layers.curve_altitude_meshes(pts, s, total, np.float32(total / base), step, tr, start_cap=bool(cs),
                                            end_cap=bool(ce))
        _same_meshes(_drawn(ref, n), want)
        if not cs:
            assert np.array_equal(_drawn(ref, n)[0][0], layers.road_strip(pts, s, width, origin, size, W))


def test_water_curve_meshes(ref, product):
    """drawCurveAltitude with the water layer's arguments (WaterElevationLayer.cpp:
    the other curves at width w, nwidth 1, no caps; rivers at TOTALWIDTH with caps)."""
    from proland_gb300 import layers
    rng = np.random.default_rng(9)
    for trial in range(16):
        W, size = 101, 2000.0 / (1 << (trial % 4))
        origin = (float(rng.uniform(-5000, 5000)), float(rng.uniform(-5000, 5000)))
        tr = layers.tile_transform(origin, size, W)
        pts, s = _polyline(rng, origin, size, 2 + trial % 4)
        w = np.float32(rng.uniform(2.0, 60.0))
        step = max(np.float32(1.0), np.float32(np.float32(1.0) / tr[3]))
        if trial % 2:
            base = layers.base_width(w, tr[3])
            width, nwidth, cs, ce = np.float32(base * np.float32(3.0)), None, trial % 3 == 0, trial % 4 == 1
            nwidth = np.float32(width / base)
        else:
            width, nwidth, cs, ce = w, np.float32(w / w), False, False
        n = ref.ref_curve_altitude(tr[0], tr[1], tr[2], np.ascontiguousarray(pts).ctypes.data, s.ctypes.data,
                                   len(pts), float(width), float(nwidth), float(step), int(cs), int(ce))
        want = layers.curve_altitude_meshes(pts, s, width, nwidth, step, tr, start_cap=cs, end_cap=ce)
        _same_meshes(_drawn(ref, n), want)


def test_curve_part_strips(ref, product):
    """GraphLayer::drawCurve(tileCoords, p, part, ...) against layers.curve_part_strip:
    the water layer's boundary parts (0, +-12, 1, 2) and random ones."""
    from proland_gb300 import layers
    rng = np.random.default_rng(10)
    for trial in range(16):
        W, size = 101, 3000.0 / (1 << (trial % 4))
        origin = (float(rng.uniform(-5000, 5000)), float(rng.uniform(-5000, 5000)))
        tr = layers.tile_transform(origin, size, W)
        pts, _ = _polyline(rng, origin, size, 2 + trial % 6)
        part = [(0.0, 12.0, 1.0, 2.0), (0.0, -12.0, 1.0, 2.0)][trial % 2] if trial < 8 else \
            tuple(float(v) for v in rng.uniform(-20, 20, 4))
        n = ref.ref_curve_part(tr[0], tr[1], tr[2], np.ascontiguousarray(pts).ctypes.data, len(pts), 10.0,
                               _p(np.float32(part)))
        got = _drawn(ref, n)
        assert len(got) == 1 and got[0][2] == 1 and got[0][1] is None
        assert np.array_equal(got[0][0], layers.curve_part_strip(pts, part, tr)), trial   # part as plain floats


@pytest.mark.parametrize("D,level,tx,ty", [(12.72e6, 0, 0, 0), (12.72e6, 1, 1, 0), (12.72e6, 3, 5, 2),
                                           (12.72e6, 12, 1000, 3000), (6.4e6, 16, 40000, 12345), (100000.0, 2, 1, 3)])
def test_sphere_patch_frames(ref, oracle_lib, product, D, level, tx, ty):
    """NormalProducer::doCreateTile's FP64 patch frame, read back from the uniforms it
    sets (NormalProducer.cpp:215-273), is the oracle's frame and the product's
    (tp_sphere_frame) bit for bit, parentToTangentFrame the oracle's."""
    u = np.empty(58, np.float32)
    assert ref.ref_sphere_uniforms(101, level, tx, ty, D, _p(u)) == 0
    C_, N_, L_, W2T, P2T, deform = u[:16], u[16:32], u[32:36], u[36:45], u[45:54], u[54:58]
    D = float(np.float32(D))     # getRootQuadSize() is a float
    f = oracle_lib.sphere_frame(D, level, tx, ty)
    assert np.array_equal(C_, np.float32(f.C)) and np.array_equal(N_, np.float32(f.N))
    assert np.array_equal(L_, np.float32(f.L)) and np.array_equal(W2T, np.float32(f.W2T))
    assert deform[2] == np.float32(f.size) and deform[3] == np.float32(f.R)
    mine = product.sphere_frame(D, level, tx, ty)
    assert np.array_equal(mine[:45], u[:45])
    if level > 0:
        assert np.array_equal(P2T, oracle_lib.parent_to_tangent(D, level, tx, ty))


DEM_FILES = ["terrain/examples/terrain4", "edit/examples/edit3", "edit/examples/edit4", "graph/examples/graph1",
             "river/examples/river1"]


@pytest.mark.parametrize("name", DEM_FILES)
@pytest.mark.parametrize("delta,zscale", [(0, 1.0), (2, 0.5), (3, 2.0)])
def test_residual_producer_on_reference_pyramids(ref, oracle_lib, product, name, delta, zscale):
    """ResidualProducer as written (ResidualProducer.cpp: init reading the .dat header
    and offsets, hasTile, doCreateTile with the deltaLevel chain of readTile and
    upsample, getTileSize / getTileId below minLevel, int16 * scale * zscale), on the
    reference's own DEM.dat pyramids, its TIFF strips inflated by zlib: every tile of
    levels 0-3 and a spread of deeper ones is the product's host residual tile
    (tp_residual_tile) bit for bit, and both answer hasTile alike.

    Only tiles the pyramid holds are read: at pyramid level p = level + delta >= minLevel,
    tx, ty < 2^(p - minLevel) (below minLevel every (tx, ty) names the level's single
    tile).  hasTile checks the root only, and the elevation producer asks for
    (level, tx / mod, ty / mod), which stays inside; the reference reads past its
    offsets table for a tile outside, where the product returns TP_E_BAD_ARG."""
    path = oracle_lib.ref_file("src/%s/DEM.dat" % name)
    if path is None:
        pytest.skip("the reference's pyramids are not on this machine")
    assert _residual_producers_agree(ref, product, path, delta, zscale, len(name) + delta) >= 20


def _residual_producers_agree(ref, product, path, delta, zscale, seed):
    """The reference's ResidualProducer and the product's on the .dat file at `path`: every
    tile of the first four pyramid levels and six random ones per deeper level alike, hasTile
    alike, and no tile past the last level.  With a root tile at level r > 0 (deltaLevel is
    then 0), pyramid level l is asked for at level r + l, at (rootTx << l, rootTy << l)
    plus the tile's place in the pyramid.  Returns the number of tiles compared."""
    import ctypes as C
    import struct
    min_level, max_level, tile_size, root_level, root_tx, root_ty = struct.unpack(
        "<6i", open(path, "rb").read(24))
    eff = delta if root_level == 0 else 0
    W = tile_size + 5
    storage = product.TileStorage(W, 1, 8, on_device=product.TileStorage.BOOKKEEPING)
    prod = product.ResidualProducer(product.TileCache(storage, "residuals"), path, delta=delta, zscale=zscale)
    rng = np.random.default_rng(seed)
    checked = 0
    for p in range(eff, max_level + 1):
        level = p - eff + root_level
        n = 1 << (p - min_level) if p >= min_level else 1 << (p - eff)
        tiles = {(x, y) for x in range(min(n, 4)) for y in range(min(n, 4))}
        tiles |= {(int(rng.integers(0, n)), int(rng.integers(0, n))) for _ in range(6)}
        for x, y in sorted(tiles):
            tx, ty = (root_tx << (p - eff)) + x, (root_ty << (p - eff)) + y
            out = np.full((W, W), np.nan, np.float32)
            has = C.c_int()
            assert ref.ref_residual_tile(path.encode(), delta, zscale, W, level, tx, ty, out.ctypes.data,
                                         C.byref(has)) == 0
            assert prod.has_tile(level, tx, ty) == bool(has.value), (level, tx, ty)
            if has.value:
                written = ~np.isnan(out)    # a tile below minLevel fills the slot's corner
                assert np.array_equal(prod.tile(level, tx, ty)[written], out[written]), (level, tx, ty)
                checked += 1
    # past the pyramid's last level, and beside a root tile above level 0: no tile on either side
    last = max_level - eff + root_level + 1
    outside = [(last, root_tx << (last - root_level), root_ty << (last - root_level)),
               (last, (root_tx << (last - root_level)) + 1, root_ty << (last - root_level))]
    if root_level > 0:
        outside.append((root_level, root_tx + 1, root_ty))
    for level, tx, ty in outside:
        has = C.c_int()
        out = np.zeros((W, W), np.float32)
        ref.ref_residual_tile(path.encode(), delta, zscale, W, level, tx, ty, out.ctypes.data, C.byref(has))
        assert not has.value and not prod.has_tile(level, tx, ty), (level, tx, ty)
    return checked


@pytest.mark.parametrize("top,ts,max_level,root,delta,zscale", [
    (6, 24, 5, (0, 0, 0), 0, 1.0), (6, 24, 5, (0, 0, 0), 2, 0.5), (6, 24, 5, (3, 5, 2), 2, 2.0),
    (24, 24, 3, (2, 1, 3), 0, 1.0), (12, 24, 4, (0, 0, 0), 1, 1.0)])
def test_residual_producer_on_generated_pyramids(ref, oracle_lib, product, tmp_path, top, ts, max_level, root,
                                                 delta, zscale):
    """The same comparison on pyramids that the reference's own preprocess writes
    (HeightMipmap::generate over a synthetic terrain): minLevel 2 and 1 with
    root tiles of 6 and 12 intervals, which ResidualProducer upsamples below minLevel;
    root tiles at levels 3 and 2 (where the deltaLevel asked for is set to 0); deltaLevel
    0-2.  (A deltaLevel above minLevel is an assertion in ResidualProducer::init and an
    error from tp_residual_producer_create.  ResidualProducer::readTile also asserts that a
    stored tile, TIFF header and directory included, is smaller than the raw tile,
    ResidualProducer.cpp:291; for tiles of 12 intervals (578 raw bytes) a noisy residual
    strip plus that overhead is not, so the stored levels here have 24 intervals.)"""
    import ctypes as C
    n = (top << max_level) + 1
    base = oracle_lib.fbm_heights(n, octaves=8, base_cells=2, seed=top + ts)
    assert ref.ref_mipmap_build_sized(base.ctypes.data_as(C.POINTER(C.c_int16)), top, ts, max_level, 1.0,
                                      str(tmp_path).encode()) == max_level
    path = str(tmp_path / "DEM.dat")
    try:
        ref.ref_mipmap_generate(*root, 1.0, path.encode())
    finally:
        ref.ref_mipmap_free()
    assert _residual_producers_agree(ref, product, path, delta, zscale, top + delta) >= 10


def test_ortho_cpu_producer_on_reference_pyramid(ref, oracle_lib, product):
    """OrthoCPUProducer as written (OrthoCPUProducer.cpp: init reading the header and
    64-bit offsets, hasTile, doCreateTile inflating the tile's TIFF strip, getTileId) on
    the reference's graph1/RGB.dat: every tile byte for byte the product's reader
    (tp_ortho_dat_read_tile), the header fields alike."""
    import ctypes as C
    path = oracle_lib.ref_file("src/graph/examples/graph1/RGB.dat")
    if path is None:
        pytest.skip("the reference's pyramids are not on this machine")
    d = product.OrthoDat(path)
    info = (C.c_int * 5)()
    checked = 0
    for level in range(0, d.max_level + 2):
        for tx in range(1 << level):
            for ty in range(1 << level):
                out = np.zeros((d.width, d.width, d.channels), np.uint8)
                has = C.c_int()
                assert ref.ref_ortho_dat_tile(path.encode(), level, tx, ty, out.ctypes.data, out.size, info,
                                              C.byref(has)) == 0
                assert list(info) == [d.max_level, d.tile_size, d.channels, 0 if d.flags & 2 else 2, d.width]
                assert bool(has.value) == (level <= d.max_level)
                if has.value:
                    assert np.array_equal(d.tile(level, tx, ty), out), (level, tx, ty)
                    checked += 1
    assert checked == sum(4 ** l for l in range(d.max_level + 1))


RIVER, ISLAND, LAKE = 0, 1, 2   # WaterElevationCurveData::riverType


def _loop(rng, cx, cy, r, n):
    a = np.sort(rng.uniform(0, 2 * np.pi, n))
    pts = np.column_stack([cx + r * np.cos(a), cy + r * np.sin(a)])
    return np.vstack([pts, pts[:1]])


def _curve_s(pts):
    return np.float32(np.concatenate([[0.0], np.cumsum(np.sqrt((np.diff(pts, axis=0) ** 2).sum(1)))]))


@pytest.mark.parametrize("seed", range(4))
def test_water_layer_pass_sequence(ref, product, seed):
    """WaterElevationLayer::doCreateTile as written (WaterElevationLayer.cpp:240-365),
    with GraphLayer::drawArea, drawCurve and drawCurveAltitude, over a stand-in graph
    (a lake with an island, a mixed area, curves of other types, rivers with caps, a
    river too narrow to draw), against proland_gb300.layers.water_layer given the
    inputs its docstring asks of the caller (areas, boundaries with the island
    orientation flipped, the other curves, the rivers -- chosen by the reference's
    filters): draw for draw, the program, the river uniform, the depth test and depth
    mask, the z / w colour masks and the fill depth match the product's mesh, program,
    state and fill depth, and every curve mesh is the product's vertex and index for
    index.  (The fill triangles are GLU's in the reference; the stand-in tessellator
    records the area contours, which are the clip-space contours of the areas.)"""
    import ctypes as C
    from proland_gb300 import layers
    tp = product
    rng = np.random.default_rng(seed)
    W, size, level = 101, 2000.0, 3
    origin = (float(rng.uniform(-3000, 3000)), float(rng.uniform(-3000, 3000)))
    ox, oy = origin
    cx, cy = ox + size / 2, oy + size / 2
    lake = _loop(rng, cx, cy, 700.0, 9)
    island = _loop(rng, cx + 60, cy - 40, 150.0, 6)
    other = np.column_stack([np.linspace(ox - 50, ox + size + 50, 5), oy + rng.uniform(0, size, 5)])
    river = np.column_stack([ox + rng.uniform(0, size, 4), np.linspace(oy - 80, oy + size + 80, 4)])
    narrow = np.column_stack([np.linspace(ox, ox + size, 3), oy + rng.uniform(0, size, 3)])
    # (points, type, has parent, in an area, cap start, cap end, width)
    curves = [(lake, LAKE, 1, 1, 0, 0, 30.0), (island, ISLAND, 1, 1, 0, 0, 20.0), (other, 3, 1, 0, 0, 0, 25.0),
              (other[::-1].copy(), ISLAND, 1, 0, 0, 0, 40.0), (river, RIVER, 1, 0, seed % 2, 1, 35.0),
              (narrow, RIVER, 1, 0, 0, 0, 1.0)]
    areas = [[(0, 0), (1, 0)], [(1, 1)], [(0, 1)]]   # mixed (island skipped), island, lake reversed
    info = np.array([[len(c[0]), c[1], c[2], c[3], c[4], c[5]] for c in curves], np.int32)
    xy = np.ascontiguousarray(np.vstack([c[0] for c in curves]), np.float64)
    s = np.concatenate([_curve_s(c[0]) for c in curves]).astype(np.float32)
    widths = np.float32([c[6] for c in curves])
    area_info = np.array(sum([[len(a)] + [v for pair in a for v in pair] for a in areas], []), np.int32)
    n = ref.ref_water_layer(ox, oy, size, W, level, len(curves), info.ctypes.data, xy.ctypes.data, s.ctypes.data,
                            _p(widths), len(areas), area_info.ctypes.data)
    assert n > 0
    # the product's inputs, chosen by the reference's rules
    tr = layers.tile_transform(origin, size, W)
    scale = tr[3]
    contour = [np.vstack([curves[k][0] if o == 0 else curves[k][0][::-1] for k, o in a]) for a in areas]
    boundaries = []
    for a in areas:
        island_area = all(curves[k][1] == ISLAND for k, _ in a)
        for k, o in a:
            if island_area:
                o = 1 - o
            elif curves[k][1] == ISLAND:
                continue
            boundaries.append((curves[k][0], o))
    others = [(c[0], _curve_s(c[0]), c[6]) for c in curves
              if not (np.float32(c[6]) * scale <= 1 or c[1] in (LAKE, RIVER) or c[3])]
    rivers = [(c[0], _curve_s(c[0]), c[6], bool(c[4]), bool(c[5])) for c in curves if c[1] == RIVER]
    want = layers.water_layer(origin, size, W, areas=[[cnt] for cnt in contour], boundaries=boundaries,
                              curves=others, rivers=rivers)
    assert len(want) == n
    drawn = _drawn(ref, n)
    for k, (v, ix, mode, prog, state, fill_depth) in enumerate(want):
        st = (C.c_int * 8)()
        un = np.empty(5, np.float32)
        assert ref.ref_water_draw(k, st, _p(un)) == 0
        fill, river, test_on, func, depth_mask, z_mask, w_mask, rmode = list(st)
        assert test_on == 1
        assert prog == (tp.LAYER_FILL if fill == 0 else 1 + river), k
        assert state == func | (0 if depth_mask else tp.NO_DEPTH_WRITE) | (0 if z_mask else tp.NO_Z_WRITE) | \
            (0 if w_mask else tp.NO_W_WRITE), k
        if fill == 0:
            assert np.float32(fill_depth) == un[0] and not np.any(un[1:]), k
            continue
        assert rmode == mode, k
        got = drawn[k]
        assert np.array_equal(got[0], np.asarray(v, np.float32)), k
        assert (got[1] is None and ix is None) or np.array_equal(got[1], ix), k
    # the areas' contours, as the tessellator received them
    for a, cnt in enumerate(contour):
        m = ref.ref_water_contour(a, None)
        pts = np.empty((m, 2), np.float64)
        ref.ref_water_contour(a, pts.ctypes.data)
        X = (cnt[:, 0] - tr[0]) * tr[2]
        Y = (cnt[:, 1] - tr[1]) * tr[2]
        assert np.array_equal(pts, np.column_stack([X, Y])), a


@pytest.mark.parametrize("seed", range(4))
def test_road_layer_draws(ref, product, seed):
    """RoadElevationLayer::doCreateTile as written (RoadElevationLayer.cpp:388-437) over a
    stand-in graph -- roads with and without caps at their ends, a road too narrow to draw,
    a curve of another type, a curve without a parent at a level above 0 -- after the
    elevation producer's LESS depth test, against proland_gb300.layers.road_layer given
    the roads the reference's filters keep: draw for draw, the road program under LESS with
    depth writes, z and w written, and every mesh vertex and index for index."""
    import ctypes as C
    from proland_gb300 import layers
    tp = product
    rng = np.random.default_rng(20 + seed)
    W, size, level = (101, 197)[seed % 2], 1500.0, 4
    ox, oy = float(rng.uniform(-4000, 4000)), float(rng.uniform(-4000, 4000))

    def road(n):
        return np.column_stack([ox + rng.uniform(-100, size + 100, n), oy + rng.uniform(-100, size + 100, n)])
    # (points, type, has parent, -, cap start, cap end, width)
    curves = [(road(4), 0, 1, 0, 1, 0, 12.0), (road(3), 0, 1, 0, 0, 1, 30.0), (road(5), 0, 1, 0, 1, 1, 8.0),
              (road(3), 0, 1, 0, 0, 0, 0.5), (road(3), 1, 1, 0, 0, 0, 20.0), (road(3), 0, 0, 0, 0, 0, 20.0)]
    info = np.array([[len(c[0]), c[1], c[2], c[3], c[4], c[5]] for c in curves], np.int32)
    xy = np.ascontiguousarray(np.vstack([c[0] for c in curves]), np.float64)
    s = np.concatenate([_curve_s(c[0]) for c in curves]).astype(np.float32)
    widths = np.float32([c[6] for c in curves])
    n = ref.ref_road_layer(ox, oy, size, W, level, len(curves), info.ctypes.data, xy.ctypes.data, s.ctypes.data,
                           _p(widths))
    kept = [(c[0], _curve_s(c[0]), c[6], bool(c[4]), bool(c[5])) for c in curves if c[1] == 0 and c[2]]
    want = layers.road_layer((ox, oy), size, W, roads=kept)
    assert len(want) == n and n >= 3
    drawn = _drawn(ref, n)
    for k, (v, ix, mode, prog, state, _) in enumerate(want):
        st = (C.c_int * 8)()
        un = np.empty(5, np.float32)
        ref.ref_water_draw(k, st, _p(un))
        _, _, test_on, func, depth_mask, z_mask, w_mask, rmode = list(st)
        assert (prog, state) == (tp.LAYER_ROAD, tp.DEPTH_LESS)
        assert (test_on, func, depth_mask, z_mask, w_mask, rmode) == (1, 0, 1, 1, 1, mode), k
        assert np.array_equal(drawn[k][0], np.asarray(v, np.float32)), k
        assert (drawn[k][1] is None and ix is None) or np.array_equal(drawn[k][1], ix), k


@pytest.mark.parametrize("channels", [1, 2, 3])
def test_ortho_tiles_with_fewer_residual_channels(ref, oracle_lib, channels):
    """A residual pyramid of 1-3 channels: OrthoProducer::doCreateTile uploads its tiles as
    RED / RG / RGB into the RGBA residual texture (the missing components 0, alpha 1, as
    GL's pixel transfer fills them); the oracle reads such a tile as rgba_words expands it.
    Tiles byte for byte alike, RGB and HSV noise."""
    import ctypes as C
    W = 196
    noise = np.empty((6, W, W, 4), np.uint8)
    ref.ref_ortho_noise(W, noise.ctypes.data)
    amps = np.float32([-1.0, 30.0, 20.0, 12.0, 8.0])
    rng = np.random.default_rng(60 + channels)
    for hsv in (False, True):
        for level, tx, ty in [(0, 0, 0), (2, 3, 1), (4, 9, 14)]:
            parent = rng.integers(0, 256, (W, W, 4)).astype(np.uint8) if level > 0 else None
            res = np.ascontiguousarray(rng.integers(0, 256, (W, W, channels)).astype(np.uint8))
            root_color = rng.uniform(0, 1, 4).astype(np.float32)
            noise_color = rng.uniform(0.2, 1.5, 4).astype(np.float32)
            out = np.empty((W, W, 4), np.float32)
            assert ref.ref_gl_ortho_tile_channels(1, W, level, tx, ty, 0, None if parent is None else parent.ctypes.data,
                                                  res.ctypes.data, channels, noise.ctypes.data, _p(amps), len(amps),
                                                  _p(root_color), _p(noise_color), int(hsv), C.c_float(2.0),
                                                  _p(out)) == 0
            rot, layer = oracle_lib.noise_select(0, level, tx, ty)
            want = oracle_lib.ortho_tile(W, level, tx, ty, parent, oracle_lib.rgba_words(res), noise[layer], rot,
                                         float(amps[level]), root_color=root_color, noise_color=noise_color,
                                         scale=2.0, hsv=hsv)
            assert np.array_equal(_unorm8_even(out), want), (channels, hsv, level)
