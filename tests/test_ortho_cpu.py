"""Ortho (colour) tiles on the CPU: the .dat reader against the reference's own
RGB.dat tiles (fixture decoded with Python's zlib), the RGBA8 noise table, and
the oracle's upsample arithmetic against known answers and an independent numpy
restatement of the shader (non-HSV path)."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
MINI = os.path.join(GOLDEN, "rgb_graph1_mini.dat")


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLDEN, "ortho_golden.npz"))


def test_oracle_reader_matches_fixture(oracle_lib, golden):
    d = oracle_lib.OrthoDatFile.open(MINI)
    assert [d.max_level, d.tile_size, d.channels, d.root, d.root_tx, d.root_ty, d.flags, d.ntiles] == \
        list(golden["header"])
    for key in ("L0_0_0", "L1_1_0"):
        lvl, tx, ty = (int(v) for v in key[1:].split("_"))
        assert np.array_equal(d.tile(lvl, tx, ty), golden[key])


def test_product_reader_matches_fixture(product, golden):
    d = product.OrthoDat(MINI)
    assert (d.max_level, d.tile_size, d.channels, d.ntiles, d.width) == (1, 192, 4, 5, 196)
    for key in ("L0_0_0", "L1_1_0"):
        lvl, tx, ty = (int(v) for v in key[1:].split("_"))
        assert np.array_equal(d.tile(lvl, tx, ty), golden[key])
        assert np.array_equal(d.tile_rgba(lvl, tx, ty), golden[key])   # already 4 channels
    # a tile left out of the mini pyramid has an empty strip: reported, not faked
    with pytest.raises(product.TPError) as e:
        d.tile(1, 0, 0)
    assert e.value.code == product.TP_E_IO
    with pytest.raises(product.TPError) as e:
        d.tile(2, 0, 0)
    assert e.value.code == product.TP_E_BAD_ARG
    d.close()


def test_rgba_expansion_of_fewer_channels(oracle_lib):
    t = np.arange(5 * 5 * 3, dtype=np.uint8).reshape(5, 5, 3)
    w = oracle_lib.rgba_words(t)
    assert np.array_equal(w[..., :3], t) and np.all(w[..., 3] == 255)
    one = oracle_lib.rgba_words(t[..., :1])
    assert np.all(one[..., 1:3] == 0) and np.all(one[..., 3] == 255)


@pytest.mark.parametrize("W", [196, 100, 36])
def test_noise_table_product_equals_oracle(product, oracle_lib, W):
    a = product.ortho_noise(W)
    b = oracle_lib.ortho_noise(W)
    assert np.array_equal(a, b)


def test_noise_table_structure(oracle_lib):
    W = 196
    t = oracle_lib.ortho_noise(W)
    # corners stay 128
    for layer in range(6):
        for (x, y) in [(0, 0), (3, 3), (W - 1, 0), (0, W - 1), (W - 1, W - 1), (W - 4, W - 4)]:
            assert np.all(t[layer, y, x] == 128)
    # border bands are mirrored: row 2 reversed is row 1, row 3 reversed is row 0
    for layer in range(6):
        assert np.array_equal(t[layer, 2, 4:W - 4], t[layer, 1, 4:W - 4][::-1])
        assert np.array_equal(t[layer, 3, 4:W - 4], t[layer, 0, 4:W - 4][::-1])
    # layers sharing an edge bit share that band; others differ
    assert np.array_equal(t[1, 2:4, 4:W - 4], t[2, 2:4, 4:W - 4])     # ids 1 and 3: bottom bit set
    assert not np.array_equal(t[0, 2:4, 4:W - 4], t[1, 2:4, 4:W - 4])
    # one centre sequence through all layers: no two centres repeat
    assert not np.array_equal(t[0, 4:W - 4, 4:W - 4], t[1, 4:W - 4, 4:W - 4])


def numpy_ortho(W, level, tx, ty, parent, residual, noise_layer, rot, amp, root, ncol, scale):
    """Non-HSV ortho tile restated with numpy float32 (independent of the C oracle)."""
    f = np.float32
    n = W - 4
    j, i = np.mgrid[0:W, 0:W]
    if residual is not None:
        r = residual.astype(f)
    elif level == 0:
        r = np.broadcast_to((np.array(root, f) * f(255.0)), (W, W, 4)).astype(f)
    else:
        r = np.full((W, W, 4), 128.0, f)
    if level > 0:
        dx, dy = (tx % 2) * (n // 2), (ty % 2) * (n // 2)
        px, py = (i + 1) // 2 + dx, (j + 1) // 2 + dy
        masks = np.array([[1, 3, 3, 9], [3, 1, 9, 3], [3, 9, 1, 3], [9, 3, 3, 1]], f)
        m = masks[(i % 2) + 2 * (j % 2)]
        p = parent.astype(f)
        s = (m[..., 0:1] * p[py, px] + m[..., 1:2] * p[py, px + 1] + m[..., 2:3] * p[py + 1, px] +
             m[..., 3:4] * p[py + 1, px + 1])
        c = np.floor(s / f(16.0))
        rs = f(scale) if residual is not None else f(-1.0)
        r = (r - f(128.0)) * rs + c
    x, y = {0: (i, j), 1: (j, W - 1 - i), 2: (W - 1 - i, W - 1 - j), 3: (W - 1 - j, i)}[rot]
    nv = noise_layer[y, x].astype(f)
    nc = (np.array(ncol, f) * f(scale) * f(amp)) / f(255.0)
    out = nc * (nv - f(128.0)) + r
    q = np.clip(out / f(255.0), f(0.0), f(1.0)) * f(255.0)
    return np.rint(q).astype(np.uint8)


@pytest.mark.parametrize("level,tx,ty,rot,with_res", [(0, 0, 0, 0, False), (0, 0, 0, 2, True), (3, 5, 2, 1, True),
                                                      (4, 10, 7, 3, False), (7, 100, 33, 0, True)])
def test_oracle_equals_numpy_restatement(oracle_lib, level, tx, ty, rot, with_res):
    W = 196
    rng = np.random.default_rng(level * 31 + tx)
    parent = rng.integers(0, 256, (W, W, 4), dtype=np.uint8)
    residual = rng.integers(0, 256, (W, W, 4), dtype=np.uint8) if with_res else None
    table = oracle_lib.ortho_noise(W)
    root, ncol = (0.3, 0.6, 0.1, 0.5), (70 / 255, 80 / 255, 100 / 255, 1.0)
    a = oracle_lib.ortho_tile(W, level, tx, ty, parent, residual, table[2], rot, 37.0, root_color=root,
                              noise_color=ncol, scale=2.0)
    b = numpy_ortho(W, level, tx, ty, parent, residual, table[2], rot, 37.0, root, ncol, 2.0)
    assert np.array_equal(a, b)


def test_known_answers(oracle_lib):
    W = 196
    table = oracle_lib.ortho_noise(W)
    # a constant parent and no residual, no noise: the masks sum to 16, so the child is that constant
    parent = np.full((W, W, 4), 77, np.uint8)
    out = oracle_lib.ortho_tile(W, 2, 1, 3, parent, None, table[0], 0, 0.0)
    assert np.all(out == 77)
    # residual 128 is zero whatever the scale
    out = oracle_lib.ortho_tile(W, 2, 1, 3, parent, np.full((W, W, 4), 128, np.uint8), table[0], 0, 0.0, scale=5.0)
    assert np.all(out == 77)
    # level 0 without residual: the root colour
    out = oracle_lib.ortho_tile(W, 0, 0, 0, None, None, table[0], 0, 0.0, root_color=(0.2, 0.4, 0.6, 1.0))
    assert np.all(out == np.round(np.array([0.2, 0.4, 0.6, 1.0], np.float32) * np.float32(255)).astype(np.uint8))
    # a horizontal ramp parent: even/odd child columns weigh (1, 3) and (3, 1)
    ramp = np.zeros((W, W, 4), np.uint8)
    ramp[..., 0] = np.arange(W, dtype=np.uint8)[None, :]
    out = oracle_lib.ortho_tile(W, 1, 0, 0, ramp, None, table[0], 0, 0.0)
    i = np.arange(W)
    px = (i + 1) // 2
    want = np.where(i % 2 == 0, (px * 4 + 3) * 4 // 16, (px * 4 + 1) * 4 // 16)   # (1 px + 3 (px+1)) etc., x4 rows
    assert np.array_equal(out[5, :, 0], want.astype(np.uint8))
    # saturation: noise pushes channels past 255 / below 0 and they clamp
    hi = np.full((W, W, 4), 250, np.uint8)
    out = oracle_lib.ortho_tile(W, 1, 0, 0, hi, None, table[0], 0, 255.0, noise_color=(1.0, 1.0, 1.0, 1.0),
                                scale=2.0)
    assert out.max() == 255 and out.min() == 0


def test_hsv_mode_keeps_grey_and_darkens_little_on_bright(oracle_lib):
    """HSV noise: a grey (zero saturation) tile keeps equal channels; the value
    factor 1 - smoothstep(0.4, 0.8, v) switches the noise off for bright texels."""
    W = 36
    table = oracle_lib.ortho_noise(W)
    grey = np.full((W, W, 4), 100, np.uint8)
    out = oracle_lib.ortho_tile(W, 1, 0, 0, grey, None, table[1], 1, 255.0, noise_color=(0.3, 0.3, 0.3, 1.0),
                                hsv=True)
    assert np.all(out[..., 0] == out[..., 1]) and np.all(out[..., 1] == out[..., 2])
    bright = np.zeros((W, W, 4), np.uint8)
    bright[..., 0], bright[..., 1], bright[..., 2] = 240, 230, 220
    out = oracle_lib.ortho_tile(W, 1, 0, 0, bright, None, table[1], 1, 255.0, noise_color=(0.3, 0.3, 0.3, 1.0),
                                hsv=True)
    assert np.abs(out[..., :3].astype(int) - bright[..., :3].astype(int)).max() <= 1


def test_ortho_producer_protocol_on_bookkeeping_storages(product):
    """getTile of an ortho tile acquires its parent chain and its residual (where the
    residual producer has one), queues them, and releases nothing until produced;
    hasTile and getBorder follow OrthoProducer / OrthoCPUProducer."""
    tp = product
    W = 196
    oc = tp.TileCache(tp.TileStorage(W, 1, 16, on_device=tp.TileStorage.BOOKKEEPING), "ortho")
    rc = tp.TileCache(tp.TileStorage(W, 1, 8, on_device=tp.TileStorage.BOOKKEEPING), "orthoCpu")
    res = tp.OrthoResidualProducer(rc, MINI)
    orth = tp.OrthoProducer(oc, res, tp.make_ortho_params(), noise_amp=[255.0] * 17, face=1, max_level=5)
    assert res.get_border() == 2 and orth.get_border() == 2
    assert res.has_tile(1, 1, 0) and not res.has_tile(2, 0, 0)          # maxLevel of the file is 1
    assert orth.has_tile(5, 31, 31) and not orth.has_tile(6, 0, 0)       # maxLevel attribute
    t = orth.get_tile(2, 3, 1)
    assert t is not None
    # the tile, its parent (1, 1, 0) and grandparent (0, 0, 0) are queued; the residual
    # producer queued the two levels it has
    assert orth.queued() == 3 and res.queued() == 2
    assert oc.get_used_tiles() == 3 and rc.get_used_tiles() == 2
    # a second request of a sibling reuses the queued parents
    t2 = orth.get_tile(2, 2, 1)
    assert orth.queued() == 4 and res.queued() == 2
    assert orth.put_tile(t2) == 0 and orth.put_tile(t) == 0
    # no file: zero tiles at levels 0 and 1 only (OrthoCPUProducer with an empty name)
    zc = tp.TileCache(tp.TileStorage(W, 1, 4, on_device=tp.TileStorage.BOOKKEEPING), "zeros")
    z = tp.OrthoResidualProducer(zc)
    assert z.has_tile(1, 1, 1) and not z.has_tile(2, 0, 0)
    with pytest.raises(tp.TPError):
        tp.OrthoProducer(tp.TileCache(tp.TileStorage(197, 1, 4, on_device=tp.TileStorage.BOOKKEEPING)), None)
