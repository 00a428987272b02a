"""Residual pyramid files: the library's own TIFF-strip parser and inflate decoder
against the reference's DEM.dat tiles (fixtures cut from the reference's files and
decoded with Python's zlib), error handling, and the residual producer's root
chain against the oracle.  No GPU needed."""
import os
import zlib

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KEPT = [(0, 0, 0), (1, 0, 0), (2, 0, 0), (3, 0, 0), (4, 0, 0)]


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLDEN, "dem_golden.npz"))


@pytest.mark.parametrize("name", ["terrain4", "edit3"])
def test_header_and_tiles_match_reference_decode(product, golden, name):
    d = product.DatPyramid(os.path.join(GOLDEN, "dem_%s_mini.dat" % name))
    h = golden["%s_header" % name]
    assert [d.min_level, d.max_level, d.tile_size, d.root_level, d.root_tx, d.root_ty, d.ntiles] == list(h)
    assert np.float32(d.scale) == golden["%s_scale" % name][0]
    for lvl, tx, ty in KEPT:
        t = d.tile_int16(lvl, tx, ty)
        want = golden["%s_L%d_%d_%d" % (name, lvl, tx, ty)]
        # tiles below minLevel are smaller: tileSize >> (minLevel - level), + 5
        ts = d.tile_size >> (d.min_level - lvl) if lvl < d.min_level else d.tile_size
        assert t.shape == (ts + 5, ts + 5)
        assert np.array_equal(t, want), (name, lvl)


def test_tile_ids_follow_residual_producer(product):
    # ResidualProducer::getTileId: level below minLevel -> level, else
    # minLevel + tx + ty * 2^l + (4^l - 1) / 3 with l = level - minLevel
    d = product.DatPyramid(os.path.join(GOLDEN, "dem_edit3_mini.dat"))
    assert d.ntiles == 3 + (4 ** 3 - 1) // 3
    with pytest.raises(product.TPError) as e:
        d.tile_int16(5, 3, 2)       # left out of the fixture: empty strip
    assert e.value.code == product.TP_E_IO
    with pytest.raises(product.TPError) as e:
        d.tile_int16(6, 0, 0)       # past maxLevel
    assert e.value.code == product.TP_E_BAD_ARG


@pytest.mark.parametrize("level", [0, 1, 6, 9])
def test_inflate_matches_zlib(product, level):
    rng = np.random.default_rng(level)
    data = rng.integers(0, 7, 40000, dtype=np.uint8).tobytes() + rng.bytes(3000) + b"proland" * 500
    assert product.inflate_zlib(zlib.compress(data, level), len(data) + 16) == data


def test_corrupt_and_truncated_streams(product, tmp_path):
    good = zlib.compress(b"x" * 1000 + bytes(range(256)) * 8, 6)
    bad = bytearray(good)
    bad[len(bad) // 2] ^= 0x5A
    with pytest.raises(product.TPError) as e:
        product.inflate_zlib(bytes(bad), 10000)
    assert e.value.code == product.TP_E_IO
    with pytest.raises(product.TPError):
        product.inflate_zlib(good[:-9], 10000)
    src = open(os.path.join(GOLDEN, "dem_edit3_mini.dat"), "rb").read()
    p = tmp_path / "short.dat"
    p.write_bytes(src[:100])            # header + part of the offset table
    with pytest.raises(product.TPError) as e:
        product.DatPyramid(str(p))
    assert e.value.code == product.TP_E_IO
    p.write_bytes(src[:len(src) - 5000])  # last strip truncated
    d = product.DatPyramid(str(p))
    with pytest.raises(product.TPError) as e:
        d.tile_int16(4, 0, 0)
    assert e.value.code == product.TP_E_IO
    with pytest.raises(product.TPError) as e:
        product.DatPyramid(str(tmp_path / "missing.dat"))
    assert e.value.code == product.TP_E_IO


@pytest.mark.parametrize("name,delta,zscale", [("edit3", 2, 0.1), ("terrain4", 2, 1.0), ("edit3", 0, 1.0)])
def test_residual_root_chain_matches_oracle(product, oracle_lib, name, delta, zscale):
    """ResidualProducer with delta: the root tile chains readTile + upsample over
    the pyramid's first levels (ResidualProducer.cpp:218-225)."""
    path = os.path.join(GOLDEN, "dem_%s_mini.dat" % name)
    storage = product.TileStorage(197, 1, 4, on_device=product.TileStorage.BOOKKEEPING)
    cache = product.TileCache(storage, "residuals")
    r = product.ResidualProducer(cache, path, delta=delta, zscale=zscale)
    got = r.tile(0, 0, 0)
    want = oracle_lib.residual_chain_root(oracle_lib.DatFile.open(path), delta, zscale)
    assert np.array_equal(got, want)
    # a tile below the root is one plain readTile at level + delta
    d = oracle_lib.DatFile.open(path)
    lvl = 3 - delta if delta else 3
    if lvl >= 1:
        t = r.tile(lvl, 0, 0)
        scale = np.float32(np.float32(d.scale) * np.float32(zscale))
        raw = d.tile_int16(lvl + delta, 0, 0).astype(np.float32) * scale
        w = raw.shape[0]
        assert np.array_equal(t[:w, :w], raw.astype(np.float32))


def test_delta_level_past_min_level_is_an_error(product):
    # ResidualProducer::init asserts deltaLevel <= minLevel (ResidualProducer.cpp:122);
    # the library refuses it with TP_E_BAD_ARG and accepts deltaLevel = minLevel
    path = os.path.join(GOLDEN, "dem_edit3_mini.dat")
    d = product.DatPyramid(path)
    W = d.tile_size + 5
    storage = product.TileStorage(W, 1, 4, on_device=product.TileStorage.BOOKKEEPING)
    product.ResidualProducer(product.TileCache(storage, "ok"), path, delta=d.min_level)
    with pytest.raises(product.TPError) as e:
        product.ResidualProducer(product.TileCache(storage, "past"), path, delta=d.min_level + 1)
    assert e.value.code == product.TP_E_BAD_ARG and "minLevel" in str(e.value)
    d.close()
