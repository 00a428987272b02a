"""The oracle's restatement against the reference's own code, compiled from its
sources by oracle/ref_build.py (oracle/_ref/libref.so): the LCG and cnoise of
math/noise.h / noise.cpp, createDemNoise's table (ElevationProducer.cpp:50-133),
the noise-layer choice (ElevationProducer.cpp:345-376), CPUElevationProducer's
residual addressing and stencil loop (CPUElevationProducer.cpp:178-245),
HeightMipmap's residual / encode / approximation functions (HeightMipmap.cpp:449-559),
its whole pyramid build (base-level tiles, decimated levels, residual chain) and the
.dat files its generate writes, read back by the library's and the oracle's readers.
Every comparison is bit for bit.  The product's host-side noise code is checked
against the same compiled reference; its CUDA kernels are checked against the
oracle by the GPU tests, which this pin anchors.

Runs where the reference tree is present (this is where the oracle is pinned);
skipped elsewhere."""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref(oracle_lib):
    L = oracle_lib.ref_lib()
    if L is None:
        pytest.skip("the reference sources are not on this machine")
    return L


def _f(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def test_lrandom_and_frandom(ref, oracle_lib):
    for seed in (1234567, 7654321, 5647381, 12345, 1, 2 ** 31 - 2):
        a, b = C.c_long(seed), C.c_long(seed)
        for _ in range(5000):
            assert ref.ref_lrandom(C.byref(a)) == oracle_lib.lib().or_lrandom(C.byref(b))
        a, b = C.c_long(seed), C.c_long(seed)
        got = [ref.ref_frandom(C.byref(a)) for _ in range(5000)]
        want = [oracle_lib.lib().or_frandom(C.byref(b)) for _ in range(5000)]
        assert np.array_equal(np.float32(got), np.float32(want))


@pytest.mark.parametrize("W", [13, 21, 37, 101, 197, 253])
def test_dem_noise_table(ref, oracle_lib, product, W):
    """createDemNoise's float table, rounded to fp16 as its R16F texture stores it,
    is the oracle's table and the product's."""
    raw = np.empty((6, W, W), np.float32)
    ref.ref_dem_noise(W, _f(raw))
    as_r16f = raw.astype(np.float16).astype(np.float32)
    assert np.array_equal(oracle_lib.dem_noise(W), as_r16f)
    assert np.array_equal(product.dem_noise(W), as_r16f)


def test_cnoise(ref, oracle_lib, product):
    rng = np.random.default_rng(1)
    pts = list(rng.uniform(-5000, 5000, (3000, 2)).astype(np.float32))
    # the points the layer choice evaluates: integers and half-integers
    pts += [(np.float32(x + h), np.float32(y + v)) for x in range(-40, 40, 3) for y in range(-40, 70, 5)
            for h in (0.0, 0.5) for v in (0.0, 0.5)]
    for x, y in pts:
        want = np.float32(ref.ref_cnoise2(float(x), float(y)))
        assert np.float32(oracle_lib.cnoise(x, y)) == want, (x, y)
        assert np.float32(product.cnoise(x, y)) == want, (x, y)


def test_noise_layer_choice(ref, oracle_lib, product):
    """Every face (0 flat, 1-6 cube faces), levels 0-12, the tile edges and random tiles."""
    rng = np.random.default_rng(2)
    r, l = C.c_int(), C.c_int()
    for face in range(7):
        for level in range(13):
            m = 1 << level
            coords = {(0, 0), (m - 1, 0), (0, m - 1), (m - 1, m - 1)}
            coords |= {(int(rng.integers(0, m)), int(rng.integers(0, m))) for _ in range(min(m * m, 40))}
            for tx, ty in coords:
                ref.ref_noise_select(face, level, tx, ty, C.byref(r), C.byref(l))
                want = (r.value, l.value)
                assert oracle_lib.noise_select(face, level, tx, ty) == want, (face, level, tx, ty)
                assert product.noise_select(face, level, tx, ty) == want, (face, level, tx, ty)


@pytest.mark.parametrize("W,Wr", [(101, 101), (101, 197), (197, 197), (21, 21), (21, 37)])
def test_cpu_elevation_loop(ref, oracle_lib, W, Wr):
    """CPUElevationProducer::doCreateTile's residual tile choice (tx / mod, ty / mod),
    offsets (rx, ry) and stencil, against the oracle's loop, for every parity of the
    tile coordinates, with and without a residual, at level 0 and below."""
    rng = np.random.default_rng(W * 1000 + Wr)
    n = W - 5
    mod = (Wr - 5) // n
    asked = (C.c_int * 3)()
    for level in (0, 1, 2, 5, 11):
        m = 1 << level
        for tx, ty in {(0, 0), (1, 0), (0, 1), (1, 1), (m - 1, m - 1),
                       (int(rng.integers(0, m)), int(rng.integers(0, m)))}:
            parent = (rng.standard_normal((W, W)) * 1000.0).astype(np.float32)
            for with_res in (True, False):
                resid = (rng.standard_normal((Wr, Wr)) * 50.0).astype(np.float32) if with_res else None
                out = np.empty((W, W), np.float32)
                ref.ref_cpu_elevation_tile(W, level, tx, ty, _f(parent), Wr, _f(resid) if with_res else None,
                                           _f(out), asked)
                assert tuple(asked) == (level, tx // mod, ty // mod)
                want = oracle_lib.cpu_elevation_tile(W, level, tx, ty, parent if level > 0 else None, resid,
                                                     (tx % mod) * n, (ty % mod) * n)
                assert np.array_equal(out, want), (level, tx, ty, with_res)
                # the shader-semantics oracle the GPU tests compare with: its zf without
                # noise is this loop's output (the reference's CPU / GPU pairing)
                if level > 0:
                    zf, _, _ = oracle_lib.elevation_tile(W, level, tx, ty, parent, np.maximum(parent, 0), resid,
                                                         rx=(tx % mod) * n, ry=(ty % mod) * n,
                                                         grid_g=max(n // 24, 1))
                    assert np.array_equal(zf, out), (level, tx, ty, with_res)


@pytest.mark.parametrize("W", [101, 197])
def test_heightmipmap_residual_encode_approx(ref, oracle_lib, W):
    """HeightMipmap's residual (fine minus the stencil of the parent approximation),
    its int16 encoding (round to nearest, little-endian bytes) and the approximation
    (stencil plus quantised residual), against the oracle's preprocess restatement."""
    rng = np.random.default_rng(W)
    n = W - 5
    for tx, ty in ((0, 0), (1, 0), (0, 1), (1, 1), (6, 3)):
        parent = (rng.standard_normal((W, W)) * 800.0).astype(np.float32)
        fine = (rng.standard_normal((W, W)) * 800.0 + 3.0).astype(np.float32)
        rq, enc, approx = oracle_lib.compute_residual(W, tx, ty, parent, fine)
        res = np.empty((W, W), np.float32)
        mx, mean = C.c_float(), C.c_float()
        ref.ref_compute_residual(n, n, _f(parent), _f(fine.copy()), 3, tx, ty, _f(res), C.byref(mx), C.byref(mean))
        raw = np.zeros((W, W, 2), np.uint8)
        ref.ref_encode_residual(n, n, 3, _f(res), raw.ctypes.data)
        assert np.array_equal(res, rq)
        assert np.array_equal(raw.reshape(-1).view("<i2").reshape(W, W), enc)
        tile = fine.copy()
        err = C.c_float()
        ref.ref_compute_approx_tile(n, n, _f(parent), _f(res), 3, tx, ty, _f(tile), C.byref(err))
        assert np.array_equal(tile, approx)


@pytest.mark.parametrize("ts,max_level,scale,seed", [(8, 5, 1.0, 3), (12, 3, 4.0, 7), (24, 2, 2.5, 11)])
def test_heightmipmap_pyramid(ref, oracle_lib, tmp_path, ts, max_level, scale, seed):
    """HeightMipmap's whole pyramid build (HeightMipmap.cpp:83-97, 131-323, 327-559, with
    AbstractTileCache.cpp's tile cache and clamped reads): the base-level tiles, each
    coarser level decimated from the one above, and the residual chain of buildResiduals
    (encoded residuals and the approximation tiles saved for the next level), against the
    oracle's level tiles (or_level_tile) and residual chain (or_compute_residual), bit for
    bit.  The (8, 5) case has 32 x 32 tiles at the finest level, two files of 16 x 16
    tiles a side."""
    base = oracle_lib.fbm_heights((ts << max_level) + 1, octaves=8, base_cells=2, seed=seed)
    assert ref.ref_mipmap_build(base.ctypes.data_as(C.POINTER(C.c_int16)), ts, max_level, scale,
                                str(tmp_path).encode()) == max_level
    W = ts + 5
    try:
        got = np.empty((W, W), np.float32)
        prev = {}
        for level in range(max_level + 1):
            cur = {}
            for ty in range(1 << level):
                for tx in range(1 << level):
                    want = oracle_lib.level_tile(base, ts, max_level, level, tx, ty, scale)
                    ref.ref_mipmap_level_tile(level, tx, ty, _f(got))
                    assert np.array_equal(got, want), (level, tx, ty)
                    if level == 0:
                        cur[tx, ty] = want
                        continue
                    _, enc, approx = oracle_lib.compute_residual(W, tx, ty, prev[tx // 2, ty // 2], want)
                    raw = np.zeros(2 * W * W, np.uint8)
                    assert ref.ref_mipmap_residual(level, tx, ty, raw.ctypes.data, raw.size) == raw.size
                    assert np.array_equal(raw.view("<i2").reshape(W, W), enc), (level, tx, ty)
                    if level < max_level:
                        ref.ref_mipmap_approx_tile(level, tx, ty, _f(got))
                        assert np.array_equal(got, approx), (level, tx, ty)
                    cur[tx, ty] = approx
            prev = cur
    finally:
        ref.ref_mipmap_free()


def _roundf(x32):
    """C's roundf (half away from zero) of float32 values, exactly."""
    x = np.asarray(x32, np.float64)
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


@pytest.mark.parametrize("top,ts,max_level,scale,root", [(8, 8, 4, 1.0, (0, 0, 0)), (6, 24, 4, 2.0, (2, 1, 3)),
                                                         (12, 12, 3, 0.5, (5, 17, 9))])
def test_heightmipmap_dat_file_reads_back(ref, oracle_lib, product, tmp_path, top, ts, max_level, scale, root):
    """HeightMipmap::generate's .dat file (HeightMipmap.cpp:99-129, 561-654: the header, the
    tile offsets in Lebesgue order, all-zero tiles sharing the first one's bytes, each tile
    a Deflate TIFF), written by the reference's code through a TIFF writer stand-in, read
    back by the library's own .dat reader and the oracle's: the header, and every tile equal to the residual
    buildResiduals encoded; the root tile is the level-0 heights over the scale, rounded.
    (6, 24) has minLevel 2: levels 0 and 1 are single tiles of 6 and 12 intervals.  The
    lower-left quadrant of the terrain is flat, so its residual tiles are all zero."""
    n = (top << max_level) + 1
    base = oracle_lib.fbm_heights(n, octaves=8, base_cells=2, seed=ts + max_level)
    base[: n // 2, : n // 2] = 1234
    assert ref.ref_mipmap_build_sized(base.ctypes.data_as(C.POINTER(C.c_int16)), top, ts, max_level, scale,
                                      str(tmp_path).encode()) == max_level
    path = str(tmp_path / "pyramid.dat")
    try:
        min_level = ref.ref_mipmap_generate(*root, scale, path.encode())
        d = product.DatPyramid(path)
        od = oracle_lib.DatFile.open(path)
        ntiles = min_level + ((1 << (2 * (max_level - min_level) + 2)) - 1) // 3
        assert [d.min_level, d.max_level, d.tile_size, d.root_level, d.root_tx, d.root_ty, d.ntiles] == \
            [min_level, max_level, ts, *root, ntiles]
        assert (1 << min_level) * top == ts and np.float32(d.scale) == np.float32(scale)
        W = ts + 5
        got = np.empty((W, W), np.float32)
        ref.ref_mipmap_level_tile(0, 0, 0, _f(got))
        root_tile = _roundf(got[: top + 5, : top + 5])
        assert np.array_equal(d.tile_int16(0, 0, 0), root_tile)
        if top == ts:
            assert np.array_equal(got, oracle_lib.level_tile(base, ts, max_level, 0, 0, 0, scale))
        zeros = 0
        raw = np.zeros(2 * W * W, np.uint8)
        for level in range(1, max_level + 1):
            w = min(top << level, ts) + 5
            for ty in range(1 << max(level - min_level, 0)):
                for tx in range(1 << max(level - min_level, 0)):
                    nb = ref.ref_mipmap_residual(level, tx, ty, raw.ctypes.data, raw.size)
                    assert nb == 2 * w * w
                    want = raw[:nb].view("<i2").reshape(w, w)
                    assert np.array_equal(d.tile_int16(level, tx, ty), want), (level, tx, ty)
                    assert np.array_equal(od.tile_int16(level, tx, ty), want), (level, tx, ty)
                    zeros += not want.any()
        assert zeros > 0 and np.abs(root_tile).max() > 0
        d.close()
    finally:
        ref.ref_mipmap_free()
