"""Residual tiles of the reference's DEM.dat pyramids decoded on the device
(tp_dat_decode_device) equal the host decode, tile by tile; zero tiles stay zero;
a corrupt strip gives TP_E_IO and leaves the other tiles intact."""
import os
import shutil

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def stored_tiles(orc_dat):
    d = orc_dat
    out = []
    for l in range(0, d.max_level + 1):
        for x in range(1 << l):
            for y in range(1 << l):
                if (l >= d.min_level or (x == 0 and y == 0)) and d.tile_id(l, x, y) < d.ntiles \
                        and len(d.strip(l, x, y)) > 0:
                    out.append((l, x, y))
    return out


@pytest.mark.parametrize("name", ["dem_terrain4_mini.dat", "dem_edit3_mini.dat"])
def test_device_decode_matches_host(gpu, oracle_lib, name):
    tp = gpu
    path = os.path.join(GOLDEN, name)
    host = tp.DatPyramid(path)
    tiles = stored_tiles(oracle_lib.DatFile.open(path))
    assert tiles
    W = host.tile_size + 5
    res = tp.TileStorage(W, 1, len(tiles) + 1)
    scale = host.scale * 0.5
    host.decode_device(tiles + [(-1, 0, 0)], scale, res, list(range(len(tiles) + 1)))
    got = res.download(0, len(tiles) + 1, 0)
    for k, (l, x, y) in enumerate(tiles):
        v = host.tile_int16(l, x, y)
        w = v.shape[0]
        want = np.zeros((W, W), np.float32)
        want[:w, :w] = v.astype(np.float32) * np.float32(scale)
        assert np.array_equal(got[k], want), (l, x, y)
    assert not np.any(got[-1])
    host.close()


def test_corrupt_strip_is_an_io_error(gpu, oracle_lib, tmp_path):
    tp = gpu
    src = os.path.join(GOLDEN, "dem_terrain4_mini.dat")
    orc = oracle_lib.DatFile.open(src)
    tiles = stored_tiles(orc)
    l, x, y = tiles[-1]
    # flip bytes inside the deflate data of the last stored tile
    tid = orc.tile_id(l, x, y)
    a, b = int(orc.offsets[2 * tid]), int(orc.offsets[2 * tid + 1])
    data = bytearray(open(src, "rb").read())
    mid = orc.header + (a + b) // 2
    for k in range(mid, mid + 64):
        data[k] ^= 0x5A
    bad = tmp_path / "corrupt.dat"
    bad.write_bytes(bytes(data))
    d = tp.DatPyramid(str(bad))
    W = d.tile_size + 5
    res = tp.TileStorage(W, 1, 2)
    with pytest.raises(tp.TPError) as e:
        d.decode_device([(l, x, y)], d.scale, res, [0])
    assert e.value.code == tp.TP_E_IO
    # an intact tile of the same file still decodes
    d.decode_device([tiles[0]], d.scale, res, [1])
    v = d.tile_int16(*tiles[0])
    assert np.array_equal(res.download(1, 1, 0)[0][:v.shape[0], :v.shape[0]], v.astype(np.float32) * np.float32(d.scale))
    d.close()
