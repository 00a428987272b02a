"""The ortho producers behind the TileCache / TileProducer protocol on the GPU:
getTile of deep tiles pulls their parent chain and the residual tiles the
reference's RGB.dat holds, one scheduler run produces them parents first, and
every tile equals the oracle's chain byte for byte."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
MINI = os.path.join(HERE, "golden", "rgb_graph1_mini.dat")


@pytest.mark.parametrize("hsv", [False, True])
def test_ortho_producer_chain_matches_oracle(gpu, oracle_lib, hsv):
    tp = gpu
    W = 196
    amps = [255.0 * 0.7 ** l for l in range(17)]
    params = tp.make_ortho_params(root_color=(60 / 255, 150 / 255, 20 / 255, 1.0),
                                  noise_color=(70 / 255, 80 / 255, 100 / 255, 1.0), scale=2.0, hsv=hsv)
    ostore = tp.TileStorage(W, 1, 32)
    rstore = tp.TileStorage(W, 1, 8)
    res = tp.OrthoResidualProducer(tp.TileCache(rstore, "orthoCpu"), MINI)
    orth = tp.OrthoProducer(tp.TileCache(ostore, "ortho"), res, params, noise_amp=amps, face=1)
    want_tiles = [(2, 2, 0), (2, 3, 0), (2, 2, 1), (2, 3, 1), (3, 6, 2)]
    tiles = orth.create_tiles(want_tiles)
    tp.stream_check()
    golden = np.load(os.path.join(HERE, "golden", "ortho_golden.npz"))
    table = oracle_lib.ortho_noise(W)

    def expect(level, tx, ty, parent):
        rot, layer = tp.noise_select(1, level, tx, ty)
        key = "L%d_%d_%d" % (level, tx, ty)
        residual = golden[key] if key in golden.files else None
        return oracle_lib.ortho_tile(W, level, tx, ty, parent, residual, table[layer], rot, amps[level],
                                     root_color=list(params.root_color), noise_color=list(params.noise_color),
                                     scale=params.scale, hsv=hsv)
    root = expect(0, 0, 0, None)
    l1 = expect(1, 1, 0, root)
    l2 = {(x, y): expect(2, x, y, l1) for x in (2, 3) for y in (0, 1)}
    l3 = expect(3, 6, 2, l2[(3, 1)])
    want = [l2[(2, 0)], l2[(3, 0)], l2[(2, 1)], l2[(3, 1)], l3]
    for t, (l, x, y), w in zip(tiles, want_tiles, want):
        got = tp.texels_to_rgba(ostore.download(t.slot, 1, 0)[0])
        assert np.array_equal(got, w), (l, x, y)
    # the parents were produced too and stay cached (unused) for the next request
    p = orth.find_tile(1, 1, 0, include_cache=True)
    assert p is not None and p.info()["done"] == 1
    assert np.array_equal(tp.texels_to_rgba(ostore.download(p.slot, 1, 0)[0]), l1)
    for t in tiles:
        orth.put_tile(t)
