"""View-driven streaming (an 8192-slot device TileCache, the seeded camera path
from 10 km down to 50 m over a level 0-14 quadtree): every frame's new tiles are
acquired and produced by one scheduler run, tiles of vanished quads released;
every new tile of each frame is compared with the oracle (zf, zc, zm bit for
bit)."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "proland-4.0_gb300"))

pytestmark = pytest.mark.gpu


def residual(level, tx, ty, width):
    rng = np.random.default_rng((level * 1000003 + tx) * 1000033 + ty)
    return (rng.standard_normal((width, width), dtype=np.float32) * np.float32(2000.0 * 0.5 ** level))


def test_streaming_camera_path(gpu, oracle_lib):
    tp, orc = gpu, oracle_lib
    from proland_gb300 import streaming as S
    W, slots = 101, 8192
    es, rs = tp.TileStorage(W, 3, slots), tp.TileStorage(W, 1, slots)
    ec, rc = tp.TileCache(es, "elevation"), tp.TileCache(rs, "residual")
    r = tp.ResidualProducer(rc, source=residual)
    amps = [300.0 * 0.55 ** l for l in range(S.MAX_LEVEL + 1)]
    e = tp.ElevationProducer(ec, r, noise_amp=amps, params=tp.make_params(), face=0)
    e.set_root_quad_size(S.ROOT_SIZE)
    streamer = S.Streamer(e)
    cams = S.camera_path(600)
    table = orc.dem_noise(W)
    memo = {}

    def want(t):
        if t not in memo:
            l, x, y = t
            p = want((l - 1, x // 2, y // 2)) if l > 0 else None
            rot, layer = orc.noise_select(0, l, x, y)
            memo[t] = orc.elevation_tile(W, l, x, y, p[0] if p else None, p[2] if p else None,
                                         residual(l, x, y, W), noise=table[layer], noise_rot=rot, noise_amp=amps[l])
        return memo[t]

    total_new = 0
    for f in list(range(0, 600, 40)) + [599]:
        req = S.quadtree_requests(cams[f])
        new = streamer.frame(req, tp.scheduler_run)
        tp.stream_check()
        total_new += len(new)
        assert ec.get_used_tiles() == len(req)
        if new:
            slots = [streamer.held[t].slot for t in new]
            got = [np.stack([es.download(s, 1, ch)[0] for s in slots]) for ch in (tp.ZF, tp.ZC, tp.ZM)]
            for i, t in enumerate(new):
                wz = want(t)
                for c, name in enumerate(("zf", "zc", "zm")):
                    assert np.array_equal(got[c][i], wz[c]), (f, t, name)
        # a later frame's new tile has its parent among this frame's tiles
        for t in [t for t in memo if t not in streamer.held]:
            del memo[t]
    assert total_new > 5000
