"""View-driven streaming through the native TileSampler (tp_sampler_update, holding
each quad's elevation and normal tiles): an
8192-slot cache per producer, synthetic residuals made on the device
(N(0, (2000 * 0.5^l)^2) stand-in), noise 300 * 0.55^l, flat normals fused into
the elevation launch, the seeded camera path from 10 km down to 50 m over a level
0-14 quadtree.  Every new tile of the frames visited is compared with the oracle:
its residual bit for bit, elevations (zf, zc, zm) bit for bit, normals within 1e-4."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "proland-4.0_gb300"))

pytestmark = pytest.mark.gpu

SEED = 4242


def make_chain(tp, S, slots=8192, W=101):
    rs, es, ns = tp.TileStorage(W, 1, slots), tp.TileStorage(W, 3, slots), tp.TileStorage(W - 4, 2, slots)
    rc, ec, nc = tp.TileCache(rs, "residual"), tp.TileCache(es, "elevation"), tp.TileCache(ns, "normal")
    r = tp.ResidualProducer(rc, synthetic=(2000.0, 0.5, SEED))
    amps = [300.0 * 0.55 ** l for l in range(S.MAX_LEVEL + 1)]
    e = tp.ElevationProducer(ec, r, noise_amp=amps, params=tp.make_params(), face=0)
    n = tp.NormalProducer(nc, e)
    for p in (e, n):
        p.set_root_quad_size(S.ROOT_SIZE)
    return (rs, es, ns), (rc, ec, nc), (r, e, n), amps


def test_sampler_streaming_every_new_tile(gpu, oracle_lib):
    tp, orc = gpu, oracle_lib
    from proland_gb300 import streaming as S
    W = 101
    (rs, es, ns), caches, (r, e, n), amps = make_chain(tp, S)
    sampler = tp.TileSampler(e, n)
    table = orc.dem_noise(W)
    memo = {}

    def residual(l, x, y):
        return orc.synthetic_residual(SEED, l, x, y, float(np.float32(2000.0 * 0.5 ** l)), W)

    def want(t):
        if t not in memo:
            l, x, y = t
            p = want((l - 1, x // 2, y // 2)) if l > 0 else None
            rot, layer = orc.noise_select(0, l, x, y)
            memo[t] = orc.elevation_tile(W, l, x, y, p[0] if p else None, p[2] if p else None, residual(l, x, y),
                                         noise=table[layer], noise_rot=rot, noise_amp=amps[l])
        return memo[t]

    cams = S.camera_path(600)
    total_new = 0
    checked_residuals = 0
    for f in list(range(0, 600, 40)) + [599]:
        req = S.quadtree_requests(cams[f])
        new = sampler.update(req)
        tp.stream_check()
        total_new += len(new)
        assert sampler.held() == len(req)
        if not new:
            continue
        eslots = [sampler.find(*t, producer=0).slot for t in new]
        nslots = [sampler.find(*t, producer=1).slot for t in new]
        # residual tiles go back to the LRU once their elevation tile is made (a quad whose
        # elevation tile came back from the LRU did not need its residual again)
        rtiles = [(t, r.find_tile(*t, include_cache=True)) for t in new[:16]]
        rtiles = [(t, h) for t, h in rtiles if h is not None]
        got = [np.stack([es.download(s, 1, ch)[0] for s in eslots]) for ch in (tp.ZF, tp.ZC, tp.ZM)]
        gnx = np.stack([ns.download(s, 1, tp.NX)[0] for s in nslots])
        gny = np.stack([ns.download(s, 1, tp.NY)[0] for s in nslots])
        for t, h in rtiles:
            assert np.array_equal(rs.download(h.slot, 1, 0)[0], residual(*t)), ("residual", f, t)
        checked_residuals += len(rtiles)
        for i, t in enumerate(new):
            wz = want(t)
            for c, name in enumerate(("zf", "zc", "zm")):
                assert np.array_equal(got[c][i], wz[c]), (f, t, name)
            enx, eny = orc.normals_flat(W, wz[2], S.ROOT_SIZE / (1 << t[0]))
            assert np.abs(gnx[i] - enx).max() <= 1e-4 and np.abs(gny[i] - eny).max() <= 1e-4, (f, t)
        for t in [t for t in memo if sampler.find(*t) is None]:
            del memo[t]
    assert total_new > 5000 and checked_residuals > 50
    sampler.close()
