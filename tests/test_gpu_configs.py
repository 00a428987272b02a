"""The benchmark configurations as parity cases: the whole levels 0-5 quadtree
(1365 tiles of 101 x 101, fBm root, residual sigma 2000 * 0.5^l, noise off,
normals for every tile) in one launch, each tile compared with the oracle and
with an FP64 evaluation of the same stencil on the same inputs."""
import sys
import os

import numpy as np
import pytest

from tilecase import assert_normals_close

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "proland-4.0_gb300"))
from proland_gb300 import workloads  # noqa: E402

pytestmark = pytest.mark.gpu


def quadtree_case(levels, W=101):
    tiles = [(l, x, y) for l in range(levels + 1) for y in range(1 << l) for x in range(1 << l)]
    resid = np.empty((len(tiles), W, W), np.float32)
    resid[0] = workloads.value_noise_fbm((W, W), octaves=8, seed=1)  # the root tile
    k = 1
    for l in range(1, levels + 1):
        m = 4 ** l
        resid[k:k + m] = workloads.residual_tiles([l] * m, W, seed=2 + l)
        k += m
    return tiles, resid


def test_config0_quadtree_levels_0_to_5(gpu, oracle_lib):
    tp, orc = gpu, oracle_lib
    W, D = 101, 50000.0
    tiles, resid = quadtree_case(5, W)
    n = len(tiles)
    assert n == 1365
    index = {t: k for k, t in enumerate(tiles)}
    elev, res, nrm = tp.TileStorage(W, 3, n), tp.TileStorage(W, 1, n), tp.TileStorage(W - 4, 2, n)
    res.upload(0, 0, resid)
    jobs = []
    for k, (l, x, y) in enumerate(tiles):
        pj = index[(l - 1, x // 2, y // 2)] if l > 0 else -1
        jobs.append(tp.make_job(l, x, y, out_slot=k, parent_slot=pj, residual_slot=k, normal_slot=k,
                                tile_meters=D / (1 << l), parent_job=pj))
    tp.elevation_batch(elev, res, nrm, tp.make_params(), jobs)
    tp.stream_check()
    zf, zc, zm = (elev.download(0, n, c) for c in (tp.ZF, tp.ZC, tp.ZM))
    nx, ny = (nrm.download(0, n, c) for c in (tp.NX, tp.NY))
    want = {}
    err64 = np.zeros(6)
    nerr64 = np.zeros(6)
    for k, (l, x, y) in enumerate(tiles):
        p = want.get((l - 1, x // 2, y // 2))
        args = (W, l, x, y, p[0] if p else None, p[2] if p else None, resid[k])
        ezf, ezc, ezm = orc.elevation_tile(*args)
        want[(l, x, y)] = (ezf, ezc, ezm)
        assert np.array_equal(zf[k], ezf), "zf %s" % (tiles[k],)
        assert np.array_equal(zc[k], ezc), "zc %s" % (tiles[k],)
        assert np.array_equal(zm[k], ezm), "zm %s" % (tiles[k],)
        enx, eny = orc.normals_flat(W, ezm, D / (1 << l))
        assert_normals_close(nx[k], enx, "nx %s" % (tiles[k],))
        assert_normals_close(ny[k], eny, "ny %s" % (tiles[k],))
        # the same stencil on the same float inputs, evaluated in FP64
        dzf, _, dzm = orc.elevation_tile(*args, f64=True)
        # error relative to the tile's height scale: single samples near zero height keep
        # the absolute cancellation error of fp32 arithmetic on heights of thousands of metres
        err64[l] = max(err64[l], float(np.max(np.abs(zf[k] - dzf)) / max(float(np.max(np.abs(dzf))), 1.0)))
        dnx, dny = orc.normals_flat_f64(W, dzm, D / (1 << l))
        nerr64[l] = max(nerr64[l], float(np.max(np.abs(nx[k] - dnx))), float(np.max(np.abs(ny[k] - dny))))
    print("max err of zf vs FP64 per level (relative to the tile's max |z|):", ["%.2e" % e for e in err64])
    print("max abs err of normals vs FP64 per level:", ["%.2e" % e for e in nerr64])
    assert err64.max() <= 1e-6 and nerr64.max() <= 1e-4
