"""The batched-frame configuration at its full size: 4096 requests with levels
uniform in 1-12, a quarter of them 197-wide, fBm parents, residuals
N(0, (2000 * 0.5^l)^2) and noise 300 * 0.55^l, produced by one persistent launch
per tile width (CUDA graph).

The oracle checks a seeded sample of the tiles bit for bit; every tile is checked
by properties that hold whatever the size: zm is exactly max(zf, 0), normals are
finite with nx^2 + ny^2 < 1, and the host-buffer pipeline (chunked copies around
the same kernel) returns the same bytes as the whole-frame launch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT_QUAD = 100000.0


def frame_class(tp, W, levels, tx, ty, seed):
    from proland_gb300 import workloads
    n = len(levels)
    uz, um = workloads.fbm_parent_tiles(min(48, n), W, seed)
    pick = np.arange(n) % uz.shape[0]
    pz, pm = np.ascontiguousarray(uz[pick]), np.ascontiguousarray(um[pick])
    res = workloads.residual_tiles(levels, W, seed + 1)
    jobs = []
    for k in range(n):
        l = int(levels[k])
        rot, layer = tp.noise_select(1, l, int(tx[k]), int(ty[k]))
        jobs.append(tp.make_job(l, int(tx[k]), int(ty[k]), out_slot=k, parent_slot=n + k, residual_slot=k,
                                normal_slot=k, noise_rot=rot, noise_layer=layer,
                                noise_amp=float(workloads.noise_amplitude(l)), tile_meters=ROOT_QUAD / (1 << l)))
    return pz, pm, res, jobs


def test_full_size_batched_frame(gpu, oracle_lib):
    tp = gpu
    from proland_gb300 import workloads
    levels, tx, ty, wide = workloads.frame_requests(4096, 2024)
    params = tp.make_params()
    classes = []
    frame = tp.Frame()
    for W, sel in ((101, ~wide), (197, wide)):
        idx = np.nonzero(sel)[0]
        pz, pm, res, jobs = frame_class(tp, W, levels[idx], tx[idx], ty[idx], 2024 + W)
        n = len(jobs)
        elev, rs, nrm = tp.TileStorage(W, 3, 2 * n), tp.TileStorage(W, 1, n), tp.TileStorage(W - 4, 2, n)
        elev.upload(n, tp.ZF, pz)
        elev.upload(n, tp.ZM, pm)
        rs.upload(0, 0, res)
        frame.add(elev, rs, nrm, params, jobs)
        classes.append((W, n, pz, pm, res, jobs, elev, rs, nrm))
    assert sum(c[1] for c in classes) == 4096
    frame.graph_launch()
    frame.graph_launch()   # replay: same inputs, same outputs
    tp.stream_check()
    rng = np.random.default_rng(5)
    for W, n, pz, pm, res, jobs, elev, rs, nrm in classes:
        zf = elev.download(0, n, tp.ZF)
        zm = elev.download(0, n, tp.ZM)
        nx = nrm.download(0, n, tp.NX)
        ny = nrm.download(0, n, tp.NY)
        # properties of every tile
        assert np.array_equal(zm, np.maximum(zf, np.float32(0.0))), "zm != max(zf, 0)"
        assert np.isfinite(zf).all() and np.isfinite(nx).all() and np.isfinite(ny).all()
        assert float((nx.astype(np.float64) ** 2 + ny.astype(np.float64) ** 2).max()) < 1.0
        # sampled tiles against the oracle, bit for bit (normals within 1e-4)
        table = oracle_lib.dem_noise(W)
        zc = elev.download(0, n, tp.ZC)
        for k in rng.choice(n, 24, replace=False):
            j = jobs[int(k)]
            ezf, ezc, ezm = oracle_lib.elevation_tile(W, j.level, j.tx, j.ty, pz[k], pm[k], res[k],
                                                      noise=table[j.noise_layer], noise_rot=j.noise_rot,
                                                      noise_amp=j.noise_amp)
            assert np.array_equal(zf[k], ezf) and np.array_equal(zc[k], ezc) and np.array_equal(zm[k], ezm), \
                "tile %d (level %d, W %d)" % (k, j.level, W)
            enx, eny = oracle_lib.normals_flat(W, ezm, float(j.tile_meters))
            assert np.abs(nx[k] - enx).max() <= 1e-4 and np.abs(ny[k] - eny).max() <= 1e-4
        # the host-buffer pipeline over all tiles of this width equals the whole-frame launch
        pipe = tp.HostPipeline(W, chunk=256 if W == 101 else 64)
        outs = [np.empty((n, W, W), np.float32) for _ in range(3)] + \
               [np.empty((n, W - 4, W - 4), np.float32) for _ in range(2)]
        pipe.run(params, jobs, pz, None, res, *outs)
        tp.stream_check()
        for name, got, want in zip(("zf", "zc", "zm", "nx", "ny"), outs, (zf, zc, zm, nx, ny)):
            assert np.array_equal(got, want), "host pipeline %s differs (W %d)" % (name, W)
        pipe.close()
    frame.close()
