"""The batched-frame configuration at its full size: 4096 requests with levels
uniform in 1-12, a quarter of them 197-wide, fBm parents, residuals
N(0, (2000 * 0.5^l)^2) and noise 300 * 0.55^l, produced by one persistent launch
per tile width (CUDA graph).

The oracle produces every tile of the frame on all host threads: each tile's zf,
zc and zm are bit-identical to it and its normals within 1e-4.  Every tile is
also checked by properties that hold whatever the size (zm is exactly max(zf, 0),
normals are finite with nx^2 + ny^2 < 1), and the host-buffer pipeline (chunked
copies around the same kernel) returns the same bytes as the whole-frame launch."""
import os

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


def oracle_frame(orc, W, pz, pm, res, jobs):
    """Every tile of one width through the oracle's threaded batch runner:
    (zf, zc, zm, nx, ny) arrays of [n, ...]."""
    n = len(jobs)
    table = orc.dem_noise(W)
    zf, zc, zm = (np.empty((n, W, W), np.float32) for _ in range(3))
    nx, ny = (np.empty((n, W - 4, W - 4), np.float32) for _ in range(2))
    fp = orc._f32p
    recs = []
    for k, j in enumerate(jobs):
        b = orc.Job()
        b.W, b.level, b.tx, b.ty = W, j.level, j.tx, j.ty
        b.parent_zf, b.parent_zm, b.parent_pitch = pz[k].ctypes.data_as(fp), pm[k].ctypes.data_as(fp), W
        b.residual, b.res_pitch, b.rx, b.ry, b.rscale = res[k].ctypes.data_as(fp), W, 0, 0, 1.0
        b.noise, b.noise_rot, b.noise_amp = table[j.noise_layer].ctypes.data_as(fp), j.noise_rot, j.noise_amp
        b.tile_meters = j.tile_meters
        b.out_zf, b.out_zc, b.out_zm = (a[k].ctypes.data_as(fp) for a in (zf, zc, zm))
        b.out_pitch = W
        b.out_nx, b.out_ny, b.nrm_pitch = nx[k].ctypes.data_as(fp), ny[k].ctypes.data_as(fp), W - 4
        recs.append(b)
    orc.run_jobs(recs, os.cpu_count() or 1)
    return zf, zc, zm, nx, ny


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
        # every tile against the oracle: elevations bit for bit, normals within 1e-4
        zc = elev.download(0, n, tp.ZC)
        ezf, ezc, ezm, enx, eny = oracle_frame(oracle_lib, W, pz, pm, res, jobs)
        for name, got, want in (("zf", zf, ezf), ("zc", zc, ezc), ("zm", zm, ezm)):
            bad = np.nonzero((got != want).reshape(n, -1).any(axis=1))[0]
            assert bad.size == 0, "%s of %d tiles differs (W %d), first %s" % (name, bad.size, W, bad[:5])
        for name, got, want in (("nx", nx, enx), ("ny", ny, eny)):
            err = np.abs(got - want).reshape(n, -1).max(axis=1)
            assert float(err.max()) <= 1e-4, "%s: %d tiles off by more than 1e-4 (W %d)" % (
                name, int((err > 1e-4).sum()), W)
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
