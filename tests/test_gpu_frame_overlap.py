"""A two-width frame gives the same tiles whether its two persistent launches run on
forked streams (the default, two parallel graph nodes) or one after the other
(tp_frame_overlap_classes(f, 0)), through both tp_frame_launch and the CUDA graph."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_overlapped_and_serial_launches_agree(gpu, oracle_lib):
    tp = gpu
    from proland_gb300 import workloads
    frame = tp.Frame()
    classes = []
    for W, n, seed in ((101, 48, 1), (197, 16, 2)):
        rng = np.random.default_rng(seed)
        levels = rng.integers(1, 9, n)
        tx = np.array([rng.integers(0, 1 << int(l)) for l in levels])
        ty = np.array([rng.integers(0, 1 << int(l)) for l in levels])
        pz, pm = workloads.fbm_parent_tiles(n, W, seed)
        res = workloads.residual_tiles(levels, W, seed + 1)
        jobs = []
        for k in range(n):
            l = int(levels[k])
            rot, layer = tp.noise_select(1, l, int(tx[k]), int(ty[k]))
            jobs.append(tp.make_job(l, int(tx[k]), int(ty[k]), out_slot=k, parent_slot=n + k, residual_slot=k,
                                    normal_slot=k, noise_rot=rot, noise_layer=layer,
                                    noise_amp=float(workloads.noise_amplitude(l)), tile_meters=100000.0 / (1 << l)))
        elev, rs, nrm = tp.TileStorage(W, 3, 2 * n), tp.TileStorage(W, 1, n), tp.TileStorage(W - 4, 2, n)
        elev.upload(n, tp.ZF, pz)
        elev.upload(n, tp.ZM, pm)
        rs.upload(0, 0, res)
        frame.add(elev, rs, nrm, tp.make_params(), jobs)
        classes.append((W, n, elev, nrm, pz, pm, res, jobs, rs))

    def outputs():
        tp.stream_check()
        return [(e.download(0, n, tp.ZF), e.download(0, n, tp.ZM), m.download(0, n, tp.NX))
                for W, n, e, m, *_ in classes]

    frame.launch()
    overlapped = outputs()
    frame.graph_launch()
    graph_overlapped = outputs()
    frame.overlap_classes(False)
    frame.launch()
    serial = outputs()
    frame.graph_launch()
    graph_serial = outputs()
    for a, b, c, d in zip(overlapped, graph_overlapped, serial, graph_serial):
        for x, y, z, w in zip(a, b, c, d):
            assert np.array_equal(x, y) and np.array_equal(x, z) and np.array_equal(x, w)
    # and one tile of each width against the oracle
    for (W, n, e, m, pz, pm, res, jobs, _), (zf, _, _) in zip(classes, overlapped):
        j = jobs[0]
        table = oracle_lib.dem_noise(W)
        ezf, _, _ = oracle_lib.elevation_tile(W, j.level, j.tx, j.ty, pz[0], pm[0], res[0],
                                              noise=table[j.noise_layer], noise_rot=j.noise_rot,
                                              noise_amp=j.noise_amp)
        assert np.array_equal(zf[0], ezf)
    frame.close()
