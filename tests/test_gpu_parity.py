"""Parity of the CUDA elevation + normal producer with the CPU oracle, through
the C ABI (tp_elevation_batch), on small seeded cases.

Elevations (zf, zc, zm) are compared within 1e-5 relative and are expected to be
bit-identical (same operation order, separately rounded operations); tile
indexing and residual addressing are integer and exact.  Normals within 1e-4
absolute.
"""
import numpy as np
import pytest

from tilecase import Case, assert_elev_close, assert_normals_close

pytestmark = pytest.mark.gpu


def run_cases(tp, oracle, cases, params, exact=True, residual_width=None, with_normals=True):
    W = cases[0].W
    Wr = residual_width or cases[0].Wr
    n = len(cases)
    elev = tp.TileStorage(W, 3, 2 * n)
    res = tp.TileStorage(Wr, 1, n)
    nrm = tp.TileStorage(W - 4, 2, n) if with_normals else None
    table = oracle.dem_noise(W)
    jobs, expect = [], []
    for k, c in enumerate(cases):
        parent_slot = -1
        if c.level > 0:
            parent_slot = n + k
            elev.upload(parent_slot, tp.ZF, c.parent_zf[None])
            elev.upload(parent_slot, tp.ZC, np.zeros_like(c.parent_zf)[None])
            elev.upload(parent_slot, tp.ZM, c.parent_zm[None])
        if c.residual is not None:
            res.upload(k, 0, c.residual[None])
        rot, layer = tp.noise_select(c.face, c.level, c.tx, c.ty)
        jobs.append(tp.make_job(c.level, c.tx, c.ty, out_slot=k, parent_slot=parent_slot,
                                residual_slot=k if c.residual is not None else -1,
                                rx=c.rx, ry=c.ry, normal_slot=k if with_normals else -1,
                                noise_rot=rot, noise_layer=layer, noise_amp=c.noise_amp,
                                rscale=c.rscale, tile_meters=float(c.tile_meters)))
        expect.append(c.oracle(oracle, table, params_dict(params), rot, layer))
    tp.elevation_batch(elev, res, nrm, params, jobs)
    tp.stream_check()
    zf = elev.download(0, n, tp.ZF)
    zc = elev.download(0, n, tp.ZC)
    zm = elev.download(0, n, tp.ZM)
    if with_normals:
        nx = nrm.download(0, n, tp.NX)
        ny = nrm.download(0, n, tp.NY)
    mism = 0
    for k, (ezf, ezc, ezm, enx, eny) in enumerate(expect):
        tag = "tile %d (level %d, %d, %d, W %d)" % (k, cases[k].level, cases[k].tx, cases[k].ty, W)
        mism += assert_elev_close(zf[k], ezf, tag + " zf")
        mism += assert_elev_close(zc[k], ezc, tag + " zc")
        mism += assert_elev_close(zm[k], ezm, tag + " zm")
        if with_normals:
            assert_normals_close(nx[k], enx, tag + " nx")
            assert_normals_close(ny[k], eny, tag + " ny")
    if exact:
        assert mism == 0, "%d elevation samples differ in their last bits" % mism
    return zf, zc, zm


def params_dict(p):
    return dict(grid_size=p.grid_size, flip=p.flip, no_clamp=p.no_clamp, noise_mode=p.noise_mode)


@pytest.mark.parametrize("W", [101, 197])
def test_stencil_residual_normals(gpu, oracle_lib, W):
    cases = [Case(W, lvl, tx, ty, seed=10 * lvl + tx + 3 * ty)
             for lvl, tx, ty in [(1, 0, 0), (1, 1, 0), (1, 0, 1), (1, 1, 1), (5, 17, 9), (7, 100, 127)]]
    run_cases(gpu, oracle_lib, cases, gpu.make_params())


@pytest.mark.parametrize("W,band_rows,stages", [(101, 26, 1), (101, 51, 2), (197, 99, 1), (197, 140, 1),
                                                 (197, 33, 2), (101, 101, 2), (197, 98, 1), (101, 50, 2),
                                                 (197, 48, 1), (197, 58, 2)])
def test_band_heights(gpu, oracle_lib, W, band_rows, stages):
    """Every band split of a tile, single- or double-buffered, produces the same bits
    (bands of band_rows rows, the last one the rest: down to one row)."""
    cases = [Case(W, lvl, tx, ty, seed=lvl + 5 * tx, noise_amp=-20.0) for lvl, tx, ty in [(1, 1, 0), (4, 7, 12), (0, 0, 0)]]
    run_cases(gpu, oracle_lib, cases, gpu.make_params(band_rows=band_rows, flip=True, stages=stages))


def test_residual_window_mod2(gpu, oracle_lib):
    """101-wide elevations on 197-wide residual tiles (terrain4): mod 2, the
    residual sub-window (tx % 2, ty % 2) * 96."""
    cases = [Case(101, 4, tx, ty, seed=tx * 7 + ty, residual_width=197) for tx in (4, 5) for ty in (8, 9)]
    run_cases(gpu, oracle_lib, cases, gpu.make_params(), residual_width=197)


def test_level0_and_no_residual(gpu, oracle_lib):
    cases = [Case(101, 0, 0, 0, seed=3), Case(101, 2, 3, 1, seed=4, with_residual=False),
             Case(101, 0, 0, 0, seed=5, with_residual=False, noise_amp=-140.0)]
    run_cases(gpu, oracle_lib, cases, gpu.make_params())


@pytest.mark.parametrize("W", [101, 197])
def test_noise_terrain1(gpu, oracle_lib, W):
    """|amp| * N with the DEM noise table, every rotation/layer the selector yields."""
    cases = [Case(W, lvl, tx, ty, seed=lvl * 13 + tx, noise_amp=a)
             for lvl, tx, ty, a in [(1, 0, 1, -140.0), (2, 3, 2, -100.0), (3, 5, 6, -15.0), (4, 9, 3, 5.0),
                                    (6, 33, 40, 2.5), (8, 200, 17, 1.0), (9, 311, 400, 0.5), (3, 7, 7, -8.0)]]
    run_cases(gpu, oracle_lib, cases, gpu.make_params())


def test_noise_modulated(gpu, oracle_lib):
    """Slope/curvature modulated noise of the demo shader (amp > 0) and the
    negative-amplitude branch."""
    cases = [Case(101, lvl, tx, ty, seed=lvl + tx, noise_amp=a, tile_meters=50000.0 / (1 << lvl))
             for lvl, tx, ty, a in [(1, 1, 1, 300.0), (3, 2, 5, 120.0), (5, 30, 2, -40.0), (0, 0, 0, 80.0)]]
    run_cases(gpu, oracle_lib, cases, gpu.make_params(noise_mode=1))


@pytest.mark.parametrize("flip,no_clamp", [(True, False), (False, True)])
def test_flip_and_noclamp(gpu, oracle_lib, flip, no_clamp):
    cases = [Case(101, lvl, tx, ty, seed=lvl * 5 + ty) for lvl, tx, ty in [(2, 1, 2), (4, 6, 11), (6, 63, 0)]]
    cases += [Case(197, 3, 5, 2, seed=77)]
    run_cases(gpu, oracle_lib, cases[:3], gpu.make_params(flip=flip, no_clamp=no_clamp))
    run_cases(gpu, oracle_lib, cases[3:], gpu.make_params(flip=flip, no_clamp=no_clamp))


def test_quadtree_waves(gpu, oracle_lib):
    """Levels 0..3 (85 tiles) in one batch: children name their parent's job and the
    batch runs in dependency waves; compared with the oracle run level by level."""
    tp, orc = gpu, oracle_lib
    W = 101
    rng = np.random.default_rng(5)
    tiles = [(l, x, y) for l in range(4) for y in range(1 << l) for x in range(1 << l)]
    index = {t: k for k, t in enumerate(tiles)}
    n = len(tiles)
    elev = tp.TileStorage(W, 3, n)
    res = tp.TileStorage(W, 1, n)
    nrm = tp.TileStorage(W - 4, 2, n)
    resid = (rng.standard_normal((n, W, W)) * np.array([2000.0 * 0.5 ** l for l, _, _ in tiles])[:, None, None]).astype(np.float32)
    res.upload(0, 0, resid)
    jobs = []
    for k, (l, x, y) in enumerate(tiles):
        pj = index[(l - 1, x // 2, y // 2)] if l > 0 else -1
        jobs.append(tp.make_job(l, x, y, out_slot=k, parent_slot=pj, residual_slot=k, normal_slot=k,
                                tile_meters=50000.0 / (1 << l), parent_job=pj))
    tp.elevation_batch(elev, res, nrm, tp.make_params(), jobs)
    tp.stream_check()
    zf = elev.download(0, n, tp.ZF)
    zm = elev.download(0, n, tp.ZM)
    nx = nrm.download(0, n, tp.NX)
    want = {}
    for k, (l, x, y) in enumerate(tiles):
        p = want.get((l - 1, x // 2, y // 2))
        ezf, ezc, ezm = orc.elevation_tile(W, l, x, y, p[0] if p else None, p[2] if p else None, resid[k])
        want[(l, x, y)] = (ezf, ezc, ezm)
        assert np.array_equal(zf[k], ezf), "zf of tile %s" % (tiles[k],)
        assert np.array_equal(zm[k], ezm)
        enx, _ = orc.normals_flat(W, ezm, 50000.0 / (1 << l))
        assert_normals_close(nx[k], enx, "nx %s" % (tiles[k],))


def test_cpu_gpu_pairing(gpu, oracle_lib):
    """The reference pairs a cpuElevationProducer and a GPU elevationProducer on the
    same residuals (edit/examples/edit3/helloworld.xml:36-56): with no noise their zf
    must agree.  The CUDA zf is compared with CPUElevationProducer's loop."""
    tp, orc = gpu, oracle_lib
    cases = [Case(101, 3, tx, ty, seed=50 + tx + ty, residual_width=197) for tx, ty in [(2, 3), (5, 4)]]
    zf, _, _ = run_cases(tp, orc, cases, tp.make_params(), residual_width=197, with_normals=False)
    for k, c in enumerate(cases):
        cpu = orc.cpu_elevation_tile(101, c.level, c.tx, c.ty, c.parent_zf, c.residual, c.rx, c.ry)
        assert np.array_equal(zf[k], cpu)


def test_errors(gpu):
    tp = gpu
    elev = tp.TileStorage(101, 3, 4)
    with pytest.raises(tp.TPError) as e:
        tp.elevation_batch(elev, None, None, tp.make_params(), [tp.make_job(2, 1, 1, out_slot=0)])
    assert e.value.code == tp.TP_E_MISSING_PARENT
    with pytest.raises(tp.TPError) as e:
        tp.elevation_batch(elev, None, None, tp.make_params(), [tp.make_job(0, 0, 0, out_slot=9)])
    assert e.value.code == tp.TP_E_BAD_ARG
    with pytest.raises(tp.TPError) as e:
        tp.elevation_batch(elev, None, None, tp.make_params(grid_size=7), [tp.make_job(0, 0, 0, out_slot=0)])
    assert e.value.code == tp.TP_E_BAD_ARG


def _class_setup(tp, orc, W, specs, seed):
    """Storages, jobs and oracle outputs of one tile width for a frame."""
    cases = [Case(W, lvl, tx, ty, seed=seed + 7 * k, noise_amp=a) for k, (lvl, tx, ty, a) in enumerate(specs)]
    n = len(cases)
    elev = tp.TileStorage(W, 3, 2 * n)
    res = tp.TileStorage(W, 1, n)
    nrm = tp.TileStorage(W - 4, 2, n)
    table = orc.dem_noise(W)
    jobs, expect = [], []
    params = tp.make_params(flip=True)
    for k, c in enumerate(cases):
        ps = -1
        if c.level > 0:
            ps = n + k
            elev.upload(ps, tp.ZF, c.parent_zf[None])
            elev.upload(ps, tp.ZM, c.parent_zm[None])
        res.upload(k, 0, c.residual[None])
        rot, layer = tp.noise_select(1, c.level, c.tx, c.ty)
        jobs.append(tp.make_job(c.level, c.tx, c.ty, out_slot=k, parent_slot=ps, residual_slot=k, normal_slot=k,
                                noise_rot=rot, noise_layer=layer, noise_amp=c.noise_amp,
                                tile_meters=float(c.tile_meters)))
        expect.append(c.oracle(orc, table, params_dict(params), rot, layer))
    return dict(elev=elev, res=res, nrm=nrm, jobs=jobs, expect=expect, params=params, n=n)


def _check_class(tp, k):
    n = k["n"]
    zf = k["elev"].download(0, n, tp.ZF)
    zc = k["elev"].download(0, n, tp.ZC)
    nx = k["nrm"].download(0, n, tp.NX)
    for i, (ezf, ezc, ezm, enx, eny) in enumerate(k["expect"]):
        assert np.array_equal(zf[i], ezf), "zf of job %d" % i
        assert np.array_equal(zc[i], ezc), "zc of job %d" % i
        assert_normals_close(nx[i], enx, "nx of job %d" % i)


def test_frame_two_widths_one_launch_and_graph(gpu, oracle_lib):
    """101- and 197-wide tiles in one persistent launch, then the same frame
    replayed from its CUDA graph (outputs cleared in between)."""
    tp, orc = gpu, oracle_lib
    a = _class_setup(tp, orc, 101, [(1, 0, 1, -140.0), (3, 5, 2, 5.0), (6, 40, 33, 0.0), (2, 3, 3, -15.0)], 100)
    b = _class_setup(tp, orc, 197, [(2, 1, 2, -100.0), (5, 17, 30, 1.5), (1, 1, 1, 0.0)], 200)
    f = tp.Frame()
    for k in (a, b):
        f.add(k["elev"], k["res"], k["nrm"], k["params"], k["jobs"])
    assert f.units() == 4 * 1 + 3 * 4
    f.launch()
    tp.stream_check()
    _check_class(tp, a)
    _check_class(tp, b)
    for k in (a, b):
        W, n = k["elev"].tile_size, k["n"]
        for c in (tp.ZF, tp.ZC, tp.ZM):
            k["elev"].upload(0, c, np.zeros((n, W, W), np.float32))
    for _ in range(3):
        f.graph_launch()
    tp.stream_check()
    _check_class(tp, a)
    _check_class(tp, b)


def test_autotuned_frame_keeps_results(gpu, oracle_lib):
    """The autotuner changes only the work-unit shape, never the produced bits."""
    tp, orc = gpu, oracle_lib
    a = _class_setup(tp, orc, 101, [(1, 0, 1, -140.0), (3, 5, 2, 5.0), (2, 3, 3, -15.0)], 300)
    b = _class_setup(tp, orc, 197, [(2, 1, 2, -100.0), (5, 17, 30, 1.5)], 400)
    f = tp.Frame()
    for k in (a, b):
        f.add(k["elev"], k["res"], k["nrm"], k["params"], k["jobs"])
    f.autotune(repeats=1)
    for i in range(2):
        cfg = f.config(i)
        assert cfg["stages"] in (1, 2) and cfg["ctas_per_sm"] in (2, 3) and cfg["band_rows"] >= 8
    f.graph_launch()
    tp.stream_check()
    _check_class(tp, a)
    _check_class(tp, b)


def test_quadtree_double_buffered(gpu, oracle_lib):
    """Parent/child ordering inside one launch with the next unit prefetched."""
    tp, orc = gpu, oracle_lib
    W = 101
    rng = np.random.default_rng(9)
    tiles = [(l, x, y) for l in range(4) for y in range(1 << l) for x in range(1 << l)]
    index = {t: k for k, t in enumerate(tiles)}
    n = len(tiles)
    elev = tp.TileStorage(W, 3, n)
    res = tp.TileStorage(W, 1, n)
    resid = (rng.standard_normal((n, W, W)) * 50.0).astype(np.float32)
    res.upload(0, 0, resid)
    jobs = []
    for k, (l, x, y) in enumerate(tiles):
        pj = index[(l - 1, x // 2, y // 2)] if l > 0 else -1
        jobs.append(tp.make_job(l, x, y, out_slot=k, parent_slot=pj, residual_slot=k,
                                tile_meters=50000.0 / (1 << l), parent_job=pj))
    tp.elevation_batch(elev, res, None, tp.make_params(band_rows=34, stages=2), jobs)
    tp.stream_check()
    zf = elev.download(0, n, tp.ZF)
    want = {}
    for k, (l, x, y) in enumerate(tiles):
        p = want.get((l - 1, x // 2, y // 2))
        ezf, ezc, ezm = orc.elevation_tile(W, l, x, y, p[0] if p else None, p[2] if p else None, resid[k])
        want[(l, x, y)] = (ezf, ezc, ezm)
        assert np.array_equal(zf[k], ezf), "zf of tile %s" % (tiles[k],)
