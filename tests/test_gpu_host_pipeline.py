"""Host-buffer batches (tp_elevation_batch_host): dense host tiles in and out
through the chunked pipeline must equal, bit for bit, the same jobs produced by
tp_elevation_batch over device slots, and the oracle on sampled tiles.

Cases: both tile widths, a job count that leaves a ragged last chunk, level-0
jobs (no parent), jobs without a residual, parent zm given or derived on the
device, with and without normals, and two calls in a row on one pipeline.
"""
import numpy as np
import pytest

from tilecase import assert_elev_close, assert_normals_close

pytestmark = pytest.mark.gpu


def make_inputs(tp, W, n, seed, no_residual_every=5):
    rng = np.random.default_rng(seed)
    levels = rng.integers(0, 10, n)
    levels[:3] = 0
    tx = np.array([rng.integers(0, 1 << int(l)) for l in levels])
    ty = np.array([rng.integers(0, 1 << int(l)) for l in levels])
    y, x = np.mgrid[0:W, 0:W].astype(np.float32)
    pz = np.empty((n, W, W), np.float32)
    for k in range(n):
        a, b, c = rng.uniform(0.02, 0.2, 3)
        pz[k] = 900.0 * np.sin(a * x + c) * np.cos(b * y) + rng.uniform(-300, 300) + \
            rng.standard_normal((W, W)).astype(np.float32) * 5.0
    pm = np.maximum(pz, 0.0).astype(np.float32)
    res = (rng.standard_normal((n, W, W)) * 50.0).astype(np.float32)
    jobs = []
    for k in range(n):
        l = int(levels[k])
        rot, layer = tp.noise_select(1, l, int(tx[k]), int(ty[k]))
        jobs.append(tp.make_job(l, int(tx[k]), int(ty[k]), out_slot=k, parent_slot=n + k if l > 0 else -1,
                                residual_slot=-1 if k % no_residual_every == 4 else k, normal_slot=k,
                                noise_rot=rot, noise_layer=layer, noise_amp=float(300.0 * 0.55 ** l),
                                tile_meters=100000.0 / (1 << l)))
    return jobs, pz, pm, res


def slot_reference(tp, W, jobs, pz, pm, res, params, normals=True):
    n = len(jobs)
    elev = tp.TileStorage(W, 3, 2 * n)
    rs = tp.TileStorage(W, 1, n)
    nrm = tp.TileStorage(W - 4, 2, n) if normals else None
    elev.upload(n, tp.ZF, pz)
    elev.upload(n, tp.ZM, pm)
    rs.upload(0, 0, res)
    if not normals:
        jobs = [tp.TileJob.from_buffer_copy(j) for j in jobs]
        for j in jobs:
            j.normal_slot = -1
    tp.elevation_batch(elev, rs, nrm, params, jobs)
    tp.stream_check()
    out = [elev.download(0, n, c) for c in (tp.ZF, tp.ZC, tp.ZM)]
    if normals:
        out += [nrm.download(0, n, c) for c in (tp.NX, tp.NY)]
    return out


def host_outputs(n, W, normals=True):
    out = [np.full((n, W, W), np.nan, np.float32) for _ in range(3)]
    if normals:
        out += [np.full((n, W - 4, W - 4), np.nan, np.float32) for _ in range(2)]
    return out


@pytest.mark.parametrize("W,n,chunk,nbuf", [(101, 37, 8, 3), (197, 11, 4, 2), (101, 5, 64, 3)])
def test_host_pipeline_equals_slot_batch(gpu, W, n, chunk, nbuf):
    tp = gpu
    params = tp.make_params()
    jobs, pz, pm, res = make_inputs(tp, W, n, seed=W + n)
    want = slot_reference(tp, W, jobs, pz, pm, res, params)
    pipe = tp.HostPipeline(W, chunk=chunk, nbuf=nbuf)
    for call in range(2):
        got = host_outputs(n, W)
        pipe.run(params, jobs, pz, pm if call == 0 else None, res, *got)
        tp.stream_check()
        for name, g, w in zip(("zf", "zc", "zm", "nx", "ny"), got, want):
            assert np.array_equal(g, w), "call %d: %s differs from the slot batch" % (call, name)
    pipe.close()


def test_host_pipeline_without_normals_and_no_clamp(gpu):
    tp = gpu
    W, n = 101, 9
    params = tp.make_params(no_clamp=True)
    jobs, pz, _, res = make_inputs(tp, W, n, seed=3)
    want = slot_reference(tp, W, jobs, pz, pz, res, params, normals=False)
    pipe = tp.HostPipeline(W, chunk=4)
    got = host_outputs(n, W, normals=False)
    pipe.run(params, jobs, pz, None, res, *got)
    tp.stream_check()
    for name, g, w in zip(("zf", "zc", "zm"), got, want):
        assert np.array_equal(g, w), name


def test_host_pipeline_matches_oracle(gpu, oracle_lib):
    tp = gpu
    W, n = 101, 6
    params = tp.make_params()
    jobs, pz, pm, res = make_inputs(tp, W, n, seed=17)
    pipe = tp.HostPipeline(W, chunk=4)
    got = host_outputs(n, W)
    pipe.run(params, jobs, pz, pm, res, *got)
    tp.stream_check()
    table = oracle_lib.dem_noise(W)
    for k, j in enumerate(jobs):
        ezf, ezc, ezm = oracle_lib.elevation_tile(
            W, j.level, j.tx, j.ty, pz[k] if j.level > 0 else None, pm[k] if j.level > 0 else None,
            res[k] if j.residual_slot >= 0 else None, noise=table[j.noise_layer], noise_rot=j.noise_rot,
            noise_amp=j.noise_amp)
        tag = "tile %d (level %d)" % (k, j.level)
        assert assert_elev_close(got[0][k], ezf, tag + " zf") == 0
        assert assert_elev_close(got[1][k], ezc, tag + " zc") == 0
        assert assert_elev_close(got[2][k], ezm, tag + " zm") == 0
        enx, eny = oracle_lib.normals_flat(W, ezm, float(j.tile_meters))
        assert_normals_close(got[3][k], enx, tag + " nx")
        assert_normals_close(got[4][k], eny, tag + " ny")


def test_host_pipeline_zf_and_normals_only(gpu):
    """zc and zm left out (NULL): zf and the normals are the full form's, and the
    arrays given for zc / zm in the full call are not what this call writes."""
    tp = gpu
    W, n = 101, 9
    params = tp.make_params()
    jobs, pz, pm, res = make_inputs(tp, W, n, seed=23)
    pipe = tp.HostPipeline(W, chunk=4)
    full = host_outputs(n, W)
    pipe.run(params, jobs, pz, pm, res, *full)
    tp.stream_check()
    zf = np.full((n, W, W), -7.0, np.float32)
    nx = np.full((n, W - 4, W - 4), -7.0, np.float32)
    ny = np.full_like(nx, -7.0)
    pipe.run(params, jobs, pz, pm, res, zf, None, None, nx, ny)
    tp.stream_check()
    assert np.array_equal(zf, full[0]) and np.array_equal(nx, full[3]) and np.array_equal(ny, full[4])
    # zm is rebuilt on the host as the kernel writes it
    assert np.array_equal(np.maximum(zf, np.float32(0.0)), full[2])
    pipe.close()


def test_host_pipeline_rejects_bad_calls(gpu):
    tp = gpu
    W = 101
    jobs, pz, pm, res = make_inputs(tp, W, 4, seed=5)
    pipe = tp.HostPipeline(W, chunk=2)
    out = host_outputs(4, W)
    dep = [tp.TileJob.from_buffer_copy(j) for j in jobs]
    dep[1].parent_job = 0
    with pytest.raises(tp.TPError) as e:
        pipe.run(tp.make_params(), dep, pz, pm, res, *out)
    assert e.value.code == tp.TP_E_BAD_ARG
    with pytest.raises(tp.TPError):
        pipe.run(tp.make_params(), jobs, pz, pm, None, *out)   # residual slots but no residual tiles
    with pytest.raises(tp.TPError):
        tp.HostPipeline(100)
