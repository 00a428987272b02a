"""Normal tiles in the reference's four formats (NormalProducer.cpp:195, demo
normalShader.glsl:93-124), flat and on the sphere, with coarse normals from the
parent normal tile, against the oracle; and the same through a NormalProducer."""
import numpy as np
import pytest

from tilecase import smooth_tile

pytestmark = pytest.mark.gpu


def check_planes(got, want, quantized, what):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    err = np.abs(got - want)
    if quantized:  # 8-bit steps: a float-rounding difference may move a value across one step
        assert err.max() <= 1.0 / 255.0 + 1e-6, (what, err.max())
        assert np.mean(err > 1e-6) < 5e-3, (what, np.mean(err > 1e-6))
        assert np.allclose(np.round(got * 255.0), got * 255.0, atol=1e-3)
    else:
        assert err.max() <= 1e-4, (what, err.max())


@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
@pytest.mark.parametrize("sphere", [False, True])
def test_formats_with_coarse_normals(gpu, oracle_lib, fmt, sphere):
    tp, orc = gpu, oracle_lib
    W = 101
    D = 12.72e6 if sphere else 40000.0
    tiles = [(2, 1, 3)] + [(3, x, y) for x in (2, 3) for y in (6, 7)]
    n = len(tiles)
    elev = tp.TileStorage(W, 3, n)
    ch = 4 if fmt <= 1 else 2
    nrm = tp.TileStorage(W - 4, ch, n)
    zm = np.stack([np.maximum(smooth_tile(W, 40 + k, amp=800.0), 0.0) for k in range(n)]).astype(np.float32)
    elev.upload(0, tp.ZM, zm)
    jobs = [tp.make_job(l, x, y, out_slot=k, normal_slot=k, tile_meters=D / (1 << l)) for k, (l, x, y) in enumerate(tiles)]
    tp.normal_batch_format(elev, nrm, jobs, fmt, parent_slots=[-1] + [0] * (n - 1),
                           root_quad_size=D if sphere else 0.0)
    tp.stream_check()
    got = [nrm.download(0, n, c) for c in range(ch)]
    quant = fmt in (1, 3)
    # the parent (level 2, no parent normal: nc = nf)
    want0 = orc.normals_full(W, zm[0], D / 4, fmt, 1, 3, None, D if sphere else 0.0, 2)
    for c in range(ch):
        check_planes(got[c][0], want0[c], quant, "parent plane %d" % c)
    # the children, coarse normals from the parent tile as stored
    parent = [got[0][0], got[1][0]]
    for k in range(1, n):
        l, x, y = tiles[k]
        want = orc.normals_full(W, zm[k], D / 8, fmt, x, y, parent, D if sphere else 0.0, l)
        for c in range(ch):
            check_planes(got[c][k], want[c], quant, "tile %s plane %d" % (tiles[k], c))
        if fmt <= 1:  # the coarse normals really come from the parent
            assert not np.allclose(got[2][k], got[0][k])


def test_producer_format_1(gpu, oracle_lib):
    tp, orc = gpu, oracle_lib
    W = 101
    es, rs, ns = tp.TileStorage(W, 3, 64), tp.TileStorage(W, 1, 64), tp.TileStorage(W - 4, 4, 64)
    r = tp.ResidualProducer(tp.TileCache(rs), source=lambda l, x, y, w: smooth_tile(w, 7 * l + x + 3 * y, 300.0 / (1 + l)))
    e = tp.ElevationProducer(tp.TileCache(es), r, noise_amp=[0.0], params=tp.make_params(), face=0)
    nc = tp.TileCache(ns)
    n = tp.NormalProducer(nc, e)
    n.set_format(1)
    n.set_root_quad_size(30000.0)
    held = [n.get_tile(2, 1, 2), n.get_tile(1, 0, 1)]
    tp.scheduler_run([n])
    tp.stream_check()
    child, parent = held
    zm = es.download(e.find_tile(2, 1, 2, include_cache=True).slot, 1, tp.ZM)[0]
    pn = [ns.download(parent.slot, 1, c)[0] for c in (0, 1)]
    want = orc.normals_full(W, zm, 30000.0 / 4, 1, 1, 2, pn)
    for c in range(4):
        check_planes(ns.download(child.slot, 1, c)[0], want[c], True, "producer plane %d" % c)
