"""tp_elevation_batch_noalloc, whose kernel scratch (work counter, completion
counts, job records, noise tables) is one static device array, against
tp_elevation_batch on the same inputs.  Several calls in a row share the array,
so each is compared with the allocating entry point.  The file sorts last so
that it also runs after every other GPU test in one process.

It exists for callers that cannot allocate device memory while they produce
tiles (a renderer whose device memory is all in its own pools, a frame loop that
must not stall on an allocation or a free): the tests also check that the calls
leave the device's free memory unchanged."""
import ctypes as C

import numpy as np
import pytest

from tilecase import assert_elev_close, assert_normals_close

pytestmark = pytest.mark.gpu


def _call_noalloc(tp, elev, res, nrm, params, jobs, stream=None):
    arr = jobs if isinstance(jobs, C.Array) else (tp.TileJob * len(jobs))(*jobs)
    return tp.lib().tp_elevation_batch_noalloc(elev.handle, res.handle if res else None,
                                               nrm.handle if nrm else None, C.byref(params), arr, len(jobs), stream)


def _compare(tp, eA, eB, nA, nB, slots, what):
    for ch, name in ((tp.ZF, "zf"), (tp.ZC, "zc"), (tp.ZM, "zm")):
        a = np.stack([eA.download(s, 1, ch)[0] for s in slots])
        b = np.stack([eB.download(s, 1, ch)[0] for s in slots])
        assert_elev_close(b, a, "%s %s" % (what, name))
    if nA is not None:
        for ch, name in ((tp.NX, "nx"), (tp.NY, "ny")):
            a = np.stack([nA.download(s, 1, ch)[0] for s in slots])
            b = np.stack([nB.download(s, 1, ch)[0] for s in slots])
            assert_normals_close(b, a, "%s %s" % (what, name))


def _storages(tp, W, cap):
    return (tp.TileStorage(W, 3, cap), tp.TileStorage(W, 3, cap),
            tp.TileStorage(W - 4, 2, cap), tp.TileStorage(W - 4, 2, cap))


def test_noalloc_batch_matches_allocating_batch(gpu):
    tp = gpu
    W = 101
    rng = np.random.default_rng(11)
    tiles = [(l, x, y) for l in range(4) for y in range(1 << l) for x in range(1 << l)]
    index = {t: k for k, t in enumerate(tiles)}
    n = len(tiles)
    cap = n + 16
    res = tp.TileStorage(W, 1, cap)
    res.upload(0, 0, (rng.standard_normal((cap, W, W)) * 300.0).astype(np.float32))
    eA, eB, nA, nB = _storages(tp, W, cap)

    # call 1: levels 0..3 in one batch, children ordered after their parents' jobs
    jobs = []
    for k, (l, x, y) in enumerate(tiles):
        pj = index[(l - 1, x // 2, y // 2)] if l > 0 else -1
        rot, layer = tp.noise_select(1, l, x, y)
        jobs.append(tp.make_job(l, x, y, out_slot=k, parent_slot=pj, residual_slot=k, normal_slot=k,
                                noise_rot=rot, noise_layer=layer, noise_amp=-40.0 * 0.5 ** l,
                                tile_meters=40000.0 / (1 << l), parent_job=pj))
    params = tp.make_params()
    tp.elevation_batch(eA, res, nA, params, jobs)
    assert _call_noalloc(tp, eB, res, nB, params, jobs) == tp.TP_OK, tp.lib().tp_last_error()
    tp.stream_check()
    _compare(tp, eA, eB, nA, nB, range(n), "call 1")

    # call 2, right after on the same array: level-4 children of resident level-3
    # parents (no in-batch dependencies), slope/curvature-modulated noise
    kids = [(4, x, y) for y in range(0, 16, 3) for x in range(0, 16, 2)]
    jobs2 = []
    for i, (l, x, y) in enumerate(kids):
        rot, layer = tp.noise_select(1, l, x, y)
        jobs2.append(tp.make_job(l, x, y, out_slot=n + (i % 16), parent_slot=index[(3, x // 2, y // 2)],
                                 residual_slot=i % cap, normal_slot=n + (i % 16), noise_rot=rot,
                                 noise_layer=layer, noise_amp=6.0, tile_meters=2500.0))
        if i == 15:
            break
    params2 = tp.make_params(noise_mode=1)
    tp.elevation_batch(eA, res, nA, params2, jobs2)
    assert _call_noalloc(tp, eB, res, nB, params2, jobs2) == tp.TP_OK, tp.lib().tp_last_error()
    tp.stream_check()
    _compare(tp, eA, eB, nA, nB, range(n, n + len(jobs2)), "call 2")


def test_noalloc_batch_other_width_then_back(gpu):
    """Each tile width's noise table is written once into the array, so a call with
    another width leaves the first width's table as it was."""
    tp = gpu
    rng = np.random.default_rng(12)
    for W, seed in ((197, 1), (101, 2)):
        cap = 8
        res = tp.TileStorage(W, 1, cap)
        res.upload(0, 0, (rng.standard_normal((cap, W, W)) * 200.0).astype(np.float32))
        eA, eB, nA, nB = _storages(tp, W, cap)
        par = (rng.standard_normal((1, W, W)) * 500.0).astype(np.float32)
        for e in (eA, eB):
            e.upload(0, tp.ZF, par)
            e.upload(0, tp.ZM, np.maximum(par, 0))
        jobs = [tp.make_job(3, 2 + (k & 1), 6 + (k >> 1), out_slot=1 + k, parent_slot=0, residual_slot=k,
                            normal_slot=1 + k, noise_rot=k % 4, noise_layer=(k + seed) % 6, noise_amp=-25.0,
                            tile_meters=5000.0) for k in range(4)]
        params = tp.make_params(flip=(W == 197))
        tp.elevation_batch(eA, res, nA, params, jobs)
        assert _call_noalloc(tp, eB, res, nB, params, jobs) == tp.TP_OK, tp.lib().tp_last_error()
        tp.stream_check()
        _compare(tp, eA, eB, nA, nB, range(1, 5), "W=%d" % W)


def test_noalloc_batch_rejects_more_jobs_than_the_scratch_holds(gpu):
    tp = gpu
    W = 101
    e = tp.TileStorage(W, 3, 4)
    jobs = [tp.make_job(0, 0, 0, out_slot=0)] * 4097
    assert _call_noalloc(tp, e, None, None, tp.make_params(), jobs) == tp.TP_E_BAD_ARG
    assert b"4096" in tp.lib().tp_last_error()


def _frame_case(tp, W, n, seed, levels=(3, 9)):
    """n independent requests of width W, each with a parent slot, a residual and
    per-level noise: storages for both entry points and the job list."""
    rng = np.random.default_rng(seed)
    res = tp.TileStorage(W, 1, n)
    res.upload(0, 0, (rng.standard_normal((n, W, W)) * 80.0).astype(np.float32))
    eA, eB, nA, nB = _storages(tp, W, 2 * n)
    npar = 8
    par = (rng.standard_normal((npar, W, W)) * 600.0).astype(np.float32)
    for e in (eA, eB):
        e.upload(n, tp.ZF, par[np.arange(n) % npar])
        e.upload(n, tp.ZM, np.maximum(par[np.arange(n) % npar], 0))
    jobs = []
    for k in range(n):
        l = int(rng.integers(levels[0], levels[1] + 1))
        x, y = int(rng.integers(0, 1 << l)), int(rng.integers(0, 1 << l))
        rot, layer = tp.noise_select(1, l, x, y)
        jobs.append(tp.make_job(l, x, y, out_slot=k, parent_slot=n + k, residual_slot=k, normal_slot=k,
                                noise_rot=rot, noise_layer=layer, noise_amp=300.0 * 0.55 ** l,
                                tile_meters=100000.0 / (1 << l)))
    return res, eA, eB, nA, nB, jobs


def test_noalloc_batch_at_the_job_limit_allocates_nothing(gpu):
    """4096 jobs (the limit) in one call, twice in a row, compared tile by tile with
    the allocating entry point; around the calls after the first, the device's free
    memory does not change."""
    import torch
    tp = gpu
    W, n = 101, 4096
    res, eA, eB, nA, nB, jobs = _frame_case(tp, W, n, 21)
    params = tp.make_params()
    arr = (tp.TileJob * n)(*jobs)
    tp.elevation_batch(eA, res, nA, params, arr)
    assert _call_noalloc(tp, eB, res, nB, params, arr) == tp.TP_OK, tp.lib().tp_last_error()   # set-up call
    tp.stream_check()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call_noalloc(tp, eB, res, nB, params, arr) == tp.TP_OK, tp.lib().tp_last_error()
    tp.stream_check()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "free device memory moved from %d to %d bytes" % (free0, free1)
    _compare(tp, eA, eB, nA, nB, range(0, n, 7), "4096 jobs")


def test_noalloc_batch_job_buffer_reused_at_once(gpu):
    """The caller refills its pinned job buffer right after the first call returns,
    without waiting for the stream, and makes a second call: each call produces the
    tiles of the jobs it was given."""
    import torch
    tp = gpu
    W, n = 101, 64
    res, eA, eB, nA, nB, jobs = _frame_case(tp, W, 2 * n, 22)
    first, second = jobs[:n], jobs[n:]
    params = tp.make_params()
    tp.elevation_batch(eA, res, nA, params, first)
    tp.elevation_batch(eA, res, nA, params, second)
    tp.stream_check()
    size = C.sizeof(tp.TileJob) * n
    pinned = torch.empty(size, dtype=torch.uint8, pin_memory=True)
    buf = (tp.TileJob * n).from_address(pinned.data_ptr())
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    for k in range(n):
        buf[k] = first[k]
    assert _call_noalloc(tp, eB, res, nB, params, buf, sh) == tp.TP_OK, tp.lib().tp_last_error()
    for k in range(n):          # refilled while the first call may still be running
        buf[k] = second[k]
    assert _call_noalloc(tp, eB, res, nB, params, buf, sh) == tp.TP_OK, tp.lib().tp_last_error()
    stream.synchronize()
    tp.stream_check(sh)
    _compare(tp, eA, eB, nA, nB, range(2 * n), "reused job buffer")


def test_noalloc_batch_noise_tables_fill_up(gpu):
    """Widths 101, 197 and 253 fill the room for noise tables; a fourth width is
    rejected with a message, and the widths already there still work."""
    tp = gpu
    for W in (101, 197, 253):
        res, eA, eB, nA, nB, jobs = _frame_case(tp, W, 2, 30 + W)
        params = tp.make_params(grid_size=24 if (W - 5) % 24 == 0 else 8)
        tp.elevation_batch(eA, res, nA, params, jobs)
        assert _call_noalloc(tp, eB, res, nB, params, jobs) == tp.TP_OK, tp.lib().tp_last_error()
        tp.stream_check()
        _compare(tp, eA, eB, nA, nB, range(2), "W=%d" % W)
    e = tp.TileStorage(21, 3, 4)
    assert _call_noalloc(tp, e, None, None, tp.make_params(grid_size=4),
                         [tp.make_job(0, 0, 0, out_slot=0)]) == tp.TP_E_BAD_ARG
    assert b"no room" in tp.lib().tp_last_error()
    res, eA, eB, nA, nB, jobs = _frame_case(tp, 197, 3, 77)
    params = tp.make_params()
    tp.elevation_batch(eA, res, nA, params, jobs)
    assert _call_noalloc(tp, eB, res, nB, params, jobs) == tp.TP_OK, tp.lib().tp_last_error()
    tp.stream_check()
    _compare(tp, eA, eB, nA, nB, range(3), "W=197 after the table space filled")
