"""Parity of the CUDA ortho (colour) tile kernel with the CPU oracle through the
C ABI (tp_ortho_batch): RGBA8 tiles must be byte-identical.

Cases: random parents and residuals at both child parities and many levels, RGB
and HSV noise, level-0 tiles with and without a residual, a parent -> child ->
grandchild chain produced in one launch, and the reference's own RGB.dat tiles
as parent and residual."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
MINI = os.path.join(HERE, "golden", "rgb_graph1_mini.dat")


def run(tp, W, jobs, tiles_in, residuals, params, capacity):
    """tiles_in: {slot: [W, W, 4] uint8}; residuals: {slot: tile}; returns the ortho storage."""
    orth = tp.TileStorage(W, 1, capacity)
    res = tp.TileStorage(W, 1, max(residuals) + 1) if residuals else None
    for slot, t in tiles_in.items():
        orth.upload(slot, 0, tp.rgba_to_texels(t)[None])
    for slot, t in (residuals or {}).items():
        res.upload(slot, 0, tp.rgba_to_texels(t)[None])
    tp.ortho_batch(orth, res, params, jobs)
    tp.stream_check()
    return orth


def get(tp, orth, slot):
    return tp.texels_to_rgba(orth.download(slot, 1, 0)[0])


def oracle_tile(oracle, W, j, parent, residual, params, table):
    return oracle.ortho_tile(W, j.level, j.tx, j.ty, parent, residual, table[j.noise_layer], j.noise_rot,
                             j.noise_amp, root_color=list(params.root_color), noise_color=list(params.noise_color),
                             scale=params.scale, hsv=bool(params.hsv))


@pytest.mark.parametrize("hsv", [False, True])
def test_random_tiles_bit_identical(gpu, oracle_lib, hsv):
    tp = gpu
    W, n = 196, 24
    rng = np.random.default_rng(5 + hsv)
    params = tp.make_ortho_params(root_color=(60 / 255, 150 / 255, 20 / 255, 0.5),
                                  noise_color=(70 / 255, 80 / 255, 100 / 255, 1.0), scale=2.0, hsv=hsv)
    table = oracle_lib.ortho_noise(W)
    parents, residuals, jobs, want = {}, {}, [], []
    for k in range(n):
        level = 0 if k < 3 else int(rng.integers(1, 14))
        tx, ty = (int(v) for v in rng.integers(0, 1 << level, 2))
        rot, layer = tp.noise_select(1, level, tx, ty)
        parent = rng.integers(0, 256, (W, W, 4), dtype=np.uint8) if level > 0 else None
        residual = rng.integers(60, 200, (W, W, 4), dtype=np.uint8) if k % 3 != 1 else None
        if parent is not None:
            parents[n + k] = parent
        if residual is not None:
            residuals[k] = residual
        j = tp.make_ortho_job(level, tx, ty, out_slot=k, parent_slot=n + k if level > 0 else -1,
                              residual_slot=k if residual is not None else -1, noise_rot=rot, noise_layer=layer,
                              noise_amp=255.0 * 0.8 ** level)
        jobs.append(j)
        want.append(oracle_tile(oracle_lib, W, j, parent, residual, params, table))
    orth = run(tp, W, jobs, parents, residuals, params, 2 * n)
    for k in range(n):
        got = get(tp, orth, k)
        diff = np.count_nonzero(got != want[k])
        assert diff == 0, "tile %d (level %d): %d bytes differ" % (k, jobs[k].level, diff)


def test_chain_in_one_launch(gpu, oracle_lib):
    """Root, child, grandchild and great-grandchild as one batch with parent_job links."""
    tp = gpu
    W = 196
    params = tp.make_ortho_params(hsv=False)
    table = oracle_lib.ortho_noise(W)
    rng = np.random.default_rng(11)
    chain = [(0, 0, 0), (1, 1, 0), (2, 3, 1), (3, 6, 3)]
    residuals = {k: rng.integers(90, 170, (W, W, 4), dtype=np.uint8) for k in range(4)}
    jobs = []
    for k, (l, x, y) in enumerate(chain):
        rot, layer = tp.noise_select(1, l, x, y)
        jobs.append(tp.make_ortho_job(l, x, y, out_slot=k, parent_slot=k - 1 if k else -1, residual_slot=k,
                                      noise_rot=rot, noise_layer=layer, noise_amp=40.0, parent_job=k - 1))
    orth = run(tp, W, jobs, {}, residuals, params, 4)
    parent = None
    for k, j in enumerate(jobs):
        want = oracle_tile(oracle_lib, W, j, parent, residuals[k], params, table)
        got = get(tp, orth, k)
        assert np.array_equal(got, want), "chain tile %d" % k
        parent = want


def test_reference_tiles_as_inputs(gpu, oracle_lib):
    """The reference's RGB.dat: the level-0 tile upsampled into its four children,
    with the decoded level-1 tile as the residual of each."""
    tp = gpu
    d = tp.OrthoDat(MINI)
    W = d.width
    root = d.tile_rgba(0, 0, 0)
    resid = d.tile_rgba(1, 1, 0)
    params = tp.make_ortho_params(scale=1.0)
    table = oracle_lib.ortho_noise(W)
    jobs = []
    for k, (x, y) in enumerate([(0, 0), (1, 0), (0, 1), (1, 1)]):
        rot, layer = tp.noise_select(1, 1, x, y)
        jobs.append(tp.make_ortho_job(1, x, y, out_slot=k, parent_slot=4, residual_slot=0, noise_rot=rot,
                                      noise_layer=layer, noise_amp=12.0))
    orth = run(tp, W, jobs, {4: root}, {0: resid}, params, 5)
    for k, j in enumerate(jobs):
        want = oracle_tile(oracle_lib, W, j, root, resid, params, table)
        assert np.array_equal(get(tp, orth, k), want), "child %d" % k


def test_bad_jobs_are_rejected(gpu):
    tp = gpu
    W = 196
    orth = tp.TileStorage(W, 1, 4)
    params = tp.make_ortho_params()
    with pytest.raises(tp.TPError) as e:
        tp.ortho_batch(orth, None, params, [tp.make_ortho_job(2, 1, 1, out_slot=0)])   # no parent
    assert e.value.code == tp.TP_E_MISSING_PARENT
    with pytest.raises(tp.TPError) as e:
        tp.ortho_batch(orth, None, params, [tp.make_ortho_job(0, 0, 0, out_slot=0, residual_slot=0)])
    assert e.value.code == tp.TP_E_BAD_ARG
    with pytest.raises(tp.TPError):
        tp.ortho_batch(tp.TileStorage(197, 1, 2), None, params, [tp.make_ortho_job(0, 0, 0, out_slot=0)])
    tp.stream_check()


@pytest.mark.parametrize("divisor", [6.0, 255.0, 0.4])
def test_known_divisor_division_is_correctly_rounded(gpu, divisor):
    """The HSV path divides by 6, 255 and 0.4 with a multiply and one FMA correction:
    it must equal the correctly rounded division for every one of the 2^32 dividends."""
    mismatches, first = gpu.division_self_test(divisor)
    assert mismatches == 0, "%d dividends differ (first 0x%08x)" % (mismatches, first)
