"""The device preprocess and the learned residual predictor against the CPU oracle:
procedural heights and pyramid tiles bit-exact; the net's forward pass, loss and
every parameter gradient within bf16 tolerances of the oracle's emulation of the
same rounding points; learned residual tiles through the elevation kernel."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "proland-4.0_gb300"))

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def L(gpu):
    from proland_gb300 import learned
    return learned


def test_fbm_heights_match_oracle(L, oracle_lib):
    for size, seed in ((257, 1), (97, 7)):
        got = L.fbm_heights(size, octaves=12, base_cells=4, amplitude=4000.0, quantum=0.25, seed=seed).cpu().numpy()
        want = oracle_lib.fbm_heights(size, 12, 4, 4000.0, 0.25, seed)
        assert np.array_equal(got, want)
        assert np.abs(got.astype(np.int64)).max() > 1000  # a real height field, not zeros


@pytest.mark.parametrize("ts,max_level", [(16, 4), (96, 2)])
def test_preprocess_pyramid_matches_oracle(L, oracle_lib, ts, max_level):
    orc = oracle_lib
    W = ts + 5
    base = L.fbm_heights((ts << max_level) + 1, seed=3)
    base_h = base.cpu().numpy()
    approx, _, _, _ = L.preprocess_level(base, ts, max_level, 0)
    want_prev = {(0, 0): orc.level_tile(base_h, ts, max_level, 0, 0, 0)}
    assert np.array_equal(approx[0].cpu().numpy(), want_prev[(0, 0)])
    for l in range(1, max_level + 1):
        approx, up, res, enc = L.preprocess_level(base, ts, max_level, l, approx)
        a, u, r, e = (t.cpu().numpy() for t in (approx, up, res, enc))
        side = 1 << l
        cur = {}
        for ty in range(side):
            for tx in range(side):
                k = ty * side + tx
                parent = want_prev[(tx // 2, ty // 2)]
                fine = orc.level_tile(base_h, ts, max_level, l, tx, ty)
                rq, enc_w, ap = orc.compute_residual(W, tx, ty, parent, fine)
                z = np.zeros((W, W), np.float32)
                orc.lib().or_residual_upsample(W, ts, tx, ty, orc._p(parent), orc._p(z))
                assert np.array_equal(r[k], rq), (l, tx, ty)
                assert np.array_equal(e[k], enc_w)
                assert np.array_equal(a[k], ap)
                assert np.array_equal(u[k], z)
                cur[(tx, ty)] = ap
        want_prev = cur


def _case(W, n, seed):
    rng = np.random.default_rng(seed)
    levels = rng.integers(1, 12, n).astype(np.int32)
    up = (rng.standard_normal((n, W, W)) * 300.0 + rng.uniform(-2000, 2000, (n, 1, 1))).astype(np.float32)
    target = (rng.standard_normal((n, W, W)) * 20.0).astype(np.float32)
    sigma_in = rng.uniform(100.0, 400.0, 24).astype(np.float32)
    sigma_out = rng.uniform(5.0, 30.0, 24).astype(np.float32)
    return levels, up, target, sigma_in, sigma_out


def _relerr(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("W,n", [(21, 3), (37, 2), (101, 1)])
def test_forward_backward_match_oracle(L, oracle_lib, W, n):
    levels, up, target, si, so = _case(W, n, seed=W)
    net = L.LearnedPredictor(tile_width=W, max_batch=4, seed=5)
    params = net.get_params()
    rng = np.random.default_rng(1)
    # non-zero biases and embedding, so that their paths are exercised too
    mask = params != 0
    params = params + np.where(mask, 0.0, 0.0).astype(np.float32)
    nz = np.arange(params.size) >= params.size - 24 * 32
    params[nz] = rng.standard_normal(nz.sum()).astype(np.float32) * 0.1
    net.set_params(params)
    net.set_sigmas(si, so)
    up_d, tg_d = torch.from_numpy(up).cuda(), torch.from_numpy(target).cuda()
    out = net.forward(up_d, levels, training=True).cpu().numpy()
    loss = net.backward(tg_d)
    g = net.get_grads()
    want_loss, want_pred, want_g = oracle_lib.learned_loss_grad(params, up, target, levels, si, so, emulate=True)
    want_out = want_pred * so[levels][:, None, None]
    assert _relerr(out, want_out) < 1e-2, _relerr(out, want_out)
    assert abs(loss - want_loss) <= 1e-2 * want_loss
    # per parameter tensor: weights and bias of every layer, the embedding
    cin, cout = [16, 32, 32, 32, 32], [32, 32, 32, 32, 16]
    off = 0
    for l in range(5):
        for name, cnt in (("W%d" % l, cout[l] * 9 * cin[l]), ("b%d" % l, cout[l])):
            e = _relerr(g[off:off + cnt], want_g[off:off + cnt])
            assert e < 3e-2, (name, e)
            off += cnt
    e = _relerr(g[off:], want_g[off:])
    assert e < 3e-2, ("embedding", e)
    net.close()


@pytest.mark.parametrize("W,n", [(21, 3), (37, 2), (101, 4)])
def test_inference_input_channels_made_in_the_first_layer(L, W, n):
    """An inference pass builds the first layer's input channels inside the first
    convolution (no input image): the same bits as the training pass, which writes the
    input image and reads it back."""
    levels, up, _, si, so = _case(W, n, seed=W + 1)
    net = L.LearnedPredictor(tile_width=W, max_batch=4, seed=7)
    net.set_sigmas(si, so)
    up_d = torch.from_numpy(up).cuda()
    train_out = net.forward(up_d, levels, training=True).clone()
    infer_out = net.forward(up_d, levels, training=False)
    torch.cuda.synchronize()
    assert torch.equal(train_out, infer_out)
    net.close()


def test_inference_passes_in_a_row(L):
    """Inference passes are enqueued without a host synchronisation and share the net's
    buffers: passes issued back to back on one stream (different inputs, levels and
    batch sizes) give the results of each pass run alone, and check() reports no
    failure."""
    W = 101
    net = L.LearnedPredictor(tile_width=W, max_batch=64, seed=11)
    cases = []
    for k, n in enumerate((64, 17, 40, 64)):
        levels, up, _, si, so = _case(W, n, seed=200 + k)
        if k == 0:
            net.set_sigmas(si, so)
        cases.append((torch.from_numpy(up).cuda(), levels))
    alone = []
    for up_d, levels in cases:
        alone.append(net.forward(up_d, levels).clone())
        net.check()
    outs = [torch.empty_like(up_d) for up_d, _ in cases]
    for (up_d, levels), out in zip(cases, outs):
        net.forward(up_d, levels, out=out)
    net.check()
    for a, b in zip(alone, outs):
        assert torch.equal(a, b)
    net.close()


@pytest.mark.parametrize("W,n", [(21, 5), (101, 256), (197, 64)])
def test_fused_pairs_give_the_per_layer_bits(L, W, n):
    """Inference by fused layer pairs (layers 0 + 1 and 2 + 3 in one launch each, the
    hidden activations kept in shared memory) gives the bits of one launch per layer,
    over batches large enough that every CTA runs many blocks through its rings."""
    rng = np.random.default_rng(W * 7 + n)
    levels = [int(v) for v in rng.integers(1, 13, n)]
    up = (rng.standard_normal((n, W, W)) * 300.0 + 1000.0).astype(np.float32)
    up += np.cumsum(rng.standard_normal((n, W, W)).astype(np.float32), axis=2)
    si = np.full(24, 300.0, np.float32)
    so = np.geomspace(200.0, 0.01, 24).astype(np.float32)
    net = L.LearnedPredictor(tile_width=W, max_batch=n, seed=5)
    net.set_sigmas(si, so)
    up_d = torch.from_numpy(up).cuda()
    net.set_fused(False)
    per_layer = net.forward(up_d, levels).clone()
    net.set_fused(True)
    fused = net.forward(up_d, levels)
    torch.cuda.synchronize()
    assert torch.isfinite(fused).all()
    diff = (fused != per_layer).sum().item()
    assert diff == 0, "%d of %d outputs differ" % (diff, fused.numel())
    net.close()


def test_adam_lowers_the_loss_of_a_fixed_batch(L):
    W, n = 37, 4
    levels, up, target, si, so = _case(W, n, seed=3)
    # a learnable target: a smooth function of the input
    target = (0.05 * (up - up.mean(axis=(1, 2), keepdims=True))).astype(np.float32)
    net = L.LearnedPredictor(tile_width=W, max_batch=n, seed=2)
    net.set_sigmas(si, so)
    up_d, tg_d = torch.from_numpy(up).cuda(), torch.from_numpy(target).cuda()
    losses = []
    for _ in range(60):
        net.forward(up_d, levels, training=True)
        losses.append(net.backward(tg_d))
        net.adam(3e-3)
    assert losses[-1] < 0.5 * losses[0], losses[::10]
    net.close()


def test_learned_residual_tiles_through_the_elevation_kernel(gpu, L, oracle_lib):
    tp, orc = gpu, oracle_lib
    W, n = 101, 6
    rng = np.random.default_rng(9)
    net = L.LearnedPredictor(tile_width=W, max_batch=8, seed=3)
    si = np.full(24, 300.0, np.float32)
    so = np.full(24, 12.0, np.float32)
    net.set_sigmas(si, so)
    elev = tp.TileStorage(W, 3, n + 1)
    res = tp.TileStorage(W, 1, n)
    parent = (rng.standard_normal((1, W, W)) * 500.0).astype(np.float32)
    elev.upload(0, tp.ZF, parent)
    elev.upload(0, tp.ZM, np.maximum(parent, 0))
    kids = [(4, 6 + (k % 2), 2 + (k // 2) % 2) for k in range(n)]
    jobs = [tp.make_job(l, x, y, out_slot=1 + k, parent_slot=0, residual_slot=k, tile_meters=3000.0)
            for k, (l, x, y) in enumerate(kids)]
    net.predict_residuals(elev, jobs, res)
    tp.elevation_batch(elev, res, None, tp.make_params(), jobs)
    tp.stream_check()
    r = res.download(0, n, 0)
    zf = elev.download(1, n, tp.ZF)
    ups = []
    for k, (l, x, y) in enumerate(kids):
        z = np.zeros((W, W), np.float32)
        orc.lib().or_residual_upsample(W, W - 5, x, y, orc._p(parent[0]), orc._p(z))
        ups.append(z)
        # the tile is the stencil plus the learned residual, bit-exact
        ezf, _, _ = orc.elevation_tile(W, l, x, y, parent[0], np.maximum(parent[0], 0), r[k])
        assert np.array_equal(zf[k], ezf)
    # the residuals are the net's prediction on the upsampled parents
    want = net.forward(torch.from_numpy(np.stack(ups)).cuda(), [l for l, _, _ in kids]).cpu().numpy()
    assert _relerr(r, want) < 1e-6
    assert float(np.abs(r).max()) > 0.0
    net.close()
