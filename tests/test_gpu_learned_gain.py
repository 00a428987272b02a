"""What the learned residual predictor gains over the method without it, on terrain
it was not trained on.

The pairs below the finest octave's cells come from tp_fbm_pairs (the procedural
fBm sampled on each tile's own window); the test first checks those pairs against
the oracle bit for bit.  Then the net is trained briefly by the library's own
kernels on a small residual pyramid (levels 1-5) plus deep pairs (levels 6-10) of
one fBm seed, and evaluated on pairs of ANOTHER seed: per level its RMS height
error must be below the plain method's (which leaves the residual out, so its
error is the residual itself), and where the field is resolved (levels 9-10) the
net must remove most of the residual."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_deep_pairs_match_oracle(gpu, oracle_lib):
    import torch
    W = 101
    arr = lambda v: (C.c_int * 1)(v)  # noqa: E731
    for l, x, y in [(1, 1, 0), (6, 21, 40), (9, 300, 17), (12, 2047, 3001)]:
        up = torch.empty((1, W, W), dtype=torch.float32, device="cuda")
        res = torch.empty_like(up)
        gpu.check(gpu.lib().tp_fbm_pairs(12, 4, 4000.0, 5, 96, arr(l), arr(x), arr(y), 1, C.c_void_p(up.data_ptr()),
                                         C.c_void_p(res.data_ptr()), None, None))
        torch.cuda.synchronize()
        wup, wres, _ = oracle_lib.fbm_pair(l, x, y, seed=5)
        assert np.array_equal(up[0].cpu().numpy(), wup), (l, x, y)
        assert np.array_equal(res[0].cpu().numpy(), wres), (l, x, y)


def test_trained_net_beats_the_plain_method_on_held_out_terrain(gpu):
    from proland_gb300 import learned as L
    train = L.merge(L.build_pyramid(5, seed=1), L.deep_pairs(range(6, 11), 384, seed=1, tile_seed=1))
    held = L.merge(L.select_levels(L.build_pyramid(5, seed=2), [3, 4, 5]),
                   L.deep_pairs(range(6, 11), 48, seed=2, tile_seed=2))
    si, so = L.level_sigmas(train)
    net = L.LearnedPredictor(101, 128, seed=3)
    net.set_sigmas(si, so)
    losses = L.train(net, train, 600, batch=128, lr=1e-3, lr_final=2e-4)
    assert np.mean(losses[-50:]) < np.mean(losses[:50])
    ev = L.evaluate(net, held, so)
    print({l: round(e["rms_over_sigma"], 3) for l, e in ev.items()})
    for l, e in ev.items():
        assert e["rms_learned"] < e["rms_plain"], (l, e)
    assert min(ev[9]["rms_over_sigma"], ev[10]["rms_over_sigma"]) < 0.5, ev
    net.close()
