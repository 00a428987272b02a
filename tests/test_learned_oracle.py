"""The oracle of the learned predictor and of the device preprocess, on the CPU:
the backward pass against central finite differences (fp64 mode), the bf16
emulation close to fp64, and the level tiles' decimation and edge clamping."""
import numpy as np

import oracle


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    W, n = 9, 2
    P = oracle.learned_param_count()
    params = (rng.standard_normal(P) * 0.2).astype(np.float32)
    up = (rng.standard_normal((n, W, W)) * 50).astype(np.float32)
    tg = (rng.standard_normal((n, W, W)) * 3).astype(np.float32)
    lv, si, so = [3, 5], np.full(24, 40.0, np.float32), np.full(24, 2.0, np.float32)
    _, _, g = oracle.learned_loss_grad(params, up, tg, lv, si, so, emulate=False)
    worst = 0.0
    for i in rng.choice(P, 40, replace=False):
        h = np.float32(1e-3 * max(1.0, abs(params[i])))
        pp, pm = params.copy(), params.copy()
        pp[i] += h
        pm[i] -= h
        lp = oracle.learned_loss_grad(pp, up, tg, lv, si, so, emulate=False, want_grad=False)[0]
        lm = oracle.learned_loss_grad(pm, up, tg, lv, si, so, emulate=False, want_grad=False)[0]
        fd = (lp - lm) / (float(pp[i]) - float(pm[i]))
        worst = max(worst, abs(fd - g[i]) / max(1e-6, abs(fd) + abs(g[i])))
    assert worst < 1e-3, worst


def test_bf16_emulation_stays_close_to_fp64():
    rng = np.random.default_rng(1)
    W, n = 13, 2
    P = oracle.learned_param_count()
    params = (rng.standard_normal(P) * 0.1).astype(np.float32)
    up = (rng.standard_normal((n, W, W)) * 100).astype(np.float32)
    tg = (rng.standard_normal((n, W, W)) * 5).astype(np.float32)
    lv, si, so = [1, 2], np.full(24, 80.0, np.float32), np.full(24, 4.0, np.float32)
    l64, p64, g64 = oracle.learned_loss_grad(params, up, tg, lv, si, so, emulate=False)
    l16, p16, g16 = oracle.learned_loss_grad(params, up, tg, lv, si, so, emulate=True)
    assert abs(l16 - l64) < 2e-2 * l64
    assert np.linalg.norm(p16 - p64) < 3e-2 * np.linalg.norm(p64)
    assert np.linalg.norm(g16 - g64) < 5e-2 * np.linalg.norm(g64)


def test_level_tiles_decimate_and_clamp():
    ts, L = 16, 3
    base = oracle.fbm_heights((ts << L) + 1, octaves=8, base_cells=2, seed=4)
    # level L is the base itself, level l takes every 2^(L-l)-th sample
    t3 = oracle.level_tile(base, ts, L, 3, 1, 2)
    assert t3[2, 2] == base[2 * ts, ts]
    t1 = oracle.level_tile(base, ts, L, 1, 1, 0)
    assert t1[2 + 3, 2 + 5] == base[(0 * ts + 3) * 4, (1 * ts + 5) * 4]
    # coordinates outside the level clamp to its edge
    t0 = oracle.level_tile(base, ts, L, 0, 0, 0)
    assert t0[0, 0] == t0[2, 2] == base[0, 0]
    assert t0[-1, -1] == base[-1, -1]
    assert np.abs(base.astype(np.int64)).max() > 100
