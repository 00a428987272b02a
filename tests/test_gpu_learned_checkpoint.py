"""Checkpoint and resume of the learned predictor's training: the state written
every k steps (parameters, Adam's moments and step count, the sigmas, the batch
sampler's random state and the losses) restores exactly into a fresh net, and a
run resumed from it continues with the same batches and rates as the run that
wrote it.  The weight gradients sum per-CTA partials with atomics, so the two
continuations agree to rounding, not bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_resume_continues_the_run(gpu, tmp_path):
    from proland_gb300 import learned as L
    data = L.merge(L.build_pyramid(3, seed=4), L.deep_pairs([8, 9], 64, seed=4, tile_seed=4))
    si, so = L.level_sigmas(data)
    a = L.LearnedPredictor(101, 32, seed=3)
    a.set_sigmas(si, so)
    ck = str(tmp_path / "ck_{step}.npz")
    la = L.train(a, data, 30, batch=32, lr=1e-3, lr_final=1e-4, seed=11, checkpoint=ck, checkpoint_every=15)
    # the state at step 15 restores exactly
    b = L.LearnedPredictor(101, 32, seed=99)
    extra = b.load_state(ck.format(step=15))
    with np.load(ck.format(step=15)) as f:
        assert np.array_equal(b.get_params(), f["params"])
        assert int(f["adam_step"]) == 15 and int(extra["train_step"]) == 15
    # a fresh net resumed from step 15 follows the original run
    c = L.LearnedPredictor(101, 32, seed=98)
    lc = L.train(c, data, 30, batch=32, lr=1e-3, lr_final=1e-4, seed=11, resume_from=ck.format(step=15))
    assert len(lc) == 30 and lc[:15] == la[:15]
    np.testing.assert_allclose(lc[15:], la[15:], rtol=2e-3)
    pa, pc = a.get_params(), c.get_params()
    assert np.abs(pa - pc).max() <= 1e-3 * np.abs(pa).max()
    with np.load(ck.format(step=30)) as f:
        assert np.array_equal(f["params"], pa)
    for n in (a, b, c):
        n.close()
