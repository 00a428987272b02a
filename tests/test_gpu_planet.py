"""Planet-scale mixed frames (6 cube faces, 197-wide tiles, levels 0-16): stored
residuals through level 10, learned residuals beyond, sphere normals.  Every tile
of a small frame equals the oracle on the same inputs; the FP64 error report per
level is within the float path's known bounds."""
import os
import sys

import numpy as np
import pytest

from tilecase import assert_normals_close

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "proland-4.0_gb300"))

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("learned", [True, False])
def test_planet_frame_matches_oracle(gpu, oracle_lib, learned):
    tp, orc = gpu, oracle_lib
    from proland_gb300 import learned as L, planet
    pf = planet.PlanetFrame(n=80, seed=5)
    pf.allocate()
    net = None
    if learned:
        net = L.LearnedPredictor(tile_width=197, max_batch=32, seed=4)
        si = np.array([900.0 * 0.5 ** l for l in range(24)], np.float32)
        so = np.array([30.0 * 0.5 ** l for l in range(24)], np.float32)
        net.set_sigmas(si, so)
    pf.build(net, chunk=32)
    pf.produce()
    tp.stream_check()
    table = orc.dem_noise(197)
    assert len(pf.learned_idx) > 10
    for k in range(pf.n):
        j = pf.all_jobs[k]
        res = pf.res.download(k, 1, 0)[0]
        if j.level > pf.stored_max:
            assert (np.abs(res).max() > 0) == learned
        else:
            assert np.array_equal(res, pf.residual[k])
        pz = pf.parent_zf[k] if j.level > 0 else None
        pm = pf.parent_zm[k] if j.level > 0 else None
        ezf, ezc, ezm = orc.elevation_tile(197, j.level, j.tx, j.ty, pz, pm, res, noise=table[j.noise_layer],
                                           noise_rot=j.noise_rot, noise_amp=j.noise_amp)
        assert np.array_equal(pf.elev.download(k, 1, tp.ZF)[0], ezf), k
        assert np.array_equal(pf.elev.download(k, 1, tp.ZM)[0], ezm), k
        enx, eny = orc.normals_sphere(197, ezm, orc.sphere_frame(pf.root, j.level, j.tx, j.ty))
        assert_normals_close(pf.nrm.download(k, 1, tp.NX)[0], enx, "nx %d" % k)
        assert_normals_close(pf.nrm.download(k, 1, tp.NY)[0], eny, "ny %d" % k)
    errs = pf.fp64_errors(orc, per_level=1)
    for l, e in errs.items():
        assert e["max_normal_angle_err"] < 2e-3, (l, e)
        assert e["max_height_err"] < 1e-2, (l, e)
    pf.close()
    if net:
        net.close()
