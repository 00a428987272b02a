"""Planet-scale mixed frames: requests on the six faces of a cube planet, 197-wide
tiles at levels 0-16, stored (synthetic) residuals through level 10 and learned
residuals (or, without a net, the plain per-level noise) beyond, sphere normals.

One frame = learned residual tiles for the deep requests (tp_learned_predict_residuals,
in chunks), one persistent elevation launch for all requests (a CUDA graph), and
the normal pass on the sphere (tp_normal_batch).  Errors per level are stated
against FP64 evaluations of the same tiles (oracle twins), see `fp64_errors`.
"""
import ctypes as C

import numpy as np

from . import TileStorage, Frame, TileJob, make_job, make_params, noise_select, normal_batch, ZF, ZM, NX, NY
from . import workloads

EARTH_ROOT = 2.0 * 6360000.0   # root quad size of a face: twice the radius (terrain2, demo earth)


class PlanetFrame:
    def __init__(self, n=16384, seed=11, W=197, max_level=16, stored_max=10, root=EARTH_ROOT, n_unique_parents=48,
                 n_residual_pool=64):
        rng = np.random.default_rng(seed)
        self.W, self.n, self.root = W, n, root
        self.stored_max = stored_max
        self.levels = rng.integers(0, max_level + 1, n)
        self.faces = rng.integers(1, 7, n)
        self.tx = np.array([rng.integers(0, 1 << int(l)) for l in self.levels])
        self.ty = np.array([rng.integers(0, 1 << int(l)) for l in self.levels])
        uz, um = workloads.fbm_parent_tiles(min(n_unique_parents, n), W, seed)
        pick = np.arange(n) % uz.shape[0]
        self.parent_zf, self.parent_zm = uz[pick], um[pick]
        # stored residuals: a pool of unit N(0, 1) tiles scaled by the level's sigma
        pool = np.random.default_rng(seed + 1).standard_normal((min(n_residual_pool, n), W, W), dtype=np.float32)
        sig = np.where(self.levels > stored_max, 0.0, 2000.0 * 0.5 ** np.minimum(self.levels, stored_max))
        self.residual = pool[np.arange(n) % pool.shape[0]] * sig.astype(np.float32)[:, None, None]
        self.learned_idx = np.nonzero(self.levels > stored_max)[0]

    def jobs(self, learned):
        """Elevation jobs: stored levels add their residual and no noise; deep levels
        add the learned residual (noise off) or, without a net, the plain noise."""
        out = []
        for k in range(self.n):
            l, x, y, f = int(self.levels[k]), int(self.tx[k]), int(self.ty[k]), int(self.faces[k])
            rot, layer = noise_select(f, l, x, y)
            deep = l > self.stored_max
            amp = 0.0 if (not deep or learned) else float(workloads.noise_amplitude(l))
            out.append(make_job(l, x, y, out_slot=k, parent_slot=self.n + k if l > 0 else -1, residual_slot=k,
                                normal_slot=k, noise_rot=rot, noise_layer=layer, noise_amp=amp,
                                tile_meters=self.root / (1 << l)))
        return out

    def allocate(self, tp=None):
        W, n = self.W, self.n
        self.elev = TileStorage(W, 3, 2 * n)
        self.res = TileStorage(W, 1, n)
        self.nrm = TileStorage(W - 4, 2, n)
        self.elev.upload(n, ZF, self.parent_zf)
        self.elev.upload(n, ZM, self.parent_zm)
        self.res.upload(0, 0, self.residual)

    def build(self, net=None, stream=None, chunk=512):
        """Jobs and the elevation frame (graph) of this planet frame."""
        self.net = net
        self.all_jobs = self.jobs(learned=net is not None)
        self.frame = Frame()
        # normals are on the sphere: not fused into the elevation launch
        flat = []
        for j in self.all_jobs:
            c = TileJob.from_buffer_copy(j)
            c.normal_slot = -1
            flat.append(c)
        self.frame.add(self.elev, self.res, None, make_params(), flat)
        self.learned_jobs = [self.all_jobs[k] for k in self.learned_idx]
        self.chunk = chunk
        # the frame's job arrays in C form, built once (a renderer keeps its requests so)
        from . import job_array
        self.all_jobs_arr = job_array(self.all_jobs)
        self.learned_chunks = [job_array(self.learned_jobs[s:s + chunk]) for s in range(0, len(self.learned_jobs), chunk)]

    def produce(self, stream=None):
        if self.net is not None:
            for arr in self.learned_chunks:
                self.net.predict_residuals(self.elev, arr, self.res, stream)
        self.frame.graph_launch(stream)
        normal_batch(self.elev, self.nrm, self.all_jobs_arr, self.root, stream)

    def fp64_errors(self, oracle, per_level=2, seed=0):
        """Per level: max / RMS height error of zf and max / RMS normal-angle error
        (radians) against FP64 evaluations of the same tiles (same parent, residual
        and noise inputs); normals from the FP64 heights on the FP64 sphere frame."""
        rng = np.random.default_rng(seed)
        table = oracle.dem_noise(self.W)
        out = {}
        for l in np.unique(self.levels):
            idx = np.nonzero(self.levels == l)[0]
            errs_h, errs_a = [], []
            for k in rng.choice(idx, min(per_level, len(idx)), replace=False):
                k = int(k)
                j = self.all_jobs[k]
                zf = self.elev.download(k, 1, ZF)[0]
                res = self.res.download(k, 1, 0)[0]
                nx = self.nrm.download(k, 1, NX)[0]
                ny = self.nrm.download(k, 1, NY)[0]
                pz = self.parent_zf[k] if j.level > 0 else None
                pm = self.parent_zm[k] if j.level > 0 else None
                dzf, _, dzm = oracle.elevation_tile(self.W, j.level, j.tx, j.ty, pz, pm, res, noise=table[j.noise_layer],
                                                    noise_rot=j.noise_rot, noise_amp=j.noise_amp, f64=True)
                errs_h.append(np.asarray(zf, np.float64) - dzf)
                dnx, dny = oracle.normals_sphere_f64(self.W, dzm, self.root, j.level, j.tx, j.ty)
                a = np.stack([nx, ny, np.sqrt(np.maximum(0.0, 1.0 - nx.astype(np.float64) ** 2 - ny.astype(np.float64) ** 2))])
                b = np.stack([dnx, dny, np.sqrt(np.maximum(0.0, 1.0 - dnx ** 2 - dny ** 2))])
                errs_a.append(np.arccos(np.clip((a * b).sum(0), -1.0, 1.0)))
            h = np.concatenate([e.ravel() for e in errs_h])
            a = np.concatenate([e.ravel() for e in errs_a])
            out[int(l)] = {"max_height_err": float(np.abs(h).max()), "rms_height_err": float(np.sqrt((h ** 2).mean())),
                           "max_normal_angle_err": float(a.max()), "rms_normal_angle_err": float(np.sqrt((a ** 2).mean())),
                           "learned": bool(l > self.stored_max and self.net is not None)}
        return out

    def close(self):
        self.frame.close()
