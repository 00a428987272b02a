"""Shared helpers of the parity tests: seeded tile inputs, a product run through
the C ABI and the same tiles through the CPU oracle."""
import numpy as np

ELEV_TOL_REL = 1e-5      # fp32 elevations vs the oracle: 1e-5 relative (asserted beside bit identity)
NORMAL_TOL_ABS = 1e-4    # normals vs the oracle


def smooth_tile(W, seed, amp=1500.0):
    """A smooth random W x W height tile with negative and positive values."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:W, 0:W].astype(np.float64) / W
    z = np.zeros((W, W))
    for k in range(6):
        fx, fy, ph = rng.uniform(0.5, 4.0), rng.uniform(0.5, 4.0), rng.uniform(0, 6.3)
        z += rng.uniform(0.3, 1.0) * np.sin(2 * np.pi * (fx * x + fy * y) + ph)
    z += 0.05 * rng.standard_normal((W, W))
    return (amp * z / 3.0).astype(np.float32)


class Case:
    """One tile to produce: inputs as host arrays plus the job fields."""

    def __init__(self, W, level, tx, ty, seed, residual_width=None, with_residual=True,
                 noise_amp=0.0, tile_meters=1000.0, rscale=1.0, face=1):
        self.W, self.level, self.tx, self.ty = W, level, tx, ty
        n = W - 5
        rng = np.random.default_rng(seed)
        self.parent_zf = smooth_tile(W, seed + 1) if level > 0 else None
        self.parent_zm = np.maximum(self.parent_zf, 0).astype(np.float32) if level > 0 else None
        self.Wr = residual_width or W
        self.mod = (self.Wr - 5) // n
        self.residual = ((rng.standard_normal((self.Wr, self.Wr)) * 40.0).astype(np.float32)
                         if with_residual else None)
        self.rx = (tx % self.mod) * n
        self.ry = (ty % self.mod) * n
        self.noise_amp = noise_amp
        self.tile_meters = np.float32(tile_meters)
        self.rscale = rscale
        self.face = face

    def oracle(self, oracle, noise_table, params, rot=0, layer=0):
        noise = noise_table[layer] if self.noise_amp != 0.0 else None
        n = self.W - 5
        mps = float(np.float32(self.tile_meters) / np.float32(n))
        g = n // params["grid_size"]
        zf, zc, zm = oracle.elevation_tile(
            self.W, self.level, self.tx, self.ty, self.parent_zf, self.parent_zm,
            self.residual, self.rx, self.ry, self.rscale, noise, rot, self.noise_amp,
            params["noise_mode"], mps, g, params["flip"], params["no_clamp"])
        nx, ny = oracle.normals_flat(self.W, zm, float(self.tile_meters))
        return zf, zc, zm, nx, ny


def assert_elev_close(got, want, what):
    """Bit-level agreement is expected; the stated tolerance is 1e-5 relative."""
    got, want = np.asarray(got), np.asarray(want)
    scale = np.maximum(np.abs(want), 1.0)
    err = np.abs(got.astype(np.float64) - want.astype(np.float64)) / scale
    assert err.max() <= ELEV_TOL_REL, "%s: max rel err %g at %s" % (what, err.max(), np.unravel_index(err.argmax(), err.shape))
    return int(np.count_nonzero(got != want))


def assert_normals_close(got, want, what):
    err = np.abs(np.asarray(got, np.float64) - np.asarray(want, np.float64))
    assert err.max() <= NORMAL_TOL_ABS, "%s: max abs err %g" % (what, err.max())
    return float(err.max())
