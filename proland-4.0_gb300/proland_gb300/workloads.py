"""Seeded synthetic inputs of the benchmark configurations (numpy only).

No public dataset is involved: parents are value-noise fBm tiles, residuals iid
normal samples, noise amplitudes per level as in the configurations:

* quadtree:  levels 0..L of W=101 tiles, root = 8-octave value-noise fBm
  (lacunarity 2, gain 0.5, amplitude 4000 m), residual at level l iid
  N(0, (2000 * 0.5^l)^2), noise off;
* frame:     n independent requests, levels uniform in 1..12, a fraction of
  them 197-wide, each with its own materialised fBm parent, residual sigma as
  above, noise amplitude 300 * 0.55^l with the DEM noise table.
"""
import numpy as np


def value_noise_fbm(shape, octaves=8, lacunarity=2.0, gain=0.5, amplitude=4000.0,
                    base_cells=4, seed=1, offset=(0.0, 0.0), scale=1.0):
    """Value-noise fBm sampled on an (H, W) grid: each octave bilinearly interpolates
    a random lattice of `base_cells * lacunarity^o` cells across the grid, with
    smoothstep weights; octave amplitudes `gain^o`, normalised to `amplitude`."""
    H, Wd = shape
    rng = np.random.default_rng(seed)
    out = np.zeros(shape, np.float64)
    norm = 0.0
    y = (np.arange(H, dtype=np.float64) * scale + offset[1])
    x = (np.arange(Wd, dtype=np.float64) * scale + offset[0])
    a = 1.0
    for o in range(octaves):
        cells = base_cells * (lacunarity ** o)
        step = max(H, Wd) / cells
        gy, gx = y / step, x / step
        ny, nx = int(np.floor(gy.max())) + 2, int(np.floor(gx.max())) + 2
        lat = rng.standard_normal((ny + 1, nx + 1))
        iy, ix = np.floor(gy).astype(int), np.floor(gx).astype(int)
        fy, fx = gy - iy, gx - ix
        fy = fy * fy * (3 - 2 * fy)
        fx = fx * fx * (3 - 2 * fx)
        v00 = lat[np.ix_(iy, ix)]
        v01 = lat[np.ix_(iy, ix + 1)]
        v10 = lat[np.ix_(iy + 1, ix)]
        v11 = lat[np.ix_(iy + 1, ix + 1)]
        fxr, fyc = fx[None, :], fy[:, None]
        out += a * ((v00 * (1 - fxr) + v01 * fxr) * (1 - fyc) + (v10 * (1 - fxr) + v11 * fxr) * fyc)
        norm += a
        a *= gain
    out *= amplitude / (2.0 * norm)
    return out.astype(np.float32)


def residual_sigma(level):
    return 2000.0 * 0.5 ** level


def noise_amplitude(level):
    return 300.0 * 0.55 ** level


def residual_tiles(levels, W, seed):
    """iid N(0, sigma(level)^2) residual tiles, one per entry of `levels`: [n, W, W]."""
    rng = np.random.default_rng(seed)
    levels = np.asarray(levels)
    sig = (2000.0 * 0.5 ** levels.astype(np.float64)).astype(np.float32)
    return (rng.standard_normal((len(levels), W, W), dtype=np.float32) * sig[:, None, None])


def fbm_parent_tiles(n, W, seed, octaves=8):
    """n different W x W fBm tiles (zf) cut from one fBm field, plus their zm = max(zf, 0)."""
    side = int(np.ceil(np.sqrt(n)))
    field = value_noise_fbm((side * W, side * W), octaves=octaves, seed=seed,
                            base_cells=max(2, side * 2))
    zf = np.empty((n, W, W), np.float32)
    for k in range(n):
        r, c = divmod(k, side)
        zf[k] = field[r * W:(r + 1) * W, c * W:(c + 1) * W]
    return zf, np.maximum(zf, 0.0).astype(np.float32)


def frame_requests(n, seed, frac_197=0.25, max_level=12):
    """Levels, tile coordinates and widths of an n-request frame."""
    rng = np.random.default_rng(seed)
    levels = rng.integers(1, max_level + 1, n)
    tx = np.array([rng.integers(0, 1 << int(l)) for l in levels])
    ty = np.array([rng.integers(0, 1 << int(l)) for l in levels])
    wide = rng.random(n) < frac_197
    return levels, tx, ty, wide
