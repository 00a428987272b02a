"""The oracle against known answers (no GPU): the stencil copies parent samples
at even/even positions and reproduces cubic polynomials exactly; the reference's
CPU producer and its GPU shader agree without noise (edit3 pairing); the LCG,
fp16 rounding and noise table; flat normals of planes; HeightMipmap's residual
relation; the FP64 twin."""
import numpy as np
import pytest


def cubic_parent(W, seed):
    """Integer cubic z(x, y) sampled on the parent grid (exact in float)."""
    rng = np.random.default_rng(seed)
    c = rng.integers(-3, 4, 10).astype(np.float64)
    y, x = np.mgrid[0:W, 0:W].astype(np.float64)
    u, v = x - W / 2, y - W / 2
    z = (c[0] + c[1] * u + c[2] * v + c[3] * u * u + c[4] * u * v + c[5] * v * v
         + (c[6] * u ** 3 + c[7] * u * u * v + c[8] * u * v * v + c[9] * v ** 3) / 8.0)
    return z, c


@pytest.mark.parametrize("W,tx,ty", [(37, 0, 0), (37, 1, 0), (37, 0, 1), (37, 1, 1), (101, 1, 1), (197, 0, 1)])
def test_stencil_reproduces_cubics_and_copies_parent(oracle_lib, W, tx, ty):
    zp, c = cubic_parent(W, W + tx + ty)
    parent = zp.astype(np.float32)
    assert np.array_equal(parent.astype(np.float64), zp)   # exactly representable
    child = oracle_lib.cpu_elevation_tile(W, 3, tx, ty, parent)
    n = W - 5
    dx, dy = (tx % 2) * n // 2, (ty % 2) * n // 2
    # child sample i sits at parent coordinate (i - 2) / 2 + dx + 2
    i = np.arange(W)
    px = (i - 2) / 2.0 + dx + 2
    py = (i - 2) / 2.0 + dy + 2
    PX, PY = np.meshgrid(px, py)
    u, v = PX - W / 2, PY - W / 2
    exact = (c[0] + c[1] * u + c[2] * v + c[3] * u * u + c[4] * u * v + c[5] * v * v
             + (c[6] * u ** 3 + c[7] * u * u * v + c[8] * u * v * v + c[9] * v ** 3) / 8.0)
    # exact in real arithmetic: only float rounding of the partial sums remains
    assert np.abs(child.astype(np.float64) - exact).max() <= 4 * 2.0 ** -24 * np.abs(exact).max()
    # even/even child samples are parent samples
    assert np.array_equal(child[::2, ::2], parent[dy + 1:dy + 1 + (W + 1) // 2, dx + 1:dx + 1 + (W + 1) // 2])


def test_cpu_and_gpu_producers_agree_without_noise(oracle_lib):
    """edit/examples/edit3/helloworld.xml:36-56 runs a cpuElevationProducer next to
    an elevationProducer on the same residuals; with no noise their zf match."""
    rng = np.random.default_rng(3)
    W, Wr = 101, 197
    parent = (rng.standard_normal((W, W)) * 300).astype(np.float32)
    res = (rng.standard_normal((Wr, Wr)) * 20).astype(np.float32)
    for tx, ty in [(4, 6), (5, 6), (4, 7), (5, 7)]:
        rx, ry = (tx % 2) * 96, (ty % 2) * 96
        cpu = oracle_lib.cpu_elevation_tile(W, 3, tx, ty, parent, res, rx, ry)
        zf, zc, zm = oracle_lib.elevation_tile(W, 3, tx, ty, parent, None, res, rx, ry)
        assert np.array_equal(cpu, zf)
        assert np.array_equal(zm, np.maximum(zf, 0))


def test_lcg_and_half_rounding(oracle_lib):
    seq = oracle_lib.lrandom_seq(1234567, 5)
    s, want = 1234567, []
    for _ in range(5):
        s = (s * 1103515245 + 12345) & 0x7FFFFFFF
        want.append(s)
    assert seq == want
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-1, 1, 20000), rng.uniform(-1e-4, 1e-4, 2000), [2 ** -23, -2 ** -24, 1.0 - 2 ** -24]])
    xs = xs.astype(np.float32)
    got = np.array([oracle_lib.half_round(x) for x in xs], np.float32)
    assert np.array_equal(got, xs.astype(np.float16).astype(np.float32))


def test_noise_table(oracle_lib):
    W = 101
    t = oracle_lib.dem_noise(W)
    assert t.shape == (6, W, W)
    assert np.all(np.abs(t) <= 1.0)
    assert np.array_equal(t, t.astype(np.float16).astype(np.float32))
    # layers 0 and 1 differ only where the bottom edge's bit differs (layer ids 0 and 1)
    assert not np.array_equal(t[0][:5, 5:W - 5], t[1][:5, 5:W - 5])
    # border bands mirror: row 2 symmetric in x
    for l in range(6):
        assert np.array_equal(t[l][2, 5:W // 2 + 1], t[l][2, W - 1 - np.arange(5, W // 2 + 1)])


def test_plane_normals(oracle_lib):
    W, meters = 101, 1000.0
    n = W - 5
    h = meters / n
    y, x = np.mgrid[0:W, 0:W].astype(np.float64)
    a, b = 0.3, -0.7
    zm = (a * x * h + b * y * h + 500.0).astype(np.float32)
    nx, ny = oracle_lib.normals_flat(W, zm, meters)
    ln = np.sqrt(a * a + b * b + 1.0)
    assert np.abs(nx + a / ln).max() < 1e-5
    assert np.abs(ny + b / ln).max() < 1e-5


def test_heightmipmap_residual_relation(oracle_lib):
    rng = np.random.default_rng(5)
    W = 101
    parent = (rng.standard_normal((W, W)) * 100).astype(np.float32)
    fine = (oracle_lib.cpu_elevation_tile(W, 1, 1, 0, parent) + rng.standard_normal((W, W)) * 30).astype(np.float32)
    rq, enc, approx = oracle_lib.compute_residual(W, 1, 0, parent, fine)
    assert np.array_equal(rq, enc.astype(np.float32))
    assert np.abs(approx - fine).max() <= 0.5 + 1e-3
    # approx = upsample(parent) + quantised residual: the elevation producer rebuilds it
    zf = oracle_lib.cpu_elevation_tile(W, 1, 1, 0, parent, rq)
    assert np.array_equal(zf, approx)


def test_fp64_twin(oracle_lib):
    rng = np.random.default_rng(8)
    W = 197
    parent = (rng.standard_normal((W, W)) * 1000).astype(np.float32)
    res = (rng.standard_normal((W, W)) * 10).astype(np.float32)
    t = oracle_lib.dem_noise(W)
    a = oracle_lib.elevation_tile(W, 5, 3, 4, parent, None, res, noise=t[2], noise_rot=3, noise_amp=-15.0)
    b = oracle_lib.elevation_tile(W, 5, 3, 4, parent, None, res, noise=t[2], noise_rot=3, noise_amp=-15.0, f64=True)
    for x, y in zip(a, b):
        assert np.abs(x - y).max() < 1e-3


def test_gl_linear_sampling_emulation(oracle_lib):
    """The reporting-only emulation of the GL path's LINEAR fetches at +0.25-texel
    offsets: on a plane it gives the texel-exact normals (finite differences of a
    plane do not depend on the sampling offset); on a rough surface it moves them."""
    import numpy as np
    W, meters = 101, 1000.0
    y, x = np.mgrid[0:W, 0:W].astype(np.float64)
    plane = (3.0 * x - 2.0 * y + 40.0).astype(np.float32)
    pnx, pny = oracle_lib.normals_flat(W, plane, meters)
    lnx, lny = oracle_lib.normals_flat_gl_linear(W, plane, meters)
    assert np.abs(pnx - lnx).max() < 1e-6 and np.abs(pny - lny).max() < 1e-6
    rough = np.random.default_rng(2).standard_normal((W, W)).astype(np.float32) * 20.0
    pnx, _ = oracle_lib.normals_flat(W, rough, meters)
    lnx, _ = oracle_lib.normals_flat_gl_linear(W, rough, meters)
    assert np.abs(pnx - lnx).max() > 1e-3
