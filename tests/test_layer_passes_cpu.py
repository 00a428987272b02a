"""The layer kernel's order-independent pass rule, restated on the CPU, equals the
oracle's in-order drawing on adversarial tiles.

The kernel (csrc/tp_layers.cu) splits a tile's meshes into passes (runs with one
pass state, a new one at each depth clear) and resolves each pass per texel over
the fragments that pass the depth test against the depth stored BEFORE the pass:
LESS with depth writes keeps the least (depth, triangle number), every other
supported state the largest triangle number.  Here that rule runs in numpy over
fragments rasterised with the oracle's arithmetic (float32, each operation
rounded), and the result is compared with or_layer_tile, which draws fragment by
fragment in order.  CPU only."""
import numpy as np

from test_gpu_water_layer import adversarial, as_batch, water_tile

f32 = np.float32


def _snap(c, W):
    w = f32(f32(f32(c) + f32(1.0)) * f32(0.5 * W)) * f32(256.0)
    return int(np.rint(w)) if abs(w) <= 8388608.0 else None


def _smooth(e0, e1, x):
    t = np.clip((x - f32(e0)) / (f32(e1) - f32(e0)), f32(0.0), f32(1.0)).astype(np.float32)
    return t * t * (f32(3.0) - f32(2.0) * t)


def _triangles(ms):
    out = []
    for mi, (v, ix, mode, *_rest) in enumerate(ms):
        v = np.asarray(v, np.float32).reshape(-1, 4)
        cnt = len(ix) if ix is not None else len(v)
        ntri = cnt // 3 if mode == 0 else max(cnt - 2, 0)
        for k in range(ntri):
            c = ((k + 1, k, k + 2) if k & 1 else (k, k + 1, k + 2)) if mode == 1 else (3 * k, 3 * k + 1, 3 * k + 2)
            out.append((mi, [v[ix[q] if ix is not None else q] for q in c]))
    return out


def _fragments(W, verts, prog, fill_depth):
    """Coverage, z, w and depth of one triangle at every texel centre."""
    X, Y = [], []
    for q in verts:
        x, y = _snap(q[0], W), _snap(q[1], W)
        if x is None or y is None:
            return None
        X.append(x)
        Y.append(y)
    a, u = [f32(q[2]) for q in verts], [f32(q[3]) for q in verts]

    def edge(xa, ya, xb, yb, px, py):
        return (xb - xa) * (py - ya) - (yb - ya) * (px - xa)
    a2 = edge(X[0], Y[0], X[1], Y[1], X[2], Y[2])
    if a2 == 0:
        return None
    if a2 < 0:
        X[1], X[2], Y[1], Y[2], a[1], a[2], u[1], u[2] = X[2], X[1], Y[2], Y[1], a[2], a[1], u[2], u[1]
        a2 = -a2
    area = f32(a2)
    j, i = np.mgrid[0:W, 0:W]
    px, py = 256 * i + 128, 256 * j + 128
    E = [edge(X[1], Y[1], X[2], Y[2], px, py), edge(X[2], Y[2], X[0], Y[0], px, py),
         edge(X[0], Y[0], X[1], Y[1], px, py)]
    inside = np.ones((W, W), bool)
    for q in range(3):
        dx, dy = X[(q + 2) % 3] - X[(q + 1) % 3], Y[(q + 2) % 3] - Y[(q + 1) % 3]
        top_left = dy < 0 or (dy == 0 and dx < 0)
        inside &= (E[q] > 0) | ((E[q] == 0) & top_left)
    l1 = (E[1].astype(np.float32) / area).astype(np.float32)
    l2 = (E[2].astype(np.float32) / area).astype(np.float32)
    A = a[0] + (a[1] - a[0]) * l1 + (a[2] - a[0]) * l2
    U = u[0] + (u[1] - u[0]) * l1 + (u[2] - u[0]) * l2
    d = np.abs(U)
    if prog == 0:
        z = A + f32(0.03) * (f32(1.0) - _smooth(0.98, 1.0, d))
        w, dp = _smooth(1.0, 2.0, d), np.clip(d * f32(0.1) + f32(0.3), 0, 1)
    elif prog == 4:
        z, w, dp = A, U, np.full((W, W), np.clip(f32(fill_depth), 0, 1), np.float32)
    else:
        river = prog - 1
        z = A if river == 0 else (A - f32(1.0)) + np.maximum(d - f32(1.0), f32(0.0))
        w = _smooth(1.0, 2.0, d)
        dp = np.full((W, W), f32(1.0)) if river == 2 else \
            np.clip(d * f32(0.1) + (f32(0.15) if river == 1 else f32(0.3)), 0, 1)
    return inside, z.astype(np.float32), w.astype(np.float32), dp.astype(np.float32)


def resolve_by_passes(W, zf, zm, ms):
    z, w, dep = zm.copy(), np.zeros_like(zm), np.ones_like(zm)
    tris = _triangles(ms)
    m = 0
    while m < len(ms):
        state, clear = ms[m][5], ms[m][3]
        m2 = m + 1
        while m2 < len(ms) and not ms[m2][3] and ms[m2][5] == state:
            m2 += 1
        if clear:
            dep[:] = 1.0
        test = state & 3
        write_depth, write_z, write_w = not state & 4, not state & 8, not state & 16
        least = test == 0 and write_depth
        hit = np.zeros((W, W), bool)
        bz, bw, bd = np.zeros_like(z), np.zeros_like(z), np.zeros_like(z)
        for mi, verts in tris:
            if not m <= mi < m2:
                continue
            fr = _fragments(W, verts, ms[mi][4], ms[mi][6])
            if fr is None:
                continue
            inside, fz, fw, fdp = fr
            ok = inside & (fdp < dep if test == 0 else (True if test == 1 else fdp != dep))
            # least: a later triangle wins only with a strictly smaller depth; last: always
            upd = ok & (~hit | (fdp < bd)) if least else ok
            bz, bw, bd = np.where(upd, fz, bz), np.where(upd, fw, bw), np.where(upd, fdp, bd)
            hit |= upd
        if write_z:
            z = np.where(hit, bz, z)
        if write_w:
            w = np.where(hit, bw, w)
        if write_depth:
            dep = np.where(hit, bd, dep)
        m = m2
    b = np.minimum(w, f32(1.0))
    return (zf * b + z * (f32(1.0) - b)).astype(np.float32)


def test_pass_rule_equals_in_order_drawing(oracle_lib):
    W = 61
    rng = np.random.default_rng(2024)
    tiles = [adversarial(rng, W, k) for k in range(10)] + [as_batch(water_tile(rng, W, k=k)) for k in range(2)]
    zr = np.random.default_rng(5)
    for k, ms in enumerate(tiles):
        zf = (zr.standard_normal((W, W)) * 60.0).astype(np.float32)
        zm = np.maximum(zf, f32(0.0))
        want = oracle_lib.layer_tile(W, zf, zm, ms, 0)
        assert not np.array_equal(want, zm), k
        assert np.array_equal(resolve_by_passes(W, zf, zm, ms), want), k
