"""Learned residual predictor and the device preprocess that makes its training data.

* `fbm_heights`, `preprocess_level`, `build_pyramid`: residual pyramids built on the
  device the way the reference's preprocess tool builds them (decimated mipmap,
  residual = sample - upsample(parent approximation), rounded to int16), from a
  procedural fBm height field;
* `LearnedPredictor`: the 5-layer BF16 convolutional net of the C ABI
  (tp_learned_*), trained by the library's own forward/backward/Adam kernels;
* `train`: the training loop over (upsampled parent, residual) pairs of a pyramid,
  with the eight symmetries of the square as augmentation;
* `evaluate`: RMS / max height error and normal-angle error per level of the
  learned residuals against the stored ones, beside the plain method (stencil +
  noise, no residual).

Device buffers are torch CUDA tensors (plumbing); every computation runs in the
library's kernels.
"""
import ctypes as C
import json
import os

import numpy as np

from ._lib import TileJob, check, lib

try:
    import torch
except ImportError:  # pragma: no cover - the GPU paths need torch for device buffers
    torch = None

_f32p = C.POINTER(C.c_float)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


# ---------------------------------------------------------------- preprocess
def fbm_heights(size, octaves=12, base_cells=4, amplitude=4000.0, quantum=0.25, seed=1):
    """int16 heights (units of `quantum` metres) of the procedural fBm on a size x size grid."""
    out = torch.empty((size, size), dtype=torch.int16, device="cuda")
    check(lib().tp_fbm_heights(size, octaves, base_cells, amplitude, quantum, seed, _ptr(out), _stream()))
    return out


def preprocess_level(base, tile_size, max_level, level, parent=None, scale=1.0, want=("up", "res", "enc")):
    """One pyramid level on the device: (approx, up, res, enc) tensors of
    [4^level, W, W] (up/res/enc None at level 0 or when not wanted)."""
    W = tile_size + 5
    n = 1 << (2 * level)
    approx = torch.empty((n, W, W), dtype=torch.float32, device="cuda")
    up = res = enc = None
    if level > 0:
        up = torch.empty_like(approx) if "up" in want else None
        res = torch.empty_like(approx) if "res" in want else None
        enc = torch.empty((n, W, W), dtype=torch.int16, device="cuda") if "enc" in want else None
    check(lib().tp_preprocess_level(_ptr(base), tile_size, max_level, level, scale, _ptr(parent), _ptr(approx),
                                    _ptr(up), _ptr(res), _ptr(enc), _stream()))
    return approx, up, res, enc


def build_pyramid(max_level, tile_size=96, octaves=12, base_cells=4, amplitude=4000.0, quantum=0.25, seed=1,
                  first_level=1):
    """Training pairs of a residual pyramid: dict with 'up' [N, W, W] (upsampled parent
    approximations, metres), 'res' [N, W, W] (residuals, metres), 'level' [N] and
    'tile' [N, 3] (level, tx, ty), for levels first_level..max_level."""
    base = fbm_heights((tile_size << max_level) + 1, octaves, base_cells, amplitude, quantum, seed)
    approx, _, _, _ = preprocess_level(base, tile_size, max_level, 0)
    ups, ress, levels, tiles = [], [], [], []
    for l in range(1, max_level + 1):
        approx, up, res, _ = preprocess_level(base, tile_size, max_level, l, approx, want=("up", "res"))
        if l >= first_level:
            ups.append(up * quantum)
            ress.append(res * quantum)
            side = 1 << l
            levels.append(np.full(side * side, l, np.int32))
            tiles.append(np.stack([np.full(side * side, l), np.arange(side * side) % side,
                                   np.arange(side * side) // side], 1))
    return {"up": torch.cat(ups), "res": torch.cat(ress), "level": np.concatenate(levels),
            "tile": np.concatenate(tiles), "quantum": quantum, "tile_size": tile_size}


def deep_pairs(levels, per_level, seed=1, tile_seed=0, tile_size=96, octaves=12, base_cells=4, amplitude=4000.0):
    """(upsampled parent, residual) pairs at any levels of the same procedural fBm
    (tp_fbm_pairs: the field sampled in double precision on each tile's window, the
    residual formed before rounding): `per_level` tiles per level at random interior
    positions (drawn with `tile_seed`), as a dict like build_pyramid's."""
    rng = np.random.default_rng(tile_seed)
    lv, txs, tys = [], [], []
    for l in levels:
        m = 1 << int(l)
        lo, hi = (1, m - 1) if m > 2 else (0, m)
        lv += [int(l)] * per_level
        txs += [int(v) for v in rng.integers(lo, hi, per_level)]
        tys += [int(v) for v in rng.integers(lo, hi, per_level)]
    n, W = len(lv), tile_size + 5
    up = torch.empty((n, W, W), dtype=torch.float32, device="cuda")
    res = torch.empty_like(up)
    arr = lambda v: (C.c_int * n)(*v)  # noqa: E731
    check(lib().tp_fbm_pairs(octaves, base_cells, amplitude, seed, tile_size, arr(lv), arr(txs), arr(tys), n, _ptr(up),
                             _ptr(res), None, _stream()))
    return {"up": up, "res": res, "level": np.array(lv, np.int32), "tile": np.stack([lv, txs, tys], 1),
            "tile_size": tile_size}


def merge(*datas):
    """One training set of several pair sets (build_pyramid / deep_pairs dicts)."""
    return {"up": torch.cat([d["up"] for d in datas]), "res": torch.cat([d["res"] for d in datas]),
            "level": np.concatenate([d["level"] for d in datas]), "tile": np.concatenate([d["tile"] for d in datas]),
            "tile_size": datas[0]["tile_size"]}


def select_levels(data, levels):
    """The pairs of `data` at the given levels."""
    idx = np.nonzero(np.isin(data["level"], list(levels)))[0]
    sel = torch.from_numpy(idx).cuda()
    return {"up": data["up"].index_select(0, sel), "res": data["res"].index_select(0, sel),
            "level": data["level"][idx], "tile": data["tile"][idx], "tile_size": data["tile_size"]}


def level_sigmas(data, nlevels=24, extrapolate=0.5):
    """Per-level input sigma (RMS of the mean-removed upsampled tile) and output sigma
    (RMS of the residual); levels without data continue the last level by the
    factor `extrapolate` per level (fBm of gain 1/2)."""
    si = np.zeros(nlevels, np.float32)
    so = np.zeros(nlevels, np.float32)
    lv = data["level"]
    for l in np.unique(lv):
        idx = torch.from_numpy(np.nonzero(lv == l)[0]).cuda()
        u = data["up"].index_select(0, idx)
        u = u - u.mean(dim=(1, 2), keepdim=True)
        si[l] = float(u.pow(2).mean().sqrt())
        so[l] = float(data["res"].index_select(0, idx).pow(2).mean().sqrt())
    known = [l for l in range(nlevels) if so[l] > 0]
    lo, hi = min(known), max(known)
    for l in range(nlevels):
        if l < lo:
            si[l], so[l] = si[lo], so[lo]
        elif l > hi:
            si[l] = si[hi] * extrapolate ** (l - hi)
            so[l] = so[hi] * extrapolate ** (l - hi)
    return np.maximum(si, 1e-6), np.maximum(so, 1e-6)


# ---------------------------------------------------------------- the net
class LearnedPredictor:
    """tp_learned: 5 x (3x3 conv, 32 features), GELU, BF16 weights and activations,
    FP32 accumulation on the tensor cores."""

    def __init__(self, tile_width=101, max_batch=256, seed=1):
        h = C.c_void_p()
        check(lib().tp_learned_create(tile_width, max_batch, C.byref(h)))
        self.handle = h
        self.W = tile_width
        self.max_batch = max_batch
        if seed != 1:
            check(lib().tp_learned_init(h, seed))

    def close(self):
        if self.handle:
            lib().tp_learned_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def param_count(self):
        return lib().tp_learned_param_count(self.handle)

    def get_params(self):
        out = np.empty(self.param_count, np.float32)
        check(lib().tp_learned_get_params(self.handle, out.ctypes.data_as(_f32p), out.size))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        check(lib().tp_learned_set_params(self.handle, p.ctypes.data_as(_f32p), p.size))

    def set_fused(self, on=True):
        """Inference by fused layer pairs, or one launch per layer (the default; same bits)."""
        check(lib().tp_learned_set_fused(self.handle, int(bool(on))))

    CHECKPOINT_FORMAT = "proland_gb300.learned/1"

    def save(self, path, **extra):
        """Writes the whole training state -- parameters, Adam's moments and step count,
        the per-level sigmas -- and any `extra` arrays to the .npz file `path`
        (through a temporary file, so that a crash leaves the previous checkpoint)."""
        n = self.param_count
        m, v, step = np.empty(n, np.float32), np.empty(n, np.float32), C.c_int()
        check(lib().tp_learned_get_state(self.handle, m.ctypes.data_as(_f32p), v.ctypes.data_as(_f32p), n,
                                         C.byref(step)))
        si, so = np.empty(24, np.float32), np.empty(24, np.float32)
        check(lib().tp_learned_get_sigmas(self.handle, si.ctypes.data_as(_f32p), so.ctypes.data_as(_f32p), 24))
        tmp = path + ".tmp.npz"
        np.savez(tmp, format=np.array(self.CHECKPOINT_FORMAT), params=self.get_params(), adam_m=m, adam_v=v,
                 adam_step=np.array(step.value), sigma_in=si, sigma_out=so, **extra)
        os.replace(tmp, path)

    def load_state(self, path):
        """Restores a state written by `save`; returns its extra entries."""
        with np.load(path, allow_pickle=False) as f:
            d = {k: f[k] for k in f.files}
        if str(d.get("format")) != self.CHECKPOINT_FORMAT:
            raise ValueError("%s: not a learned-predictor checkpoint" % path)
        if d["params"].size != self.param_count:
            raise ValueError("%s: %d parameters, the net has %d" % (path, d["params"].size, self.param_count))
        self.set_params(d["params"])
        m, v = np.ascontiguousarray(d["adam_m"], np.float32), np.ascontiguousarray(d["adam_v"], np.float32)
        check(lib().tp_learned_set_state(self.handle, m.ctypes.data_as(_f32p), v.ctypes.data_as(_f32p), m.size,
                                         int(d["adam_step"])))
        self.set_sigmas(d["sigma_in"], d["sigma_out"])
        return {k: d[k] for k in d if k not in ("format", "params", "adam_m", "adam_v", "adam_step", "sigma_in",
                                                "sigma_out")}

    def get_grads(self):
        out = np.empty(self.param_count, np.float32)
        check(lib().tp_learned_get_grads(self.handle, out.ctypes.data_as(_f32p), out.size))
        return out

    def set_sigmas(self, sigma_in, sigma_out):
        si = np.ascontiguousarray(sigma_in, np.float32)
        so = np.ascontiguousarray(sigma_out, np.float32)
        check(lib().tp_learned_set_sigmas(self.handle, si.ctypes.data_as(_f32p), so.ctypes.data_as(_f32p), si.size))

    def forward(self, up, levels, training=False, out=None):
        """Residuals (metres) predicted for the upsampled tiles `up` [n, W, W].  An
        inference pass is enqueued on the current stream (a kernel failure in it is
        raised by the next synchronising call, e.g. check())."""
        n = up.shape[0]
        lv = (C.c_int * n)(*[int(v) for v in levels])
        if out is None:
            out = torch.empty_like(up)
        check(lib().tp_learned_forward(self.handle, _ptr(up), lv, n, int(training), _ptr(out), _stream()))
        return out

    def check(self):
        """Waits for the current stream and raises a kernel failure of earlier passes."""
        check(lib().tp_learned_check(self.handle, _stream()))

    def backward(self, target):
        loss = C.c_float()
        check(lib().tp_learned_backward(self.handle, _ptr(target), C.byref(loss), _stream()))
        return loss.value

    def adam(self, lr):
        check(lib().tp_learned_adam(self.handle, lr, _stream()))

    def gather(self, up_src, res_src, src, dihedral, up_out, res_out):
        n = len(src)
        s = (C.c_int * n)(*[int(v) for v in src])
        d = (C.c_int * n)(*[int(v) for v in dihedral])
        check(lib().tp_learned_gather(self.handle, _ptr(up_src), _ptr(res_src), up_src.shape[0], s, d, n, _ptr(up_out),
                                      _ptr(res_out),
                                      _stream()))

    def predict_residuals(self, elev, jobs, residuals, stream=None):
        """jobs: a list of TileJob, or a ctypes TileJob array built once by the caller."""
        arr = jobs if isinstance(jobs, C.Array) else (TileJob * len(jobs))(*jobs)
        check(lib().tp_learned_predict_residuals(self.handle, elev.handle, arr, len(jobs), residuals.handle, stream))


def train(net, data, steps, batch=256, lr=3e-4, seed=0, log_every=0, lr_final=None, balance_levels=True,
          checkpoint=None, checkpoint_every=0, resume_from=None):
    """Adam on random (tile, symmetry) pairs of `data`; returns the loss history.
    With lr_final the rate decays geometrically to it over the run; with
    balance_levels each sample first draws a level uniformly (a pyramid holds 4x
    more tiles per level), then a tile of that level.  Every `checkpoint_every`
    steps the training state (net.save, plus the step, the sampler's random state
    and the losses so far) goes to `checkpoint` (a path, formatted with step=...);
    `resume_from` continues a run from such a file with the same batches and rates."""
    rng = np.random.default_rng(seed)
    N = data["up"].shape[0]
    W = net.W
    by_level = [np.nonzero(data["level"] == l)[0] for l in np.unique(data["level"])]
    up_b = torch.empty((batch, W, W), dtype=torch.float32, device="cuda")
    res_b = torch.empty_like(up_b)
    losses, start = [], 0
    if resume_from is not None:
        extra = net.load_state(resume_from)
        start = int(extra["train_step"])
        rng.bit_generator.state = json.loads(str(extra["rng_state"]))
        losses = [float(x) for x in extra["losses"]]
    for s in range(start, steps):
        if balance_levels:
            pick = rng.integers(0, len(by_level), batch)
            src = np.array([by_level[k][rng.integers(0, len(by_level[k]))] for k in pick])
        else:
            src = rng.integers(0, N, batch)
        dih = rng.integers(0, 8, batch)
        net.gather(data["up"], data["res"], src, dih, up_b, res_b)
        net.forward(up_b, data["level"][src], training=True)
        losses.append(net.backward(res_b))
        rate = lr if lr_final is None else lr * (lr_final / lr) ** (s / max(1, steps - 1))
        net.adam(rate)
        if log_every and (s + 1) % log_every == 0:
            print("step %d loss %.4f" % (s + 1, float(np.mean(losses[-log_every:]))))
        if checkpoint and checkpoint_every and (s + 1) % checkpoint_every == 0:
            net.save(checkpoint.format(step=s + 1), train_step=np.array(s + 1),
                     rng_state=np.array(json.dumps(rng.bit_generator.state)), losses=np.array(losses))
    return losses


def evaluate(net, data, sigma_out, batch=None):
    """Per level: RMS and max height error of the learned residuals, of the plain
    method without residual (error = the residual itself), and the RMS of the
    normal-angle error of both (finite differences over the interior).  `sigma` is
    the RMS of the residuals evaluated (the plain method's RMS error), and
    `rms_over_sigma` the learned error in that unit."""
    lv = data["level"]
    batch = min(batch or net.max_batch, net.max_batch)
    out = {}
    for l in np.unique(lv):
        idx = np.nonzero(lv == l)[0]
        se_l = se_p = 0.0
        mx_l = mx_p = 0.0
        ang_l = ang_p = 0.0
        count = 0
        h = 2.0 * (50000.0 / (1 << int(l))) / (net.W - 5)
        for k in range(0, len(idx), batch):
            sel = torch.from_numpy(idx[k:k + batch]).cuda()
            up = data["up"].index_select(0, sel)
            res = data["res"].index_select(0, sel)
            pred = net.forward(up, lv[idx[k:k + batch]])
            e_l = pred - res
            se_l += float(e_l.pow(2).sum())
            se_p += float(res.pow(2).sum())
            mx_l = max(mx_l, float(e_l.abs().max()))
            mx_p = max(mx_p, float(res.abs().max()))
            ang_l += float(_angle_sq(up + pred, up + res, h).sum())
            ang_p += float(_angle_sq(up, up + res, h).sum())
            count += res.numel()
        ni = count * ((net.W - 2) / net.W) ** 2
        out[int(l)] = {"rms_learned": (se_l / count) ** 0.5, "rms_plain": (se_p / count) ** 0.5,
                       "max_learned": mx_l, "max_plain": mx_p, "sigma": (se_p / count) ** 0.5,
                       "rms_over_sigma": (se_l / max(se_p, 1e-30)) ** 0.5, "tiles": int(len(idx)),
                       "angle_rms_learned": (ang_l / ni) ** 0.5, "angle_rms_plain": (ang_p / ni) ** 0.5}
    return out


def _angle_sq(za, zb, h):
    """Squared angle between central-difference normals of za and zb (interior samples)."""
    def nrm(z):
        dx = z[:, 1:-1, 2:] - z[:, 1:-1, :-2]
        dy = z[:, 2:, 1:-1] - z[:, :-2, 1:-1]
        v = torch.stack([-dx, -dy, torch.full_like(dx, h)], 0)
        return v / v.norm(dim=0, keepdim=True)
    c = (nrm(za) * nrm(zb)).sum(0).clamp(-1.0, 1.0)
    return torch.acos(c) ** 2
