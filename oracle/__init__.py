"""CPU oracle for the terrain tile-production path -- TEST INFRASTRUCTURE ONLY.

ctypes bindings over oracle/_build/liboracle.so (the C restatement in
oracle.c) plus a pure-Python reader of the reference's ``.dat`` residual
pyramids.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline
leg use this package, always as the reference results; the product does not import it.
"""
import ctypes as C
import os
import struct
import zlib

import numpy as np

from . import build as _build

_LIB = None
_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)


class ElevTile(C.Structure):
    _fields_ = [
        ("W", C.c_int), ("level", C.c_int), ("tx", C.c_int), ("ty", C.c_int),
        ("parent_zf", _f32p), ("parent_zm", _f32p), ("parent_pitch", C.c_int),
        ("residual", _f32p), ("res_pitch", C.c_int), ("rx", C.c_int), ("ry", C.c_int),
        ("rscale", C.c_float),
        ("noise", _f32p), ("noise_rot", C.c_int), ("noise_amp", C.c_float),
        ("noise_mode", C.c_int), ("meters_per_sample", C.c_float),
        ("grid_g", C.c_int), ("flip", C.c_int), ("no_clamp", C.c_int),
        ("out_zf", _f32p), ("out_zc", _f32p), ("out_zm", _f32p), ("out_pitch", C.c_int),
    ]


class SphereFrame(C.Structure):
    _fields_ = [("C", C.c_float * 16), ("N", C.c_float * 16), ("L", C.c_float * 4),
                ("W2T", C.c_float * 9), ("R", C.c_float), ("size", C.c_float)]


class Job(C.Structure):
    _fields_ = [
        ("W", C.c_int), ("level", C.c_int), ("tx", C.c_int), ("ty", C.c_int),
        ("parent_zf", _f32p), ("parent_zm", _f32p), ("parent_pitch", C.c_int),
        ("residual", _f32p), ("res_pitch", C.c_int), ("rx", C.c_int), ("ry", C.c_int),
        ("rscale", C.c_float),
        ("noise", _f32p), ("noise_rot", C.c_int), ("noise_amp", C.c_float),
        ("tile_meters", C.c_float),
        ("out_zf", _f32p), ("out_zc", _f32p), ("out_zm", _f32p), ("out_pitch", C.c_int),
        ("out_nx", _f32p), ("out_ny", _f32p), ("nrm_pitch", C.c_int),
    ]


class OrthoJob(C.Structure):
    _fields_ = [
        ("W", C.c_int), ("level", C.c_int), ("tx", C.c_int), ("ty", C.c_int),
        ("parent", C.c_void_p), ("residual", C.c_void_p), ("noise", C.c_void_p),
        ("noise_rot", C.c_int), ("noise_amp", C.c_float),
        ("root_color", C.c_float * 4), ("noise_color", C.c_float * 4),
        ("scale", C.c_float), ("hsv", C.c_int), ("out", C.c_void_p),
    ]


class LayerMesh(C.Structure):
    _fields_ = [("first_vertex", C.c_int), ("count", C.c_int), ("first_index", C.c_int), ("mode", C.c_int),
                ("clear_depth", C.c_int), ("program", C.c_int), ("state", C.c_int), ("fill_depth", C.c_float)]


def lib():
    global _LIB
    if _LIB is None:
        path = _build.LIB
        if not os.path.exists(path):
            path = _build.build()
        L = C.CDLL(path)
        L.or_lrandom.argtypes = [C.POINTER(C.c_long)]
        L.or_lrandom.restype = C.c_long
        L.or_frandom.argtypes = [C.POINTER(C.c_long)]
        L.or_frandom.restype = C.c_float
        L.or_half_round.argtypes = [C.c_float]
        L.or_half_round.restype = C.c_float
        L.or_dem_noise.argtypes = [C.c_int, _f32p]
        L.or_cnoise2.argtypes = [C.c_float, C.c_float]
        L.or_cnoise2.restype = C.c_float
        L.or_noise_select.argtypes = [C.c_int] * 4 + [C.POINTER(C.c_int)] * 2
        L.or_ortho_noise.argtypes = [C.c_int, C.c_void_p]
        L.or_ortho_tile.argtypes = [C.POINTER(OrthoJob)]
        L.or_ortho_tile_id.argtypes = [C.c_int, C.c_int, C.c_int]
        L.or_ortho_tile_id.restype = C.c_int
        L.or_layer_tile.argtypes = [C.c_int, _f32p, _f32p, C.POINTER(LayerMesh), C.c_int, _f32p,
                                    C.POINTER(C.c_uint32), C.c_int, _f32p]
        L.or_layer_fragment.argtypes = [C.c_int, C.c_float, C.c_float, C.c_float, _f32p]
        L.or_layer_blend.argtypes = [C.c_int, _f32p, _f32p, _f32p, C.c_int, _f32p]
        L.or_elevation_tile.argtypes = [C.POINTER(ElevTile)]
        L.or_elevation_tile_f64.argtypes = [C.POINTER(ElevTile), _f64p, _f64p, _f64p]
        L.or_cpu_elevation_tile.argtypes = [C.c_int] * 4 + [_f32p, C.c_int, _f32p, C.c_int,
                                                            C.c_int, C.c_int, _f32p, C.c_int]
        L.or_normals_flat.argtypes = [C.c_int, _f32p, C.c_int, C.c_float, C.c_int, _f32p, _f32p, C.c_int]
        L.or_normals_flat_gl_linear.argtypes = [C.c_int, _f32p, C.c_int, C.c_float, _f32p, _f32p, C.c_int]
        L.or_normals_flat_f64.argtypes = [C.c_int, _f64p, C.c_int, C.c_double, _f64p, _f64p, C.c_int]
        L.or_sphere_frame_make.argtypes = [C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(SphereFrame)]
        L.or_normals_sphere.argtypes = [C.c_int, _f32p, C.c_int, C.POINTER(SphereFrame), _f32p, _f32p, C.c_int]
        L.or_run_jobs.argtypes = [C.POINTER(Job), C.c_int, C.c_int]
        L.or_residual_upsample.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _f32p, _f32p]
        L.or_compute_residual.argtypes = [C.c_int, C.c_int, C.c_int, _f32p, _f32p, _f32p,
                                          C.POINTER(C.c_int16), _f32p]
        L.or_normals_sphere_f64.argtypes = [C.c_int, _f64p, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int,
                                            _f64p, _f64p, C.c_int]
        L.or_parent_to_tangent.argtypes = [C.c_double, C.c_int, C.c_int, C.c_int, _f32p]
        L.or_normals_full.argtypes = [C.c_int, _f32p, C.c_int, C.c_float, C.POINTER(SphereFrame), _f32p, C.c_int,
                                      C.c_int, C.c_int, C.c_int, _f32p, _f32p, C.c_int, _f32p, _f32p, _f32p, _f32p,
                                      C.c_int]
        _i16p = C.POINTER(C.c_int16)
        L.or_fbm_heights.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_uint32, _i16p]
        L.or_fbm_pair.argtypes = [C.c_int, C.c_int, C.c_float, C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_int,
                                  _f32p, _f32p, _f32p]
        L.or_synthetic_residual.argtypes = [C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, _f32p]
        L.or_level_tile.argtypes = [_i16p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, _f32p]
        L.or_learned_param_count.restype = C.c_int
        L.or_learned_loss_grad.argtypes = [C.c_int, C.c_int, _f32p, _f32p, _f32p, C.POINTER(C.c_int), _f32p, _f32p,
                                           C.c_int, _f32p, _f64p]
        L.or_learned_loss_grad.restype = C.c_double
        _LIB = L
    return _LIB


def _p(a, t=_f32p):
    return None if a is None else a.ctypes.data_as(t)


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


# ---------------------------------------------------------------- noise
def lrandom_seq(seed, n):
    s = C.c_long(seed)
    return [lib().or_lrandom(C.byref(s)) for _ in range(n)]


def half_round(x):
    return lib().or_half_round(float(x))


def dem_noise(W):
    out = np.empty((6, W, W), np.float32)
    lib().or_dem_noise(W, _p(out))
    return out


def cnoise(x, y):
    return lib().or_cnoise2(float(x), float(y))


def noise_select(face, level, tx, ty):
    r, l = C.c_int(), C.c_int()
    lib().or_noise_select(face, level, tx, ty, C.byref(r), C.byref(l))
    return r.value, l.value


# ---------------------------------------------------------------- ortho
def ortho_noise(W):
    """createOrthoNoise: [6, W, W, 4] uint8."""
    out = np.empty((6, W, W, 4), np.uint8)
    lib().or_ortho_noise(W, out.ctypes.data)
    return out


def ortho_tile(W, level, tx, ty, parent, residual, noise_layer, noise_rot, noise_amp, root_color=(0.5,) * 4,
               noise_color=(1.0,) * 4, scale=2.0, hsv=False):
    """One ortho tile ([W, W, 4] uint8) as OrthoProducer::doCreateTile + the
    upsample shader make it; parent None at level 0, residual None without one."""
    out = np.empty((W, W, 4), np.uint8)
    keep = []

    def ptr(a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, np.uint8)
        keep.append(a)
        return a.ctypes.data
    j = OrthoJob()
    j.W, j.level, j.tx, j.ty = W, level, tx, ty
    j.parent = ptr(parent) if level > 0 else None
    j.residual = ptr(residual)
    j.noise = ptr(noise_layer)
    j.noise_rot, j.noise_amp = noise_rot, noise_amp
    j.root_color[:] = [float(v) for v in root_color]
    j.noise_color[:] = [float(v) for v in noise_color]
    j.scale, j.hsv = scale, int(bool(hsv))
    j.out = out.ctypes.data
    lib().or_ortho_tile(C.byref(j))
    return out


def layer_tile(W, zf, zm, meshes, blend_mode=0):
    """zm of one elevation tile after its layers (or_layer_tile): meshes is a list of
    (vertices [n, 4] (x, y, a, u) in clip coordinates, indices or None, mode
    (0 triangles, 1 strip), clear_depth[, program, state, fill_depth])."""
    verts, idx, ms = [], [], []
    nv = ni = 0
    for mesh in meshes:
        v, ix, mode, clear = mesh[:4]
        program, state, fill_depth = tuple(mesh[4:]) if len(mesh) > 4 else (0, 0, 0.0)
        v = np.ascontiguousarray(v, np.float32).reshape(-1, 4)
        m = LayerMesh(nv, v.shape[0], -1, mode, int(clear), int(program), int(state), float(fill_depth))
        if ix is not None:
            ix = np.ascontiguousarray(ix, np.uint32)
            m.first_index, m.count = ni, ix.size
            idx.append(ix)
            ni += ix.size
        verts.append(v)
        nv += v.shape[0]
        ms.append(m)
    va = np.concatenate(verts) if verts else np.zeros((1, 4), np.float32)
    ia = np.concatenate(idx) if idx else np.zeros(1, np.uint32)
    arr = (LayerMesh * max(1, len(ms)))(*ms)
    out = np.empty((W, W), np.float32)
    lib().or_layer_tile(W, _p(_f32(zf)), _p(_f32(zm)), arr, len(ms), _p(va), _p(ia, C.POINTER(C.c_uint32)),
                        blend_mode, _p(out))
    return out


def layer_fragment(program, a, u, fill_depth=0.0):
    """(depth clamped to [0, 1], z, w) of one fragment of a layer program."""
    out = np.empty(3, np.float32)
    lib().or_layer_fragment(int(program), float(fill_depth), float(a), float(u), _p(out))
    return tuple(float(v) for v in out)


def layer_blend(W, zf, z, w, blend_mode=0):
    """The blend pass alone: zm from zf and the layers' z and w planes."""
    out = np.empty((W, W), np.float32)
    lib().or_layer_blend(W, _p(_f32(zf)), _p(_f32(z)), _p(_f32(w)), blend_mode, _p(out))
    return out


class OrthoDatFile:
    """Reader of OrthoCPUProducer's .dat pyramid (OrthoCPUProducer.cpp:82-114,
    170-236): a 7-word int32 header {maxLevel, tileSize, channels, root, tx, ty,
    flags} (flags bit 0: DXT tiles, bit 1: no border), 2 * ntiles int64 [start,
    end) offsets relative to the end of the header, ntiles = (4^(maxLevel+1) - 1) / 3,
    then one single-strip deflate TIFF of (tileSize + 2 border)^2 x channels bytes
    per tile.  Pure Python (struct + zlib)."""

    def __init__(self, data: bytes):
        self.data = data
        (self.max_level, self.tile_size, self.channels, self.root, self.root_tx, self.root_ty,
         self.flags) = struct.unpack_from("<7i", data, 0)
        self.dxt = (self.flags & 1) != 0
        self.border = 0 if (self.flags & 2) else 2
        self.ntiles = ((1 << (self.max_level * 2 + 2)) - 1) // 3
        self.header = 7 * 4 + 2 * self.ntiles * 8
        self.offsets = np.frombuffer(data, "<i8", self.ntiles * 2, 28)

    @classmethod
    def open(cls, path):
        with open(path, "rb") as f:
            return cls(f.read())

    def tile_id(self, level, tx, ty):
        return lib().or_ortho_tile_id(level, tx, ty)

    def strip(self, level, tx, ty):
        tid = self.tile_id(level, tx, ty)
        a, b = int(self.offsets[2 * tid]), int(self.offsets[2 * tid + 1])
        return self.data[self.header + a:self.header + b]

    def tile(self, level, tx, ty):
        """Decoded tile, shape (w, w, channels) uint8."""
        w = self.tile_size + 2 * self.border
        raw = decode_tiff_strip(self.strip(level, tx, ty))
        return np.frombuffer(raw[:w * w * self.channels], np.uint8).reshape(w, w, self.channels)


def rgba_words(tile):
    """An (w, w, c) uint8 residual tile as the RGBA texels a GL texture of fewer
    components returns: missing green / blue read 0, missing alpha 255."""
    w, _, c = tile.shape
    out = np.zeros((w, w, 4), np.uint8)
    out[..., 3] = 255
    out[..., :c] = tile
    return out


# ---------------------------------------------------------------- elevation
def _elev_struct(W, level, tx, ty, parent_zf, parent_zm, residual, rx, ry, rscale,
                 noise, noise_rot, noise_amp, noise_mode, meters_per_sample,
                 grid_g, flip, no_clamp, outs):
    t = ElevTile()
    t.W, t.level, t.tx, t.ty = W, level, tx, ty
    if level > 0:
        t.parent_zf, t.parent_zm = _p(parent_zf), _p(parent_zm)
        t.parent_pitch = parent_zf.shape[1]
    t.residual = _p(residual)
    t.res_pitch = 0 if residual is None else residual.shape[1]
    t.rx, t.ry, t.rscale = rx, ry, rscale
    t.noise = _p(noise)
    t.noise_rot, t.noise_amp, t.noise_mode = noise_rot, noise_amp, noise_mode
    t.meters_per_sample = meters_per_sample
    t.grid_g = grid_g if grid_g else (W - 5) // 24
    t.flip, t.no_clamp = int(flip), int(no_clamp)
    t.out_zf, t.out_zc, t.out_zm = [_p(o) for o in outs]
    t.out_pitch = W
    return t


def elevation_tile(W, level, tx, ty, parent_zf=None, parent_zm=None, residual=None,
                   rx=0, ry=0, rscale=1.0, noise=None, noise_rot=0, noise_amp=0.0,
                   noise_mode=0, meters_per_sample=1.0, grid_g=0, flip=False,
                   no_clamp=False, f64=False):
    """One elevation tile; returns (zf, zc, zm) W x W arrays (float32, or float64 if f64)."""
    parent_zf, parent_zm, residual, noise = map(_f32, (parent_zf, parent_zm, residual, noise))
    if level > 0 and parent_zm is None:
        parent_zm = np.maximum(parent_zf, 0).astype(np.float32)
    outs32 = [np.empty((W, W), np.float32) for _ in range(3)]
    t = _elev_struct(W, level, tx, ty, parent_zf, parent_zm, residual, rx, ry, rscale,
                     noise, noise_rot, noise_amp, noise_mode, meters_per_sample,
                     grid_g, flip, no_clamp, outs32)
    if f64:
        o = [np.empty((W, W), np.float64) for _ in range(3)]
        lib().or_elevation_tile_f64(C.byref(t), _p(o[0], _f64p), _p(o[1], _f64p), _p(o[2], _f64p))
        return tuple(o)
    lib().or_elevation_tile(C.byref(t))
    return tuple(outs32)


def cpu_elevation_tile(W, level, tx, ty, parent=None, residual=None, rx=0, ry=0):
    parent, residual = _f32(parent), _f32(residual)
    out = np.empty((W, W), np.float32)
    lib().or_cpu_elevation_tile(W, level, tx, ty, _p(parent), 0 if parent is None else parent.shape[1],
                                _p(residual), 0 if residual is None else residual.shape[1], rx, ry,
                                _p(out), W)
    return out


def normals_flat(W, zm, tile_meters, fmt=2):
    zm = _f32(zm)
    n1 = W - 4
    nx = np.empty((n1, n1), np.float32)
    ny = np.empty((n1, n1), np.float32)
    lib().or_normals_flat(W, _p(zm), zm.shape[1], float(tile_meters), fmt, _p(nx), _p(ny), n1)
    return nx, ny


def normals_flat_gl_linear(W, zm, tile_meters):
    """Normals as the GL path samples zm (LINEAR storage, +0.25-texel offsets): for
    reporting the difference to the texel-exact finite differences only."""
    zm = _f32(zm)
    n1 = W - 4
    nx = np.empty((n1, n1), np.float32)
    ny = np.empty((n1, n1), np.float32)
    lib().or_normals_flat_gl_linear(W, _p(zm), zm.shape[1], float(tile_meters), _p(nx), _p(ny), n1)
    return nx, ny


def normals_flat_f64(W, zm, tile_meters):
    zm = np.ascontiguousarray(zm, np.float64)
    n1 = W - 4
    nx = np.empty((n1, n1), np.float64)
    ny = np.empty((n1, n1), np.float64)
    lib().or_normals_flat_f64(W, _p(zm, _f64p), zm.shape[1], float(tile_meters),
                              _p(nx, _f64p), _p(ny, _f64p), n1)
    return nx, ny


def sphere_frame(root_quad_size, level, tx, ty):
    f = SphereFrame()
    lib().or_sphere_frame_make(float(root_quad_size), level, tx, ty, C.byref(f))
    return f


def normals_sphere(W, zm, frame):
    zm = _f32(zm)
    n1 = W - 4
    nx = np.empty((n1, n1), np.float32)
    ny = np.empty((n1, n1), np.float32)
    lib().or_normals_sphere(W, _p(zm), zm.shape[1], C.byref(frame), _p(nx), _p(ny), n1)
    return nx, ny


def normals_sphere_f64(W, zm, root_quad_size, level, tx, ty):
    zm = np.ascontiguousarray(zm, np.float64)
    n1 = W - 4
    nx = np.empty((n1, n1), np.float64)
    ny = np.empty((n1, n1), np.float64)
    lib().or_normals_sphere_f64(W, _p(zm, _f64p), zm.shape[1], float(root_quad_size), level, tx, ty,
                                _p(nx, _f64p), _p(ny, _f64p), n1)
    return nx, ny


def parent_to_tangent(root_quad_size, level, tx, ty):
    out = np.empty(9, np.float32)
    lib().or_parent_to_tangent(float(root_quad_size), level, tx, ty, _p(out))
    return out


def normals_full(W, zm, tile_meters, fmt, tx, ty, parent=None, root_quad_size=0.0, level=0, grid_mesh=24):
    """Normal tile planes of format `fmt` (4 planes for 0/1, 2 for 2/3); `parent`:
    the parent normal tile's first two planes (nx, ny) or None."""
    zm = _f32(zm)
    Wn = W - 4
    outs = [np.zeros((Wn, Wn), np.float32) for _ in range(4)]
    frame = sphere_frame(root_quad_size, level, tx, ty) if root_quad_size > 0 else None
    p2t = parent_to_tangent(root_quad_size, level, tx, ty) if (root_quad_size > 0 and level > 0) else None
    pnx = _f32(parent[0]) if parent is not None else None
    pny = _f32(parent[1]) if parent is not None else None
    lib().or_normals_full(W, _p(zm), zm.shape[1], float(tile_meters), C.byref(frame) if frame else None, _p(p2t),
                          fmt, grid_mesh, tx, ty, _p(pnx), _p(pny), Wn, *[_p(o) for o in outs], Wn)
    return outs[:4] if fmt in (0, 1) else outs[:2]


def compute_residual(W, tx, ty, parent_approx, fine):
    parent_approx, fine = _f32(parent_approx), _f32(fine)
    rq = np.empty((W, W), np.float32)
    enc = np.empty((W, W), np.int16)
    approx = np.empty((W, W), np.float32)
    lib().or_compute_residual(W, tx, ty, _p(parent_approx), _p(fine), _p(rq),
                              enc.ctypes.data_as(C.POINTER(C.c_int16)), _p(approx))
    return rq, enc, approx


_TUNED = None


def tuned_lib():
    """The oracle built at -O3 on this machine (the timed CPU baseline)."""
    global _TUNED
    if _TUNED is None:
        L = C.CDLL(_build.build_tuned())
        L.or_run_jobs.argtypes = [C.POINTER(Job), C.c_int, C.c_int]
        _TUNED = L
    return _TUNED


def run_jobs(jobs, nthreads, tuned=False):
    arr = (Job * len(jobs))(*jobs)
    (tuned_lib() if tuned else lib()).or_run_jobs(arr, len(jobs), int(nthreads))


# ---------------------------------------------------------------- .dat pyramid
class DatFile:
    """Reader of ResidualProducer's .dat pyramid (ResidualProducer.cpp:93-107,
    253-340): a 7-word header {minLevel, maxLevel, tileSize, rootLevel, rootTx,
    rootTy: int32, scale: float32}, then 2 * ntiles uint32 [start, end) offsets
    relative to the end of the header, then one single-strip deflate TIFF per tile.
    Pure Python (struct + zlib), independent of the product's C++ reader."""

    def __init__(self, data: bytes):
        self.data = data
        (self.min_level, self.max_level, self.tile_size, self.root_level,
         self.root_tx, self.root_ty) = struct.unpack_from("<6i", data, 0)
        (self.scale,) = struct.unpack_from("<f", data, 24)
        l = max(self.max_level - self.min_level, 0)
        self.ntiles = self.min_level + ((1 << (l * 2 + 2)) - 1) // 3
        self.header = 4 + 4 * (6 + self.ntiles * 2)
        self.offsets = np.frombuffer(data, "<u4", self.ntiles * 2, 28)

    @classmethod
    def open(cls, path):
        with open(path, "rb") as f:
            return cls(f.read())

    def tile_width(self, level):
        ts = self.tile_size >> (self.min_level - level) if level < self.min_level else self.tile_size
        return ts + 5

    def tile_id(self, level, tx, ty):
        if level < self.min_level:
            return level
        l = level - self.min_level
        return self.min_level + tx + ty * (1 << l) + ((1 << (2 * l)) - 1) // 3

    def strip(self, level, tx, ty):
        tid = self.tile_id(level, tx, ty)
        a, b = int(self.offsets[2 * tid]), int(self.offsets[2 * tid + 1])
        return self.data[self.header + a:self.header + b]

    def tile_int16(self, level, tx, ty):
        """Decoded int16 samples of one tile, shape (w, w)."""
        w = self.tile_width(level)
        raw = decode_tiff_strip(self.strip(level, tx, ty))
        return np.frombuffer(raw[:2 * w * w], "<i2").reshape(w, w)


def decode_tiff_strip(blob: bytes) -> bytes:
    """Decodes strip 0 of a little- or big-endian TIFF with deflate (8 or 32946)
    or no compression; returns the raw strip bytes."""
    bo = "<" if blob[:2] == b"II" else ">"
    (ifd,) = struct.unpack_from(bo + "I", blob, 4)
    (count,) = struct.unpack_from(bo + "H", blob, ifd)
    tags = {}
    sizes = {1: 1, 2: 1, 3: 2, 4: 4, 5: 8}
    for k in range(count):
        tag, typ, n, val = struct.unpack_from(bo + "HHI4s", blob, ifd + 2 + 12 * k)
        fmt = {3: "H", 4: "I"}.get(typ)
        if fmt is None:
            continue
        if sizes[typ] * n <= 4:
            vals = struct.unpack_from(bo + fmt * n, val, 0)
        else:
            (off,) = struct.unpack_from(bo + "I", val, 0)
            vals = struct.unpack_from(bo + fmt * n, blob, off)
        tags[tag] = vals
    comp = tags.get(259, (1,))[0]
    off = tags[273][0]
    cnt = tags[279][0]
    data = blob[off:off + cnt]
    if comp in (8, 32946):
        return zlib.decompress(data)
    if comp == 1:
        return data
    raise ValueError("unsupported TIFF compression %d" % comp)


def residual_chain_root(dat, delta, zscale=1.0):
    """The root residual tile of a producer started `delta` levels below the
    pyramid's first level: readTile(0), then for i = 1..delta upsample and add
    readTile(i) (ResidualProducer.cpp:218-225, 268-384)."""
    W = dat.tile_size + 5
    scale = np.float32(np.float32(dat.scale) * np.float32(zscale))
    out = np.zeros((W, W), np.float32)
    t0 = dat.tile_int16(0, 0, 0)
    w = t0.shape[0]
    out[:w, :w] = (t0.astype(np.float32) * scale).astype(np.float32)
    tmp = np.zeros((W, W), np.float32)
    for i in range(1, delta + 1):
        ts = dat.tile_size >> (dat.min_level - i) if i < dat.min_level else dat.tile_size
        lib().or_residual_upsample(W, ts, 0, 0, _p(out), _p(tmp))
        ti = dat.tile_int16(i, 0, 0)
        w = ti.shape[0]
        out = tmp.copy()
        out[:w, :w] = (tmp[:w, :w] + (ti.astype(np.float32) * scale)).astype(np.float32)
    return out


# ---------------------------------------------------------------- preprocess and learned net
def fbm_pair(level, tx, ty, seed=1, tile_size=96, octaves=12, base_cells=4, amplitude=4000.0):
    """(up, res, fine) of one tile of the procedural fBm at any level (tp_fbm_pairs)."""
    W = tile_size + 5
    out = [np.empty((W, W), np.float32) for _ in range(3)]
    lib().or_fbm_pair(octaves, base_cells, amplitude, C.c_uint32(seed), tile_size, level, tx, ty, *[_p(o) for o in out])
    return tuple(out)


def synthetic_residual(seed, level, tx, ty, sigma, W):
    """The product's synthetic residual tile (tp_residual_producer_set_synthetic) for a
    tile of standard deviation `sigma` (a float32 value)."""
    out = np.empty((W, W), np.float32)
    lib().or_synthetic_residual(C.c_uint32(seed), level, tx, ty, C.c_float(sigma), W, _p(out))
    return out


def fbm_heights(size, octaves=12, base_cells=4, amplitude=4000.0, quantum=0.25, seed=1):
    """The device preprocess's procedural fBm height field as int16 (size x size)."""
    out = np.empty((size, size), np.int16)
    lib().or_fbm_heights(size, octaves, base_cells, amplitude, quantum, seed,
                         out.ctypes.data_as(C.POINTER(C.c_int16)))
    return out


def level_tile(base, ts, max_level, level, tx, ty, scale=1.0):
    """HeightMipmap::getTile of a decimated level of `base` (int16, ts * 2^max_level + 1 square)."""
    base = np.ascontiguousarray(base, np.int16)
    out = np.empty((ts + 5, ts + 5), np.float32)
    lib().or_level_tile(base.ctypes.data_as(C.POINTER(C.c_int16)), ts, max_level, level, tx, ty, scale, _p(out))
    return out


def learned_param_count():
    return lib().or_learned_param_count()


def learned_loss_grad(params, up, target, levels, sigma_in, sigma_out, emulate=True, want_grad=True):
    """Loss (mean squared error in sigma units), normalised predictions [n, W, W] and
    the gradient (float64, flat like the parameters) of the learned net."""
    params, up, target = _f32(params), _f32(up), _f32(target)
    n, W = up.shape[0], up.shape[1]
    lv = np.ascontiguousarray(levels, np.int32)
    si, so = _f32(sigma_in), _f32(sigma_out)
    pred = np.empty((n, W, W), np.float32)
    grad = np.empty(learned_param_count(), np.float64) if want_grad else None
    loss = lib().or_learned_loss_grad(W, n, _p(params), _p(up), _p(target), lv.ctypes.data_as(C.POINTER(C.c_int)),
                                      _p(si), _p(so), int(emulate), _p(pred), _p(grad, _f64p))
    return loss, pred, grad


def quadtree_requests(cam, root, max_level, split, dist_factor=1.0, ground=0.0):
    """TerrainQuad::update's split rule (TerrainQuad.cpp:80-138) with
    TerrainNode::getCameraDist (TerrainNode.cpp:92-97): the quads of the tree,
    parents first, children near to far; every quad visible."""
    cx, cy, cz = (float(v) for v in cam)
    zmin, zmax = min(0.0, ground), max(0.0, ground)
    order = {(0, 0): (0, 1, 2, 3), (0, 1): (1, 0, 3, 2), (1, 0): (2, 0, 3, 1), (1, 1): (3, 1, 2, 0)}
    out = []

    def visit(level, tx, ty, ox, oy, l):
        out.append((level, tx, ty))
        d = max(abs(cz - zmax) / dist_factor, max(min(abs(cx - ox), abs(cx - (ox + l))),
                                                   min(abs(cy - oy), abs(cy - (oy + l)))))
        dist = float(np.float32(d))
        if not (dist < l * float(np.float32(split)) and level < max_level):
            return
        for c in order[(0 if cy < oy + l / 2.0 else 1, 0 if cx < ox + l / 2.0 else 1)]:
            i, j = c & 1, c >> 1
            visit(level + 1, 2 * tx + i, 2 * ty + j, ox + i * l / 2.0, oy + j * l / 2.0, l / 2.0)

    visit(0, 0, 0, -root / 2.0, -root / 2.0, root)
    return out


# ---------------------------------------------------------------- the reference's own code
_REF = None


def ref_file(rel):
    """A file of the reference tree (path relative to its root) where the tree is on
    this machine, else None: the reference's own data for the pin tests."""
    from . import ref_build
    path = os.path.join(ref_build.DEFAULT_ROOT, rel)
    return path if os.path.exists(path) else None


def ref_lib():
    """oracle/_ref/libref.so: pieces of the reference's C++ compiled from its sources by
    oracle/ref_build.py (noise.cpp, createDemNoise, the noise-layer choice, the CPU
    elevation loop, HeightMipmap's residual functions, and the GPU producers'
    doCreateTile functions running their shaders as C++), or None where the reference
    tree is absent.  Used only to check the oracle's restatement."""
    global _REF
    if _REF is None:
        from . import ref_build
        path = ref_build.build()
        if path is None or not os.path.exists(path):
            return None
        L = C.CDLL(path)
        L.ref_lrandom.argtypes = [C.POINTER(C.c_long)]
        L.ref_lrandom.restype = C.c_long
        L.ref_frandom.argtypes = [C.POINTER(C.c_long)]
        L.ref_frandom.restype = C.c_float
        L.ref_cnoise2.argtypes = [C.c_float, C.c_float]
        L.ref_cnoise2.restype = C.c_float
        L.ref_dem_noise.argtypes = [C.c_int, _f32p]
        L.ref_noise_select.argtypes = [C.c_int] * 4 + [C.POINTER(C.c_int)] * 2
        L.ref_cpu_elevation_tile.argtypes = [C.c_int] * 4 + [_f32p, C.c_int, _f32p, _f32p, C.POINTER(C.c_int)]
        L.ref_compute_residual.argtypes = [C.c_int, C.c_int, _f32p, _f32p, C.c_int, C.c_int, C.c_int, _f32p,
                                           _f32p, _f32p]
        L.ref_encode_residual.argtypes = [C.c_int, C.c_int, C.c_int, _f32p, C.c_void_p]
        L.ref_compute_approx_tile.argtypes = [C.c_int, C.c_int, _f32p, _f32p, C.c_int, C.c_int, C.c_int, _f32p,
                                              _f32p]
        L.ref_mipmap_build.argtypes = [C.POINTER(C.c_int16), C.c_int, C.c_int, C.c_float, C.c_char_p]
        L.ref_mipmap_level_tile.argtypes = [C.c_int] * 3 + [_f32p]
        L.ref_mipmap_approx_tile.argtypes = [C.c_int] * 3 + [_f32p]
        L.ref_mipmap_residual.argtypes = [C.c_int] * 3 + [C.c_void_p, C.c_int]
        L.ref_mipmap_build_sized.argtypes = [C.POINTER(C.c_int16), C.c_int, C.c_int, C.c_int, C.c_float, C.c_char_p]
        L.ref_mipmap_generate.argtypes = [C.c_int] * 3 + [C.c_float, C.c_char_p]
        L.ref_gl_elevation_tile.argtypes = [C.c_int] * 6 + [_f32p, _f32p, C.c_int, _f32p, _f32p, C.c_int,
                                                            C.c_float, C.c_int, C.c_int, _f32p]
        L.ref_gl_normal_tile.argtypes = [C.c_int] * 5 + [_f32p, C.c_int, _f32p, C.c_float, C.c_int, C.c_int, _f32p]
        L.ref_gl_elevation_tile_layers.argtypes = [C.c_int] * 7 + [_f32p, _f32p, C.c_int, _f32p, _f32p, C.c_int,
                                                                   C.c_float, C.c_int, C.c_int, _f32p, _f32p, _f32p]
        L.ref_gl_layer_fragment.argtypes = [C.c_int, C.c_int, C.c_float, _f32p, C.c_float, C.c_float, _f32p,
                                            C.POINTER(C.c_float)]
        L.ref_ortho_noise.argtypes = [C.c_int, C.c_void_p]
        L.ref_gl_ortho_tile_channels.argtypes = [C.c_int] * 6 + [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, _f32p,
                                                                 C.c_int, _f32p, _f32p, C.c_int, C.c_float, _f32p]
        L.ref_sphere_uniforms.argtypes = [C.c_int] * 4 + [C.c_float, _f32p]
        L.ref_residual_tile.argtypes = [C.c_char_p, C.c_int, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_void_p, C.POINTER(C.c_int)]
        L.ref_ortho_dat_tile.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                         C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.ref_cache_create.argtypes = [C.c_int, C.c_int]
        L.ref_cache_get.argtypes = [C.c_int] * 4 + [C.POINTER(C.c_int)]
        L.ref_cache_put.argtypes = [C.c_int] * 4
        L.ref_cache_find.argtypes = [C.c_int] * 5
        L.ref_cache_prefetch.argtypes = [C.c_int] * 4
        L.ref_cache_counts.argtypes = [C.POINTER(C.c_int)] * 3
        L.ref_quadtree.argtypes = [C.c_double, C.c_int, C.c_float, C.c_float, C.c_double, C.c_double, C.c_double,
                                   C.c_float, C.c_void_p, C.c_int]
        L.ref_sampler_create.argtypes = [C.c_double, C.c_int, C.c_float, C.c_int]
        L.ref_sampler_frame.argtypes = [C.c_double] * 3 + [C.c_void_p]
        L.ref_sampler_users.argtypes = [C.c_int] * 3
        L.ref_water_layer.argtypes = [C.c_double] * 3 + [C.c_int] * 3 + [C.c_void_p, C.c_void_p, C.c_void_p,
                                                                         _f32p, C.c_int, C.c_void_p]
        L.ref_water_draw.argtypes = [C.c_int, C.POINTER(C.c_int), _f32p]
        L.ref_road_layer.argtypes = [C.c_double] * 3 + [C.c_int] * 3 + [C.c_void_p, C.c_void_p, C.c_void_p, _f32p]
        L.ref_water_contour.argtypes = [C.c_int, C.c_void_p]
        L.ref_deps_create.argtypes = [C.c_int] * 3
        L.ref_deps_get.argtypes = [C.c_int] * 4
        L.ref_deps_users.argtypes = [C.c_int] * 4
        L.ref_deps_counts.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.ref_road_meshes.argtypes = [C.c_double] * 3 + [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                                         C.c_float, C.c_int, C.c_int, C.POINTER(C.c_float)]
        L.ref_curve_altitude.argtypes = [C.c_double] * 3 + [C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_float,
                                                            C.c_float, C.c_int, C.c_int]
        L.ref_curve_part.argtypes = [C.c_double] * 3 + [C.c_void_p, C.c_int, C.c_float, _f32p]
        L.ref_drawn_mesh.argtypes = [C.c_int] + [C.POINTER(C.c_int)] * 3 + [C.c_void_p, C.c_void_p]
        L.ref_gl_ortho_tile.argtypes = [C.c_int] * 6 + [C.c_void_p] * 3 + [_f32p, C.c_int, _f32p, _f32p, C.c_int,
                                                                            C.c_float, _f32p]
        _REF = L
    return _REF
