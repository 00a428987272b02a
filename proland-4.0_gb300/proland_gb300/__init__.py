"""proland_gb300: Python view of the GB300 terrain tile producer.

Thin wrappers over the C ABI (include/proland_gb300.h) that mirror Proland's
TileStorage / TileCache / TileProducer classes; every computation runs in the
CUDA library, which must be built (there is no CPU fallback).
"""
import ctypes as C

import numpy as np

from ._lib import (ElevParams, HostTiles, LAYER_FN, LayerJob, LayerMesh, OrthoJob, OrthoParams, TileJob, TPError, check, lib, LIB_PATH, RESIDUAL_SOURCE,  # noqa: F401
                   TP_OK, TP_E_BAD_ARG, TP_E_CACHE_FULL, TP_E_MISSING_PARENT,
                   TP_E_TIMEOUT, TP_E_CUDA, TP_E_IO, TP_E_NO_DEVICE, TP_E_BOUNDS)

ZF, ZC, ZM = 0, 1, 2      # planes of an elevation slot (the reference's RGB32F texel)
NX, NY = 0, 1             # planes of a normal slot (format 2)


def device_available():
    return bool(lib().tp_device_available())


class TileStorage:
    """A pool of tile slots (GPUTileStorage / CPUTileStorage,
    core/.../producer/TileStorage.h:140-182)."""

    DEVICE, PINNED_HOST, BOOKKEEPING = 1, 0, 2

    def __init__(self, tile_size, channels, capacity, on_device=True):
        h = C.c_void_p()
        kind = on_device if isinstance(on_device, int) and not isinstance(on_device, bool) else int(bool(on_device))
        check(lib().tp_storage_create(tile_size, channels, capacity, kind, C.byref(h)))
        self.handle = h
        self.tile_size = tile_size
        self.channels = channels
        self.capacity = capacity
        self.pitch = lib().tp_storage_pitch(h)

    def close(self):
        if self.handle:
            lib().tp_storage_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_tile_size(self):
        return lib().tp_storage_tile_size(self.handle)

    def get_capacity(self):
        return lib().tp_storage_capacity(self.handle)

    def get_free_slots(self):
        return lib().tp_storage_free_slots(self.handle)

    def new_slot(self):
        return lib().tp_storage_new_slot(self.handle)

    def delete_slot(self, slot):
        check(lib().tp_storage_delete_slot(self.handle, slot))

    def plane_ptr(self, slot, channel):
        return lib().tp_storage_plane(self.handle, slot, channel)

    def upload(self, first_slot, channel, host, stream=None):
        """host: float32 array [count, W, W] (pinned memory for asynchronous copies)."""
        a = np.ascontiguousarray(host, dtype=np.float32)
        W = self.tile_size
        a = a.reshape(-1, W, W)
        check(lib().tp_storage_upload(self.handle, first_slot, a.shape[0], channel,
                                      a.ctypes.data, stream))
        return a

    def download(self, first_slot, count, channel, out=None, stream=None):
        W = self.tile_size
        if out is None:
            out = np.empty((count, W, W), np.float32)
        check(lib().tp_storage_download(self.handle, first_slot, count, channel,
                                        out.ctypes.data, stream))
        return out


def make_params(grid_size=24, flip=False, no_clamp=False, noise_mode=0, normal_format=2, band_rows=0,
                stages=0):
    p = ElevParams()
    p.grid_size, p.flip, p.no_clamp = grid_size, int(flip), int(no_clamp)
    p.noise_mode, p.normal_format, p.band_rows, p.stages = noise_mode, normal_format, band_rows, stages
    return p


def stream_check(stream=None):
    """Synchronises `stream` and raises if a kernel reported a failure."""
    check(lib().tp_stream_check(stream))


def make_job(level, tx, ty, out_slot, parent_slot=-1, residual_slot=-1, rx=0, ry=0,
             normal_slot=-1, noise_rot=0, noise_layer=0, noise_amp=0.0, rscale=1.0,
             tile_meters=1000.0, parent_job=-1):
    j = TileJob()
    j.level, j.tx, j.ty = level, tx, ty
    j.out_slot, j.parent_slot, j.residual_slot = out_slot, parent_slot, residual_slot
    j.rx, j.ry, j.normal_slot = rx, ry, normal_slot
    j.noise_rot, j.noise_layer, j.noise_amp = noise_rot, noise_layer, noise_amp
    j.rscale, j.tile_meters, j.parent_job = rscale, tile_meters, parent_job
    return j


def elevation_batch(elev, residuals, normals, params, jobs, stream=None):
    """Produces the jobs (a list or ctypes array of TileJob) in one batch (tp_elevation_batch)."""
    arr = job_array(jobs)
    check(lib().tp_elevation_batch(elev.handle, residuals.handle if residuals else None,
                                   normals.handle if normals else None, C.byref(params),
                                   arr, len(jobs), stream))


def job_array(jobs):
    """A ctypes TileJob array of a job list (build once, pass to the batch calls)."""
    return jobs if isinstance(jobs, C.Array) else (TileJob * len(jobs))(*jobs)


def normal_batch(elev, normals, jobs, root_quad_size=0.0, stream=None):
    """Normal tiles of produced elevation tiles (tp_normal_batch); sphere normals
    when root_quad_size > 0.  jobs: a list of TileJob or a job_array."""
    arr = job_array(jobs)
    check(lib().tp_normal_batch(elev.handle, normals.handle, arr, len(jobs), float(root_quad_size), stream))


def normal_batch_format(elev, normals, jobs, fmt, parent_slots=None, root_quad_size=0.0, grid_mesh=24, stream=None):
    """Normal tiles in format 0-3 with coarse normals from parent normal slots
    (tp_normal_batch_format)."""
    arr = (TileJob * len(jobs))(*jobs)
    ps = (C.c_int * len(jobs))(*parent_slots) if parent_slots is not None else None
    check(lib().tp_normal_batch_format(elev.handle, normals.handle, arr, len(jobs), float(root_quad_size), fmt, ps,
                                       grid_mesh, stream))


def elevation_batch_device(elev, residuals, normals, params, jobs_dev_ptr, n, stream=None):
    check(lib().tp_elevation_batch_device(elev.handle, residuals.handle if residuals else None,
                                          normals.handle if normals else None, C.byref(params),
                                          jobs_dev_ptr, n, stream))


class HostPipeline:
    """Host-buffer batches (tp_pipeline_*, tp_elevation_batch_host): dense host
    tile arrays in, dense host tile arrays out, the copies of neighbouring chunks
    overlapping the elevation launches.  Arrays should be pinned (e.g. from
    torch.empty(..., pin_memory=True).numpy()) for the copies to overlap."""

    def __init__(self, tile_width, chunk=256, nbuf=3):
        h = C.c_void_p()
        check(lib().tp_pipeline_create(tile_width, chunk, nbuf, C.byref(h)))
        self.handle = h
        self.tile_width = tile_width

    def close(self):
        if self.handle:
            lib().tp_pipeline_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, params, jobs, parent_zf, parent_zm, residual, zf, zc, zm, nx=None, ny=None, stream=None):
        """Enqueues the batch; synchronise `stream` (or call stream_check) before
        reading the outputs, and keep every array alive until then (the copies read
        and write them asynchronously).  Arrays must be C-contiguous float32
        [n, W, W] ([n, W-4, W-4] for nx, ny); parent_zm and residual may be None."""
        n = len(jobs)
        W = self.tile_width
        io = HostTiles()

        def ptr(a, side):
            if a is None:
                return None
            if a.dtype != np.float32 or not a.flags["C_CONTIGUOUS"] or a.shape[0] < n or a.shape[1:] != (side, side):
                raise ValueError("host tiles must be contiguous float32 [n, %d, %d]" % (side, side))
            return a.ctypes.data
        io.parent_zf, io.parent_zm, io.residual = ptr(parent_zf, W), ptr(parent_zm, W), ptr(residual, W)
        io.zf, io.zc, io.zm = ptr(zf, W), ptr(zc, W), ptr(zm, W)
        io.nx, io.ny = ptr(nx, W - 4), ptr(ny, W - 4)
        self._arr = (TileJob * n)(*jobs)
        self._io = io
        check(lib().tp_elevation_batch_host(self.handle, C.byref(params), self._arr, n, C.byref(io), stream))


# ---------------------------------------------------------------- elevation layers
TRIANGLES, TRIANGLE_STRIP = 0, 1
# fragment programs: the road layer's, the water layer's with river = 0, 1, 2, the fill
LAYER_ROAD, LAYER_WATER, LAYER_WATER_RIVER, LAYER_WATER_LARGE, LAYER_FILL = 0, 1, 2, 3, 4
# pass state: a depth test and write masks (0: LESS, depth, z and w written)
DEPTH_LESS, DEPTH_ALWAYS, DEPTH_NOTEQUAL = 0, 1, 2
NO_DEPTH_WRITE, NO_Z_WRITE, NO_W_WRITE = 4, 8, 16


class LayerBatch:
    """The meshes of a layer pass, packed once for tp_elevation_layers.  tiles: list of
    (slot, meshes), meshes a list of (vertices [n, 4] float32 (x, y, a, u) in clip
    coordinates, indices or None, mode, clear_depth[, program, state, fill_depth]);
    without the last three, the road layer's program and state."""

    def __init__(self, tiles):
        verts, idx, meshes, jobs = [], [], [], []
        nv = ni = 0
        for slot, ms in tiles:
            jobs.append(LayerJob(slot, len(meshes), len(ms), 0))
            for mesh in ms:
                v, ix, mode, clear = mesh[:4]
                program, state, fill_depth = tuple(mesh[4:]) if len(mesh) > 4 else (LAYER_ROAD, 0, 0.0)
                v = np.ascontiguousarray(v, np.float32).reshape(-1, 4)
                m = LayerMesh()
                m.first_vertex, m.mode, m.clear_depth = nv, mode, int(clear)
                m.program, m.state, m.fill_depth = int(program), int(state), float(fill_depth)
                if ix is None:
                    m.first_index, m.count = -1, v.shape[0]
                else:
                    ix = np.ascontiguousarray(ix, np.uint32)
                    m.first_index, m.count = ni, ix.size
                    idx.append(ix)
                    ni += ix.size
                verts.append(v)
                nv += v.shape[0]
                meshes.append(m)
        self.vertices = np.concatenate(verts) if verts else np.zeros((0, 4), np.float32)
        self.indices = np.concatenate(idx) if idx else np.zeros(0, np.uint32)
        self.jobs = (LayerJob * max(1, len(jobs)))(*jobs)
        self.meshes = (LayerMesh * max(1, len(meshes)))(*meshes)
        self.n_jobs, self.n_meshes, self.n_vertices, self.n_indices = len(jobs), len(meshes), nv, ni

    def pin(self, torch):
        """Moves the vertex and index arrays into pinned host memory (asynchronous uploads)."""
        for name in ("vertices", "indices"):
            a = getattr(self, name)
            t = torch.empty(a.shape, dtype=torch.float32 if a.dtype == np.float32 else torch.int32,
                            pin_memory=True)
            pinned = t.numpy().view(a.dtype)
            pinned[...] = a
            setattr(self, name, pinned)
            setattr(self, "_" + name + "_pinned", t)
        return self

    def to_device(self, torch):
        """Device copies of the vertex and index arrays, for run_device."""
        self._dv = torch.from_numpy(np.ascontiguousarray(self.vertices)).cuda()
        self._di = torch.from_numpy(np.ascontiguousarray(self.indices).view(np.int32)).cuda()
        return self

    def run(self, elev, blend_mode=0, stream=None):
        check(lib().tp_elevation_layers(elev.handle, self.jobs, self.n_jobs, self.meshes, self.n_meshes,
                                        self.vertices.ctypes.data, self.n_vertices, self.indices.ctypes.data,
                                        self.n_indices, blend_mode, stream))

    def run_device(self, elev, blend_mode=0, stream=None):
        check(lib().tp_elevation_layers_device(elev.handle, self.jobs, self.n_jobs, self.meshes, self.n_meshes,
                                               C.c_void_p(self._dv.data_ptr()), self.n_vertices,
                                               C.c_void_p(self._di.data_ptr()), self.n_indices, blend_mode, stream))


def elevation_layers(elev, tiles, blend_mode=0, stream=None):
    """Road and water layer meshes drawn into produced elevation tiles and blended
    into zm (tp_elevation_layers); tiles as for LayerBatch."""
    LayerBatch(tiles).run(elev, blend_mode, stream)


# ---------------------------------------------------------------- ortho tiles
def division_self_test(divisor):
    """(mismatches, first mismatching dividend bits) of the ortho kernel's known-divisor
    division against the correctly rounded one, over all 2^32 dividends."""
    n, first = C.c_ulonglong(), C.c_uint32()
    check(lib().tp_division_self_test(divisor, C.byref(n), C.byref(first)))
    return n.value, first.value


def ortho_noise(tile_width):
    """createOrthoNoise: [6, W, W, 4] uint8."""
    out = np.empty((6, tile_width, tile_width, 4), np.uint8)
    check(lib().tp_ortho_noise(tile_width, out.ctypes.data))
    return out


def make_ortho_params(root_color=(0.5, 0.5, 0.5, 0.5), noise_color=(1.0, 1.0, 1.0, 1.0), scale=2.0, hsv=False):
    """tp_ortho_params; colours in [0, 1] (the reference's rnoise / cnoise over 255)."""
    p = OrthoParams()
    p.root_color[:] = [float(v) for v in root_color]
    p.noise_color[:] = [float(v) for v in noise_color]
    p.scale, p.hsv = float(scale), int(bool(hsv))
    return p


def make_ortho_job(level, tx, ty, out_slot, parent_slot=-1, residual_slot=-1, noise_rot=0, noise_layer=0,
                   noise_amp=0.0, parent_job=-1):
    j = OrthoJob()
    j.level, j.tx, j.ty = level, tx, ty
    j.out_slot, j.parent_slot, j.residual_slot = out_slot, parent_slot, residual_slot
    j.noise_rot, j.noise_layer, j.noise_amp, j.parent_job = noise_rot, noise_layer, float(noise_amp), parent_job
    return j


def ortho_batch(ortho, residuals, params, jobs, stream=None):
    """Produces ortho jobs (a list of OrthoJob) in one launch (tp_ortho_batch)."""
    arr = (OrthoJob * len(jobs))(*jobs)
    check(lib().tp_ortho_batch(ortho.handle, residuals.handle if residuals else None, C.byref(params), arr,
                               len(jobs), stream))


def ortho_batch_device(ortho, residuals, params, jobs_dev_ptr, n, stream=None):
    check(lib().tp_ortho_batch_device(ortho.handle, residuals.handle if residuals else None, C.byref(params),
                                      jobs_dev_ptr, n, stream))


def rgba_to_texels(tiles):
    """[..., W, W, 4] uint8 -> [..., W, W] float32 view of the packed RGBA8 texels
    (the storage's element type), for tp_storage_upload."""
    a = np.ascontiguousarray(tiles, np.uint8)
    return a.view(np.uint32).reshape(a.shape[:-1]).view(np.float32)


def texels_to_rgba(texels):
    """Inverse of rgba_to_texels."""
    a = np.ascontiguousarray(texels, np.float32)
    return a.view(np.uint8).reshape(a.shape + (4,))


class OrthoDat:
    """OrthoCPUProducer's .dat pyramid (tp_ortho_dat_*)."""

    def __init__(self, path):
        h = C.c_void_p()
        check(lib().tp_ortho_dat_open(path.encode(), C.byref(h)))
        self.handle = h
        info = (C.c_int * 8)()
        check(lib().tp_ortho_dat_info(h, info))
        (self.max_level, self.tile_size, self.channels, self.root, self.root_tx, self.root_ty, self.flags,
         self.ntiles) = list(info)
        self.width = self.tile_size + (0 if self.flags & 2 else 4)

    def close(self):
        if self.handle:
            lib().tp_ortho_dat_close(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tile(self, level, tx, ty):
        w = self.width
        out = np.empty((w, w, self.channels), np.uint8)
        got = C.c_int()
        check(lib().tp_ortho_dat_read_tile(self.handle, level, tx, ty, out.ctypes.data, out.size, C.byref(got)))
        return out

    def tile_rgba(self, level, tx, ty):
        w = self.width
        out = np.empty((w, w, 4), np.uint8)
        got = C.c_int()
        check(lib().tp_ortho_dat_read_rgba(self.handle, level, tx, ty, out.ctypes.data, w * w, C.byref(got)))
        return out


class Frame:
    """All requests of a frame (up to two tile widths) produced by one persistent
    launch, optionally replayed from a CUDA graph (tp_frame_*)."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().tp_frame_create(C.byref(h)))
        self.handle = h
        self._keep = []

    def close(self):
        if self.handle:
            lib().tp_frame_destroy(self.handle)
            self.handle = None
        self._keep = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, elev, residuals, normals, params, jobs):
        arr = (TileJob * len(jobs))(*jobs)
        check(lib().tp_frame_add(self.handle, elev.handle, residuals.handle if residuals else None,
                                 normals.handle if normals else None, C.byref(params), arr, len(jobs)))
        self._keep.append((elev, residuals, normals))  # the launches read these storages

    def add_device(self, elev, residuals, normals, params, jobs_dev_ptr, n, has_dependencies=True):
        check(lib().tp_frame_add_device(self.handle, elev.handle, residuals.handle if residuals else None,
                                        normals.handle if normals else None, C.byref(params), jobs_dev_ptr, n,
                                        int(has_dependencies)))
        self._keep.append((elev, residuals, normals))

    def launch(self, stream=None):
        check(lib().tp_frame_launch(self.handle, stream))

    def graph_launch(self, stream=None):
        check(lib().tp_frame_graph_launch(self.handle, stream))

    def overlap_classes(self, on=True):
        """Two tile widths' launches on forked streams (default) or one after the other."""
        check(lib().tp_frame_overlap_classes(self.handle, int(bool(on))))

    def units(self):
        return check(lib().tp_frame_units(self.handle))

    def autotune(self, stream=None, repeats=3):
        check(lib().tp_frame_autotune(self.handle, stream, repeats))

    def config(self, klass):
        b, s, m = C.c_int(), C.c_int(), C.c_int()
        check(lib().tp_frame_config(self.handle, klass, C.byref(b), C.byref(s), C.byref(m)))
        return {"band_rows": b.value, "stages": s.value, "ctas_per_sm": m.value}


def dem_noise(tile_width):
    out = np.empty((6, tile_width, tile_width), np.float32)
    check(lib().tp_dem_noise(tile_width, out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


def cnoise(x, y):
    return lib().tp_cnoise(float(x), float(y))


def noise_select(face, level, tx, ty):
    r, l = C.c_int(), C.c_int()
    check(lib().tp_noise_select(face, level, tx, ty, C.byref(r), C.byref(l)))
    return r.value, l.value


# ------------------------------------------------------------------ cache and producers
class TileCache:
    """TileCache (core/.../producer/TileCache.h:201-309) over a TileStorage."""

    def __init__(self, storage, name=""):
        h = C.c_void_p()
        check(lib().tp_cache_create(storage.handle, name.encode(), C.byref(h)))
        self.handle, self.storage = h, storage

    def close(self):
        if self.handle:
            lib().tp_cache_destroy(self.handle)
            self.handle = None

    def get_used_tiles(self):
        return check(lib().tp_cache_used_tiles(self.handle))

    def get_unused_tiles(self):
        return check(lib().tp_cache_unused_tiles(self.handle))

    def stats(self):
        q, m = C.c_longlong(), C.c_longlong()
        check(lib().tp_cache_stats(self.handle, C.byref(q), C.byref(m)))
        return q.value, m.value


class Tile:
    """A tile handle (TileCache::Tile)."""

    def __init__(self, handle):
        self.handle = handle

    def info(self):
        v = [C.c_int() for _ in range(6)]
        check(lib().tp_tile_info(self.handle, *[C.byref(x) for x in v]))
        return dict(zip(("level", "tx", "ty", "slot", "users", "done"), (x.value for x in v)))

    @property
    def slot(self):
        return self.info()["slot"]


class TileProducer:
    """Common TileProducer calls (core/.../producer/TileProducer.h:68-378)."""

    def __init__(self, handle, cache):
        self.handle, self.cache = handle, cache

    def close(self):
        if self.handle:
            lib().tp_producer_destroy(self.handle)
            self.handle = None

    def get_id(self):
        return lib().tp_producer_id(self.handle)

    def get_border(self):
        return lib().tp_producer_border(self.handle)

    def set_root_quad_size(self, size):
        check(lib().tp_producer_set_root_quad_size(self.handle, float(size)))

    def has_tile(self, level, tx, ty):
        return bool(check(lib().tp_producer_has_tile(self.handle, level, tx, ty)))

    def get_tile(self, level, tx, ty):
        h = lib().tp_producer_get_tile(self.handle, level, tx, ty)
        return Tile(h) if h else None

    def find_tile(self, level, tx, ty, include_cache=False, done=False):
        h = lib().tp_producer_find_tile(self.handle, level, tx, ty, int(include_cache), int(done))
        return Tile(h) if h else None

    def put_tile(self, tile):
        return check(lib().tp_producer_put_tile(self.handle, tile.handle))

    def prefetch_tile(self, level, tx, ty):
        return check(lib().tp_producer_prefetch_tile(self.handle, level, tx, ty))

    def invalidate_tiles(self):
        check(lib().tp_producer_invalidate_tiles(self.handle))

    def queued(self):
        return check(lib().tp_producer_queued(self.handle))

    def create_tiles(self, requests, stream=None):
        """Batched doCreateTile (tp_create_tiles): [(level, tx, ty), ...] -> produced
        tiles, each holding one user."""
        n = len(requests)
        flat = (C.c_int32 * (3 * n))(*[int(v) for r in requests for v in r])
        out = (C.c_void_p * n)()
        check(lib().tp_create_tiles(self.handle, flat, n, out, stream))
        return [Tile(out[i]) for i in range(n)]

    def create_tile(self, level, tx, ty, stream=None):
        h = C.c_void_p()
        check(lib().tp_create_tile(self.handle, level, tx, ty, C.byref(h), stream))
        return Tile(h.value)


class TileSampler:
    """The TileSamplers of one terrain node (tp_sampler_*) over one or more producers
    (e.g. an elevation and a normal producer): `update` takes the next frame's
    quadtree requests (parents first), releases the tiles of quads that disappeared,
    acquires and produces the new quads' tiles in one scheduler run, and returns the
    new quads [(level, tx, ty), ...]."""

    def __init__(self, *producers):
        h = C.c_void_p()
        arr = (C.c_void_p * len(producers))(*[p.handle for p in producers])
        check(lib().tp_sampler_create(arr, len(producers), C.byref(h)))
        self.handle, self.producers = h, producers

    def update(self, requests, stream=None):
        reqs = np.ascontiguousarray(np.asarray(requests, np.int32).reshape(-1, 3))
        n = C.c_int()
        check(lib().tp_sampler_update(self.handle, reqs.ctypes.data_as(C.POINTER(C.c_int32)), reqs.shape[0],
                                      stream, C.byref(n)))
        out = np.empty((max(n.value, 1), 3), np.int32)
        check(lib().tp_sampler_new_tiles(self.handle, out.ctypes.data_as(C.POINTER(C.c_int32)), n.value))
        return [tuple(int(v) for v in r) for r in out[:n.value]]

    def held(self):
        return check(lib().tp_sampler_held(self.handle))

    def find(self, level, tx, ty, producer=0):
        """The held tile (level, tx, ty) of producer number `producer`, or None."""
        h = lib().tp_sampler_find(self.handle, producer, level, tx, ty)
        return Tile(h) if h else None

    def close(self):
        if self.handle:
            lib().tp_sampler_destroy(self.handle)
            self.handle = None


def trace_set(flags):
    """Tracing flags (tp_trace_set): bit 0 NVTX ranges, bit 1 host phase timers."""
    return check(lib().tp_trace_set(int(flags)))


def trace_host_times(reset=False):
    """{phase: (seconds, calls)} of the host phase timers (tp_trace_host_times)."""
    n = 16
    secs, calls = (C.c_double * n)(), (C.c_longlong * n)()
    k = check(lib().tp_trace_host_times(secs, calls, n, int(reset)))
    return {lib().tp_trace_phase_name(i).decode(): (secs[i], calls[i]) for i in range(k)}


class ResidualProducer(TileProducer):
    """ResidualProducer: a .dat pyramid, a host callback or zero residuals."""

    def __init__(self, cache, file="", delta=0, zscale=1.0, source=None, device_decode=False, synthetic=None):
        """synthetic: (sigma0, ratio, seed) for synthetic tiles of standard deviation
        sigma0 * ratio^level made on the device (tp_residual_producer_set_synthetic)."""
        h = C.c_void_p()
        check(lib().tp_residual_producer_create(cache.handle, (file or "").encode(), delta, zscale, C.byref(h)))
        super().__init__(h, cache)
        self._source = None
        if source is not None:
            self.set_source(source)
        if device_decode:
            check(lib().tp_residual_producer_set_device_decode(h, 1))
        if synthetic is not None:
            sigma0, ratio, seed = synthetic
            check(lib().tp_residual_producer_set_synthetic(h, float(sigma0), float(ratio), int(seed)))

    def tile(self, level, tx, ty):
        """The residual tile as computed on the host (tp_residual_tile)."""
        W = self.cache.storage.tile_size
        out = np.empty((W, W), np.float32)
        check(lib().tp_residual_tile(self.handle, level, tx, ty, out.ctypes.data_as(C.POINTER(C.c_float)), W))
        return out

    def set_source(self, fn):
        """fn(level, tx, ty, width) -> float32 array [width, width]."""
        def cb(user, level, tx, ty, out, width):
            try:
                a = np.ascontiguousarray(fn(level, tx, ty, width), dtype=np.float32).reshape(width, width)
                C.memmove(out, a.ctypes.data, a.nbytes)
                return 0
            except Exception:
                return 1
        self._source = RESIDUAL_SOURCE(cb)
        check(lib().tp_residual_producer_set_source(self.handle, self._source, None))


class ElevationProducer(TileProducer):
    def __init__(self, cache, residuals=None, noise_amp=(), params=None, face=0):
        h = C.c_void_p()
        amps = (C.c_float * max(1, len(noise_amp)))(*noise_amp)
        check(lib().tp_elevation_producer_create(cache.handle, residuals.handle if residuals else None, amps,
                                                 len(noise_amp), C.byref(params or make_params()), face, C.byref(h)))
        super().__init__(h, cache)
        self.residuals = residuals
        self._layers = []

    def add_layer(self, fn):
        """TileProducer::addLayer with a road or water elevation layer: fn(level, tx, ty)
        returns the meshes it draws on that tile, a list of (vertices [n, 4] float32,
        indices or None, mode[, program, state, fill_depth]) -- see elevation_layers."""
        def cb(user, level, tx, ty, builder):
            try:
                for mesh in fn(level, tx, ty):
                    verts, idx, mode = mesh[:3]
                    program, state, fill_depth = tuple(mesh[3:]) if len(mesh) > 3 else (LAYER_ROAD, 0, 0.0)
                    rc = lib().tp_layer_builder_set_pass(builder, int(program), int(state), float(fill_depth))
                    if rc:
                        return rc
                    v = np.ascontiguousarray(verts, np.float32).reshape(-1, 4)
                    ix = None if idx is None else np.ascontiguousarray(idx, np.uint32)
                    rc = lib().tp_layer_builder_add_mesh(builder, v.ctypes.data, v.shape[0],
                                                         None if ix is None else ix.ctypes.data,
                                                         0 if ix is None else ix.size, mode)
                    if rc:
                        return rc
                return 0
            except Exception:
                return -1
        c = LAYER_FN(cb)
        self._layers.append(c)
        check(lib().tp_elevation_producer_add_layer(self.handle, c, None))

    def set_blend(self, mode):
        """0: graph1/edit3 blendShader, 1: the demo's 3x3 filtered blend."""
        check(lib().tp_elevation_producer_set_blend(self.handle, mode))


class NormalProducer(TileProducer):
    def __init__(self, cache, elevations, deform=False):
        h = C.c_void_p()
        check(lib().tp_normal_producer_create(cache.handle, elevations.handle, int(deform), C.byref(h)))
        super().__init__(h, cache)
        self.elevations = elevations

    def set_format(self, fmt, grid_mesh=24):
        """Output format 0-3 (NormalProducer.cpp:195): 0/1 carry the coarse normals."""
        check(lib().tp_normal_producer_set_format(self.handle, fmt, grid_mesh))


class OrthoResidualProducer(TileProducer):
    """OrthoCPUProducer: RGBA8 tiles of an ortho .dat pyramid (or zero tiles without a
    file) in a one-channel cache of width tileSize + 2 border."""

    def __init__(self, cache, file=""):
        h = C.c_void_p()
        check(lib().tp_ortho_residual_producer_create(cache.handle, (file or "").encode(), C.byref(h)))
        super().__init__(h, cache)


class OrthoProducer(TileProducer):
    """OrthoProducer: colour tiles upsampled from their parent, plus residuals and noise."""

    def __init__(self, cache, residuals=None, params=None, noise_amp=(), face=1, max_level=-1):
        h = C.c_void_p()
        amps = (C.c_float * max(1, len(noise_amp)))(*noise_amp)
        check(lib().tp_ortho_producer_create(cache.handle, residuals.handle if residuals else None,
                                             C.byref(params or make_ortho_params()), amps, len(noise_amp), face,
                                             max_level, C.byref(h)))
        super().__init__(h, cache)
        self.residuals = residuals


def scheduler_run(producers, stream=None):
    """Produces every queued tile of the producers (tp_scheduler_run)."""
    arr = (C.c_void_p * len(producers))(*[p.handle for p in producers])
    check(lib().tp_scheduler_run(arr, len(producers), stream))


# ------------------------------------------------------------------ residual files
class DatPyramid:
    """A residual pyramid file (tp_dat_*)."""

    def __init__(self, path):
        h = C.c_void_p()
        check(lib().tp_dat_open(path.encode(), C.byref(h)))
        self.handle = h
        info = (C.c_int * 7)()
        sc = C.c_float()
        check(lib().tp_dat_info(h, info, C.byref(sc)))
        (self.min_level, self.max_level, self.tile_size, self.root_level, self.root_tx, self.root_ty,
         self.ntiles) = list(info)
        self.scale = sc.value

    def close(self):
        if self.handle:
            lib().tp_dat_close(self.handle)
            self.handle = None

    def decode_device(self, tiles, scale, residuals, slots, stream=None):
        """Decodes [(level, tx, ty), ...] on the device into residual slots (tp_dat_decode_device)."""
        n = len(tiles)
        lv = (C.c_int * n)(*[t[0] for t in tiles])
        xs = (C.c_int * n)(*[t[1] for t in tiles])
        ys = (C.c_int * n)(*[t[2] for t in tiles])
        sl = (C.c_int * n)(*slots)
        check(lib().tp_dat_decode_device(self.handle, lv, xs, ys, n, scale, residuals.handle, sl, stream))

    def tile_int16(self, level, tx, ty):
        cap = (self.tile_size + 5) ** 2
        out = np.empty(cap, np.int16)
        w = C.c_int()
        check(lib().tp_dat_read_tile(self.handle, level, tx, ty, out.ctypes.data_as(C.POINTER(C.c_int16)), cap,
                                     C.byref(w)))
        return out[:w.value * w.value].reshape(w.value, w.value)


def inflate_zlib(data, capacity):
    out = np.empty(capacity, np.uint8)
    n = C.c_size_t()
    src = np.frombuffer(data, np.uint8)
    check(lib().tp_inflate_zlib(src.ctypes.data, len(data), out.ctypes.data, capacity, C.byref(n)))
    return out[:n.value].tobytes()


def sphere_frame(root_quad_size, level, tx, ty):
    """The 47 floats of a tile's spherical frame (tp_sphere_frame)."""
    out = np.empty(47, np.float32)
    check(lib().tp_sphere_frame(float(root_quad_size), level, tx, ty, out.ctypes.data_as(C.POINTER(C.c_float))))
    return out
