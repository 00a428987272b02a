"""ctypes binding of libproland_gb300.so (the C ABI declared in include/proland_gb300.h).

The shared library is the product: every compute call goes through it and there
is no CPU fallback.  Loading fails loudly when the library has not been built.
"""
import ctypes as C
import os

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# PROLAND_GB300_DEBUG=1 selects the debug build (device-side bounds checks, storage guards)
DEBUG = os.environ.get("PROLAND_GB300_DEBUG", "0") == "1"
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libproland_gb300_debug.so" if DEBUG else "libproland_gb300.so")

TP_OK = 0
TP_E_BAD_ARG = -1
TP_E_CACHE_FULL = -2
TP_E_MISSING_PARENT = -3
TP_E_TIMEOUT = -4
TP_E_CUDA = -5
TP_E_IO = -6
TP_E_NO_DEVICE = -7
TP_E_BOUNDS = -8

ERROR_NAMES = {
    TP_E_BAD_ARG: "TP_E_BAD_ARG", TP_E_CACHE_FULL: "TP_E_CACHE_FULL",
    TP_E_MISSING_PARENT: "TP_E_MISSING_PARENT", TP_E_TIMEOUT: "TP_E_TIMEOUT",
    TP_E_CUDA: "TP_E_CUDA", TP_E_IO: "TP_E_IO", TP_E_NO_DEVICE: "TP_E_NO_DEVICE", TP_E_BOUNDS: "TP_E_BOUNDS",
}


class TPError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERROR_NAMES.get(code, "TP_E_?"), code, msg))
        self.code = code


class TileJob(C.Structure):
    """tp_tile_job"""
    _fields_ = [
        ("level", C.c_int32), ("tx", C.c_int32), ("ty", C.c_int32),
        ("out_slot", C.c_int32), ("parent_slot", C.c_int32), ("residual_slot", C.c_int32),
        ("rx", C.c_int32), ("ry", C.c_int32), ("normal_slot", C.c_int32),
        ("noise_rot", C.c_int32), ("noise_layer", C.c_int32),
        ("noise_amp", C.c_float), ("rscale", C.c_float), ("tile_meters", C.c_float),
        ("parent_job", C.c_int32), ("reserved", C.c_int32),
    ]


class ElevParams(C.Structure):
    """tp_elev_params"""
    _fields_ = [
        ("grid_size", C.c_int32), ("flip", C.c_int32), ("no_clamp", C.c_int32),
        ("noise_mode", C.c_int32), ("normal_format", C.c_int32), ("band_rows", C.c_int32),
        ("stages", C.c_int32), ("reserved", C.c_int32),
    ]


class OrthoJob(C.Structure):
    """tp_ortho_job"""
    _fields_ = [
        ("level", C.c_int32), ("tx", C.c_int32), ("ty", C.c_int32),
        ("out_slot", C.c_int32), ("parent_slot", C.c_int32), ("residual_slot", C.c_int32),
        ("noise_rot", C.c_int32), ("noise_layer", C.c_int32), ("noise_amp", C.c_float),
        ("parent_job", C.c_int32), ("reserved", C.c_int32 * 2),
    ]


class OrthoParams(C.Structure):
    """tp_ortho_params"""
    _fields_ = [
        ("root_color", C.c_float * 4), ("noise_color", C.c_float * 4), ("scale", C.c_float),
        ("hsv", C.c_int32), ("reserved", C.c_int32 * 2),
    ]


class HostTiles(C.Structure):
    """tp_host_tiles"""
    _fields_ = [(n, C.c_void_p) for n in ("parent_zf", "parent_zm", "residual", "zf", "zc", "zm", "nx", "ny")]


class LayerMesh(C.Structure):
    """tp_layer_mesh"""
    _fields_ = [("first_vertex", C.c_int32), ("count", C.c_int32), ("first_index", C.c_int32),
                ("mode", C.c_int32), ("clear_depth", C.c_int32), ("program", C.c_int32), ("state", C.c_int32),
                ("fill_depth", C.c_float)]


class LayerJob(C.Structure):
    """tp_layer_job"""
    _fields_ = [("slot", C.c_int32), ("first_mesh", C.c_int32), ("n_meshes", C.c_int32), ("reserved", C.c_int32)]


LAYER_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p)
RESIDUAL_SOURCE = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float), C.c_int)

_LIB = None
_vp = C.c_void_p
_i = C.c_int
_f32p = C.POINTER(C.c_float)


def lib():
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise ImportError("libproland_gb300.so is not built (%s): run "
                          "`python -c \"import __graft_entry__ as g; g.build()\"`" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    sig = {
        "tp_last_error": ([], C.c_char_p),
        "tp_version": ([], _i),
        "tp_build_is_debug": ([], _i),
        "tp_storage_check_guards": ([_vp], _i),
        "tp_debug_check_capacity": ([_vp, _i], _i),
        "tp_device_available": ([], _i),
        "tp_storage_create": ([_i, _i, _i, _i, C.POINTER(_vp)], _i),
        "tp_storage_destroy": ([_vp], _i),
        "tp_storage_tile_size": ([_vp], _i),
        "tp_storage_capacity": ([_vp], _i),
        "tp_storage_free_slots": ([_vp], _i),
        "tp_storage_channels": ([_vp], _i),
        "tp_storage_pitch": ([_vp], _i),
        "tp_storage_new_slot": ([_vp], _i),
        "tp_storage_delete_slot": ([_vp, _i], _i),
        "tp_storage_plane": ([_vp, _i, _i], _vp),
        "tp_storage_upload": ([_vp, _i, _i, _i, _vp, _vp], _i),
        "tp_storage_download": ([_vp, _i, _i, _i, _vp, _vp], _i),
        "tp_elevation_batch": ([_vp, _vp, _vp, C.POINTER(ElevParams), C.POINTER(TileJob), _i, _vp], _i),
        "tp_elevation_batch_device": ([_vp, _vp, _vp, C.POINTER(ElevParams), _vp, _i, _vp], _i),
        "tp_normal_batch": ([_vp, _vp, C.POINTER(TileJob), _i, C.c_double, _vp], _i),
        "tp_normal_batch_format": ([_vp, _vp, C.POINTER(TileJob), _i, C.c_double, _i, C.POINTER(_i), _i, _vp], _i),
        "tp_normal_producer_set_format": ([_vp, _i, _i], _i),
        "tp_elevation_batch_noalloc": ([_vp, _vp, _vp, C.POINTER(ElevParams), C.POINTER(TileJob), _i, _vp], _i),
        "tp_pipeline_create": ([_i, _i, _i, C.POINTER(_vp)], _i),
        "tp_pipeline_destroy": ([_vp], _i),
        "tp_elevation_batch_host": ([_vp, C.POINTER(ElevParams), C.POINTER(TileJob), _i, C.POINTER(HostTiles), _vp],
                                    _i),
        "tp_ortho_noise": ([_i, _vp], _i),
        "tp_ortho_batch": ([_vp, _vp, C.POINTER(OrthoParams), C.POINTER(OrthoJob), _i, _vp], _i),
        "tp_ortho_batch_device": ([_vp, _vp, C.POINTER(OrthoParams), _vp, _i, _vp], _i),
        "tp_ortho_residual_producer_create": ([_vp, C.c_char_p, C.POINTER(_vp)], _i),
        "tp_ortho_producer_create": ([_vp, _vp, C.POINTER(OrthoParams), _f32p, _i, _i, _i, C.POINTER(_vp)], _i),
        "tp_division_self_test": ([C.c_float, C.POINTER(C.c_ulonglong), C.POINTER(C.c_uint32)], _i),
        "tp_sphere_division_self_test": ([C.c_ulonglong, C.c_uint, _f32p, _i, C.POINTER(C.c_ulonglong),
                                          C.POINTER(C.c_ulonglong)], _i),
        "tp_ortho_dat_open": ([C.c_char_p, C.POINTER(_vp)], _i),
        "tp_ortho_dat_close": ([_vp], _i),
        "tp_ortho_dat_info": ([_vp, C.POINTER(_i)], _i),
        "tp_ortho_dat_read_tile": ([_vp, _i, _i, _i, _vp, _i, C.POINTER(_i)], _i),
        "tp_ortho_dat_read_rgba": ([_vp, _i, _i, _i, _vp, _i, C.POINTER(_i)], _i),
        "tp_frame_create": ([C.POINTER(_vp)], _i),
        "tp_frame_destroy": ([_vp], _i),
        "tp_frame_clear": ([_vp], _i),
        "tp_frame_add": ([_vp, _vp, _vp, _vp, C.POINTER(ElevParams), C.POINTER(TileJob), _i], _i),
        "tp_frame_add_device": ([_vp, _vp, _vp, _vp, C.POINTER(ElevParams), _vp, _i, _i], _i),
        "tp_frame_launch": ([_vp, _vp], _i),
        "tp_frame_graph_launch": ([_vp, _vp], _i),
        "tp_frame_units": ([_vp], _i),
        "tp_frame_overlap_classes": ([_vp, _i], _i),
        "tp_frame_autotune": ([_vp, _vp, _i], _i),
        "tp_frame_config": ([_vp, _i, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i)], _i),
        "tp_status": ([C.POINTER(_i), _i], _i),
        "tp_stream_check": ([_vp], _i),
        "tp_cache_create": ([_vp, C.c_char_p, C.POINTER(_vp)], _i),
        "tp_cache_destroy": ([_vp], _i),
        "tp_cache_used_tiles": ([_vp], _i),
        "tp_cache_unused_tiles": ([_vp], _i),
        "tp_cache_stats": ([_vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)], _i),
        "tp_residual_producer_create": ([_vp, C.c_char_p, _i, C.c_float, C.POINTER(_vp)], _i),
        "tp_residual_producer_set_source": ([_vp, RESIDUAL_SOURCE, _vp], _i),
        "tp_elevation_producer_create": ([_vp, _vp, _f32p, _i, C.POINTER(ElevParams), _i, C.POINTER(_vp)], _i),
        "tp_normal_producer_create": ([_vp, _vp, _i, C.POINTER(_vp)], _i),
        "tp_producer_destroy": ([_vp], _i),
        "tp_producer_id": ([_vp], _i),
        "tp_producer_border": ([_vp], _i),
        "tp_producer_set_root_quad_size": ([_vp, C.c_float], _i),
        "tp_producer_has_tile": ([_vp, _i, _i, _i], _i),
        "tp_producer_get_tile": ([_vp, _i, _i, _i], _vp),
        "tp_producer_find_tile": ([_vp, _i, _i, _i, _i, _i], _vp),
        "tp_producer_put_tile": ([_vp, _vp], _i),
        "tp_producer_prefetch_tile": ([_vp, _i, _i, _i], _i),
        "tp_producer_invalidate_tiles": ([_vp], _i),
        "tp_producer_queued": ([_vp], _i),
        "tp_tile_info": ([_vp] + [C.POINTER(_i)] * 6, _i),
        "tp_scheduler_run": ([C.POINTER(_vp), _i, _vp], _i),
        "tp_create_tiles": ([_vp, C.POINTER(C.c_int32), _i, C.POINTER(_vp), _vp], _i),
        "tp_create_tile": ([_vp, _i, _i, _i, C.POINTER(_vp), _vp], _i),
        "tp_quadtree_requests": ([C.c_double, _i, C.c_float, C.c_float, C.c_double, C.c_double, C.c_double,
                                  C.c_double, C.POINTER(C.c_int32), _i, C.POINTER(_i)], _i),
        "tp_residual_tile": ([_vp, _i, _i, _i, _f32p, _i], _i),
        "tp_sphere_frame": ([C.c_double, _i, _i, _i, _f32p], _i),
        "tp_dat_open": ([C.c_char_p, C.POINTER(_vp)], _i),
        "tp_dat_close": ([_vp], _i),
        "tp_dat_info": ([_vp, C.POINTER(_i), C.POINTER(C.c_float)], _i),
        "tp_dat_read_tile": ([_vp, _i, _i, _i, C.POINTER(C.c_int16), _i, C.POINTER(_i)], _i),
        "tp_dat_decode_device": ([_vp, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), _i, C.c_float, _vp,
                                  C.POINTER(_i), _vp], _i),
        "tp_residual_producer_set_device_decode": ([_vp, _i], _i),
        "tp_residual_producer_set_synthetic": ([_vp, C.c_double, C.c_double, C.c_uint], _i),
        "tp_sampler_create": ([C.POINTER(_vp), _i, C.POINTER(_vp)], _i),
        "tp_sampler_destroy": ([_vp], _i),
        "tp_sampler_update": ([_vp, C.POINTER(C.c_int32), _i, _vp, C.POINTER(_i)], _i),
        "tp_sampler_new_tiles": ([_vp, C.POINTER(C.c_int32), _i], _i),
        "tp_sampler_held": ([_vp], _i),
        "tp_sampler_find": ([_vp, _i, _i, _i, _i], _vp),
        "tp_trace_set": ([_i], _i),
        "tp_trace_host_times": ([C.POINTER(C.c_double), C.POINTER(C.c_longlong), _i, _i], _i),
        "tp_trace_phase_name": ([_i], C.c_char_p),
        "tp_inflate_zlib": ([_vp, C.c_size_t, _vp, C.c_size_t, C.POINTER(C.c_size_t)], _i),
        "tp_dem_noise": ([_i, _f32p], _i),
        "tp_cnoise": ([C.c_float, C.c_float], C.c_float),
        "tp_noise_select": ([_i, _i, _i, _i, C.POINTER(_i), C.POINTER(_i)], _i),
        "tp_fbm_heights": ([_i, _i, _i, C.c_float, C.c_float, C.c_uint32, _vp, _vp], _i),
        "tp_preprocess_level": ([_vp, _i, _i, _i, C.c_float, _vp, _vp, _vp, _vp, _vp, _vp], _i),
        "tp_fbm_pairs": ([_i, _i, C.c_float, C.c_uint32, _i, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), _i, _vp, _vp,
                          _vp, _vp], _i),
        "tp_learned_create": ([_i, _i, C.POINTER(_vp)], _i),
        "tp_learned_destroy": ([_vp], _i),
        "tp_learned_param_count": ([_vp], _i),
        "tp_learned_init": ([_vp, C.c_uint32], _i),
        "tp_learned_get_params": ([_vp, _f32p, _i], _i),
        "tp_learned_set_params": ([_vp, _f32p, _i], _i),
        "tp_learned_get_grads": ([_vp, _f32p, _i], _i),
        "tp_learned_set_sigmas": ([_vp, _f32p, _f32p, _i], _i),
        "tp_learned_set_fused": ([_vp, _i], _i),
        "tp_learned_get_state": ([_vp, _vp, _vp, _i, C.POINTER(_i)], _i),
        "tp_learned_set_state": ([_vp, _vp, _vp, _i, _i], _i),
        "tp_learned_get_sigmas": ([_vp, _vp, _vp, _i], _i),
        "tp_learned_forward": ([_vp, _vp, C.POINTER(_i), _i, _i, _vp, _vp], _i),
        "tp_learned_check": ([_vp, _vp], _i),
        "tp_learned_backward": ([_vp, _vp, _f32p, _vp], _i),
        "tp_learned_adam": ([_vp, C.c_float, _vp], _i),
        "tp_learned_gather": ([_vp, _vp, _vp, _i, C.POINTER(_i), C.POINTER(_i), _i, _vp, _vp, _vp], _i),
        "tp_elevation_layers": ([_vp, C.POINTER(LayerJob), _i, C.POINTER(LayerMesh), _i, _vp, _i, _vp, _i, _i, _vp],
                                _i),
        "tp_elevation_layers_device": ([_vp, C.POINTER(LayerJob), _i, C.POINTER(LayerMesh), _i, _vp, _i, _vp, _i,
                                        _i, _vp], _i),
        "tp_layer_builder_add_mesh": ([_vp, _vp, _i, _vp, _i, _i], _i),
        "tp_layer_builder_set_pass": ([_vp, _i, _i, C.c_float], _i),
        "tp_elevation_producer_add_layer": ([_vp, LAYER_FN, _vp], _i),
        "tp_elevation_producer_set_blend": ([_vp, _i], _i),
        "tp_learned_predict_residuals": ([_vp, _vp, C.POINTER(TileJob), _i, _vp, _vp], _i),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _LIB = L
    return L


def check(rc):
    """Raises TPError for a negative return code, else returns it."""
    if rc < 0:
        raise TPError(rc, lib().tp_last_error().decode(errors="replace"))
    return rc
