"""ctypes view of the C ABI declared in include/vgb.h.

The structs below mirror include/vgb.h field for field; ``load()`` opens the in-tree
``libvgb.so`` and raises if it is missing, so nothing silently falls back to another path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

MAX_BANDS = 8
NO_HIT = 0xFFFFFFFF

STATUS = {
    0: "VGB_OK",
    1: "VGB_ERR_INVALID_ARGUMENT",
    2: "VGB_ERR_CUDA",
    3: "VGB_ERR_OUT_OF_MEMORY",
    4: "VGB_ERR_NOT_READY",
    5: "VGB_ERR_DEVICE_LIMIT",
    6: "VGB_ERR_INTERNAL",
}


class VgbError(RuntimeError):
    """A vgb_* call returned a status other than VGB_OK."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


DISTORTION_NONE, DISTORTION_BROWN, DISTORTION_OPENCV, DISTORTION_OWEN = 0, 1, 2, 3


class Camera(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32),
        ("origin", C.c_float * 3), ("rotation", C.c_float * 9), ("kinv", C.c_float * 6),
        ("z_dir", C.c_float), ("power_scale", C.c_float * MAX_BANDS),
        ("distortion", C.c_uint32), ("distortion_coeffs", C.c_float * 12), ("interpolate_directions", C.c_uint32),
        ("depth_of_field", C.c_uint32), ("aperture_radius", C.c_float), ("focal_length", C.c_float),
        ("focus_distance", C.c_float),
        ("sensor_size", C.c_float * 2), ("velocity", C.c_float * 3), ("angular_rate", C.c_float * 3),
        ("rot_origin", C.c_float * 3),
    ]


class Light(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("radius", C.c_float), ("radiance", C.c_float * MAX_BANDS)]


class DenoiseOptions(C.Structure):
    _fields_ = [("levels_direct", C.c_uint32), ("levels_indirect", C.c_uint32), ("depth_threshold", C.c_float),
                ("normal_threshold", C.c_float), ("min_normal_weight", C.c_float), ("epsilon", C.c_float)]


class PtOptions(C.Structure):
    _fields_ = [
        ("samples", C.c_uint32), ("bounces", C.c_uint32), ("show_background", C.c_uint32),
        ("simulate_lighting", C.c_uint32), ("smooth_shading", C.c_uint32),
        ("deterministic_light", C.c_uint32), ("rr_depth", C.c_uint32), ("has_ambient", C.c_uint32),
        ("seed", C.c_uint64), ("frame", C.c_uint32), ("nbands", C.c_uint32),
        ("ambient", C.c_float * MAX_BANDS), ("background", C.c_float * MAX_BANDS),
        ("adaptive_sampling", C.c_uint32), ("samples_per_batch", C.c_uint32), ("sampling_tolerance", C.c_float),
        ("samples_to_detect_miss", C.c_uint32), ("denoise", C.c_uint32), ("denoiser", DenoiseOptions),
    ]


class Film(C.Structure):
    _fields_ = [
        ("total_radiance", C.c_void_p), ("direct_radiance", C.c_void_p), ("indirect_radiance", C.c_void_p),
        ("received_power", C.c_void_p), ("albedo", C.c_void_p), ("normal_global", C.c_void_p),
        ("depth", C.c_void_p), ("alpha", C.c_void_p), ("triangle_id", C.c_void_p),
        ("pixel_solid_angle", C.c_void_p), ("on_device", C.c_int32),
        ("velocity_global", C.c_void_p), ("velocity_camera", C.c_void_p), ("triangle_size", C.c_void_p),
    ]


class InstanceMotion(C.Structure):
    _fields_ = [("first_triangle", C.c_uint32), ("velocity", C.c_float * 3), ("angular_rate", C.c_float * 3),
                ("position", C.c_float * 3)]


class Frame(C.Structure):
    _fields_ = [("camera", Camera), ("lights", Light * 8), ("nlights", C.c_uint32), ("samples", C.c_uint32),
                ("frame", C.c_uint32), ("film", Film)]


class View(C.Structure):
    _fields_ = [("camera", Camera), ("lights", Light * 8), ("nlights", C.c_uint32), ("samples", C.c_uint32),
                ("frame", C.c_uint32), ("pad", C.c_uint32), ("target", C.c_void_p), ("radiance", C.c_void_p)]


class Sensor(C.Structure):
    _fields_ = [("exposure_time", C.c_float), ("photon_energy", C.c_float * 8), ("quantum_efficiency", C.c_float * 8),
                ("gain", C.c_float), ("max_adu", C.c_float), ("simulate_photon_noise", C.c_uint32),
                ("noise_model", C.c_uint32), ("dark_current", C.c_float), ("readout_noise_mean", C.c_float),
                ("readout_noise_std", C.c_float), ("horizontal_scale", C.c_float), ("vertical_scale", C.c_float),
                ("horizontal_pattern_period", C.c_uint32), ("vertical_pattern_period", C.c_uint32),
                ("frame", C.c_uint32), ("seed", C.c_uint64), ("filter_mosaic", C.c_void_p)]


class RgbConversion(C.Structure):
    _fields_ = [("band_min", C.c_float * 8), ("band_max", C.c_float * 8), ("rgb_min", C.c_float * 3),
                ("rgb_max", C.c_float * 3), ("rgb_bandwidth", C.c_float * 3), ("rgb_photon_energy", C.c_float * 3),
                ("rgb_quantum_efficiency", C.c_float * 3)]


class BatchOptions(C.Structure):
    _fields_ = [("autotune", C.c_uint32), ("use_graph", C.c_uint32), ("block_threads", C.c_uint32),
                ("blocks_per_sm", C.c_uint32), ("tiles_per_grab", C.c_uint32)]


class BvhOptions(C.Structure):
    _fields_ = [("max_leaf_size", C.c_uint32), ("builder", C.c_uint32), ("threads", C.c_uint32),
                ("layout", C.c_uint32)]


class Stats(C.Structure):
    _fields_ = [
        ("rays_closest", C.c_uint64), ("rays_shadow", C.c_uint64), ("nodes_visited", C.c_uint64),
        ("tris_tested", C.c_uint64), ("nodes_closest", C.c_uint64), ("tris_closest", C.c_uint64),
        ("hits_closest", C.c_uint64), ("bvh_nodes", C.c_uint32), ("bvh_node_bytes", C.c_uint32),
        ("tri_record_bytes", C.c_uint32), ("kernel_launches", C.c_uint32), ("device_error", C.c_uint32),
        ("ms_last", C.c_float), ("ms_trace", C.c_float), ("ms_shade", C.c_float), ("ms_shadow", C.c_float),
        ("ms_film", C.c_float), ("launches_trace", C.c_uint32), ("launches_shade", C.c_uint32),
        ("launches_shadow", C.c_uint32), ("launches_film", C.c_uint32),
    ]


class RasterOptions(C.Structure):
    _fields_ = [("intrinsic", C.c_float * 6), ("simulate_lighting", C.c_uint32), ("smooth_shading", C.c_uint32),
                ("nbands", C.c_uint32), ("pad", C.c_uint32)]


QUIPU_MAX_LODS = 64
QUIPU_NO_ALBEDO = 0xFFFFFFFF


class QuipuHeader(C.Structure):
    _fields_ = [("class_id", C.c_uint16), ("num_lods", C.c_uint16), ("has_albedos", C.c_uint32),
                ("position", C.c_double * 3), ("rotation", C.c_double * 9), ("scale", C.c_double * 3),
                ("normal", C.c_float * 3), ("cone_angle", C.c_float)]


class QuipuProjection(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("pixel_scale", C.c_double * 2),
                ("tile_definitions", C.c_uint32 * 2), ("tile_row", C.c_uint32), ("tile_col", C.c_uint32),
                ("xoff", C.c_double), ("yoff", C.c_double), ("dx", C.c_double), ("dy", C.c_double),
                ("is_ogr", C.c_uint32), ("pad", C.c_uint32), ("row_col_rotation", C.c_double * 2),
                ("model_tie_point", C.c_double * 2)]


class QuipuLodInfo(C.Structure):
    _fields_ = [("gsd", C.c_double), ("offset", C.c_uint64), ("width", C.c_uint32), ("height", C.c_uint32),
                ("projection", QuipuProjection), ("height_min", C.c_float), ("height_max", C.c_float),
                ("precision", C.c_uint32), ("compressed", C.c_uint32), ("albedo_type", C.c_uint32),
                ("albedo_channels", C.c_uint32)]


class QuipuReadOptions(C.Structure):
    _fields_ = [("nbands", C.c_uint32), ("read_albedos", C.c_uint32), ("default_albedo", C.c_float),
                ("albedo_profile", C.c_float * MAX_BANDS)]


class QuipuLodData(C.Structure):
    _fields_ = [("projection", QuipuProjection), ("heights", C.c_void_p), ("albedo_type", C.c_uint32),
                ("nbands", C.c_uint32), ("albedo", C.c_void_p)]


# exported symbol -> (restype, argtypes); the symbol list is the one include/vgb.h declares
_P = C.c_void_p
_U32 = C.c_uint32
SIGNATURES = {
    "vgb_context_create": (C.c_int, [C.POINTER(_P), C.c_int]),
    "vgb_context_destroy": (C.c_int, [_P]),
    "vgb_last_error": (C.c_char_p, [_P]),
    "vgb_version": (C.c_char_p, []),
    "vgb_set_stream": (C.c_int, [_P, _P]),
    "vgb_synchronize": (C.c_int, [_P]),
    "vgb_compute_vertex_normals": (C.c_int, [_P, _U32, _P, _U32, _P]),
    "vgb_dem_triangulate": (C.c_int, [_P, _U32, _U32, C.c_double, C.c_double, _P, _P, C.POINTER(_U32)]),
    "vgb_camera_intrinsics": (C.c_int, [C.c_float, C.c_float, C.c_float, _U32, _U32, C.c_float, C.c_float,
                                        C.c_float, C.c_float, C.c_float, C.POINTER(C.c_float)]),
    "vgb_scene_upload": (C.c_int, [_P, _P, _U32, _P, _U32, _U32, _P, _P, _P, _P, _U32, _U32]),
    "vgb_bvh_build": (C.c_int, [_P, C.POINTER(BvhOptions)]),
    "vgb_scene_update_positions": (C.c_int, [_P, _P, _P, C.c_int]),
    "vgb_pixel_solid_angle": (C.c_int, [_P, C.POINTER(Camera), _P, C.c_int]),
    "vgb_render": (C.c_int, [_P, C.POINTER(Camera), _P, _U32, C.POINTER(PtOptions), C.POINTER(Film)]),
    "vgb_render_noalloc": (C.c_int, [_P, C.POINTER(Camera), _P, _U32, C.POINTER(PtOptions), C.POINTER(Film)]),
    "vgb_trace_rays": (C.c_int, [_P, _P, _P, _P, _U32, C.c_int, _P, _P, _P, C.c_int]),
    "vgb_render_batch": (C.c_int, [_P, _P, _U32, C.POINTER(PtOptions), C.POINTER(BatchOptions)]),
    "vgb_batch_tuning": (C.c_int, [_P, C.POINTER(_U32), C.POINTER(_U32), C.POINTER(_U32)]),
    "vgb_adjoint": (C.c_int, [_P, C.POINTER(Camera), _P, _U32, C.POINTER(PtOptions), _P, _P, _P, C.c_int]),
    "vgb_dem_triangulate_gpu": (C.c_int, [_P, _P, _U32, _U32, C.c_double, C.c_double, _P, _P, C.POINTER(_U32), C.c_int]),
    "vgb_compute_vertex_normals_gpu": (C.c_int, [_P, _P, _U32, _P, _U32, _P, C.c_int]),
    "vgb_sensor_simulate": (C.c_int, [_P, _P, _U32, _U32, _U32, C.POINTER(Sensor), _P, C.c_int]),
    "vgb_psf_convolve": (C.c_int, [_P, _P, _U32, _U32, _U32, _P, _U32, _U32, C.c_int]),
    "vgb_denoise": (C.c_int, [_P, _P, _P, _P, _P, _P, _U32, _U32, _U32, _P, C.c_int]),
    "vgb_adjoint_positions": (C.c_int, [_P, C.POINTER(Camera), _P, _U32, C.POINTER(PtOptions), _P, _P, _P, C.c_int]),
    "vgb_render_adjoint_batch": (C.c_int, [_P, _P, _U32, C.POINTER(PtOptions), _P, _P, C.POINTER(C.c_double)]),
    "vgb_texture_update": (C.c_int, [_P, _P, _U32, _U32]),
    "vgb_scene_normal_map": (C.c_int, [_P, _P, _U32, _U32]),
    "vgb_scene_motion": (C.c_int, [_P, _P, _U32]),
    "vgb_get_stats": (C.c_int, [_P, C.POINTER(Stats)]),
    "vgb_set_count_pass": (C.c_int, [_P, C.c_int]),
    "vgb_set_profiling": (C.c_int, [_P, C.c_int]),
    "vgb_set_traversal_limit": (C.c_int, [_P, C.c_uint32]),
    "vgb_sensor_simulate_rgb": (C.c_int, [_P, _P, _U32, _U32, _U32, _P, _P, _P, C.c_int]),
    "vgb_set_wavefront_tuning": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32]),
    "vgb_measure_l2_read": (C.c_int, [_P, C.c_uint64, C.c_uint32, C.c_uint32, C.POINTER(C.c_double)]),
    "vgb_rasterize": (C.c_int, [_P, C.POINTER(Camera), _P, _U32, C.POINTER(RasterOptions), C.POINTER(Film)]),
    "vgb_quipu_open": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "vgb_quipu_close": (None, [_P]),
    "vgb_quipu_last_error": (C.c_char_p, []),
    "vgb_quipu_get_header": (C.c_int, [_P, C.POINTER(QuipuHeader)]),
    "vgb_quipu_get_lod": (C.c_int, [_P, _U32, C.POINTER(QuipuLodInfo)]),
    "vgb_quipu_select_lod": (_U32, [_P, C.c_double]),
    "vgb_quipu_read_heights": (C.c_int, [_P, _U32, _P]),
    "vgb_quipu_read_albedo": (C.c_int, [_P, _U32, _U32, _P]),
    "vgb_quipu_read_mesh": (C.c_int, [_P, _P, _U32, C.POINTER(QuipuReadOptions), _P, _P, _P, _P, C.POINTER(_U32),
                                      C.c_int]),
    "vgb_quipu_write": (C.c_int, [C.c_char_p, _P, _U32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double), C.c_int, C.c_int]),
    "vgb_lz4_decompress": (C.c_int64, [_P, C.c_uint64, _P, C.c_uint64]),
    "vgb_lz4_bound": (C.c_uint64, [C.c_uint64]),
    "vgb_lz4_compress": (C.c_uint64, [_P, C.c_uint64, _P, C.c_uint64]),
}

_LIB = None


def library_path() -> Path:
    return Path(__file__).resolve().parent / "_build" / "libvgb.so"


def load(build_if_missing: bool = True):
    """Open libvgb.so (building it first if it is missing or stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if build_if_missing:
        from . import build as _build
        _build.build()
    if not path.exists():
        raise RuntimeError(f"libvgb.so not found at {path}: run vira_gb300.build.build()")
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int, ctx=None, what: str = ""):
    if status != 0:
        msg = what
        if ctx:
            m = load().vgb_last_error(ctx)
            msg = (what + ": " if what else "") + (m.decode() if m else "")
        raise VgbError(status, msg)


def ptr(a) -> int | None:
    """Raw pointer of a numpy array or torch tensor (None passes NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data
