"""ctypes mirror of include/bonsai_gpu.h (the C ABI of libbonsai_gpu.so).

The structures here must match the header field for field; tests/test_abi.py checks sizes and the
exported symbol list.  Nothing here computes: it loads the in-tree shared library and declares the
signatures.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "lib" / "libbonsai_gpu.so"

BG_OK = 0
BG_ERR_INVALID = 1
BG_ERR_CUDA = 2
BG_ERR_OOM = 3
BG_ERR_TIMEOUT = 4
BG_ERR_DEVICE = 5
BG_ERR_UNSUPPORTED = 6
BG_ERR_NO_DEVICE = 7

BG_MODE_REF_COMPAT = 0
BG_MODE_PBRT = 1

BG_MAT_MATTE = 0
BG_MAT_PLASTIC = 1
BG_MAT_CONDUCTOR = 2
BG_MAT_DIELECTRIC = 3

BG_BVH_WIDE = 0
BG_BVH_REFERENCE = 1
BG_BVH_REFERENCE_FIXED = 2
BG_BVH_WIDE2 = 3

BG_RENDER_ACCUMULATE = 1
BG_RENDER_NO_READBACK = 2
BG_RENDER_GRAPH = 4
BG_RENDER_STAGE_TIMING = 8
BG_TUNE_SORT_RAYS = 1
BG_TUNE_L2_PERSIST = 2
BG_TUNE_TILE_PIXELS = 4
BG_TUNE_SHADOW_QUEUE_HALF = 8
BG_TUNE_CONCURRENT_SHADE = 16
BG_SAMPLER_INDEPENDENT, BG_SAMPLER_STRATIFIED = 0, 1

BG_TEXTURE_IMAGE = 0
BG_TEXTURE_UV = 1
BG_WRAP_REPEAT = 0
BG_WRAP_BLACK = 1
BG_WRAP_CLAMP = 2
BG_MAPPING_UV = 0
BG_MAPPING_SPHERICAL = 1
BG_MAPPING_CYLINDRICAL = 2
BG_MAPPING_PLANAR = 3
BG_INTEGRATOR_PATH = 0
BG_INTEGRATOR_WHITTED = 1
BG_INTEGRATOR_DIRECT = 2
BG_LIGHT_UNIFORM_ALL = 0
BG_LIGHT_UNIFORM_ONE = 1
BG_TRI_REVERSE_ORIENTATION = 1
BG_TRI_SWAPS_HANDEDNESS = 2

BG_NOALLOC_MAX_PIXELS = 512 * 512
BG_NOALLOC_WAVE_PATHS = 65536
BG_NOALLOC_SCRATCH_BYTES = 29099008

BG_GUIDE_PARAMS = 28160
BG_GUIDE_QUERY_FLOATS = 9
BG_GUIDE_OUTPUTS = 82
BG_GUIDE_SAMPLE_FLOATS = 16
BG_GUIDE_NO_FALLBACK = 1
BG_GUIDE_NO_TRAIN = 2
BG_GUIDE_NO_CONTINUATION = 4
BG_GUIDE_NO_NEE = 8

F3 = C.c_float * 3


class bg_material(C.Structure):
    _fields_ = [("type", C.c_uint32), ("kd", F3), ("ks", F3), ("roughness", C.c_float),
                ("remap_roughness", C.c_uint32), ("eta", F3), ("k", F3), ("ior", C.c_float),
                ("sigma", C.c_float), ("kd_texture", C.c_uint32), ("ks_texture", C.c_uint32)]


class bg_texture(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("wrap", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("rgb", C.c_void_p), ("mapping", C.c_uint32), ("uv_scale", C.c_float * 2),
                ("uv_delta", C.c_float * 2), ("world_to_texture", C.c_float * 12), ("vs", F3), ("vt", F3),
                ("ds", C.c_float), ("dt", C.c_float)]


class bg_infinite_light(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("rgb", C.c_void_p), ("intensity", F3),
                ("light_to_world", C.c_float * 12)]


class bg_obj_info(C.Structure):
    _fields_ = [("ntri", C.c_size_t), ("has_normals", C.c_uint32), ("has_uvs", C.c_uint32),
                ("flags", C.c_uint32)]


class bg_area_light(C.Structure):
    _fields_ = [("intensity", F3), ("two_sided", C.c_uint32)]


class bg_sphere(C.Structure):
    _fields_ = [("center", F3), ("radius", C.c_float), ("material_id", C.c_uint32),
                ("light_id", C.c_int32)]


class bg_quadric(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("reverse_orientation", C.c_uint32), ("object_to_world", C.c_float * 12),
                ("world_to_object", C.c_float * 12), ("radius", C.c_float), ("inner_radius", C.c_float),
                ("z_min", C.c_float), ("z_max", C.c_float), ("height", C.c_float), ("phi_max_deg", C.c_float),
                ("material_id", C.c_uint32), ("light_id", C.c_int32)]


class bg_camera(C.Structure):
    _fields_ = [("position", F3), ("look_at", F3), ("up", F3), ("fov_deg", C.c_float),
                ("near_plane", C.c_float), ("far_plane", C.c_float), ("lens_radius", C.c_float),
                ("focal_distance", C.c_float), ("width", C.c_uint32), ("height", C.c_uint32)]


class bg_render_opts(C.Structure):
    _fields_ = [("spp", C.c_uint32), ("max_depth", C.c_uint32), ("rr_threshold", C.c_float),
                ("mode", C.c_uint32), ("seed", C.c_uint64), ("first_sample", C.c_uint32),
                ("flags", C.c_uint32), ("integrator", C.c_uint32), ("light_strategy", C.c_uint32),
                ("sampler", C.c_uint32), ("x_pixel_samples", C.c_uint32), ("y_pixel_samples", C.c_uint32),
                ("sampled_dimensions", C.c_uint32), ("jitter_samples", C.c_uint32), ("reserved", C.c_uint32)]


class bg_render_stats(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("trace_ms", C.c_double), ("shadow_ms", C.c_double),
                ("shade_ms", C.c_double), ("samples", C.c_uint64), ("extension_rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("launches", C.c_uint64), ("nan_samples", C.c_uint64),
                ("error_word", C.c_uint32), ("reserved", C.c_uint32)]


class bg_ray(C.Structure):
    _fields_ = [("org", F3), ("tmax", C.c_float), ("dir", F3), ("pad", C.c_float)]


class bg_hit(C.Structure):
    _fields_ = [("prim", C.c_int32), ("t", C.c_float)]


class bg_device_opts(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_queue_paths", C.c_uint32),
                ("memory_cap_bytes", C.c_uint64), ("block_size", C.c_uint32),
                ("reserved", C.c_uint32)]


class bg_tuning(C.Structure):
    _fields_ = [("wave_paths", C.c_uint32), ("blocks_per_sm", C.c_uint32), ("refill", C.c_uint32),
                ("flags", C.c_uint32)]


class bg_build_stats(C.Structure):
    _fields_ = [("build_ms", C.c_double), ("nodes", C.c_uint64), ("prims", C.c_uint64),
                ("device_bytes", C.c_uint64)]


class bg_guide_opts(C.Structure):
    _fields_ = [("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
                ("alpha", C.c_float), ("batch_size", C.c_uint32), ("samples_per_pass", C.c_uint32),
                ("warmup_passes", C.c_uint32), ("flags", C.c_uint32), ("seed", C.c_uint64),
                ("pass_paths", C.c_uint32), ("epochs", C.c_uint32)]


class bg_guide_stats(C.Structure):
    _fields_ = [("passes", C.c_uint32), ("guided_passes", C.c_uint32), ("fallback", C.c_uint32),
                ("adam_steps", C.c_uint32), ("render_ms", C.c_double), ("train_ms", C.c_double),
                ("last_loss", C.c_double), ("relvar_plain", C.c_double), ("relvar_guided", C.c_double),
                ("ms_plain", C.c_double), ("ms_guided", C.c_double), ("records", C.c_uint64),
                ("pool_samples", C.c_uint64)]


class bg_batch_item(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", bg_camera), ("opts", bg_render_opts), ("rgb_out", C.c_void_p)]


P = C.c_void_p
PP = C.POINTER(C.c_void_p)
ST = C.c_int  # bg_status

# name -> (restype, argtypes); the C-ABI surface declared in include/bonsai_gpu.h
SIGNATURES = {
    "bg_create": (ST, [C.POINTER(bg_device_opts), PP]),
    "bg_destroy": (None, [P]),
    "bg_last_error": (C.c_char_p, [P]),
    "bg_status_string": (C.c_char_p, [C.c_int]),
    "bg_flush_l2": (ST, [P]),
    "bg_synchronize": (ST, [P]),
    "bg_scene_create": (ST, [P, PP]),
    "bg_scene_destroy": (None, [P]),
    "bg_scene_add_material": (ST, [P, C.POINTER(bg_material), C.POINTER(C.c_uint32)]),
    "bg_scene_add_area_light": (ST, [P, C.POINTER(bg_area_light), C.POINTER(C.c_uint32)]),
    "bg_scene_add_triangles": (ST, [P, P, C.c_size_t, P, P]),
    "bg_scene_add_triangle_mesh": (ST, [P, P, C.c_size_t, P, P, P, P, C.c_uint32]),
    "bg_scene_add_texture": (ST, [P, C.POINTER(bg_texture), C.POINTER(C.c_uint32)]),
    "bg_scene_add_infinite_light": (ST, [P, C.POINTER(bg_infinite_light)]),
    "bg_scene_add_spheres": (ST, [P, P, C.c_size_t]),
    "bg_scene_add_quadrics": (ST, [P, P, C.c_size_t]),
    "bg_scene_commit": (ST, [P, C.c_uint32, C.POINTER(bg_build_stats)]),
    "bg_render": (ST, [P, P, C.POINTER(bg_camera), C.POINTER(bg_render_opts), P,
                       C.POINTER(bg_render_stats)]),
    "bg_film_moments": (ST, [P, P, P, P]),
    "bg_trace_closest": (ST, [P, P, P, C.c_size_t, P]),
    "bg_trace_any": (ST, [P, P, P, C.c_size_t, P]),
    "bg_trace_closest_device": (ST, [P, P, P, C.c_size_t, P, C.POINTER(C.c_float)]),
    "bg_trace_any_device": (ST, [P, P, P, C.c_size_t, P, C.POINTER(C.c_float)]),
    "bg_device_alloc": (ST, [P, C.c_size_t, PP]),
    "bg_device_free": (ST, [P, P]),
    "bg_memcpy_h2d": (ST, [P, P, P, C.c_size_t]),
    "bg_memcpy_d2h": (ST, [P, P, P, C.c_size_t]),
    "bg_render_noalloc": (ST, [P, C.POINTER(bg_camera), C.POINTER(bg_render_opts), P, P]),
    "bg_get_tuning": (ST, [P, C.POINTER(bg_tuning)]),
    "bg_set_tuning": (ST, [P, C.POINTER(bg_tuning)]),
    "bg_guide_create": (ST, [P, C.POINTER(bg_guide_opts), PP]),
    "bg_guide_destroy": (None, [P]),
    "bg_guide_get_params": (ST, [P, P]),
    "bg_guide_set_params": (ST, [P, P]),
    "bg_guide_set_wait_limit": (ST, [P, C.c_uint64]),
    "bg_guide_forward": (ST, [P, P, C.c_size_t, P]),
    "bg_guide_gradient": (ST, [P, P, C.c_size_t, P, C.POINTER(C.c_float)]),
    "bg_guide_train": (ST, [P, P, C.c_size_t, C.POINTER(C.c_float)]),
    "bg_guide_mixture_eval": (ST, [P, P, P, P, P, C.c_size_t, P]),
    "bg_guide_pool": (ST, [P, P, C.c_size_t, C.POINTER(C.c_size_t)]),
    "bg_guide_time": (ST, [P, P, C.c_size_t, P, C.c_size_t, C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "bg_obj_read": (ST, [C.c_char_p, P, P, C.c_size_t, C.POINTER(C.c_size_t), C.c_char_p, C.c_size_t]),
    "bg_scene_add_obj": (ST, [P, C.c_char_p, P, C.c_uint32, C.c_int32, C.POINTER(C.c_size_t)]),
    "bg_obj_read_mesh": (ST, [C.c_char_p, P, P, P, P, C.c_size_t, C.POINTER(bg_obj_info), C.c_char_p,
                              C.c_size_t]),
    "bg_write_exr": (ST, [C.c_char_p, P, C.c_uint32, C.c_uint32]),
    "bg_film_write_exr": (ST, [P, C.c_char_p]),
    "bg_render_batch": (ST, [P, C.POINTER(bg_batch_item), C.c_size_t, C.POINTER(bg_render_stats)]),
    "bg_render_guided": (ST, [P, P, P, C.POINTER(bg_camera), C.POINTER(bg_render_opts), P,
                              C.POINTER(bg_render_stats), C.POINTER(bg_guide_stats)]),
}

_LIB = None


def load(path: os.PathLike | str | None = None) -> C.CDLL:
    """Load the in-tree libbonsai_gpu.so and declare every entry point.

    Raises OSError when the library has not been built: there is no fallback path.
    """
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise OSError(f"{p} is missing: build it with __graft_entry__.build()")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib
