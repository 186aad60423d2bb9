"""ctypes binding of the skyfall C-ABI (include/skyfall.h).

Loads the in-tree libskyfall.so built by skyfall.build.  There is no CPU
fallback: if the library is missing or no CUDA device is present, calls
raise SkyError.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

SKY_OK = 0
SKY_ERR_ARG = -1
SKY_ERR_OOM = -2
SKY_ERR_CUDA = -3
SKY_ERR_TIMEOUT = -4
SKY_ERR_CAPACITY = -5
SKY_ERR_STATE = -6
SKY_ERR_INJECTED = -7

SKY_PLANE_POS = 0
SKY_PLANE_LOGSCALE = 3
SKY_PLANE_ROT = 6
SKY_PLANE_OPACITY = 10
SKY_PLANE_SH = 11
SKY_NUM_PLANES = 59

SKY_BWD_EXACT = 0
SKY_BWD_REFERENCE = 1

BUF = dict(
    records=1, counts=2, cumsum=3, keys_emit=4, keys_sorted=5, vals_sorted=6, flatten=7,
    tile_offsets=8, color=9, alpha=10, last_ids=11, residual=12, partials=13, tile_grads=14,
    grads=15, groups=16, step_scalars=17, depth_radius=18, view_rgba=19, item_order=20,
    pair_counts=21,
)
BUF_DTYPE = dict(
    records=np.float32, counts=np.uint32, cumsum=np.uint32, keys_emit=np.uint32,
    keys_sorted=np.uint32, vals_sorted=np.uint32, flatten=np.uint32, tile_offsets=np.uint32,
    color=np.float32, alpha=np.float32, last_ids=np.uint32, residual=np.float32,
    partials=np.float32, tile_grads=np.int32, grads=np.float32, groups=np.uint32,
    step_scalars=np.float32, depth_radius=np.float32, view_rgba=np.float32, item_order=np.uint32,
    pair_counts=np.uint64,
)

ERROR_NAMES = {
    SKY_ERR_ARG: "SKY_ERR_ARG", SKY_ERR_OOM: "SKY_ERR_OOM", SKY_ERR_CUDA: "SKY_ERR_CUDA",
    SKY_ERR_TIMEOUT: "SKY_ERR_TIMEOUT", SKY_ERR_CAPACITY: "SKY_ERR_CAPACITY",
    SKY_ERR_STATE: "SKY_ERR_STATE", SKY_ERR_INJECTED: "SKY_ERR_INJECTED",
}


class SkyError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


class SkyCamera(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("proj", C.c_float * 16), ("focal", C.c_float * 2),
                ("width", C.c_uint32), ("height", C.c_uint32)]


class SkyConfig(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("tile_size", C.c_uint32), ("sh_degree", C.c_uint32),
        ("sh_degree_interval", C.c_uint32), ("near_plane", C.c_float), ("far_plane", C.c_float),
        ("radius_clip", C.c_float), ("eps2d", C.c_float), ("background", C.c_float * 3),
        ("w_l2", C.c_float), ("w_l1", C.c_float), ("w_ssim", C.c_float),
        ("lr_means", C.c_float), ("lr_means_final", C.c_float), ("lr_means_delay_mult", C.c_float),
        ("lr_means_max_steps", C.c_uint32), ("lr_sh", C.c_float), ("lr_opacity", C.c_float),
        ("lr_scale", C.c_float), ("lr_rotation", C.c_float), ("beta1", C.c_float),
        ("beta2", C.c_float), ("adam_eps", C.c_float), ("sh_update_interval", C.c_uint32),
        ("round_params_f16", C.c_uint32), ("backward_mode", C.c_uint32), ("use_graph", C.c_uint32),
        ("max_views_per_step", C.c_uint32), ("seed", C.c_uint64),
        ("fwd_batch", C.c_uint32), ("bwd_batch", C.c_uint32), ("tile_cull", C.c_uint32),
        ("batch_scaling", C.c_uint32),
    ]


class SkyStepStats(C.Structure):
    _fields_ = [("iteration", C.c_uint64), ("num_intersections", C.c_uint64), ("loss", C.c_double),
                ("num_gaussians", C.c_uint32), ("num_views", C.c_uint32), ("sh_degree", C.c_uint32),
                ("sh_updated", C.c_uint32)]


class SkyStatus(C.Structure):
    _fields_ = [("iteration", C.c_uint64), ("adam_steps", C.c_uint64),
                ("last_intersections", C.c_uint64), ("device_bytes", C.c_uint64),
                ("num_gaussians", C.c_uint32), ("capacity", C.c_uint32), ("num_cameras", C.c_uint32),
                ("error_flags", C.c_uint32), ("kernel_launches", C.c_uint64),
                ("graph_replays", C.c_uint64), ("graph_captures", C.c_uint64),
                ("scene_extent", C.c_float), ("scored_views", C.c_uint32),
                ("densify_runs", C.c_uint32), ("prune_runs", C.c_uint32),
                ("step_h2d_bytes", C.c_uint64), ("step_d2h_bytes", C.c_uint64)]


STAGES = ["preprocess", "scan", "emit", "sort", "ranges", "forward", "backward", "geom_adam"]


class SkyPruneParams(C.Structure):
    _fields_ = [("min_opacity", C.c_float), ("max_scale", C.c_float), ("max_remove_ratio", C.c_float),
                ("reserved", C.c_uint32)]


class SkyDensifyParams(C.Structure):
    _fields_ = [("grad_threshold", C.c_float), ("grad_abs_threshold", C.c_float),
                ("size_threshold", C.c_float), ("min_visibility", C.c_float),
                ("importance_threshold", C.c_float), ("max_new_ratio", C.c_float),
                ("pixel_width", C.c_float), ("reserved", C.c_uint32)]


class SkyScoredPruneParams(C.Structure):
    _fields_ = [("min_opacity", C.c_float), ("max_scale", C.c_float),
                ("max_screen_radius", C.c_float), ("use_screen_size", C.c_uint32),
                ("prune_ratio", C.c_float), ("max_ratio", C.c_float),
                ("opacity_bonus", C.c_float), ("scale_bonus", C.c_float),
                ("screen_bonus", C.c_float), ("use_last_scores", C.c_uint32)]


class SkySchedule(C.Structure):
    _fields_ = [("enabled", C.c_uint32), ("densify_from", C.c_uint32),
                ("densify_until", C.c_uint32), ("densify_interval", C.c_uint32),
                ("prune_from", C.c_uint32), ("prune_until", C.c_uint32),
                ("prune_interval", C.c_uint32), ("opacity_reset_interval", C.c_uint32),
                ("opacity_reset_value", C.c_float), ("min_opacity", C.c_float),
                ("max_screen_size", C.c_float), ("max_scale_ratio", C.c_float),
                ("max_scale_absolute", C.c_float), ("scene_extent", C.c_float),
                ("densify", SkyDensifyParams)]


class SkyViewSettings(C.Structure):
    _fields_ = [("gaussian_scaling", C.c_float), ("sh_degree", C.c_uint32),
                ("round_params_f16", C.c_uint32), ("reserved", C.c_uint32)]


P = C.c_void_p
U32 = C.c_uint32
U64 = C.c_uint64
I32 = C.c_int

# name -> (restype, argtypes)
PROTOTYPES = {
    "sky_version": (I32, []),
    "sky_last_error": (C.c_char_p, []),
    "sky_config_default": (None, [C.POINTER(SkyConfig)]),
    "sky_create": (I32, [C.POINTER(SkyConfig), C.POINTER(C.c_void_p)]),
    "sky_destroy": (I32, [P]),
    "sky_set_config": (I32, [P, C.POINTER(SkyConfig)]),
    "sky_get_config": (I32, [P, C.POINTER(SkyConfig)]),
    "sky_camera_pinhole": (I32, [P, C.c_double, C.c_double, C.c_double, C.c_double, U32, U32,
                                 C.POINTER(SkyCamera)]),
    "sky_load_points": (I32, [P, P, U32, U64]),
    "sky_load_packed": (I32, [P, P, P, U32]),
    "sky_load_ply": (I32, [P, C.c_char_p, C.POINTER(U32), C.POINTER(U32)]),
    "sky_save_ply": (I32, [P, C.c_char_p, U32]),
    "sky_ply_read_host": (I32, [C.c_char_p, C.POINTER(U32), C.POINTER(U32), P, U64,
                                C.POINTER(C.c_double)]),
    "sky_save_checkpoint": (I32, [P, C.c_char_p]),
    "sky_load_checkpoint": (I32, [P, C.c_char_p]),
    "sky_knn_init": (I32, [P, C.c_float, P]),
    "sky_set_cameras": (I32, [P, C.POINTER(SkyCamera), U32]),
    "sky_set_target": (I32, [P, U32, P, U32, U32]),
    "sky_render": (I32, [P, P, U32, P, P]),
    "sky_forward": (I32, [P, P, U32, C.POINTER(C.c_double)]),
    "sky_backward": (I32, [P, P, U64]),
    "sky_step": (I32, [P, P, U32, C.POINTER(SkyStepStats)]),
    "sky_train": (I32, [P, U32, U32, C.POINTER(SkyStepStats)]),
    "sky_prune": (I32, [P, C.POINTER(SkyPruneParams), P, C.POINTER(U32)]),
    "sky_densify_stats": (I32, [P, P, P]),
    "sky_densify": (I32, [P, C.POINTER(SkyDensifyParams), C.POINTER(U32), C.POINTER(U32)]),
    "sky_densify_default": (None, [C.POINTER(SkyDensifyParams)]),
    "sky_score_views": (I32, [P, P, U32, P, P]),
    "sky_scored_prune_default": (None, [C.POINTER(SkyScoredPruneParams)]),
    "sky_prune_scored": (I32, [P, C.POINTER(SkyScoredPruneParams), C.POINTER(U32)]),
    "sky_schedule_default": (None, [C.POINTER(SkySchedule)]),
    "sky_set_schedule": (I32, [P, C.POINTER(SkySchedule)]),
    "sky_reset_opacity": (I32, [P, C.c_float]),
    "sky_view_settings_default": (None, [C.POINTER(SkyViewSettings)]),
    "sky_view_render": (I32, [P, C.POINTER(SkyCamera), C.POINTER(SkyViewSettings), P, P]),
    "sky_get_params": (I32, [P, P, U64]),
    "sky_get_moments": (I32, [P, P, P, U64]),
    "sky_get_count": (I32, [P, C.POINTER(U32)]),
    "sky_get_status": (I32, [P, C.POINTER(SkyStatus)]),
    "sky_read_buffer": (I32, [P, I32, P, U64, C.POINTER(U64)]),
    "sky_sync": (I32, [P]),
    "sky_sort_pairs": (I32, [P, P, P, P, U32, U32, P]),
    "sky_sort_pairs_noalloc": (I32, [P, P, P, P, U32, U32, P]),
    "sky_get_stream": (I32, [P, C.POINTER(C.c_void_p)]),
    "sky_set_profiling": (I32, [P, I32]),
    "sky_get_stage_times": (I32, [P, C.POINTER(C.c_double), U32, C.POINTER(U64)]),
}

LIB_PATH = Path(__file__).resolve().parent / "libskyfall.so"
_lib = None


def lib():
    """The loaded library (loading it on first use)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise SkyError(SKY_ERR_STATE, f"{LIB_PATH} is not built; run skyfall.build.build()")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != SKY_OK:
        msg = lib().sky_last_error().decode(errors="replace")
        raise SkyError(rc, msg)


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def read_ply(path) -> tuple[np.ndarray, int, float]:
    """The PLY import into host memory (no GPU needed): ((59, N) f32 planes,
    SH degree of the file, scene extent)."""
    n, d, ext = C.c_uint32(), C.c_uint32(), C.c_double()
    b = str(path).encode()
    check(lib().sky_ply_read_host(b, C.byref(n), C.byref(d), None, 0, C.byref(ext)))
    planes = np.empty((SKY_NUM_PLANES, n.value), np.float32)
    check(lib().sky_ply_read_host(b, C.byref(n), C.byref(d), ptr(planes), planes.size, C.byref(ext)))
    return planes, d.value, ext.value


def default_config(**overrides) -> SkyConfig:
    cfg = SkyConfig()
    lib().sky_config_default(C.byref(cfg))
    for k, v in overrides.items():
        if k == "background":
            cfg.background = (C.c_float * 3)(*v)
        else:
            setattr(cfg, k, v)
    return cfg
