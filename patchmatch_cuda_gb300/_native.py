"""ctypes binding of the engine's C ABI (include/patchmatch_gb300.h).

The shared library is built in-tree by ``patchmatch_cuda_gb300.build``. Loading fails loudly
when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_DIR = Path(__file__).resolve().parent / "lib"
ENGINE_PATH = LIB_DIR / "libpatchmatch_gb300.so"
SCENE_PATH = LIB_DIR / "libpm_scene.so"

PM_OK = 0
STATUS_NAMES = {
    0: "PM_OK", 1: "PM_ERR_INVALID_ARGUMENT", 2: "PM_ERR_WINDOW_SIZE", 3: "PM_ERR_TOO_FEW_VIEWS",
    4: "PM_ERR_TOO_MANY_VIEWS", 5: "PM_ERR_IMAGE", 6: "PM_ERR_CAMERA", 7: "PM_ERR_CUDA",
    8: "PM_ERR_OUT_OF_MEMORY", 9: "PM_ERR_IO", 10: "PM_ERR_NO_DEVICE", 11: "PM_ERR_STATE",
    12: "PM_ERR_UNSUPPORTED", 13: "PM_ERR_SCRATCH_LIMIT",
}

PREFILTER_NONE, PREFILTER_BOX, PREFILTER_GAUSSIAN = 0, 1, 2
PRECISION_FP32, PRECISION_MIXED = 0, 1
SAMPLER_EXACT, SAMPLER_HARDWARE = 0, 1
TEXELS_AUTO, TEXELS_U8, TEXELS_F16, TEXELS_F32 = 0, 1, 2, 4
INIT_RANDOM, INIT_PROPOSAL = 0, 1
DIR_LEFT_TO_RIGHT, DIR_TOP_TO_BOTTOM, DIR_RIGHT_TO_LEFT, DIR_BOTTOM_TO_TOP = 0, 1, 2, 3

# Every symbol include/patchmatch_gb300.h declares.
EXPORTED_SYMBOLS = [
    "pm_default_params", "pm_status_string", "pm_last_error", "pm_create", "pm_destroy", "pm_run",
    "pm_run_async", "pm_synchronize", "pm_run_batch", "pm_get_depth", "pm_get_view_selection",
    "pm_save_depth", "pm_get_stats", "pm_get_stream", "pm_get_size", "pm_init_depth",
    "pm_compute_costs", "pm_run_sweep", "pm_set_depth", "pm_get_costs", "pm_set_costs",
    "pm_get_ref_maps", "pm_get_source_texels", "pm_eval_costs", "pm_sample_source",
    "pm_transpose_layers", "pm_philox", "pm_box_moments_noalloc", "pm_check_reciprocal",
    "pm_gemm_bf16", "pm_gemm_error", "pm_net_create", "pm_net_destroy", "pm_net_num_params",
    "pm_net_get_params", "pm_net_set_params", "pm_net_forward", "pm_net_gradients", "pm_net_train_step",
    "pm_net_layout", "pm_net_size", "pm_set_proposal", "pm_proposal_input", "pm_batch_create",
    "pm_batch_run", "pm_batch_info", "pm_batch_destroy", "pm_texture_peak", "pm_default_fuse_params",
    "pm_fusion_create", "pm_fusion_create_from_engines", "pm_fusion_run", "pm_fusion_info",
    "pm_fusion_get_points", "pm_fusion_get_depth", "pm_fusion_geometry", "pm_fusion_write_ply",
    "pm_fusion_last_error", "pm_fusion_destroy", "pm_refine", "pm_get_slopes", "pm_set_slopes",
    "pm_get_normals", "pm_eval_costs_planes", "pm_struct_sizes",
]

MAX_FUSE_REFS = 256


class PmView(C.Structure):
    _fields_ = [
        ("gray", C.c_void_p), ("width", C.c_int), ("height", C.c_int), ("stride", C.c_int),
        ("K", C.c_float * 9), ("R", C.c_float * 9), ("t", C.c_float * 3),
    ]


class PmParams(C.Structure):
    _fields_ = [
        ("depth_near", C.c_float), ("depth_far", C.c_float), ("half_window", C.c_int),
        ("num_samples", C.c_int), ("sp_alpha", C.c_float), ("gaussian_sigma", C.c_float),
        ("prefilter", C.c_int), ("num_iterations", C.c_int), ("orientation_x", C.c_float),
        ("orientation_z", C.c_float), ("seed", C.c_uint64), ("precision", C.c_int),
        ("init_mode", C.c_int), ("threads_per_line", C.c_int), ("quirks", C.c_int),
        ("gpu_id", C.c_int), ("block_dim_x", C.c_int), ("block_dim_y", C.c_int),
        ("sampler", C.c_int), ("texel_format", C.c_int), ("num_sweeps", C.c_int),
        ("proposal_threshold", C.c_float), ("perturbation", C.c_float), ("refine_trials", C.c_int),
        ("refine_sigma", C.c_float), ("planes", C.c_int), ("plane_depth_step", C.c_float),
        ("plane_slope_step", C.c_float),
    ]


class PmStats(C.Structure):
    _fields_ = [
        ("cost_evals", C.c_ulonglong), ("cost_evals_done", C.c_ulonglong),
        ("ms_prepare", C.c_float), ("ms_init", C.c_float), ("ms_sweeps", C.c_float),
        ("ms_total", C.c_float), ("threads_per_line", C.c_int), ("texel_bytes", C.c_int),
        ("warps_per_line", C.c_int * 4),
    ]


class PmFuseParams(C.Structure):
    _fields_ = [("max_reproj_px", C.c_float), ("max_rel_depth", C.c_float), ("min_consistent", C.c_int)]


class PmDepthView(C.Structure):
    _fields_ = [
        ("depth", C.c_void_p), ("gray", C.c_void_p), ("width", C.c_int), ("height", C.c_int),
        ("K", C.c_float * 9), ("R", C.c_float * 9), ("t", C.c_float * 3),
    ]


class PatchMatchError(RuntimeError):
    def __init__(self, status: int, message: str = ""):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}" if message else STATUS_NAMES.get(status, str(status)))


_lib = None


def load_engine() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not ENGINE_PATH.exists():
        raise RuntimeError(
            f"CUDA engine not built: {ENGINE_PATH} is missing (run python -m patchmatch_cuda_gb300.build)")
    lib = C.CDLL(str(ENGINE_PATH))
    H = C.c_void_p
    P = C.c_void_p
    sig = {
        "pm_default_params": (None, [P]),
        "pm_status_string": (C.c_char_p, [C.c_int]),
        "pm_last_error": (C.c_char_p, [H]),
        "pm_create": (C.c_int, [P, C.c_int, C.c_int, P, C.POINTER(C.c_void_p)]),
        "pm_destroy": (C.c_int, [H]),
        "pm_run": (C.c_int, [H]),
        "pm_run_async": (C.c_int, [H]),
        "pm_synchronize": (C.c_int, [H]),
        "pm_run_batch": (C.c_int, [P, C.c_int]),
        "pm_get_depth": (C.c_int, [H, P, C.c_size_t]),
        "pm_get_view_selection": (C.c_int, [H, P]),
        "pm_save_depth": (C.c_int, [H, C.c_char_p]),
        "pm_get_stats": (C.c_int, [H, P]),
        "pm_get_stream": (C.c_int, [H, C.POINTER(C.c_void_p)]),
        "pm_get_size": (C.c_int, [H, P, P, P]),
        "pm_init_depth": (C.c_int, [H]),
        "pm_compute_costs": (C.c_int, [H, C.c_int]),
        "pm_run_sweep": (C.c_int, [H, C.c_int, C.c_uint32, C.c_int, C.c_int]),
        "pm_refine": (C.c_int, [H, C.c_int, C.c_float, C.c_uint32, C.c_int, C.c_int]),
        "pm_set_depth": (C.c_int, [H, P]),
        "pm_get_costs": (C.c_int, [H, P]),
        "pm_set_costs": (C.c_int, [H, P]),
        "pm_get_ref_maps": (C.c_int, [H, P, P, P]),
        "pm_get_source_texels": (C.c_int, [H, C.c_int, P]),
        "pm_eval_costs": (C.c_int, [H, C.c_int, P, P, P, P, P, P]),
        "pm_eval_costs_planes": (C.c_int, [H, C.c_int, P, P, P, P, P, P, P]),
        "pm_get_slopes": (C.c_int, [H, P]),
        "pm_set_slopes": (C.c_int, [H, P]),
        "pm_get_normals": (C.c_int, [H, P]),
        "pm_sample_source": (C.c_int, [H, C.c_int, C.c_int, P, P, P]),
        "pm_transpose_layers": (C.c_int, [P, C.c_size_t, P, C.c_size_t, C.c_int, C.c_int, C.c_int, P]),
        "pm_philox": (C.c_int, [C.c_uint64, C.c_int, P, P]),
        "pm_check_reciprocal": (C.c_int, [C.c_int, P]),
        "pm_struct_sizes": (C.c_int, [P, C.c_int]),
        "pm_gemm_bf16": (C.c_int, [P, C.c_int, P, C.c_int, C.c_int, C.c_int, C.c_int, P, C.c_int, C.c_int, P,
                                   C.c_int, C.c_int, P]),
        "pm_gemm_error": (C.c_int, [P, C.c_int]),
        "pm_net_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_uint64, P]),
        "pm_net_destroy": (C.c_int, [P]),
        "pm_net_num_params": (C.c_int, [P, P]),
        "pm_net_get_params": (C.c_int, [P, P, C.c_size_t]),
        "pm_net_set_params": (C.c_int, [P, P, C.c_size_t]),
        "pm_net_forward": (C.c_int, [P, P, P, P]),
        "pm_net_gradients": (C.c_int, [P, P, P, C.c_float, C.c_float, P, C.c_size_t, P]),
        "pm_net_train_step": (C.c_int, [P, P, P, C.c_float, C.c_float, C.c_float, P]),
        "pm_net_layout": (C.c_int, [P, P, P, C.c_int]),
        "pm_net_size": (C.c_int, [P, P, P, P]),
        "pm_set_proposal": (C.c_int, [H, P]),
        "pm_proposal_input": (C.c_int, [H, P, P, P]),
        "pm_batch_create": (C.c_int, [P, C.c_int, P]),
        "pm_batch_run": (C.c_int, [P]),
        "pm_batch_info": (C.c_int, [P, P, P, P, C.c_int]),
        "pm_batch_destroy": (C.c_int, [P]),
        "pm_texture_peak": (C.c_int, [P]),
        "pm_default_fuse_params": (None, [P]),
        "pm_fusion_create": (C.c_int, [P, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
        "pm_fusion_create_from_engines": (C.c_int, [P, C.c_int, C.POINTER(C.c_void_p)]),
        "pm_fusion_run": (C.c_int, [P, P]),
        "pm_fusion_info": (C.c_int, [P, P, P, P, P]),
        "pm_fusion_get_points": (C.c_int, [P, P, C.c_int64]),
        "pm_fusion_get_depth": (C.c_int, [P, C.c_int, P, P]),
        "pm_fusion_geometry": (C.c_int, [P, P, P]),
        "pm_fusion_write_ply": (C.c_int, [P, C.c_char_p]),
        "pm_fusion_last_error": (C.c_char_p, [P]),
        "pm_fusion_destroy": (C.c_int, [P]),
        "pm_box_moments_noalloc": (C.c_int, [P, C.c_size_t, C.c_int, C.c_int, C.c_int, P, P, P, C.c_size_t, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


_scene = None


def load_scene() -> C.CDLL:
    global _scene
    if _scene is not None:
        return _scene
    if not SCENE_PATH.exists():
        raise RuntimeError(f"scene generator not built: {SCENE_PATH} is missing")
    lib = C.CDLL(str(SCENE_PATH))
    P = C.c_void_p
    lib.pm_scene_create.restype = C.c_void_p
    lib.pm_scene_create.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                    C.c_int, C.c_double]
    lib.pm_scene_destroy.restype = None
    lib.pm_scene_destroy.argtypes = [P]
    lib.pm_scene_camera.restype = None
    lib.pm_scene_camera.argtypes = [P, C.c_double, C.c_double, C.c_int, C.c_int, C.c_double, P, P, P]
    lib.pm_scene_render.restype = C.c_int
    lib.pm_scene_render.argtypes = [P, P, P, P, C.c_int, C.c_int, P, P]
    lib.pm_scene_pivot_depth.restype = C.c_double
    lib.pm_scene_pivot_depth.argtypes = [P]
    _scene = lib
    return lib


def check(status: int, handle=None) -> None:
    if status != PM_OK:
        msg = ""
        if handle is not None and _lib is not None:
            raw = _lib.pm_last_error(handle)
            msg = raw.decode() if raw else ""
        raise PatchMatchError(status, msg)
