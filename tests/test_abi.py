"""The C-ABI library loads, exports every symbol include/*.h declares, and rejects invalid
arguments before touching a device (CPU-only: no compute calls)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names.update(re.findall(r"\b(pm_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_the_documented_surface():
    syms = declared_symbols()
    for required in ["pm_create", "pm_run", "pm_get_depth", "pm_get_view_selection", "pm_save_depth",
                     "pm_destroy", "pm_run_batch", "pm_last_error"]:
        assert required in syms


def test_library_exports_every_declared_symbol(engine_lib):
    from patchmatch_cuda_gb300 import _native
    missing = [s for s in declared_symbols() if not hasattr(engine_lib, s)]
    assert not missing, missing
    assert sorted(_native.EXPORTED_SYMBOLS) == declared_symbols()


def test_default_params_mirror_main_cpp(engine_lib):
    from patchmatch_cuda_gb300 import default_params
    p = default_params()
    assert (p.orientation_x, p.orientation_z) == (0.0, 1.0)  # main.cpp:72-76
    assert p.gpu_id == -1                                    # main.cpp:56-59
    assert p.quirks == 1 and p.prefilter == 0
    # slanted planes per pixel are off: one normal for every pixel, as the reference runs
    assert p.planes == 0 and abs(p.plane_depth_step - 0.02) < 1e-7 and abs(p.plane_slope_step - 0.25) < 1e-7


def _views(n=3, w=32, h=24):
    from patchmatch_cuda_gb300 import Image
    imgs = [np.full((h, w), 100, np.uint8) for _ in range(n)]
    K = np.array([[30.0, 0, 16], [0, 30.0, 12], [0, 0, 1]])
    return [Image(K, np.eye(3), np.array([0.1 * i, 0, 0]), imgs[i]) for i in range(n)]


def _create(views, ref_id, **over):
    from patchmatch_cuda_gb300 import _native, default_params
    lib = _native.load_engine()
    p = default_params()
    p.depth_near, p.depth_far = 1.0, 5.0
    for k, v in over.items():
        setattr(p, k, v)
    arr = (_native.PmView * len(views))(*[v.to_view() for v in views])
    h = C.c_void_p()
    st = lib.pm_create(arr, len(views), ref_id, C.byref(p), C.byref(h))
    if st == 0:
        lib.pm_destroy(h)
    return st


@pytest.mark.parametrize("over,status", [
    (dict(half_window=0), 2), (dict(half_window=23), 2), (dict(num_samples=0), 1),
    (dict(num_samples=33), 1), (dict(depth_near=-1.0, depth_far=-1.0), 1), (dict(depth_far=0.5), 1),
    (dict(sp_alpha=0.0), 1), (dict(num_iterations=0), 1), (dict(prefilter=7), 1),
    (dict(prefilter=2, gaussian_sigma=0.0), 1), (dict(precision=5), 1),
    (dict(refine_trials=-1), 1), (dict(refine_trials=257), 1), (dict(refine_trials=4, refine_sigma=0.0), 1),
    (dict(refine_trials=4, refine_sigma=float("inf")), 1),
    (dict(planes=2), 1), (dict(planes=1, plane_depth_step=1.0), 1), (dict(planes=1, plane_depth_step=-0.1), 1),
    (dict(planes=1, plane_slope_step=2.5), 1), (dict(planes=1, plane_slope_step=float("nan")), 1),
])
def test_invalid_parameters_are_rejected(engine_lib, over, status):
    assert _create(_views(), 0, **over) == status


def test_view_count_limits(engine_lib):
    assert _create(_views(1), 0) == 3          # at least 2 images (patchMatch.cu:137-142)
    assert _create(_views(34), 0) == 4         # more than 32 source views
    assert _create(_views(3), 3) == 1          # reference index out of range


def test_bad_camera_and_image(engine_lib):
    v = _views()
    v[1].K = np.full((3, 3), np.nan, np.float32)
    assert _create(v, 0) == 6
    v = _views()
    v[0].K = np.zeros((3, 3), np.float32)      # singular reference K
    v[0].K[2, 2] = 1
    st = _create(v, 0)
    assert st in (6, 10)                        # camera error, or no device on a CPU host


def test_status_strings(engine_lib):
    assert engine_lib.pm_status_string(0) == b"ok"
    assert engine_lib.pm_status_string(2) == b"window size out of range"
    assert engine_lib.pm_status_string(99) == b"unknown status"


def test_fusion_arguments_are_checked_before_the_device(engine_lib):
    """pm_fusion_create rejects bad counts, missing depth maps and cameras without a GPU."""
    from patchmatch_cuda_gb300 import _native
    lib = _native.load_engine()
    d = np.ones((4, 5), np.float32)
    views = (_native.PmDepthView * 2)()
    for v in views:
        v.depth, v.width, v.height = d.ctypes.data, 5, 4
        v.K[:] = [5.0, 0, 2.5, 0, 5.0, 2.0, 0, 0, 1]
        v.R[:] = [1.0, 0, 0, 0, 1, 0, 0, 0, 1]
    h = C.c_void_p()
    assert lib.pm_fusion_create(views, 0, -1, C.byref(h)) == 1
    assert lib.pm_fusion_create(views, 257, -1, C.byref(h)) == 1
    views[1].depth = None
    assert lib.pm_fusion_create(views, 2, -1, C.byref(h)) == 5
    views[1].depth = d.ctypes.data
    views[1].width = 0
    assert lib.pm_fusion_create(views, 2, -1, C.byref(h)) == 5
    views[1].width = 5
    views[1].t[0] = float("nan")
    assert lib.pm_fusion_create(views, 2, -1, C.byref(h)) == 6
    assert lib.pm_fusion_create_from_engines(None, 1, C.byref(h)) == 1
    assert not h.value
    p = _native.PmFuseParams()
    lib.pm_default_fuse_params(C.byref(p))
    assert (p.max_reproj_px, round(p.max_rel_depth, 6), p.min_consistent) == (1.0, 0.01, 2)



def test_struct_mirrors_match_the_library(engine_lib):
    """The ctypes mirrors of the public structs have the library's sizes (a mirror that is too
    small would let pm_get_stats or pm_create read or write past it)."""
    import ctypes as C
    from patchmatch_cuda_gb300 import _native
    sizes = (C.c_size_t * 5)()
    assert engine_lib.pm_struct_sizes(sizes, 5) == 5
    mirrors = [_native.PmView, _native.PmParams, _native.PmStats, _native.PmFuseParams, _native.PmDepthView]
    assert [C.sizeof(m) for m in mirrors] == list(sizes)
