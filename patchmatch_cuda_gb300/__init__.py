"""GB300-native PatchMatch multi-view stereo.

Python mirror of the reference's driver surface (yhsa678/patchMatch_cuda):

    images = read_middlebury("scene_par.txt")              # image.cpp:64-93
    pm = PatchMatch(images, near, far, half_window, 32, 16, ref_id, num_samples,
                    sp_alpha, gaussian_sigma, num_iterations, orientation_x, orientation_z)
    pm.runPatchMatch()                                       # patchMatch.cu:263-407
    pm.depth_map                                             # _depthMap, H x W float32
    pm.save_to_file("depth.bin")                             # array2d_wrapper.h:51-70

All compute runs in the CUDA engine (lib/libpatchmatch_gb300.so) through its C ABI.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path
from typing import Sequence

import numpy as np

from . import _native
from ._native import (DIR_BOTTOM_TO_TOP, DIR_LEFT_TO_RIGHT, DIR_RIGHT_TO_LEFT, DIR_TOP_TO_BOTTOM,
                      PRECISION_FP32, PRECISION_MIXED, PREFILTER_BOX, PREFILTER_GAUSSIAN,
                      PREFILTER_NONE, INIT_PROPOSAL, INIT_RANDOM, PatchMatchError, PmFuseParams, PmParams,
                      PmStats, PmView)

__all__ = [
    "Image", "PatchMatch", "Engine", "Batch", "Fusion", "default_fuse_params", "run_batch", "read_middlebury", "read_nvm", "read_pnm", "write_pgm", "default_params",
    "load_depth_file", "PatchMatchError", "PREFILTER_NONE", "PREFILTER_BOX", "PREFILTER_GAUSSIAN",
    "PRECISION_FP32", "PRECISION_MIXED", "DIR_LEFT_TO_RIGHT", "DIR_TOP_TO_BOTTOM",
    "DIR_RIGHT_TO_LEFT", "DIR_BOTTOM_TO_TOP", "INIT_RANDOM", "INIT_PROPOSAL",
]


class Image:
    """One calibrated view: Image::updateCamParam (image.cpp:39-61).

    K, R (3x3) and T (3,) with pixel ~ K (R X + T); image is an HxW uint8 array."""

    def __init__(self, K=None, R=None, T=None, image=None):
        if K is not None:
            self.update_cam_param(K, R, T, image)

    def update_cam_param(self, K, R, T, image) -> None:
        self.K = np.asarray(K, np.float32).reshape(3, 3)
        self.R = np.asarray(R, np.float32).reshape(3, 3)
        self.T = np.asarray(T, np.float32).reshape(3)
        img = np.asarray(image)
        if img.ndim == 3:  # BGR to gray with BT.601 luma weights (cvtColor BGR2GRAY)
            b, g, r = (img[..., i].astype(np.uint32) for i in range(3))
            img = ((r * 4899 + g * 9617 + b * 1868 + 8192) >> 14).astype(np.uint8)
        self.image = np.ascontiguousarray(img, dtype=np.uint8)
        self.C = -self.R.T @ self.T
        self.proj = self.K @ np.concatenate([self.R, self.T[:, None]], axis=1)

    updateCamParam = update_cam_param

    def to_view(self) -> PmView:
        v = PmView()
        v.gray = self.image.ctypes.data
        v.height, v.width = self.image.shape
        v.stride = self.image.strides[0]
        v.K[:] = [float(x) for x in self.K.ravel()]
        v.R[:] = [float(x) for x in self.R.ravel()]
        v.t[:] = [float(x) for x in self.T.ravel()]
        return v


def read_pnm(path) -> np.ndarray:
    """8-bit binary PGM (P5) or PPM (P6, converted to gray)."""
    data = Path(path).read_bytes()
    tokens, pos = [], 0
    while len(tokens) < 4:
        while data[pos:pos + 1].isspace():
            pos += 1
        if data[pos:pos + 1] == b"#":
            pos = data.index(b"\n", pos) + 1
            continue
        end = pos
        while not data[end:end + 1].isspace():
            end += 1
        tokens.append(data[pos:end])
        pos = end
    magic, w, h, mx = tokens[0], int(tokens[1]), int(tokens[2]), int(tokens[3])
    pos += 1
    if mx != 255 or magic not in (b"P5", b"P6"):
        raise ValueError(f"{path}: only 8-bit P5/P6 images are supported")
    ch = 1 if magic == b"P5" else 3
    arr = np.frombuffer(data, np.uint8, w * h * ch, pos)
    if ch == 1:
        return arr.reshape(h, w).copy()
    rgb = arr.reshape(h, w, 3).astype(np.uint32)
    return ((rgb[..., 0] * 4899 + rgb[..., 1] * 9617 + rgb[..., 2] * 1868 + 8192) >> 14).astype(np.uint8)


def write_pgm(path, img: np.ndarray) -> None:
    img = np.ascontiguousarray(img, dtype=np.uint8)
    Path(path).write_bytes(b"P5\n%d %d\n255\n" % (img.shape[1], img.shape[0]) + img.tobytes())


def read_middlebury(path) -> list[Image]:
    """readMiddleBurry (image.cpp:64-93): image count, then per image
    '<file> k11..k33 r11..r33 t1 t2 t3'. Image paths resolve against the list's folder."""
    path = Path(path)
    toks = path.read_text().split()
    n = int(toks[0])
    out, i = [], 1
    for _ in range(n):
        name = toks[i]
        vals = [float(x) for x in toks[i + 1:i + 22]]
        i += 22
        p = Path(name)
        if not p.exists():
            p = path.parent / name
        out.append(Image(np.array(vals[0:9]), np.array(vals[9:18]), np.array(vals[18:21]), read_pnm(p)))
    return out


def read_nvm(path) -> tuple[list[Image], list[tuple[float, float] | None]]:
    """readNVM (image.cpp:130-245) with the per-camera depth ranges returned (the reference
    fills a by-value copy and loses them). 'NVM_V3', the camera count (> 1), per camera
    '<file> f qw qx qy qz cx cy cz d0 d1' (quaternion to R as image.cpp:95-118, T = -R C as
    image.cpp:122-128, K = [f 0 W/2; 0 f H/2; 0 0 1]), then the 3D points, each
    'x y z r g b n' followed by n projections 'camera feature u v'. A camera's range spans
    the positive depths of the points it sees, widened by a quarter of its size on both sides
    (the near side by less while it would reach zero, image.cpp:222-235); a camera that sees
    no point has None. Raises ValueError for a file that is not NVM_V3."""
    path = Path(path)
    toks = path.read_text().split()
    if not toks or not toks[0].startswith("NVM_V3"):
        raise ValueError(f"{path}: not an NVM_V3 file")
    ncam = int(toks[1])
    if ncam <= 1:
        raise ValueError(f"{path}: an NVM_V3 file needs at least two cameras")
    out, i = [], 2
    for _ in range(ncam):
        name = toks[i]
        f = float(toks[i + 1])
        q = [float(x) for x in toks[i + 2:i + 6]]
        c = [float(x) for x in toks[i + 6:i + 9]]
        i += 11
        # scalar double arithmetic in the reference's order, so the C++ reader agrees bit for bit
        qq = math.sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3])
        w, x, y, z = (q[0] / qq, q[1] / qq, q[2] / qq, q[3] / qq) if qq > 0 else (1.0, 0.0, 0.0, 0.0)
        R = [w * w + x * x - z * z - y * y, 2 * x * y - 2 * z * w, 2 * y * w + 2 * z * x,
             2 * x * y + 2 * w * z, y * y + w * w - z * z - x * x, 2 * z * y - 2 * x * w,
             2 * x * z - 2 * y * w, 2 * y * z + 2 * w * x, z * z + w * w - y * y - x * x]
        T = [-(R[3 * r] * c[0] + R[3 * r + 1] * c[1] + R[3 * r + 2] * c[2]) for r in range(3)]
        p = Path(name)
        if not p.exists():
            p = path.parent / name
        img = read_pnm(p)
        h, wd = img.shape
        K = np.array([[f, 0.0, wd / 2.0], [0.0, f, h / 2.0], [0.0, 0.0, 1.0]])
        out.append(Image(K, R, T, img))
    npoint = int(toks[i])
    i += 1
    if npoint <= 0:
        raise ValueError(f"{path}: no 3D points")
    lo = np.full(ncam, np.inf, np.float32)
    hi = np.full(ncam, -np.inf, np.float32)
    for _ in range(npoint):
        pt = [float(np.float32(v)) for v in toks[i:i + 3]]
        npj = int(toks[i + 6])
        i += 7
        for _ in range(npj):
            cidx = int(toks[i])
            i += 4
            if not 0 <= cidx < ncam:
                raise ValueError(f"{path}: projection names camera {cidx} of {ncam}")
            im = out[cidx]
            r2 = [float(v) for v in im.R[2]]
            depth = np.float32(r2[0] * pt[0] + r2[1] * pt[1] + r2[2] * pt[2] + float(im.T[2]))
            if depth <= 0:
                continue
            lo[cidx] = min(lo[cidx], depth)
            hi[cidx] = max(hi[cidx], depth)
    ranges: list[tuple[float, float] | None] = []
    for a, b in zip(lo, hi):
        if a > b:
            ranges.append(None)
            continue
        size = np.float32(b - a)
        ratio = np.float32(0.25)
        near = np.float32(a - ratio * size)
        while near <= 0:
            ratio = np.float32(ratio / np.float32(1.1))
            near = np.float32(a - ratio * size)
        ranges.append((float(near), float(np.float32(b + np.float32(0.25) * size))))
    return out, ranges


def write_middlebury(path, names: Sequence[str], images: Sequence[Image]) -> None:
    lines = [str(len(images))]
    for name, im in zip(names, images):
        vals = list(im.K.ravel()) + list(im.R.ravel()) + list(im.T.ravel())
        lines.append(name + " " + " ".join(repr(float(v)) for v in vals))
    Path(path).write_text("\n".join(lines) + "\n")


def load_depth_file(path) -> np.ndarray:
    """Reads the '<W>&<H>&<D>&' + raw float32 format written by saveToFile."""
    data = Path(path).read_bytes()
    parts = data.split(b"&", 3)
    w, h, d = int(parts[0]), int(parts[1]), int(parts[2])
    return np.frombuffer(parts[3], np.float32, w * h * d).reshape(d, h, w).squeeze(0) if d == 1 else \
        np.frombuffer(parts[3], np.float32, w * h * d).reshape(d, h, w)


def default_params() -> PmParams:
    p = PmParams()
    _native.load_engine().pm_default_params(C.byref(p))
    return p


class Engine:
    """Owns one pm_handle: every entry point of the C ABI as a method."""

    def __init__(self, images: Sequence[Image], ref_id: int, params: PmParams):
        self._lib = _native.load_engine()
        self.images = list(images)
        self.ref_id = ref_id
        self.params = params
        views = (PmView * len(self.images))(*[im.to_view() for im in self.images])
        h = C.c_void_p()
        st = self._lib.pm_create(views, len(self.images), ref_id, C.byref(params), C.byref(h))
        _native.check(st)
        self.h = h
        w, hh, v = C.c_int(), C.c_int(), C.c_int()
        self._lib.pm_get_size(self.h, C.byref(w), C.byref(hh), C.byref(v))
        self.width, self.height, self.n_src = w.value, hh.value, v.value

    def close(self) -> None:
        if getattr(self, "h", None):
            self._lib.pm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _chk(self, st):
        _native.check(st, self.h)

    def run(self) -> None:
        self._chk(self._lib.pm_run(self.h))

    def run_async(self) -> None:
        self._chk(self._lib.pm_run_async(self.h))

    def synchronize(self) -> None:
        self._chk(self._lib.pm_synchronize(self.h))

    def depth(self) -> np.ndarray:
        out = np.empty((self.height, self.width), np.float32)
        self._chk(self._lib.pm_get_depth(self.h, out.ctypes.data, 0))
        return out

    def view_selection(self) -> np.ndarray:
        out = np.empty((self.params.num_samples, self.height, self.width), np.uint8)
        self._chk(self._lib.pm_get_view_selection(self.h, out.ctypes.data))
        return out

    def save_depth(self, path) -> None:
        self._chk(self._lib.pm_save_depth(self.h, str(path).encode()))

    def proposal_shape(self) -> tuple:
        """(height, width) of the learned proposal's network input for this reference."""
        hh, ww = C.c_int(), C.c_int()
        self._chk(self._lib.pm_proposal_input(self.h, None, C.byref(hh), C.byref(ww)))
        return hh.value, ww.value

    def proposal_input(self, d_out: int) -> None:
        """Writes the network input (FP32 [height][width][17]) to DEVICE address d_out."""
        self._chk(self._lib.pm_proposal_input(self.h, C.c_void_p(d_out), None, None))

    def set_proposal(self, net) -> None:
        """Attaches a proposal network (patchmatch_cuda_gb300.proposal.ProposalNet sized for
        this reference, batch 1) used by runs with init_mode = INIT_PROPOSAL; None detaches."""
        self._proposal = net
        self._chk(self._lib.pm_set_proposal(self.h, net.h if net is not None else None))

    def stats(self) -> PmStats:
        s = PmStats()
        self._chk(self._lib.pm_get_stats(self.h, C.byref(s)))
        return s

    def stream(self) -> int:
        s = C.c_void_p()
        self._chk(self._lib.pm_get_stream(self.h, C.byref(s)))
        return s.value or 0

    def init_depth(self) -> None:
        self._chk(self._lib.pm_init_depth(self.h))

    def compute_costs(self, axis: int = 1) -> None:
        self._chk(self._lib.pm_compute_costs(self.h, axis))

    def run_sweep(self, direction: int, sweep_id: int, num_samples: int = 0, record_views: bool = False) -> None:
        self._chk(self._lib.pm_run_sweep(self.h, direction, sweep_id, num_samples, int(record_views)))

    def refine(self, trials: int = 10, sigma: float = 0.05, sweep_id: int = 0, num_samples: int = 0,
               axis: int = 0) -> None:
        """pm_refine: depth refinement on the view-selection map's sampled views."""
        self._chk(self._lib.pm_refine(self.h, trials, sigma, sweep_id, num_samples, axis))

    def set_depth(self, depth: np.ndarray) -> None:
        d = np.ascontiguousarray(depth, np.float32)
        assert d.shape == (self.height, self.width)
        self._chk(self._lib.pm_set_depth(self.h, d.ctypes.data))

    def costs(self) -> np.ndarray:
        out = np.empty((self.height, self.width, self.n_src), np.float32)
        self._chk(self._lib.pm_get_costs(self.h, out.ctypes.data))
        return out

    def set_costs(self, costs: np.ndarray) -> None:
        c = np.ascontiguousarray(costs, np.float32)
        assert c.shape == (self.height, self.width, self.n_src)
        self._chk(self._lib.pm_set_costs(self.h, c.ctypes.data))

    def ref_maps(self):
        ref = np.empty((self.height, self.width), np.float32)
        si, sii = np.empty_like(ref), np.empty_like(ref)
        self._chk(self._lib.pm_get_ref_maps(self.h, ref.ctypes.data, si.ctypes.data, sii.ctypes.data))
        return ref, si, sii

    def source_texels(self, view: int) -> np.ndarray:
        src = [im for i, im in enumerate(self.images) if i != self.ref_id][view]
        out = np.empty(src.image.shape, np.float32)
        self._chk(self._lib.pm_get_source_texels(self.h, view, out.ctypes.data))
        return out

    def eval_costs(self, xs, ys, views, depths, axes) -> np.ndarray:
        xs = np.ascontiguousarray(xs, np.int32).ravel()
        ys = np.ascontiguousarray(np.broadcast_to(ys, xs.shape), np.int32)
        vs = np.ascontiguousarray(np.broadcast_to(views, xs.shape), np.int32)
        ds = np.ascontiguousarray(np.broadcast_to(depths, xs.shape), np.float32)
        ax = np.ascontiguousarray(np.broadcast_to(axes, xs.shape), np.int32)
        out = np.empty(xs.shape, np.float32)
        self._chk(self._lib.pm_eval_costs(self.h, xs.size, xs.ctypes.data, ys.ctypes.data, vs.ctypes.data,
                                          ds.ctypes.data, ax.ctypes.data, out.ctypes.data))
        return out

    # ---- slanted-plane mode (params.planes = 1) ---------------------------------------------
    def slopes(self) -> np.ndarray:
        """Per-pixel plane slopes (a, b), normal ~ (a, b, 1): (height, width, 2) float32."""
        out = np.empty((self.height, self.width, 2), np.float32)
        self._chk(self._lib.pm_get_slopes(self.h, out.ctypes.data))
        return out

    def set_slopes(self, slopes: np.ndarray) -> None:
        s = np.ascontiguousarray(slopes, np.float32)
        assert s.shape == (self.height, self.width, 2)
        self._chk(self._lib.pm_set_slopes(self.h, s.ctypes.data))

    def normals(self) -> np.ndarray:
        """Unit plane normals in the reference camera: (height, width, 3) float32."""
        out = np.empty((self.height, self.width, 3), np.float32)
        self._chk(self._lib.pm_get_normals(self.h, out.ctypes.data))
        return out

    def eval_costs_planes(self, xs, ys, views, depths, slopes, axes) -> np.ndarray:
        xs = np.ascontiguousarray(xs, np.int32).ravel()
        ys = np.ascontiguousarray(np.broadcast_to(ys, xs.shape), np.int32)
        vs = np.ascontiguousarray(np.broadcast_to(views, xs.shape), np.int32)
        ds = np.ascontiguousarray(np.broadcast_to(depths, xs.shape), np.float32)
        sl = np.ascontiguousarray(np.broadcast_to(slopes, xs.shape + (2,)), np.float32)
        ax = np.ascontiguousarray(np.broadcast_to(axes, xs.shape), np.int32)
        out = np.empty(xs.shape, np.float32)
        self._chk(self._lib.pm_eval_costs_planes(self.h, xs.size, xs.ctypes.data, ys.ctypes.data, vs.ctypes.data,
                                                 ds.ctypes.data, sl.ctypes.data, ax.ctypes.data, out.ctypes.data))
        return out

    def sample_source(self, view: int, xs, ys) -> np.ndarray:
        xs = np.ascontiguousarray(xs, np.float32).ravel()
        ys = np.ascontiguousarray(np.broadcast_to(ys, xs.shape), np.float32)
        out = np.empty(xs.shape, np.float32)
        self._chk(self._lib.pm_sample_source(self.h, view, xs.size, xs.ctypes.data, ys.ctypes.data,
                                             out.ctypes.data))
        return out


def run_batch(engines: Sequence[Engine]) -> None:
    lib = _native.load_engine()
    arr = (C.c_void_p * len(engines))(*[e.h for e in engines])
    _native.check(lib.pm_run_batch(arr, len(engines)))


class Batch:
    """A reusable batch of engines (pm_batch): tuned warps per line, schedule captured as one
    CUDA graph. The engines must stay open while the batch lives."""

    def __init__(self, engines: Sequence[Engine]):
        self._lib = _native.load_engine()
        self.engines = list(engines)
        arr = (C.c_void_p * len(self.engines))(*[e.h for e in self.engines])
        self.h = C.c_void_p()
        _native.check(self._lib.pm_batch_create(arr, len(self.engines), C.byref(self.h)))

    def run(self) -> None:
        _native.check(self._lib.pm_batch_run(self.h))

    def info(self) -> dict:
        launches, groups = C.c_int(), C.c_int()
        wpl = (C.c_int * 128)()
        _native.check(self._lib.pm_batch_info(self.h, C.byref(launches), C.byref(groups), wpl, 64))
        return {"launches": launches.value, "groups": groups.value,
                "warps_per_line": [(wpl[2 * i], wpl[2 * i + 1]) for i in range(groups.value)]}

    def close(self) -> None:
        if getattr(self, "h", None):
            self._lib.pm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def default_fuse_params(**over) -> PmFuseParams:
    """Consistency thresholds: max_reproj_px 1, max_rel_depth 0.01, min_consistent 2."""
    p = PmFuseParams()
    _native.load_engine().pm_default_fuse_params(C.byref(p))
    for k, v in over.items():
        setattr(p, k, v)
    return p


class Fusion:
    """Consistency filtering and fusion of several references' depth maps (pm_fusion): no
    counterpart in the reference, the step after the path.

    Fusion(engines) reads the engines' device depth maps in place at every run;
    Fusion.from_depth_maps(depths, images) copies host depth maps (with the Image cameras and
    intensities) to the device."""

    def __init__(self, engines: Sequence[Engine] | None = None, *, _handle=None, _sizes=None):
        self._lib = _native.load_engine()
        self.h = C.c_void_p()
        if _handle is not None:
            self.h = _handle
            self.sizes = list(_sizes)
        else:
            self.engines = list(engines)
            arr = (C.c_void_p * len(self.engines))(*[e.h for e in self.engines])
            _native.check(self._lib.pm_fusion_create_from_engines(arr, len(self.engines), C.byref(self.h)))
            self.sizes = [(e.height, e.width) for e in self.engines]
        self.n = len(self.sizes)

    @classmethod
    def from_depth_maps(cls, depths: Sequence[np.ndarray], images: Sequence[Image], gpu_id: int = -1) -> "Fusion":
        lib = _native.load_engine()
        n = len(depths)
        views = (_native.PmDepthView * n)()
        keep = []   # alive until pm_fusion_create has copied them
        for k, (d, im) in enumerate(zip(depths, images)):
            d = np.ascontiguousarray(d, np.float32)
            g = np.ascontiguousarray(im.image, np.uint8) if im.image is not None else None
            v = views[k]
            v.depth = d.ctypes.data
            v.gray = g.ctypes.data if g is not None else None
            v.height, v.width = d.shape
            if g is not None and g.shape != d.shape:
                raise ValueError("intensity image and depth map differ in size")
            v.K[:] = [float(x) for x in im.K.ravel()]
            v.R[:] = [float(x) for x in im.R.ravel()]
            v.t[:] = [float(x) for x in im.T.ravel()]
            keep.append((d, g))
        h = C.c_void_p()
        _native.check(lib.pm_fusion_create(views, n, gpu_id, C.byref(h)))
        return cls(_handle=h, _sizes=[d.shape for d, _ in keep])

    def _chk(self, st: int) -> None:
        if st != 0:
            raw = self._lib.pm_fusion_last_error(self.h)
            raise PatchMatchError(st, raw.decode() if raw else "")

    def run(self, params: PmFuseParams | None = None) -> int:
        self._chk(self._lib.pm_fusion_run(self.h, C.byref(params or default_fuse_params())))
        return self.info()["points"]

    def info(self) -> dict:
        n, t1, t2, l = C.c_int64(), C.c_float(), C.c_float(), C.c_int()
        self._chk(self._lib.pm_fusion_info(self.h, C.byref(n), C.byref(t1), C.byref(t2), C.byref(l)))
        return {"points": n.value, "ms_check": t1.value, "ms_total": t2.value, "launches": l.value}

    def points(self) -> np.ndarray:
        """(n, 4) float32: x, y, z and intensity in [0, 1]."""
        n = self.info()["points"]
        out = np.empty((n, 4), np.float32)
        self._chk(self._lib.pm_fusion_get_points(self.h, out.ctypes.data, n))
        return out

    def depth(self, ref: int) -> tuple[np.ndarray, np.ndarray]:
        """Fused depth (0 where not kept) and the count of agreeing references."""
        h, w = self.sizes[ref]
        fused = np.empty((h, w), np.float32)
        count = np.empty((h, w), np.uint8)
        self._chk(self._lib.pm_fusion_get_depth(self.h, ref, fused.ctypes.data, count.ctypes.data))
        return fused, count

    def geometry(self) -> tuple[np.ndarray, np.ndarray]:
        pairs = np.empty((self.n, self.n, 12), np.float32)
        bp = np.empty((self.n, 12), np.float32)
        self._chk(self._lib.pm_fusion_geometry(self.h, pairs.ctypes.data, bp.ctypes.data))
        return pairs, bp

    def write_ply(self, path) -> None:
        self._chk(self._lib.pm_fusion_write_ply(self.h, str(path).encode()))

    def close(self) -> None:
        if getattr(self, "h", None):
            self._lib.pm_fusion_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PatchMatch:
    """Mirror of the reference class PatchMatch (patchMatch.h:20-103).

    Constructor arguments follow patchMatch.h:71-72; blockDim_x/blockDim_y are accepted and
    unused (the engine sizes its own launches). Extra keyword arguments set pm_params fields
    (prefilter, seed, precision, quirks, ...)."""

    def __init__(self, allImage: Sequence[Image], nearRange: float, farRange: float, halfWindowSize: int,
                 blockDim_x: int = 32, blockDim_y: int = 16, refImageId: int = 0, numOfSamples: int = 3,
                 SPMAlpha: float = 0.45, gaussianSigma: float = 1.0, numOfIterations: int = 3,
                 orientationX: float = 0.0, orientationZ: float = 1.0, **engine_options):
        p = default_params()
        p.depth_near, p.depth_far = nearRange, farRange
        p.half_window, p.num_samples = halfWindowSize, numOfSamples
        p.sp_alpha, p.gaussian_sigma = SPMAlpha, gaussianSigma
        p.num_iterations = numOfIterations
        p.orientation_x, p.orientation_z = orientationX, orientationZ
        p.block_dim_x, p.block_dim_y = blockDim_x, blockDim_y
        for k, v in engine_options.items():
            if not hasattr(p, k):
                raise TypeError(f"unknown engine option {k!r}")
            setattr(p, k, v)
        self.engine = Engine(allImage, refImageId, p)

    def runPatchMatch(self) -> None:
        self.engine.run()

    run_patch_match = runPatchMatch

    @property
    def depth_map(self) -> np.ndarray:
        return self.engine.depth()

    _depthMap = depth_map

    @property
    def used_imgs_id(self) -> np.ndarray:
        return self.engine.view_selection()

    def save_to_file(self, path) -> None:
        self.engine.save_depth(path)

    saveToFile = save_to_file

    def close(self) -> None:
        self.engine.close()
