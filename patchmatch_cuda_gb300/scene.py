"""Seeded synthetic multi-view scenes standing in for the benchmark inputs.

The workloads are named by what they are; each returns calibrated 8-bit views, the reference
index, the reference's ground-truth z-depth and the engine parameters.

    plane3_320x240     3 slanted planes, 1 ref + 4 sources on a 15 degree arc, f = 300 px,
                       depth [2, 8], 11x11 window, box prefilter sigma 1, 3 iterations
    box200_1280x720    12 planes + 200 boxes, 1 ref + 10 sources, depth [1, 20], 15x15 window,
                       5 iterations, no prefilter (the reference's runtime never calls its blur)
    batch24_mixed      24 references of 640x480 / 1280x720 / 1920x1080 with 6-12 sources each
                       from one scene of 40 planes + 500 boxes, 15x15 window, 5 iterations
    box2000_3072x2048  60 planes + 2000 boxes, 1 ref + 20 sources, depth [0.5, 50], 19x19 window
    full8_3072x2048    8 such references from one scene (make_full_batch), batched

Parameters the workloads leave open are fixed once: numOfSamples 3 for up to 4 sources else 5,
SPMAlpha 0.45, plane normal (0, 0, 1).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import Image, PREFILTER_BOX, PREFILTER_NONE, _native

ARC_DEGREES = 15.0


@dataclass
class Workload:
    name: str
    width: int
    height: int
    n_src: int
    half_window: int
    iterations: int
    depth_near: float
    depth_far: float
    n_planes: int
    n_boxes: int
    prefilter: int = PREFILTER_BOX
    gaussian_sigma: float = 1.0
    sp_alpha: float = 0.45
    seed: int = 1
    extra: dict = field(default_factory=dict)

    @property
    def num_samples(self) -> int:
        return 3 if self.n_src <= 4 else 5

    @property
    def focal(self) -> float:
        return 300.0 * self.width / 320.0

    def params(self, **over):
        from . import default_params
        p = default_params()
        p.depth_near, p.depth_far = self.depth_near, self.depth_far
        p.half_window, p.num_samples = self.half_window, self.num_samples
        p.sp_alpha, p.gaussian_sigma = self.sp_alpha, self.gaussian_sigma
        p.prefilter, p.num_iterations = self.prefilter, self.iterations
        p.seed = self.seed
        for k, v in over.items():
            setattr(p, k, v)
        return p


WORKLOADS = {
    "plane3_320x240": Workload("plane3_320x240", 320, 240, 4, 5, 3, 2.0, 8.0, 3, 0, seed=11),
    "box200_1280x720": Workload("box200_1280x720", 1280, 720, 10, 7, 5, 1.0, 20.0, 12, 200,
                                prefilter=PREFILTER_NONE, seed=22),
    "box2000_3072x2048": Workload("box2000_3072x2048", 3072, 2048, 20, 9, 5, 0.5, 50.0, 60, 2000,
                                  prefilter=PREFILTER_NONE, seed=55),
}


@dataclass
class SceneViews:
    images: list
    ref_id: int
    gt_depth: np.ndarray
    workload: Workload


class Scene:
    """A seeded scene (planes + boxes) from which calibrated views are rendered."""

    def __init__(self, seed: int, n_planes: int, n_boxes: int, depth_near: float, depth_far: float,
                 width: int, height: int, focal: float):
        self._lib = _native.load_scene()
        self.h = self._lib.pm_scene_create(seed, n_planes, n_boxes, depth_near, depth_far, width, height, focal)
        if not self.h:
            raise ValueError("invalid scene parameters")

    def close(self):
        if self.h:
            self._lib.pm_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def camera(self, yaw: float, pitch: float, width: int, height: int, focal: float):
        K, R, t = np.zeros(9), np.zeros(9), np.zeros(3)
        self._lib.pm_scene_camera(self.h, yaw, pitch, width, height, focal, K.ctypes.data, R.ctypes.data,
                                  t.ctypes.data)
        return K.reshape(3, 3), R.reshape(3, 3), t

    def render(self, K, R, t, width: int, height: int):
        K = np.ascontiguousarray(K, np.float64)
        R = np.ascontiguousarray(R, np.float64)
        t = np.ascontiguousarray(t, np.float64)
        img = np.empty((height, width), np.uint8)
        depth = np.empty((height, width), np.float32)
        self._lib.pm_scene_render(self.h, K.ctypes.data, R.ctypes.data, t.ctypes.data, width, height,
                                  img.ctypes.data, depth.ctypes.data)
        return img, depth

    def view(self, yaw: float, pitch: float, width: int, height: int, focal: float):
        K, R, t = self.camera(yaw, pitch, width, height, focal)
        img, depth = self.render(K, R, t, width, height)
        return Image(K.astype(np.float32), R.astype(np.float32), t.astype(np.float32), img), depth


def arc_yaws(n_views: int, center: float = 0.0, span: float = ARC_DEGREES) -> list[float]:
    if n_views == 1:
        return [center]
    return [center - span / 2 + span * i / (n_views - 1) for i in range(n_views)]


def make_views(w: Workload, seed: int | None = None) -> SceneViews:
    """Reference (the middle camera) and n_src sources on a 15 degree arc."""
    sc = Scene(w.seed if seed is None else seed, w.n_planes, w.n_boxes, w.depth_near, w.depth_far,
               w.width, w.height, w.focal)
    yaws = arc_yaws(w.n_src + 1)
    ref_id = w.n_src // 2
    images, gt = [], None
    for i, yaw in enumerate(yaws):
        im, d = sc.view(yaw, 0.0, w.width, w.height, w.focal)
        images.append(im)
        if i == ref_id:
            gt = d
    sc.close()
    return SceneViews(images, ref_id, gt, w)


def crop_reference(sv: SceneViews, x0: int, y0: int, width: int, height: int) -> SceneViews:
    """The same cameras with the reference cut to the rectangle [x0, x0 + width) x
    [y0, y0 + height): its principal point moves by (-x0, -y0), the sources stay whole. The
    crop keeps the full image's pixel scale and texture, so a smaller problem has the same
    statistics as the full one."""
    ref = sv.images[sv.ref_id]
    h, w = ref.image.shape
    if not (0 <= x0 and 0 <= y0 and width > 0 and height > 0 and x0 + width <= w and y0 + height <= h):
        raise ValueError("crop rectangle outside the reference image")
    K = ref.K.astype(np.float64).copy()
    K[0, 2] -= x0
    K[1, 2] -= y0
    crop = Image(K.astype(np.float32), ref.R, ref.T, np.ascontiguousarray(ref.image[y0:y0 + height, x0:x0 + width]))
    images = list(sv.images)
    images[sv.ref_id] = crop
    wl = sv.workload
    cw = Workload(f"{wl.name}_crop{width}x{height}", width, height, wl.n_src, wl.half_window, wl.iterations,
                  wl.depth_near, wl.depth_far, wl.n_planes, wl.n_boxes, wl.prefilter, wl.gaussian_sigma,
                  wl.sp_alpha, wl.seed, dict(wl.extra))
    gt = np.ascontiguousarray(sv.gt_depth[y0:y0 + height, x0:x0 + width])
    return SceneViews(images, sv.ref_id, gt, cw)


BATCH_SIZES = [(640, 480), (1280, 720), (1920, 1080)]


def make_batch(n_refs: int = 24, seed: int = 33, half_window: int = 7, iterations: int = 5,
               depth_near: float = 1.0, depth_far: float = 20.0, n_planes: int = 40,
               n_boxes: int = 500) -> list[SceneViews]:
    """References of uneven size and source count from one scene (the batched workload)."""
    rng = np.random.default_rng(seed)
    sc = Scene(seed, n_planes, n_boxes, depth_near, depth_far, 1280, 720, 1200.0)
    out = []
    for r in range(n_refs):
        w_, h_ = BATCH_SIZES[int(rng.integers(0, 3))]
        n_src = int(rng.integers(6, 13))
        yaw_c = float(rng.uniform(-20.0, 20.0))
        pitch = float(rng.uniform(-4.0, 4.0))
        f = 300.0 * w_ / 320.0
        wl = Workload(f"batch{r}", w_, h_, n_src, half_window, iterations, depth_near, depth_far,
                      n_planes, n_boxes, prefilter=PREFILTER_NONE, seed=seed * 1000 + r)
        yaws = arc_yaws(n_src + 1, yaw_c)
        ref_id = n_src // 2
        images, gt = [], None
        for i, yaw in enumerate(yaws):
            im, d = sc.view(yaw, pitch, w_, h_, f)
            images.append(im)
            if i == ref_id:
                gt = d
        out.append(SceneViews(images, ref_id, gt, wl))
    sc.close()
    return out


def make_full_batch(n_refs: int = 8, seed: int = 55, width: int = 3072, height: int = 2048, n_src: int = 20,
                    half_window: int = 9, iterations: int = 5, depth_near: float = 0.5,
                    depth_far: float = 50.0, n_planes: int = 60, n_boxes: int = 2000) -> list[SceneViews]:
    """The full-scale workload: references of 3072x2048 with 20 sources each (19x19 window,
    depth [0.5, 50]) from one scene of 60 planes + 2000 boxes, their arcs centred on yaws
    spread over 30 degrees."""
    f = 300.0 * width / 320.0
    sc = Scene(seed, n_planes, n_boxes, depth_near, depth_far, width, height, f)
    out = []
    for r in range(n_refs):
        yaw_c = -15.0 + 30.0 * r / max(1, n_refs - 1)
        wl = Workload(f"full{r}", width, height, n_src, half_window, iterations, depth_near, depth_far,
                      n_planes, n_boxes, prefilter=PREFILTER_NONE, seed=seed * 1000 + r)
        yaws = arc_yaws(n_src + 1, yaw_c)
        ref_id = n_src // 2
        images, gt = [], None
        for i, yaw in enumerate(yaws):
            im, d = sc.view(yaw, 0.0, width, height, f)
            images.append(im)
            if i == ref_id:
                gt = d
        out.append(SceneViews(images, ref_id, gt, wl))
    sc.close()
    return out


def scene_views(specs, seed: int = 7, n_planes: int = 4, n_boxes: int = 6, depth_near: float = 2.0,
                depth_far: float = 8.0) -> list[tuple[Image, np.ndarray]]:
    """Views of one scene, specs = [(yaw, pitch, width, height, focal)], each with its ground
    truth z-depth (the references of a fusion)."""
    w0, h0, f0 = specs[0][2], specs[0][3], specs[0][4]
    sc = Scene(seed, n_planes, n_boxes, depth_near, depth_far, w0, h0, f0)
    out = [sc.view(*spec) for spec in specs]
    sc.close()
    return out


def bad_pixel_rate(depth: np.ndarray, gt: np.ndarray, rel: float = 0.01) -> float:
    """Share of pixels with |d - d_gt| / d_gt > rel."""
    valid = gt > 0
    err = np.abs(depth[valid] - gt[valid]) / gt[valid]
    return float(np.mean(err > rel))


def rotation_to_quaternion(R) -> tuple[float, float, float, float]:
    """(w, x, y, z) of a rotation matrix (Shepperd's method), the inverse of the NVM reader's
    quaternion-to-rotation formula."""
    R = np.asarray(R, np.float64).reshape(3, 3)
    tr = R[0, 0] + R[1, 1] + R[2, 2]
    if tr > 0:
        s = 2.0 * np.sqrt(tr + 1.0)
        return 0.25 * s, (R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s
    i = int(np.argmax(np.diag(R)))
    j, k = (i + 1) % 3, (i + 2) % 3
    s = 2.0 * np.sqrt(1.0 + R[i, i] - R[j, j] - R[k, k])
    q = [0.0, 0.0, 0.0]
    q[i] = 0.25 * s
    q[j] = (R[j, i] + R[i, j]) / s
    q[k] = (R[k, i] + R[i, k]) / s
    return (R[k, j] - R[j, k]) / s, q[0], q[1], q[2]


def write_nvm(path, names, images, points, visible=None) -> None:
    """An NVM_V3 model of calibrated views: per camera its file, focal length K[0][0],
    quaternion and centre -R^T T (the reader puts the principal point at the image centre),
    then the 3D points [n, 3], each with its projection into every camera it lies in front
    of (visible[i] lists the cameras of point i where given)."""
    lines = ["NVM_V3", "", str(len(images))]
    for name, im in zip(names, images):
        R = np.asarray(im.R, np.float64)
        c = -R.T @ np.asarray(im.T, np.float64)
        q = rotation_to_quaternion(R)
        lines.append(" ".join([name, repr(float(im.K[0, 0]))] + [repr(float(v)) for v in q] +
                              [repr(float(v)) for v in c] + ["0", "0"]))
    pts = np.asarray(points, np.float64).reshape(-1, 3)
    lines += ["", str(len(pts))]
    for i, p in enumerate(pts):
        cams = range(len(images)) if visible is None else visible[i]
        proj = []
        for cidx in cams:
            im = images[cidx]
            u = np.asarray(im.K, np.float64) @ (np.asarray(im.R, np.float64) @ p + np.asarray(im.T, np.float64))
            if visible is None and u[2] <= 0:
                continue
            proj.append(f"{cidx} {i} {u[0] / u[2]:.3f} {u[1] / u[2]:.3f}")
        lines.append(" ".join([repr(float(v)) for v in p] + ["128", "128", "128", str(len(proj))] + proj))
    lines += ["", "0", ""]
    Path(path).write_text("\n".join(lines))


def nvm_points(sv: SceneViews, step: int = 8) -> np.ndarray:
    """3D points of the reference's ground truth on a pixel grid (a stand-in for a structure
    from motion point cloud)."""
    im = sv.images[sv.ref_id]
    K, R, T = (np.asarray(a, np.float64) for a in (im.K, im.R, im.T))
    h, w = sv.gt_depth.shape
    ys, xs = np.mgrid[step // 2:h:step, step // 2:w:step]
    d = sv.gt_depth[ys, xs].astype(np.float64)
    keep = d > 0
    pix = np.stack([xs[keep] + 0.5, ys[keep] + 0.5, np.ones(int(keep.sum()))], axis=0)
    cam = np.linalg.solve(K, pix) * d[keep]
    return (R.T @ (cam - T[:, None])).T

