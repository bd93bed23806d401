"""ctypes wrapper of the CPU oracle (pm_oracle.c). TEST INFRASTRUCTURE ONLY.

`Oracle(problem_inputs, fp32=False)` holds one problem: reference texels, source texels,
homographies (double), K^-1 terms, parameters. Parity status: pinned to the reference's own
kernels run on the CPU (oracle/pm_ref.py, ref_host.cpp) through the golden vectors they wrote
(tests/golden/ref_*.npz), plus code-derived known-answer tests and synthetic ground truth.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"

DIR_LR, DIR_TB, DIR_RL, DIR_BT = 0, 1, 2, 3
RNG_INIT, RNG_BWD, RNG_FWD_PRE, RNG_FWD_POST, RNG_RAND_DEPTH, RNG_SAMPLE = 1, 2, 3, 4, 5, 6


def build() -> None:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")


class _Problem(C.Structure):
    _fields_ = [
        ("width", C.c_int), ("height", C.c_int), ("n_src", C.c_int), ("half_window", C.c_int),
        ("ref", C.c_void_p), ("src", C.c_void_p), ("src_width", C.c_void_p), ("src_height", C.c_void_p),
        ("hh", C.c_void_p), ("inv_k", C.c_double * 4), ("orientation", C.c_double * 3),
        ("depth_near", C.c_double), ("depth_far", C.c_double), ("sp_alpha", C.c_float),
        ("seed", C.c_uint64), ("batch_id", C.c_uint32), ("quirks", C.c_int),
        ("sampler", C.c_int), ("perturbation", C.c_float),
        ("planes", C.c_int), ("ee", C.c_void_p), ("plane_depth_step", C.c_float),
        ("plane_slope_step", C.c_float), ("rng_stream", C.c_int), ("rng_counts", C.c_void_p),
    ]

# Slanted-plane mode's constants (pm_oracle.h)
SLOPE_DRAW, SLOPE_MAX, SCALE_MIN = 1.0, 2.0, 0.0625


_libs: dict[bool, C.CDLL] = {}


def load(fp32: bool = False) -> C.CDLL:
    if fp32 in _libs:
        return _libs[fp32]
    path = BUILD / ("liboracle_f32.so" if fp32 else "liboracle_f64.so")
    if not path.exists():
        build()
    lib = C.CDLL(str(path))
    P = C.c_void_p
    lib.pmo_philox4x32_10.argtypes = [P, P, P]
    lib.pmo_uniform.restype = C.c_double
    lib.pmo_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]
    lib.pmo_init_relative.argtypes = [P, P, P, P, P, P, C.c_double, C.c_double, P, P]
    lib.pmo_prefilter.restype = C.c_int
    lib.pmo_prefilter.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_float, P]
    lib.pmo_box_moments.argtypes = [P, C.c_int, C.c_int, C.c_int, P, P]
    lib.pmo_sample.argtypes = [P, C.c_int, C.c_int, P, P, P]
    lib.pmo_ncc.restype = C.c_double
    lib.pmo_ncc.argtypes = [P, P, P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int]
    lib.pmo_ncc_batch.argtypes = [P, P, P, C.c_int, P, P, P, P, P, P]
    lib.pmo_init_depth.argtypes = [P, P]
    lib.pmo_refine.restype = C.c_longlong
    lib.pmo_refine.argtypes = [P, P, P, P, P, C.c_int, C.c_int, C.c_float, C.c_uint32, C.c_int]
    lib.pmo_initial_costs.restype = C.c_longlong
    lib.pmo_initial_costs.argtypes = [P, P, P, P, P]
    lib.pmo_sweep.restype = C.c_longlong
    lib.pmo_sweep.argtypes = [P, P, P, P, P, C.c_int, C.c_uint32, C.c_int, P, C.c_int, C.c_int]
    lib.pmo_run.restype = C.c_longlong
    lib.pmo_run.argtypes = [P, C.c_int, C.c_int, P, P, P, P, P]
    lib.pmo_translation_term.argtypes = [P, P, P, P, P, P]
    lib.pmo_init_planes.argtypes = [P, P]
    lib.pmo_ncc_plane.restype = C.c_double
    lib.pmo_ncc_plane.argtypes = [P, P, P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_float, C.c_float, C.c_int]
    lib.pmo_ncc_plane_batch.argtypes = [P, P, P, C.c_int, P, P, P, P, P, P, P]
    lib.pmo_initial_costs_planes.restype = C.c_longlong
    lib.pmo_initial_costs_planes.argtypes = [P, P, P, P, P, P]
    lib.pmo_sweep_planes.restype = C.c_longlong
    lib.pmo_sweep_planes.argtypes = [P, P, P, P, P, P, C.c_int, C.c_uint32, C.c_int, P, C.c_int, C.c_int]
    lib.pmo_refine_planes.restype = C.c_longlong
    lib.pmo_refine_planes.argtypes = [P, P, P, P, P, P, C.c_int, C.c_int, C.c_float, C.c_uint32, C.c_int]
    lib.pmo_run_planes.restype = C.c_longlong
    lib.pmo_run_planes.argtypes = [P, C.c_int, C.c_int, P, P, P, P, P, P]
    lib.pmo_msg_forward.restype = C.c_double
    lib.pmo_msg_forward.argtypes = [C.c_double, C.c_double, C.c_double, C.c_float]
    lib.pmo_msg_backward.restype = C.c_double
    lib.pmo_msg_backward.argtypes = [C.c_double, C.c_double, C.c_double, C.c_float]
    lib.pmo_find_min_cost.restype = C.c_int
    lib.pmo_find_min_cost.argtypes = [P]
    lib.pmo_num_threads.restype = C.c_int
    lib.pmo_real_bytes.restype = C.c_int
    _libs[fp32] = lib
    return lib


def philox(counter, key) -> np.ndarray:
    lib = load()
    c = np.ascontiguousarray(counter, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib.pmo_philox4x32_10(c.ctypes.data, k.ctypes.data, out.ctypes.data)
    return out


def uniform(seed: int, c0: int, c1: int, c2: int, c3: int = 0) -> float:
    return load().pmo_uniform(seed, c0, c1, c2, c3)


def init_relative(K_ref, R_ref, t_ref, K_src, R_src, t_src, nx=0.0, nz=1.0):
    lib = load()
    arrs = [np.ascontiguousarray(a, np.float64).ravel() for a in (K_ref, R_ref, t_ref, K_src, R_src, t_src)]
    hh = np.zeros(18)
    ik = np.zeros(4)
    lib.pmo_init_relative(*[a.ctypes.data for a in arrs], nx, nz, hh.ctypes.data, ik.ctypes.data)
    return hh, ik


def translation_term(R_ref, t_ref, K_src, R_src, t_src) -> np.ndarray:
    """e = K_s R_s (C_s - C_r), the slanted-plane mode's translation term."""
    lib = load()
    arrs = [np.ascontiguousarray(a, np.float64).ravel() for a in (R_ref, t_ref, K_src, R_src, t_src)]
    e = np.zeros(3)
    lib.pmo_translation_term(*[a.ctypes.data for a in arrs], e.ctypes.data)
    return e


def prefilter(img: np.ndarray, mode: int, sigma: float, fp32: bool = False) -> np.ndarray:
    lib = load(fp32)
    a = np.ascontiguousarray(img, np.float32)
    out = np.empty_like(a)
    if lib.pmo_prefilter(a.ctypes.data, a.shape[1], a.shape[0], mode, sigma, out.ctypes.data) != 0:
        raise ValueError("invalid prefilter arguments")
    return out


def box_moments(img: np.ndarray, half_window: int, fp32: bool = False):
    lib = load(fp32)
    a = np.ascontiguousarray(img, np.float32)
    si = np.empty(a.shape, np.float64)
    sii = np.empty(a.shape, np.float64)
    lib.pmo_box_moments(a.ctypes.data, a.shape[1], a.shape[0], half_window, si.ctypes.data, sii.ctypes.data)
    return si, sii


def msg_forward(m, cost, u_if_two, sp_alpha):
    return load().pmo_msg_forward(m, cost, u_if_two, sp_alpha)


def msg_backward(m, cost, u_if_two, sp_alpha):
    return load().pmo_msg_backward(m, cost, u_if_two, sp_alpha)


def find_min_cost(c) -> int:
    a = np.ascontiguousarray(c, np.float64)
    return load().pmo_find_min_cost(a.ctypes.data)


class Oracle:
    """One reference image and its sources, as the CUDA engine sees them."""

    def __init__(self, ref: np.ndarray, sources: list[np.ndarray], hh: np.ndarray, inv_k,
                 half_window: int, depth_near: float, depth_far: float, sp_alpha: float, seed: int,
                 orientation=(0.0, 0.0, 1.0), quirks: bool = True, batch_id: int = 0,
                 fp32: bool = False, sampler: int = 0, ee: np.ndarray | None = None):
        self.lib = load(fp32)
        self.ref = np.ascontiguousarray(ref, np.float32)
        self.sources = [np.ascontiguousarray(s, np.float32) for s in sources]
        self.hh = np.ascontiguousarray(hh, np.float64).reshape(len(sources), 18)
        self.H, self.W = self.ref.shape
        self.V = len(sources)
        self._src_ptrs = (C.c_void_p * self.V)(*[s.ctypes.data for s in self.sources])
        self._sw = np.array([s.shape[1] for s in self.sources], np.int32)
        self._sh = np.array([s.shape[0] for s in self.sources], np.int32)
        p = _Problem()
        p.width, p.height, p.n_src, p.half_window = self.W, self.H, self.V, half_window
        p.ref = self.ref.ctypes.data
        p.src = C.cast(self._src_ptrs, C.c_void_p)
        p.src_width, p.src_height = self._sw.ctypes.data, self._sh.ctypes.data
        p.hh = self.hh.ctypes.data
        p.inv_k[:] = [float(x) for x in inv_k]
        p.orientation[:] = [float(x) for x in orientation]
        p.depth_near, p.depth_far = depth_near, depth_far
        p.sp_alpha = sp_alpha
        p.seed, p.batch_id, p.quirks = seed, batch_id, int(quirks)
        p.sampler = int(sampler)
        p.perturbation = 0.0
        # slanted-plane mode's per-view translation terms (enabled with set_planes)
        self.ee = np.ascontiguousarray(ee if ee is not None else np.zeros((self.V, 3)), np.float64).reshape(self.V, 3)
        p.ee = self.ee.ctypes.data
        p.planes = 0
        p.plane_depth_step, p.plane_slope_step = 0.0, 0.0
        self.p = p
        self.half_window = half_window
        self.sum_i, self.sum_ii = box_moments(self.ref, half_window, fp32)

    @property
    def _pp(self):
        return C.byref(self.p)

    def set_moments(self, sum_i, sum_ii):
        self.sum_i = np.ascontiguousarray(sum_i, np.float64)
        self.sum_ii = np.ascontiguousarray(sum_ii, np.float64)

    def sample(self, view, xs, ys) -> np.ndarray:
        xs = np.ascontiguousarray(xs, np.float32).ravel()
        ys = np.ascontiguousarray(np.broadcast_to(ys, xs.shape), np.float32)
        out = np.empty(xs.shape, np.float64)
        self.lib.pmo_sample(self._pp, view, xs.size, xs.ctypes.data, ys.ctypes.data, out.ctypes.data)
        return out

    def ncc(self, x, y, view, depth, axis) -> float:
        return self.lib.pmo_ncc(self._pp, self.sum_i.ctypes.data, self.sum_ii.ctypes.data, x, y, view, depth, axis)

    def ncc_batch(self, xs, ys, views, depths, axes) -> np.ndarray:
        xs = np.ascontiguousarray(xs, np.int32).ravel()
        ys = np.ascontiguousarray(np.broadcast_to(ys, xs.shape), np.int32)
        vs = np.ascontiguousarray(np.broadcast_to(views, xs.shape), np.int32)
        ds = np.ascontiguousarray(np.broadcast_to(depths, xs.shape), np.float64)
        ax = np.ascontiguousarray(np.broadcast_to(axes, xs.shape), np.int32)
        out = np.empty(xs.shape, np.float64)
        self.lib.pmo_ncc_batch(self._pp, self.sum_i.ctypes.data, self.sum_ii.ctypes.data, xs.size, xs.ctypes.data,
                               ys.ctypes.data, vs.ctypes.data, ds.ctypes.data, ax.ctypes.data, out.ctypes.data)
        return out

    def init_depth(self) -> np.ndarray:
        d = np.empty((self.H, self.W), np.float64)
        self.lib.pmo_init_depth(self._pp, d.ctypes.data)
        return d

    def initial_costs(self, depth: np.ndarray) -> np.ndarray:
        depth = np.ascontiguousarray(depth, np.float64)
        c = np.empty((self.H, self.W, self.V), np.float64)
        self.lib.pmo_initial_costs(self._pp, self.sum_i.ctypes.data, self.sum_ii.ctypes.data, depth.ctypes.data,
                                   c.ctypes.data)
        return c

    def sweep(self, depth: np.ndarray, cost: np.ndarray, direction: int, sweep_id: int, num_samples: int,
              view_sel: np.ndarray | None = None, lines: tuple[int, int] = (0, -1)) -> int:
        """In-place on float64 depth (H, W) and cost (H, W, V). Returns the evaluation count."""
        assert depth.dtype == np.float64 and depth.flags.c_contiguous
        assert cost.dtype == np.float64 and cost.flags.c_contiguous
        vs = view_sel.ctypes.data if view_sel is not None else None
        return self.lib.pmo_sweep(self._pp, self.sum_i.ctypes.data, self.sum_ii.ctypes.data, depth.ctypes.data,
                                  cost.ctypes.data, direction, sweep_id, num_samples, vs, lines[0], lines[1])

    def refine(self, depth: np.ndarray, view_sel: np.ndarray, num_samples: int, trials: int, sigma: float,
               sweep_id: int, axis: int) -> int:
        """In-place on float64 depth (H, W) from a uint8 view-selection map (S, H, W)."""
        assert depth.dtype == np.float64 and depth.flags.c_contiguous
        vs = np.ascontiguousarray(view_sel, np.uint8)
        return self.lib.pmo_refine(self._pp, self.sum_i.ctypes.data, self.sum_ii.ctypes.data, depth.ctypes.data,
                                   vs.ctypes.data, num_samples, trials, sigma, sweep_id, axis)

    # ---- slanted-plane mode -----------------------------------------------------------
    def set_planes(self, on: bool = True, depth_step: float = 0.0, slope_step: float = 0.0):
        self.p.planes = int(on)
        self.p.plane_depth_step = depth_step
        self.p.plane_slope_step = slope_step

    def init_planes(self) -> np.ndarray:
        s = np.empty((self.H, self.W, 2), np.float32)
        self.lib.pmo_init_planes(self._pp, s.ctypes.data)
        return s

    def ncc_plane(self, x, y, view, depth, a, b, axis) -> float:
        return self.lib.pmo_ncc_plane(self._pp, self.sum_i.ctypes.data, self.sum_ii.ctypes.data, x, y, view, depth,
                                      a, b, axis)

    def ncc_plane_batch(self, xs, ys, views, depths, slopes, axes) -> np.ndarray:
        xs = np.ascontiguousarray(xs, np.int32).ravel()
        ys = np.ascontiguousarray(np.broadcast_to(ys, xs.shape), np.int32)
        vs = np.ascontiguousarray(np.broadcast_to(views, xs.shape), np.int32)
        ds = np.ascontiguousarray(np.broadcast_to(depths, xs.shape), np.float64)
        sl = np.ascontiguousarray(np.broadcast_to(slopes, xs.shape + (2,)), np.float32)
        ax = np.ascontiguousarray(np.broadcast_to(axes, xs.shape), np.int32)
        out = np.empty(xs.shape, np.float64)
        self.lib.pmo_ncc_plane_batch(self._pp, self.sum_i.ctypes.data, self.sum_ii.ctypes.data, xs.size,
                                     xs.ctypes.data, ys.ctypes.data, vs.ctypes.data, ds.ctypes.data, sl.ctypes.data,
                                     ax.ctypes.data, out.ctypes.data)
        return out

    def initial_costs_planes(self, depth: np.ndarray, slopes: np.ndarray) -> np.ndarray:
        depth = np.ascontiguousarray(depth, np.float64)
        slopes = np.ascontiguousarray(slopes, np.float32)
        c = np.empty((self.H, self.W, self.V), np.float64)
        self.lib.pmo_initial_costs_planes(self._pp, self.sum_i.ctypes.data, self.sum_ii.ctypes.data,
                                          depth.ctypes.data, slopes.ctypes.data, c.ctypes.data)
        return c

    def sweep_planes(self, depth: np.ndarray, slopes: np.ndarray, cost: np.ndarray, direction: int, sweep_id: int,
                     num_samples: int, view_sel: np.ndarray | None = None, lines: tuple[int, int] = (0, -1)) -> int:
        """In place on float64 depth (H, W), float32 slopes (H, W, 2) and float64 cost (H, W, V)."""
        assert depth.dtype == np.float64 and depth.flags.c_contiguous
        assert slopes.dtype == np.float32 and slopes.flags.c_contiguous
        assert cost.dtype == np.float64 and cost.flags.c_contiguous
        vs = view_sel.ctypes.data if view_sel is not None else None
        return self.lib.pmo_sweep_planes(self._pp, self.sum_i.ctypes.data, self.sum_ii.ctypes.data,
                                         depth.ctypes.data, slopes.ctypes.data, cost.ctypes.data, direction, sweep_id,
                                         num_samples, vs, lines[0], lines[1])

    def refine_planes(self, depth: np.ndarray, slopes: np.ndarray, view_sel: np.ndarray, num_samples: int,
                      trials: int, sigma: float, sweep_id: int, axis: int) -> int:
        assert depth.dtype == np.float64 and depth.flags.c_contiguous
        slopes = np.ascontiguousarray(slopes, np.float32)
        vs = np.ascontiguousarray(view_sel, np.uint8)
        return self.lib.pmo_refine_planes(self._pp, self.sum_i.ctypes.data, self.sum_ii.ctypes.data,
                                          depth.ctypes.data, slopes.ctypes.data, vs.ctypes.data, num_samples, trials,
                                          sigma, sweep_id, axis)

    def run_planes(self, iterations: int, num_samples: int):
        depth = np.empty((self.H, self.W), np.float64)
        slopes = np.empty((self.H, self.W, 2), np.float32)
        cost = np.empty((self.H, self.W, self.V), np.float64)
        vsel = np.full((num_samples, self.H, self.W), 255, np.uint8)
        n = self.lib.pmo_run_planes(self._pp, iterations, num_samples, self.sum_i.ctypes.data,
                                    self.sum_ii.ctypes.data, depth.ctypes.data, slopes.ctypes.data, cost.ctypes.data,
                                    vsel.ctypes.data)
        return depth, slopes, cost, vsel, n

    def set_stream(self, counts: np.ndarray | None) -> None:
        """Stream mode (the reference's order of draws from per-pixel random states) with the
        uint32 (H, W) draw counts `counts`, updated in place by later calls; None: keyed draws."""
        if counts is None:
            self.p.rng_stream, self.p.rng_counts, self._counts = 0, None, None
            return
        assert counts.dtype == np.uint32 and counts.shape == (self.H, self.W) and counts.flags.c_contiguous
        self._counts = counts
        self.p.rng_stream, self.p.rng_counts = 1, counts.ctypes.data

    def run(self, iterations: int, num_samples: int):
        depth = np.empty((self.H, self.W), np.float64)
        cost = np.empty((self.H, self.W, self.V), np.float64)
        vsel = np.full((num_samples, self.H, self.W), 255, np.uint8)
        n = self.lib.pmo_run(self._pp, iterations, num_samples, self.sum_i.ctypes.data, self.sum_ii.ctypes.data,
                             depth.ctypes.data, cost.ctypes.data, vsel.ctypes.data)
        return depth, cost, vsel, n


def num_threads(fp32: bool = False) -> int:
    return load(fp32).pmo_num_threads()


def from_images(images, ref_id: int, params, source_texels=None, ref_texels=None, fp32=False) -> Oracle:
    """Oracle for the engine's inputs: FP64 camera setup from the views, texels either given
    (as the engine stores them) or derived here (u8/255, then the prefilter)."""
    ref_im = images[ref_id]
    srcs = [im for i, im in enumerate(images) if i != ref_id]
    hh, ee, ik = [], [], None
    for s in srcs:
        h_, ik = init_relative(ref_im.K, ref_im.R, ref_im.T, s.K, s.R, s.T, params.orientation_x,
                               params.orientation_z)
        hh.append(h_)
        ee.append(translation_term(ref_im.R, ref_im.T, s.K, s.R, s.T))

    def texels(im):
        t = im.image.astype(np.float32) / np.float32(255.0)
        if params.prefilter:
            t = prefilter(t, params.prefilter, params.gaussian_sigma)
        return t

    ref_t = ref_texels if ref_texels is not None else texels(ref_im)
    src_t = source_texels if source_texels is not None else [texels(s) for s in srcs]
    orc = Oracle(ref_t, src_t, np.array(hh), ik, params.half_window, params.depth_near, params.depth_far,
                 params.sp_alpha, params.seed, (params.orientation_x, 0.0, params.orientation_z),
                 bool(params.quirks), 0, fp32, getattr(params, "sampler", 0), np.array(ee))
    orc.p.perturbation = float(getattr(params, "perturbation", 0.0))
    if getattr(params, "planes", 0):
        orc.set_planes(True, float(params.plane_depth_step), float(params.plane_slope_step))
    return orc
