"""ctypes wrapper of the reference's own kernels run on the CPU (ref_host.cpp). TEST
INFRASTRUCTURE ONLY: it pins the oracle (pm_oracle.c) to the reference's code, writes the
golden vectors under tests/golden/ (make_ref_golden.py) and is bench.py's CPU baseline.

The libraries are built from the reference's sources (`make -C oracle ref`, ref_extract.sh) or,
where the sources are absent, from the kernels ref_extract.sh already copied out of them into
oracle/_ref/ref_kernels.inc (`make -C oracle ref-libs`; the file is not committed, it travels
with a working tree). Where neither is present `available()` is False and the committed golden
vectors stand in for them. bench.py times this build (the reference's own code) as its CPU
baseline where it is available.

    lib = load(wide)        wide=False: the reference as written (float arithmetic);
                            wide=True: the same code with its floats widened to double.
    ref = RefProblem.from_images(images, ref_id, params, wide=...)
    ref.box_moments(), ref.ncc(...), ref.initial_costs(depth), ref.sweep(...), ref.run(...)
    blur(img, sigma, wide)  GaussianBlurCUDA::Filter as written (box taps, clamped edges)

Random numbers: the reference's curand states become sequential Philox streams, one per pixel
state as in array2d_psng (draw k of state id = Philox4x32-10 of counter (id, k, 0x5EED << 16, 0));
`counts` holds each state's draws so far. pm_oracle's stream mode draws the same numbers.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_OUT = HERE / "_ref"
REFERENCE_ROOT = Path(os.environ.get("PM_REFERENCE_ROOT", "/root/reference"))


class _RefProblem(C.Structure):
    _fields_ = [
        ("width", C.c_int), ("height", C.c_int), ("n_src", C.c_int), ("half_window", C.c_int),
        ("ref", C.c_void_p), ("src", C.c_void_p), ("src_width", C.c_int), ("src_height", C.c_int),
        ("hh", C.c_void_p), ("orientation", C.c_double * 3), ("inv_k", C.c_double * 4),
        ("depth_near", C.c_double), ("depth_far", C.c_double), ("sp_alpha", C.c_double),
        ("seed", C.c_uint64), ("fixed_point_weights", C.c_int),
    ]


def sources_present() -> bool:
    return (REFERENCE_ROOT / "src" / "patchMatch.cu").exists()


def build() -> None:
    """Builds oracle/_ref from the reference's sources, or, where they are absent, from the
    kernels already extracted from them into oracle/_ref."""
    target = "ref" if sources_present() else "ref-libs"
    r = subprocess.run(["make", "-s", "-C", str(HERE), target, f"REF_ROOT={REFERENCE_ROOT}"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")


def extracted_present() -> bool:
    """The reference's kernels extracted from its sources (ref_kernels.inc, ref_blur.inc) are here: the
    libraries can be built even where the sources are not."""
    return all((REF_OUT / f).exists() for f in ("ref_kernels.inc", "ref_blur.inc"))


def available() -> bool:
    return sources_present() or extracted_present()


_libs: dict[bool, C.CDLL] = {}


def load(wide: bool = False) -> C.CDLL:
    if wide in _libs:
        return _libs[wide]
    path = REF_OUT / ("libpm_ref_f64.so" if wide else "libpm_ref_f32.so")
    if not path.exists():
        build()
    lib = C.CDLL(str(path))
    P = C.c_void_p
    lib.pmr_real_bytes.restype = C.c_int
    lib.pmr_box_moments.argtypes = [P, P, P, P]
    lib.pmr_init_depth.argtypes = [P, P, P]
    lib.pmr_initial_costs.argtypes = [P, P, P]
    lib.pmr_sweep.restype = C.c_longlong
    lib.pmr_sweep.argtypes = [P, C.c_int, C.c_int, P, P, P, P, C.c_int, C.c_int, P, P]
    lib.pmr_run.restype = C.c_longlong
    lib.pmr_run.argtypes = [P, C.c_int, C.c_int, P, P, P]
    lib.pmr_ncc.argtypes = [P, C.c_int, P, P, P, P, P, P]
    lib.pmr_messages.argtypes = [C.c_int, C.c_int, P, P, C.c_double, C.c_uint64, C.c_uint32, P]
    lib.pmr_find_min_cost.argtypes = [P]
    lib.pmr_blur.argtypes = [C.c_int, C.c_int, C.c_double, P, P, P]
    _libs[wide] = lib
    return lib


class RefProblem:
    """One reference image and its sources as the reference's PatchMatch object holds them: the
    u8 reference, the sources packed into zero-padded layers of the largest source size
    (copyData, patchMatch.cu:51-130), H1/H2 per source (Image::init_relative, formed in double
    and rounded to the build's float type), K^-1 terms and the parameters."""

    def __init__(self, ref_u8, sources_u8, hh, inv_k, half_window, depth_near, depth_far, sp_alpha, seed,
                 orientation=(0.0, 0.0, 1.0), fixed_point_weights=False, wide=False):
        self.lib = load(wide)
        self.ref = np.ascontiguousarray(ref_u8, np.uint8)
        self.H, self.W = self.ref.shape
        self.V = len(sources_u8)
        sw = max(s.shape[1] for s in sources_u8)
        sh = max(s.shape[0] for s in sources_u8)
        self.src = np.zeros((self.V, sh, sw), np.uint8)
        for v, s in enumerate(sources_u8):
            self.src[v, :s.shape[0], :s.shape[1]] = s
        self.hh = np.ascontiguousarray(hh, np.float64).reshape(self.V, 18)
        p = _RefProblem()
        p.width, p.height, p.n_src, p.half_window = self.W, self.H, self.V, half_window
        p.ref, p.src = self.ref.ctypes.data, self.src.ctypes.data
        p.src_width, p.src_height = sw, sh
        p.hh = self.hh.ctypes.data
        p.orientation[:] = [float(x) for x in orientation]
        p.inv_k[:] = [float(x) for x in inv_k]
        p.depth_near, p.depth_far, p.sp_alpha = depth_near, depth_far, sp_alpha
        p.seed = seed
        p.fixed_point_weights = int(bool(fixed_point_weights))
        self.p = p
        self.half_window = half_window

    @classmethod
    def from_images(cls, images, ref_id, params, wide=False, fixed_point_weights=None):
        from oracle import pm_oracle
        ref_im = images[ref_id]
        srcs = [im for i, im in enumerate(images) if i != ref_id]
        hh, ik = [], None
        for s in srcs:
            h_, ik = pm_oracle.init_relative(ref_im.K, ref_im.R, ref_im.T, s.K, s.R, s.T, params.orientation_x,
                                             params.orientation_z)
            hh.append(h_)
        fpw = getattr(params, "sampler", 0) == 1 if fixed_point_weights is None else fixed_point_weights
        return cls(ref_im.image, [s.image for s in srcs], np.array(hh), ik, params.half_window,
                   params.depth_near, params.depth_far, params.sp_alpha, params.seed,
                   (params.orientation_x, 0.0, params.orientation_z), fpw, wide)

    @property
    def _pp(self):
        return C.byref(self.p)

    def box_moments(self):
        img, si, sii = (np.empty((self.H, self.W), np.float64) for _ in range(3))
        assert self.lib.pmr_box_moments(self._pp, img.ctypes.data, si.ctypes.data, sii.ctypes.data) == 0
        return img, si, sii

    def init_depth(self, counts=None):
        counts = np.zeros((self.H, self.W), np.uint32) if counts is None else counts
        d = np.empty((self.H, self.W), np.float64)
        assert self.lib.pmr_init_depth(self._pp, counts.ctypes.data, d.ctypes.data) == 0
        return d, counts

    def initial_costs(self, depth):
        depth = np.ascontiguousarray(depth, np.float64)
        c = np.empty((self.H, self.W, self.V), np.float64)
        assert self.lib.pmr_initial_costs(self._pp, depth.ctypes.data, c.ctypes.data) == 0
        return c

    def sweep(self, depth, cost, counts, direction, num_samples, view_sel=None, lines=(0, -1),
              with_evals=False):
        """In place on float64 depth (H, W), cost (H, W, V) and uint32 counts (H, W); returns
        the homography-table fetches outside the table (samples that found no view), and with
        with_evals also the number of NCC evaluations and the kernel launch's wall time in
        seconds. Only the reference's blocks of 32 lines that hold `lines` run."""
        for a, t in ((depth, np.float64), (cost, np.float64), (counts, np.uint32)):
            assert a.dtype == t and a.flags.c_contiguous
        vs = view_sel.ctypes.data if view_sel is not None else None
        ev, sec = C.c_longlong(0), C.c_double(0.0)
        n = self.lib.pmr_sweep(self._pp, direction, num_samples, depth.ctypes.data, cost.ctypes.data,
                               counts.ctypes.data, vs, lines[0], lines[1], C.byref(ev), C.byref(sec))
        assert n >= 0
        return (n, ev.value, sec.value) if with_evals else n

    def run(self, iterations, num_samples):
        depth = np.empty((self.H, self.W), np.float64)
        cost = np.empty((self.H, self.W, self.V), np.float64)
        vsel = np.full((num_samples, self.H, self.W), 255, np.uint8)
        n = self.lib.pmr_run(self._pp, iterations, num_samples, depth.ctypes.data, cost.ctypes.data,
                             vsel.ctypes.data)
        assert n >= 0
        return depth, cost, vsel, n

    def ncc(self, xs, ys, views, depths, axes):
        xs = np.ascontiguousarray(xs, np.int32).ravel()
        ys = np.ascontiguousarray(np.broadcast_to(ys, xs.shape), np.int32)
        vs = np.ascontiguousarray(np.broadcast_to(views, xs.shape), np.int32)
        ds = np.ascontiguousarray(np.broadcast_to(depths, xs.shape), np.float64)
        ax = np.ascontiguousarray(np.broadcast_to(axes, xs.shape), np.int32)
        out = np.empty(xs.shape, np.float64)
        assert self.lib.pmr_ncc(self._pp, xs.size, xs.ctypes.data, ys.ctypes.data, vs.ctypes.data, ds.ctypes.data,
                                ax.ctypes.data, out.ctypes.data) == 0
        return out


def messages(forward: bool, msg, cost, sp_alpha: float, seed: int, state_id: int, count: int, wide=False):
    """computeMessageForward / computeMessageBackward for one pixel: (new messages, new count)."""
    lib = load(wide)
    m = np.ascontiguousarray(msg, np.float64).copy()
    c = np.ascontiguousarray(cost, np.float64)
    n = C.c_uint32(count)
    assert lib.pmr_messages(int(forward), m.size, m.ctypes.data, c.ctypes.data, sp_alpha, seed, state_id,
                            C.byref(n)) == 0
    return m, n.value


def find_min_cost(c, wide=False) -> int:
    a = np.ascontiguousarray(c, np.float64)
    return load(wide).pmr_find_min_cost(a.ctypes.data)


def blur(img, sigma: float, wide: bool = False):
    """GaussianBlurCUDA::Filter(dst, src) (GaussianBlurCUDA.cu:185-191) of a float image for an
    object made with this sigma. Returns (filtered image as float64, the filter width)."""
    lib = load(wide)
    a = np.ascontiguousarray(img, np.float64)
    out = np.empty_like(a)
    taps = C.c_int(0)
    if lib.pmr_blur(a.shape[1], a.shape[0], float(sigma), a.ctypes.data, out.ctypes.data, C.byref(taps)) != 0:
        raise ValueError(f"GaussianBlurCUDA runs no pass for sigma {sigma} (width {taps.value})")
    return out, taps.value
