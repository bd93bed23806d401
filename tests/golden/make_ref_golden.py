"""Writes tests/golden/ref_box200_96x64.npz: outputs of the REFERENCE'S OWN KERNELS
(yhsa678/patchMatch_cuda's patchMatch.cu, array2d_refImg.cu, array2d_wrapper.cu and
GaussianBlurCUDA.cu, run on the CPU by oracle/ref_host.cpp) on a 96x64 crop of the benchmarked
scene (box200_1280x720: 12 planes + 200 boxes) with its window, view count and sample count
(15x15, 10 sources, numOfSamples 5, depth [1, 20], no prefilter); each source is cut to where
the crop can project (crop_views). The oracle (pm_oracle.c) must reproduce them
(tests/test_ref_pin.py); the engine is checked against the parts that draw no random numbers on
the GPU (tests/test_gpu_refpin.py). Two builds of the reference write them: "f32" computes as the reference is written,
"f64" is the same code with its floats widened to double (the reference's rules without float
rounding, which the FP64 oracle must agree with to rounding level).

Needs the reference's sources (it builds oracle/_ref from them):

    python tests/golden/make_ref_golden.py

Contents (arrays of the f64 build are stored in float64 unless named otherwise):
  image_<i>, K, R, T, ref_id, gt_depth       the views (u8, sources of their own sizes), cameras
  sum_i_*, sum_ii_*                          Array2d_refImg::filterImage's window sums
  q_x, q_y, q_view, q_depth, q_axis          NCC queries (borders included)
  ncc_f32, ncc_f64                           computeNCC, exact bilinear weights
  ncc_f64_fixed                              the same with the texture unit's 1/256 weights
  depth0_*, counts0                          randNumGen's initial depth, the states' draw counts
  costs0_f64 (float32)                       computeAllCostGivenDepth at depth0_f64
  sweep{d}_band{b}_{depth,counts}_*          one sweep in direction d with S = 5 from the start
  sweep{d}_band{b}_costs_f64 (float32)       state (depth0_f64 and costs0_f64 as floats,
                                             counts0), on two bands of 16 lines
  sweep3_band{b}_view_sel_*                  usedImgsID of the bottom-to-top sweeps
  sweep{d}_outside_*                         samples that found no view (NaN posterior CDF)
  msg_*                                      computeMessageForward/Backward cases
  min_cost_in, min_cost_idx                  findMinCost on ties and orderings
  run_depth_*, run_view_sel_*                a 3-iteration run (random states in stream order)
  blur{i}_*, blur_sigma, blur_taps           GaussianBlurCUDA::Filter of the reference image
                                             (u8 / 255) for each sigma, and its filter width
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import pm_ref  # noqa: E402
from patchmatch_cuda_gb300 import PmParams, scene  # noqa: E402

OUT = Path(__file__).resolve().parent / "ref_box200_96x64.npz"
# the crop of the benchmarked scene (box200_1280x720) the fixture holds: the reference's
# rectangle, and the depths [2.2, 9] (the scene's surfaces lie in [2.4, 8.2]) whose projections
# into each source, widened by CROP_MARGIN pixels, give that source's rectangle
CROP = (592, 328, 96, 64)
CROP_DEPTHS = (2.2, 9.0)
CROP_MARGIN = 16
WORKLOAD = scene.Workload("ref_box200_96x64", 96, 64, 10, 7, 3, 1.0, 20.0, 12, 200, prefilter=0, seed=2024)
BAND = 16
# GaussianBlurCUDA objects: the smallest width (5 taps), a middle one and the largest (45)
BLUR_SIGMAS = (1.0, 2.0, 9.5)


def params(w=WORKLOAD):
    p = PmParams()
    p.depth_near, p.depth_far, p.half_window = w.depth_near, w.depth_far, w.half_window
    p.num_samples, p.sp_alpha, p.gaussian_sigma = w.num_samples, w.sp_alpha, w.gaussian_sigma
    p.prefilter, p.num_iterations, p.orientation_x, p.orientation_z = 0, w.iterations, 0.0, 1.0
    p.seed, p.quirks, p.sampler = w.seed, 1, 0
    return p


def crop_views(sv, rect=CROP, depths=CROP_DEPTHS, margin=CROP_MARGIN):
    """The reference cut to `rect` (scene.crop_reference) and every source cut to the bounding
    box of where that rectangle projects for depths in `depths`, widened by `margin` and
    clipped to the image, each source's principal point moved with its cut."""
    from patchmatch_cuda_gb300 import Image
    cut = scene.crop_reference(sv, *rect)
    ref = cut.images[cut.ref_id]
    Kr, Rr, tr = (np.asarray(a, np.float64) for a in (ref.K, ref.R, ref.T))
    Kri = np.linalg.inv(Kr)
    corners = [np.array([x, y, 1.0]) for x in (0.0, rect[2]) for y in (0.0, rect[3])]
    images = []
    for i, im in enumerate(cut.images):
        if i == cut.ref_id:
            images.append(im)
            continue
        Ks, Rs, ts = (np.asarray(a, np.float64) for a in (im.K, im.R, im.T))
        pts = []
        for d in depths:
            for c in corners:
                X = Rr.T @ (d * (Kri @ c) - tr)
                q = Ks @ (Rs @ X + ts)
                pts.append(q[:2] / q[2])
        pts = np.array(pts)
        h, w = im.image.shape
        x0, y0 = (max(0, int(np.floor(v)) - margin) for v in pts.min(0))
        x1, y1 = min(w, int(np.ceil(pts[:, 0].max())) + margin), min(h, int(np.ceil(pts[:, 1].max())) + margin)
        K = Ks.copy()
        K[0, 2] -= x0
        K[1, 2] -= y0
        images.append(Image(K.astype(np.float32), im.R, im.T, np.ascontiguousarray(im.image[y0:y1, x0:x1])))
    return scene.SceneViews(images, cut.ref_id, cut.gt_depth, WORKLOAD)


def views():
    return crop_views(scene.make_views(scene.WORKLOADS["box200_1280x720"]))


def stored_views(g):
    """The fixture's views as Images (sources of different sizes: keys image_<i>)."""
    from patchmatch_cuda_gb300 import Image
    n = len(g["K"])
    return [Image(g["K"][i], g["R"][i], g["T"][i], g[f"image_{i}"]) for i in range(n)]


def queries(w=WORKLOAD, n=1024):
    rng = np.random.default_rng(77)
    xs = rng.integers(0, w.width, n)
    ys = rng.integers(0, w.height, n)
    hw = w.half_window
    xs[:128] = rng.integers(0, hw + 1, 128)
    ys[128:256] = rng.integers(0, hw + 1, 128)
    xs[256:384] = rng.integers(w.width - hw - 1, w.width, 128)
    ys[384:512] = rng.integers(w.height - hw - 1, w.height, 128)
    vs = rng.integers(0, w.n_src, n)
    ds = rng.uniform(w.depth_near, w.depth_far, n).astype(np.float32).astype(np.float64)
    ax = rng.integers(0, 2, n)
    return xs.astype(np.int32), ys.astype(np.int32), vs.astype(np.int32), ds, ax.astype(np.int32)


def bands(direction, w=WORKLOAD):
    n_lines = w.height if direction in (0, 2) else w.width
    return [(0, BAND), (n_lines // 2, n_lines // 2 + BAND)]


def band_rows(a, direction, band):
    """The band's lines of a (H, W, ...) array, as (lines, steps, ...)."""
    lo, hi = band
    return a[lo:hi] if direction in (0, 2) else np.swapaxes(a[:, lo:hi], 0, 1)


def message_cases(n=64, V=10):
    rng = np.random.default_rng(5)
    msg = rng.uniform(0.0, 1.0, (n, V))
    cost = rng.uniform(0.0, 2.0, (n, V))
    cost[rng.random((n, V)) < 0.15] = 2.0          # the cost-2 replacement draws
    cost[:4] = rng.uniform(2.0, 12.0, (4, V))        # leading-edge values beyond [0, 2]
    msg[4:8] = rng.choice([0.0, 1.0, 0.5], (4, V))
    return msg, cost


MIN_COST_IN = np.array([[0.5, 0.5, 0.5], [0.2, 0.2, 0.9], [0.9, 0.2, 0.2], [0.2, 0.9, 0.2], [0.1, 0.2, 0.3],
                        [0.3, 0.2, 0.1], [0.2, 0.1, 0.3], [0.3, 0.1, 0.1], [0.1, 0.3, 0.1], [0.1, 0.1, 0.3]])


def start_state(out):
    """The state every sweep starts from: the f64 build's initial depth and costs rounded to
    float (the stored costs0_f64), the states' counts after the initial depth."""
    return (out["depth0_f64"].astype(np.float32).astype(np.float64), out["costs0_f64"].astype(np.float64),
            out["counts0"])


def compute(sv, wide: bool, start=None) -> dict:
    w = WORKLOAD
    S = w.num_samples
    tag = "f64" if wide else "f32"
    ft = np.float64 if wide else np.float32
    p = params()
    rp = pm_ref.RefProblem.from_images(sv.images, sv.ref_id, p, wide=wide, fixed_point_weights=False)
    out = {}
    _, si, sii = rp.box_moments()
    out[f"sum_i_{tag}"], out[f"sum_ii_{tag}"] = si.astype(ft), sii.astype(ft)
    out[f"ncc_{tag}"] = rp.ncc(*queries()).astype(ft)
    if wide:
        rpf = pm_ref.RefProblem.from_images(sv.images, sv.ref_id, p, wide=True, fixed_point_weights=True)
        out["ncc_f64_fixed"] = rpf.ncc(*queries())
    d0, counts0 = rp.init_depth()
    out[f"depth0_{tag}"] = d0.astype(ft)
    if wide:
        out["counts0"] = counts0
        out["costs0_f64"] = rp.initial_costs(d0).astype(np.float32)
        start = start_state(out)
    d0s, c0s, cnt0 = start
    for direction in range(4):
        d, c, cnt = d0s.copy(), c0s.copy(), cnt0.copy()
        vs = np.full((S, w.height, w.width), 255, np.uint8)
        out[f"sweep{direction}_outside_{tag}"] = np.int64(rp.sweep(d, c, cnt, direction, S, vs))
        for b, band in enumerate(bands(direction)):
            out[f"sweep{direction}_band{b}_depth_{tag}"] = band_rows(d, direction, band).astype(ft)
            if wide:
                out[f"sweep{direction}_band{b}_costs_f64"] = band_rows(c, direction, band).astype(np.float32)
            out[f"sweep{direction}_band{b}_counts_{tag}"] = (cnt[band[0]:band[1], 0] if direction in (0, 2)
                                                          else cnt[0, band[0]:band[1]]).copy()
            if direction == 3:
                out[f"sweep3_band{b}_view_sel_{tag}"] = band_rows(np.moveaxis(vs, 0, -1), 3, band).copy()
    msg, cost = message_cases()
    for fwd in (0, 1):
        res, counts = [], []
        for i in range(len(msg)):
            m, n = pm_ref.messages(bool(fwd), msg[i], cost[i], w.sp_alpha, w.seed, 1000 + i, 0, wide=wide)
            res.append(m)
            counts.append(n)
        out[f"msg_{'fwd' if fwd else 'bwd'}_{tag}"] = np.array(res, ft)
        out[f"msg_{'fwd' if fwd else 'bwd'}_draws_{tag}"] = np.array(counts, np.uint32)
    out[f"min_cost_idx_{tag}"] = np.array([pm_ref.find_min_cost(c, wide=wide) for c in MIN_COST_IN], np.int32)
    depth, _, vsel, outside = rp.run(w.iterations, S)
    out[f"run_depth_{tag}"] = depth.astype(np.float32)
    out[f"run_view_sel_{tag}"] = vsel
    out[f"run_outside_{tag}"] = np.int64(outside)
    img = sv.images[sv.ref_id].image.astype(np.float32) / np.float32(255)
    taps = []
    for i, sigma in enumerate(BLUR_SIGMAS):
        b, kw = pm_ref.blur(img, sigma, wide=wide)
        out[f"blur{i}_{tag}"] = b.astype(ft)
        taps.append(kw)
    out["blur_sigma"], out["blur_taps"] = np.array(BLUR_SIGMAS), np.array(taps, np.int32)
    return out


def main():
    pm_ref.build()
    sv = views()
    q = queries()
    msg, cost = message_cases()
    out = {f"image_{i}": im.image for i, im in enumerate(sv.images)}
    out.update(K=np.stack([im.K for im in sv.images]), R=np.stack([im.R for im in sv.images]),
               T=np.stack([im.T for im in sv.images]), ref_id=np.int64(sv.ref_id), gt_depth=sv.gt_depth,
               q_x=q[0], q_y=q[1], q_view=q[2], q_depth=q[3], q_axis=q[4], msg_in=msg, msg_cost=cost,
               min_cost_in=MIN_COST_IN)
    wide = compute(sv, True)
    out.update(wide)
    out.update(compute(sv, False, start_state(wide)))
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
