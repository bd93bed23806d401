"""Edge cases of the CUDA path against the oracle (needs a GPU): every code path of the
windowed NCC (3x3, the half-warp layout up to 15x15, one column per lane from 17x17, two
columns per lane beyond 32), the most source views and view samples the ABI accepts, source
images whose sizes differ from the reference's (the reference zero-pads them into one layered
array, patchMatch.cu:72-95), odd image sizes, and images smaller than the window.

Tolerances are those of the stage-by-stage parity tests: NCC 1e-4 (exact sampler; relative
beyond |cost| > 1) and 5e-4 at the 99.9th percentile for texture filtering; full runs at least
99.5 % of depths within 0.1 % of the oracle (99 % with 32 views and 32 samples, see that test).
"""
import numpy as np
import pytest

from parity_util import NCC_TOL, first_divergence, ncc_err

pytestmark = pytest.mark.gpu


def views_of(width, height, n_src, seed, src_sizes=None, n_planes=3, n_boxes=0, near=2.0, far=8.0):
    """A seeded scene seen by a reference of width x height and n_src sources on the 15 degree
    arc; src_sizes (one (w, h) per source) renders the sources at other sizes."""
    from patchmatch_cuda_gb300 import scene
    sc = scene.Scene(seed, n_planes, n_boxes, near, far, width, height, 300.0 * width / 320.0)
    yaws = scene.arc_yaws(n_src + 1)
    ref_id = n_src // 2
    images, gt, k = [], None, 0
    for i, yaw in enumerate(yaws):
        if i == ref_id:
            w, h = width, height
        else:
            w, h = src_sizes[k] if src_sizes else (width, height)
            k += 1
        im, d = sc.view(yaw, 0.0, w, h, 300.0 * w / 320.0)
        images.append(im)
        if i == ref_id:
            gt = d
    sc.close()
    return images, ref_id, gt


def params(**over):
    from patchmatch_cuda_gb300 import default_params
    p = default_params()
    p.depth_near, p.depth_far, p.half_window, p.num_samples, p.num_iterations = 2.0, 8.0, 3, 3, 2
    p.sp_alpha, p.seed = 0.45, 7
    for k, v in over.items():
        setattr(p, k, v)
    return p


def engine_and_oracle(images, ref_id, p):
    from oracle import pm_oracle
    from patchmatch_cuda_gb300 import Engine
    eng = Engine(images, ref_id, p)
    src = [eng.source_texels(v) for v in range(eng.n_src)]
    ref, _, _ = eng.ref_maps()
    return eng, pm_oracle.from_images(images, ref_id, p, source_texels=src, ref_texels=ref)


def ncc_queries(width, height, n_src, hw, gt, near, far, n=2048, seed=0):
    rng = np.random.default_rng(seed)
    xs = rng.integers(0, width, n)
    ys = rng.integers(0, height, n)
    xs[: n // 8] = rng.integers(0, min(hw + 1, width), n // 8)          # leading edges
    ys[n // 8: n // 4] = rng.integers(max(0, height - hw - 1), height, n // 8)  # trailing edges
    vs = rng.integers(0, n_src, n)
    ds = np.where(rng.random(n) < 0.5, gt[ys, xs], rng.uniform(near, far, n)).astype(np.float32)
    ax = rng.integers(0, 2, n)
    return xs, ys, vs, ds, ax


def assert_ncc(err, sampler, what):
    if sampler == 0:
        assert err.max() <= NCC_TOL, f"{what}: max NCC error {err.max():.3g}"
    else:
        assert np.quantile(err, 0.999) <= 5 * NCC_TOL and err.max() <= 20 * NCC_TOL, \
            f"{what}: NCC error q999 {np.quantile(err, 0.999):.3g} max {err.max():.3g}"


@pytest.fixture(scope="module")
def scene160():
    return views_of(160, 120, 3, seed=31)


@pytest.mark.parametrize("sampler", [0, 1])
@pytest.mark.parametrize("hw", [1, 8, 9, 16, 22])
def test_ncc_parity_across_window_sides(scene160, hw, sampler, parity_log):
    images, ref_id, gt = scene160
    eng, orc = engine_and_oracle(images, ref_id, params(half_window=hw, sampler=sampler))
    q = ncc_queries(160, 120, 3, hw, gt, 2.0, 8.0, seed=hw)
    err = ncc_err(eng.eval_costs(*q), orc.ncc_batch(*q))
    parity_log(f"edge_ncc_w{2 * hw + 1}_sampler{sampler}", err_max=float(err.max()),
               err_q999=float(np.quantile(err, 0.999)))
    assert_ncc(err, sampler, f"window {2 * hw + 1}")
    eng.close()


@pytest.mark.parametrize("sampler", [0, 1])
@pytest.mark.parametrize("hw,direction", [(9, 1), (9, 2), (22, 0), (22, 3)])
def test_sweep_lockstep_wide_windows(scene160, hw, direction, sampler, parity_log):
    """One sweep of the whole-warp NCC layout (19x19: one column per lane; 45x45: two) from
    the same state as the oracle."""
    images, ref_id, gt = scene160
    eng, orc = engine_and_oracle(images, ref_id, params(half_window=hw, sampler=sampler))
    eng.init_depth()
    eng.compute_costs(1)
    d0, c0 = eng.depth().astype(np.float64), eng.costs().astype(np.float64)
    eng.run_sweep(direction, 4 + direction, 3)
    gd, gc = eng.depth(), eng.costs()
    od, oc = d0.copy(), c0.copy()
    orc.sweep(od, oc, direction, 4 + direction, 3)
    prefix, nsteps = first_divergence(gd, od, direction)
    events = int(np.sum(prefix < nsteps))
    decisions = int(np.sum(np.minimum(prefix + 1, nsteps)))
    parity_log(f"edge_lockstep_w{2 * hw + 1}_dir{direction}_sampler{sampler}", divergence_events=events,
               decisions=decisions)
    assert events <= max(2, int(2e-4 * decisions)), f"{events} divergences in {decisions} decisions"
    eng.close()


def test_most_views_and_samples(parity_log):
    """32 source views (the ABI's maximum) and 32 view samples per pixel: one sweep per direction
    from the same state as the oracle (measured: 1 divergence in 27,624 decisions), then a full
    run. Each decision averages 32 FP32 costs against the oracle's FP64 ones, so the rare
    near-tie flip is carried along its line and into later sweeps: the full-run bar is 99 %
    (measured 99.36 %, bad-pixel rates 47.32 % against the oracle's 47.38 %)."""
    from patchmatch_cuda_gb300 import scene
    images, ref_id, gt = views_of(96, 72, 32, seed=41)
    p = params(num_samples=32, sampler=1)
    eng, orc = engine_and_oracle(images, ref_id, p)
    eng.init_depth()
    eng.compute_costs(1)
    d0, c0 = eng.depth().astype(np.float64), eng.costs().astype(np.float64)
    events = decisions = 0
    for direction in range(4):
        eng.set_depth(d0.astype(np.float32))
        eng.set_costs(c0.astype(np.float32))
        eng.run_sweep(direction, 4 + direction, 32)
        od, oc = d0.copy(), c0.copy()
        orc.sweep(od, oc, direction, 4 + direction, 32)
        prefix, nsteps = first_divergence(eng.depth(), od, direction)
        events += int(np.sum(prefix < nsteps))
        decisions += int(np.sum(np.minimum(prefix + 1, nsteps)))
    eng.run()
    gd = eng.depth()
    od, oc, ovs, n = orc.run(p.num_iterations, p.num_samples)
    frac = float(np.mean(np.abs(gd - od) / od <= 1e-3))
    vs = eng.view_selection()
    parity_log("edge_32_views_32_samples", within_0p1pct=frac, lockstep_events=events, lockstep_decisions=decisions,
               bad1_gpu=scene.bad_pixel_rate(gd, gt),
               bad1_oracle=scene.bad_pixel_rate(od.astype(np.float32), gt))
    assert events <= max(2, int(2e-4 * decisions)), f"{events} divergences in {decisions} decisions"
    assert frac >= 0.99
    assert vs.shape == (32, 72, 96) and vs[vs != 255].max() < 32
    eng.close()


@pytest.mark.parametrize("sampler", [0, 1])
def test_sources_of_other_sizes(sampler, parity_log):
    """Sources larger and smaller than the reference: the texture-filtering sampler reads them
    from one layered array zero-padded to the largest, the exact sampler from one array each."""
    images, ref_id, gt = views_of(160, 120, 3, seed=51, src_sizes=[(200, 150), (120, 90), (176, 96)])
    p = params(half_window=4, sampler=sampler)
    eng, orc = engine_and_oracle(images, ref_id, p)
    q = ncc_queries(160, 120, 3, 4, gt, 2.0, 8.0, seed=5)
    err = ncc_err(eng.eval_costs(*q), orc.ncc_batch(*q))
    assert_ncc(err, sampler, "ragged sources")
    eng.run()
    gd = eng.depth()
    od, *_ = orc.run(p.num_iterations, p.num_samples)
    frac = float(np.mean(np.abs(gd - od) / od <= 1e-3))
    parity_log(f"edge_ragged_sources_sampler{sampler}", err_max=float(err.max()), within_0p1pct=frac)
    assert frac >= 0.995
    eng.close()


def test_odd_sizes_full_run(parity_log):
    images, ref_id, gt = views_of(97, 61, 2, seed=61)
    p = params(half_window=4, sampler=1)
    eng, orc = engine_and_oracle(images, ref_id, p)
    eng.run()
    gd = eng.depth()
    od, *_ = orc.run(p.num_iterations, p.num_samples)
    frac = float(np.mean(np.abs(gd - od) / od <= 1e-3))
    parity_log("edge_odd_97x61", within_0p1pct=frac)
    assert frac >= 0.995
    eng.close()


@pytest.mark.parametrize("sampler", [0, 1])
def test_image_smaller_than_the_window(sampler, parity_log):
    """A 24x18 reference with a 45x45 window: every window is cut on all four sides."""
    images, ref_id, gt = views_of(24, 18, 2, seed=71)
    p = params(half_window=22, sampler=sampler)
    eng, orc = engine_and_oracle(images, ref_id, p)
    eng.init_depth()
    eng.compute_costs(1)
    c = eng.costs()
    oc = orc.initial_costs(eng.depth().astype(np.float64))
    err = ncc_err(c, oc)
    parity_log(f"edge_tiny_24x18_w45_sampler{sampler}", err_max=float(err.max()))
    assert_ncc(err.ravel(), sampler, "24x18 image, 45x45 window")
    eng.run()
    d = eng.depth()
    assert np.all(np.isfinite(d)) and d.min() >= 2.0 and d.max() <= 8.0
    eng.close()
