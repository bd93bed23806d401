"""The oracle's slanted-plane mode (no counterpart in the reference, whose plane normal is one
constant, patchMatch.cu:32) on the CPU: it reduces to the reference's rule for fronto-parallel
planes, its state is deterministic and line-independent, and it sharpens depths on slanted
surfaces."""
import numpy as np
import pytest

from oracle import pm_oracle as O


@pytest.fixture(scope="module")
def plane_scene():
    from patchmatch_cuda_gb300 import scene
    w = scene.WORKLOADS["plane3_320x240"]
    return scene.make_views(w)


def oracle(sv, fp32=False, **over):
    p = sv.workload.params(**over)
    return O.from_images(sv.images, sv.ref_id, p, fp32=fp32)


def test_translation_term_is_the_h2_column_vector(oracle_lib, plane_scene):
    """H2 = e n^T K^-1 (image.cpp:4-13): for n = (0, 0, 1) its last column is e."""
    ims = plane_scene.images
    r, s = ims[plane_scene.ref_id], ims[(plane_scene.ref_id + 1) % len(ims)]
    hh, _ = O.init_relative(r.K, r.R, r.T, s.K, s.R, s.T, 0.0, 1.0)
    e = O.translation_term(r.R, r.T, s.K, s.R, s.T)
    np.testing.assert_array_equal(hh[9:].reshape(3, 3)[:, 2], e)
    np.testing.assert_array_equal(hh[9:].reshape(3, 3)[:, :2], 0.0)


@pytest.mark.parametrize("sampler", [0, 1])
def test_fronto_parallel_planes_reduce_to_the_reference_rule(oracle_lib, plane_scene, sampler):
    orc = oracle(plane_scene, sampler=sampler)
    rng = np.random.default_rng(3)
    w = plane_scene.workload
    n = 2000
    xs, ys = rng.integers(0, w.width, n), rng.integers(0, w.height, n)
    vs = rng.integers(0, w.n_src, n)
    ds = rng.uniform(w.depth_near, w.depth_far, n).astype(np.float32).astype(np.float64)
    ax = rng.integers(0, 2, n)
    ref_mode = orc.ncc_batch(xs, ys, vs, ds, ax)
    planes = orc.ncc_plane_batch(xs, ys, vs, ds, np.zeros((n, 2), np.float32), ax)
    np.testing.assert_array_equal(planes, ref_mode)


def test_initial_slopes_are_seeded_and_bounded(oracle_lib, plane_scene):
    a = oracle(plane_scene, planes=1).init_planes()
    b = oracle(plane_scene, planes=1).init_planes()
    c = oracle(plane_scene, planes=1, seed=12345).init_planes()
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
    assert np.all(np.abs(a) <= O.SLOPE_DRAW)
    assert abs(float(a.mean())) < 0.01 and 0.3 < float(a.std()) < 0.65  # uniform in [-1, 1]


@pytest.mark.parametrize("direction", [0, 1, 2, 3])
def test_plane_sweep_lines_are_independent(oracle_lib, plane_scene, direction):
    """A sweep over a subset of lines changes exactly those lines, as the whole sweep does."""
    orc = oracle(plane_scene, planes=1, fp32=True)
    d = orc.init_depth()
    s = orc.init_planes()
    c = orc.initial_costs_planes(d, s)
    full = (d.copy(), s.copy(), c.copy())
    orc.sweep_planes(*full, direction, 9, 3)
    part = (d.copy(), s.copy(), c.copy())
    lines = (d.shape[0] if direction in (0, 2) else d.shape[1])
    orc.sweep_planes(*part, direction, 9, 3, lines=(5, lines // 2))
    sel = (slice(5, lines // 2), slice(None)) if direction in (0, 2) else (slice(None), slice(5, lines // 2))
    np.testing.assert_array_equal(part[0][sel], full[0][sel])
    np.testing.assert_array_equal(part[1][sel], full[1][sel])
    untouched = np.ones(d.shape, bool)
    untouched[sel] = False
    np.testing.assert_array_equal(part[0][untouched], d[untouched])
    np.testing.assert_array_equal(part[1][untouched], s[untouched])


def test_planes_sharpen_depths_on_slanted_surfaces(oracle_lib, plane_scene):
    """6 iterations on three slanted planes (FP32 restatement): a lower median depth error than
    one fronto-parallel normal, at no worse 1 % bad-pixel rate."""
    from patchmatch_cuda_gb300 import scene
    w = plane_scene.workload
    gt = plane_scene.gt_depth
    d_ref, *_ = oracle(plane_scene, fp32=True).run(6, w.num_samples)
    d_pl, slopes, *_ = oracle(plane_scene, fp32=True, planes=1).run_planes(6, w.num_samples)
    med_ref = float(np.median(np.abs(d_ref - gt) / gt))
    med_pl = float(np.median(np.abs(d_pl - gt) / gt))
    assert med_pl < 0.85 * med_ref, (med_pl, med_ref)
    assert scene.bad_pixel_rate(d_pl.astype(np.float32), gt) <= scene.bad_pixel_rate(d_ref.astype(np.float32), gt)
    assert np.all(np.abs(slopes) <= O.SLOPE_MAX)


def test_the_true_plane_scores_better_than_fronto_and_mirrored_planes(oracle_lib, plane_scene):
    """Sign and convention check of the plane geometry on the scene's slanted planes: the plane
    taken from the ground truth's inverse-depth gradient (1/d = g_u u + g_v v + 1/rho in
    normalised coordinates, slopes (a, b) = rho (g_u, g_v)) scores a lower median NCC at the true
    depth than the fronto-parallel plane, and beats the mirrored slopes (-a, -b) on most pixels.
    With 11x11 windows and a 15 degree arc the differences are small (about 2 % of the cost; the
    scene's planes tilt by up to 25 degrees), so the test uses many pixels with slopes above
    0.25."""
    w = plane_scene.workload
    gt = plane_scene.gt_depth.astype(np.float64)
    orc = oracle(plane_scene, planes=1)
    ik00, ik02, ik11, ik12 = orc.p.inv_k
    inv = 1.0 / gt
    gx = np.zeros_like(inv)
    gy = np.zeros_like(inv)
    gx[:, 1:-1] = (inv[:, 2:] - inv[:, :-2]) / 2.0
    gy[1:-1, :] = (inv[2:, :] - inv[:-2, :]) / 2.0
    # smooth interiors only: the second differences of 1/d vanish on one plane
    lap = np.full_like(inv, np.inf)
    lap[1:-1, 1:-1] = np.abs(inv[1:-1, 2:] + inv[1:-1, :-2] - 2 * inv[1:-1, 1:-1]) + \
        np.abs(inv[2:, 1:-1] + inv[:-2, 1:-1] - 2 * inv[1:-1, 1:-1])
    hw = w.half_window
    ys, xs = np.nonzero(lap < 1e-7)
    keep = (xs > hw + 2) & (xs < w.width - hw - 3) & (ys > hw + 2) & (ys < w.height - hw - 3)
    ys, xs = ys[keep], xs[keep]
    g_u, g_v = gx[ys, xs] / ik00, gy[ys, xs] / ik11        # per unit of normalised coordinate
    u = ik00 * (xs + 0.5) + ik02
    v = ik11 * (ys + 0.5) + ik12
    rho = 1.0 / (inv[ys, xs] - g_u * u - g_v * v)
    slopes = np.stack([rho * g_u, rho * g_v], axis=1).astype(np.float32)
    slanted = np.hypot(slopes[:, 0], slopes[:, 1]) > 0.25
    assert slanted.sum() > 5000
    xs, ys, slopes = xs[slanted], ys[slanted], slopes[slanted]
    rng = np.random.default_rng(8)
    pick = rng.choice(len(xs), 2000, replace=False)
    xs, ys, slopes = xs[pick], ys[pick], slopes[pick]
    depth = gt[ys, xs].astype(np.float32).astype(np.float64)
    views = rng.integers(0, w.n_src, len(xs))
    true = orc.ncc_plane_batch(xs, ys, views, depth, slopes, 1)
    fronto = orc.ncc_plane_batch(xs, ys, views, depth, np.zeros_like(slopes), 1)
    mirrored = orc.ncc_plane_batch(xs, ys, views, depth, -slopes, 1)
    assert np.median(true) < np.median(fronto) < np.median(mirrored)
    assert np.mean(true < mirrored) > 0.58
