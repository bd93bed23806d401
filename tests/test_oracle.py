"""Known-answer tests of the CPU oracle against rules read from the reference code (CPU only).

The reference ships no tests or fixtures, so these pins come from its source: Philox published
vectors, the NCC special values (patchMatch.cu:594-610), the tie rule (:613-618), the message
formulas (:669-715), box moments (array2d_refImg.cu:11-67), prefilter widths
(GaussianBlurCUDA.cu:99-130) and the homographies (image.cpp:4-13).
"""
import numpy as np
import pytest

from oracle import pm_oracle as O

F = float(np.float32(0.999))
C = float(np.float32(1.0) - np.float32(0.999))


def test_philox_published_vectors(oracle_lib):
    # Random123 known-answer vectors for philox4x32-10
    assert list(O.philox([0, 0, 0, 0], [0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert list(O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_uniform_interval_and_formula(oracle_lib):
    seed = 0xABCDEF0123
    for c in range(200):
        u = O.uniform(seed, c, 7, (6 << 16) | 3, 1)
        x = O.philox([c, 7, (6 << 16) | 3, 1], [seed & 0xFFFFFFFF, seed >> 32])[0]
        assert u == ((int(x) >> 8) + 1) / 2 ** 24
        assert 0.0 < u <= 1.0


@pytest.mark.parametrize("cost,idx", [((1, 1, 1), 2), ((0.5, 1, 1), 0), ((1, 0.5, 0.5), 2), ((1, 0.5, 0.7), 1),
                                      ((0.2, 0.2, 0.9), 1), ((0.1, 0.2, 0.1), 2)])
def test_find_min_cost_ties_go_to_the_later_index(oracle_lib, cost, idx):
    assert O.find_min_cost(cost) == idx


def test_messages_match_the_reference_formulas(oracle_lib):
    a2 = float(np.float32(0.45) * np.float32(0.45))
    u = np.exp(-0.5 * float(np.float32(0.83)) ** 2 / a2)
    for m in (0.1, 0.5, 0.9):
        for c in (0.0, 0.3, 1.1):
            e = float(np.float32(np.exp(-0.5 * c * c / a2)))
            fwd = (m * F + (1 - m) * C) * e / ((m * F + (1 - m) * C) * e + (m * C + (1 - m) * F) * u)
            bwd = (m * e * F + (1 - m) * u * C) / (m * e * F + (1 - m) * u * C + m * e * C + (1 - m) * u * F)
            assert O.msg_forward(m, c, 0.5, 0.45) == pytest.approx(fwd, rel=1e-12)
            assert O.msg_backward(m, c, 0.5, 0.45) == pytest.approx(bwd, rel=1e-12)
    # a cost of exactly 2 (window outside the source) is replaced by 2 U (patchMatch.cu:680-682)
    assert O.msg_forward(0.5, 2.0, 0.25, 0.45) == pytest.approx(O.msg_forward(0.5, 0.5, 0.9, 0.45))
    # emissions below the smallest normal float are zero: the forward message then collapses
    assert O.msg_forward(0.7, 9.0, 0.5, 0.45) == 0.0


def test_box_moments_against_brute_force(oracle_lib):
    rng = np.random.default_rng(0)
    img = rng.random((23, 31)).astype(np.float32)
    for hw in (1, 3, 5):
        si, sii = O.box_moments(img, hw)
        pad = np.pad(img.astype(np.float64), hw)
        for y in range(img.shape[0]):
            for x in range(img.shape[1]):
                win = pad[y:y + 2 * hw + 1, x:x + 2 * hw + 1]
                assert si[y, x] == pytest.approx(win.sum(), rel=1e-12, abs=1e-12)
                assert sii[y, x] == pytest.approx((win ** 2).sum(), rel=1e-12, abs=1e-12)


@pytest.mark.parametrize("sigma,taps", [(1.0, 5), (0.1, 5), (1.4, 7), (3.0, 15), (20.0, 45)])
def test_prefilter_box_width_and_weights(oracle_lib, sigma, taps):
    img = np.zeros((61, 61), np.float32)
    img[30, 30] = 1.0
    out = O.prefilter(img, 1, sigma)
    r = taps // 2
    # separable box of 1/taps per pass: a centred square of 1/taps^2
    assert np.count_nonzero(out) == taps * taps
    np.testing.assert_allclose(out[30 - r:31 + r, 30 - r:31 + r], 1.0 / taps ** 2, rtol=1e-6)  # float output


def test_prefilter_gaussian_is_normalised(oracle_lib):
    img = np.zeros((41, 41), np.float32)
    img[20, 20] = 1.0
    out = O.prefilter(img, 2, 1.0)
    assert out.sum() == pytest.approx(1.0, rel=1e-6)
    assert out[20, 20] == out.max()
    with pytest.raises(ValueError):
        O.prefilter(img, 2, 0.0)


def test_homographies_map_plane_points(oracle_lib):
    """H1 - H2 / (d s) maps a reference pixel to where its point on the plane with normal n,
    at z-depth d, projects in the source (image.cpp:4-13 with patchMatch.cu:462-474)."""
    rng = np.random.default_rng(1)
    Kr = np.array([[300.0, 0, 160], [0, 300.0, 120], [0, 0, 1]])
    Ks = np.array([[320.0, 0, 150], [0, 310.0, 125], [0, 0, 1]])
    ang = 0.1
    Rr = np.eye(3)
    tr = np.array([0.1, -0.2, 0.05])
    Rs = np.array([[np.cos(ang), 0, np.sin(ang)], [0, 1, 0], [-np.sin(ang), 0, np.cos(ang)]])
    ts = np.array([-0.5, 0.1, 0.2])
    nx, nz = 0.3, 0.9
    hh, ik = O.init_relative(Kr, Rr, tr, Ks, Rs, ts, nx, nz)
    H1, H2 = hh[:9].reshape(3, 3), hh[9:].reshape(3, 3)
    for _ in range(20):
        x, y, d = rng.uniform(0, 320), rng.uniform(0, 240), rng.uniform(2, 8)
        ray = np.linalg.inv(Kr) @ np.array([x, y, 1.0])
        Xc = d * ray                                # ref camera coordinates at z-depth d
        Xw = Rr.T @ (Xc - tr)
        ps = Ks @ (Rs @ Xw + ts)
        scale = nx * (ik[0] * x + ik[1]) + nz       # n^T K^-1 (x, y, 1) with n_y = 0
        q = (H1 - H2 / d / scale) @ np.array([x, y, 1.0])
        np.testing.assert_allclose(q[:2] / q[2], ps[:2] / ps[2], rtol=1e-9, atol=1e-7)


def _kat_oracle(kind, quirks=True):
    rng = np.random.default_rng(4)
    ref = rng.integers(0, 256, (40, 48)).astype(np.float32) / np.float32(255)
    if kind == "identical":
        src = ref.copy()
    elif kind == "flat":
        ref = np.full_like(ref, 90 / 255)
        src = ref.copy()
    else:
        src = np.zeros_like(ref)
    K = np.array([[50.0, 0, 24], [0, 50.0, 20], [0, 0, 1]])
    Ks = K.copy()
    Ks[0, 2] -= 0.5
    Ks[1, 2] -= 0.5
    hh, ik = O.init_relative(K, np.eye(3), np.zeros(3), Ks, np.eye(3), np.zeros(3))
    return O.Oracle(ref, [src], hh[None], ik, 3, 1.0, 10.0, 0.45, 1, quirks=quirks)


@pytest.mark.parametrize("kind,expected", [("identical", 0.0), ("flat", 1.0), ("black", 2.0)])
def test_ncc_special_values(oracle_lib, kind, expected):
    o = _kat_oracle(kind)
    xs, ys = np.meshgrid(np.arange(3, 45), np.arange(3, 37))
    got = o.ncc_batch(xs.ravel(), ys.ravel(), 0, np.full(xs.size, 4.0), 0)
    np.testing.assert_allclose(got, expected, atol=1e-12)


def test_leading_edge_misalignment(oracle_lib):
    """With the reference's pairing (patchMatch.cu:546) a window cut by the leading edge pairs
    source samples with shifted reference values, so identical images no longer score 0 there;
    aligned windows still do."""
    o = _kat_oracle("identical", quirks=True)
    a = _kat_oracle("identical", quirks=False)
    assert o.ncc(1, 20, 0, 4.0, 0) > 0.05          # x < hw, vertical-sweep pairing
    assert a.ncc(1, 20, 0, 4.0, 0) == pytest.approx(0.0, abs=1e-12)
    assert o.ncc(20, 1, 0, 4.0, 0) == pytest.approx(0.0, abs=1e-12)  # the shift is along x only
    assert o.ncc(20, 1, 0, 4.0, 1) > 0.05          # ... and along y for horizontal sweeps


def test_hardware_weight_model(oracle_lib):
    """Texture-unit weights: fractions rounded half-up to 1/256, cross term likewise."""
    ramp = np.zeros((2, 4), np.float32)
    ramp[:, 1] = 1.0
    K = np.eye(3)
    hh = np.zeros((1, 18))
    o = O.Oracle(np.zeros((4, 4), np.float32), [ramp], hh, [1, 0, 1, 0], 1, 1.0, 2.0, 0.45, 1, sampler=1)
    f = np.arange(0, 4096, dtype=np.float32) / 4096
    got = o.sample(0, f, np.zeros_like(f))
    np.testing.assert_array_equal(got, np.floor(f.astype(np.float64) * 256 + 0.5) / 256)


def test_sweep_invariants_and_convergence(oracle_lib):
    from patchmatch_cuda_gb300 import scene
    w = scene.Workload("cpu_small", 96, 72, 3, 3, 2, 2.0, 8.0, 3, 0, seed=9)
    sv = scene.make_views(w)
    o = O.from_images(sv.images, sv.ref_id, _params(w))
    d, c, vs, n = o.run(w.iterations, w.num_samples)
    assert n > 0
    assert d.min() >= w.depth_near and d.max() <= w.depth_far
    assert np.all((vs < w.n_src) | (vs == 255))
    assert np.all(np.isfinite(c))
    # propagation improves on the random start (the ground truth pins convergence)
    start = o.init_depth()
    assert scene.bad_pixel_rate(d.astype(np.float32), sv.gt_depth, 0.05) < \
        0.5 * scene.bad_pixel_rate(start.astype(np.float32), sv.gt_depth, 0.05)


def _params(w):
    from patchmatch_cuda_gb300 import PmParams
    p = PmParams()
    p.depth_near, p.depth_far, p.half_window = w.depth_near, w.depth_far, w.half_window
    p.num_samples, p.sp_alpha, p.gaussian_sigma = w.num_samples, w.sp_alpha, w.gaussian_sigma
    p.prefilter, p.num_iterations, p.orientation_x, p.orientation_z = w.prefilter, w.iterations, 0.0, 1.0
    p.seed, p.quirks = w.seed, 1
    return p


def test_refinement_never_raises_the_sampled_views_mean_cost(oracle_lib):
    """The refinement restatement: with no trials or no sampled views a depth stays; otherwise
    the mean cost over the pixel's sampled views never rises, and depths stay in range."""
    from patchmatch_cuda_gb300 import scene
    w = scene.Workload("cpu_small", 96, 72, 3, 3, 2, 2.0, 8.0, 3, 0, seed=9)
    sv = scene.make_views(w)
    o = O.from_images(sv.images, sv.ref_id, _params(w))
    d, c, vs, _ = o.run(w.iterations, w.num_samples)
    d = d.astype(np.float32).astype(np.float64)
    S = w.num_samples
    same = d.copy()
    assert o.refine(same, vs, S, 0, 0.05, 99, 0) > 0 and np.array_equal(same, d)
    none = np.full_like(vs, 255)
    same = d.copy()
    assert o.refine(same, none, S, 10, 0.05, 99, 0) == 0 and np.array_equal(same, d)
    r = d.copy()
    o.refine(r, vs, S, 10, 0.2, 99, 0)
    assert r.min() >= w.depth_near and r.max() <= w.depth_far
    changed = np.argwhere(r != d)
    assert len(changed) > 0.02 * d.size
    rng = np.random.default_rng(0)
    for y, x in changed[rng.choice(len(changed), 40, replace=False)]:
        views = [int(v) for v in vs[:S, y, x] if v < w.n_src]
        before = np.mean([o.ncc(int(x), int(y), v, float(d[y, x]), 0) for v in views])
        after = np.mean([o.ncc(int(x), int(y), v, float(r[y, x]), 0) for v in views])
        assert after < before
