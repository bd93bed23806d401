"""Parity of the CUDA kernels against the CPU oracle, stage by stage (needs a GPU).

Tolerances: source sampling 2e-6 absolute (FP32 weights vs FP64); NCC 1e-4 absolute for
costs in [0, 2] and 1e-4 relative beyond (windows at a leading edge, where the reference's
misaligned pairing of reference and source samples lets 1 - NCC leave [0, 2]); box moments
1e-5 relative; Philox bit-exact.
"""
import numpy as np
import pytest

from parity_util import (EXACT_TAIL_TOL, NCC_TOL, divergence_stats, first_divergence, matched_mask, ncc_err,  # noqa: F401
                         view_selection_mismatches)

pytestmark = pytest.mark.gpu


def bilinear_ref(img, xs, ys):
    """Exact bilinear at (xs, ys), texel i at coordinate i, zero border (float64)."""
    h, w = img.shape
    out = np.zeros(xs.shape, np.float64)
    for i, (x, y) in enumerate(zip(xs.astype(np.float64), ys.astype(np.float64))):
        if not (-1 < x < w and -1 < y < h):
            continue
        x0, y0 = int(np.floor(x)), int(np.floor(y))
        ax, ay = x - x0, y - y0

        def t(a, b):
            return float(img[b, a]) if 0 <= a < w and 0 <= b < h else 0.0
        out[i] = ((1 - ax) * (1 - ay) * t(x0, y0) + ax * (1 - ay) * t(x0 + 1, y0)
                  + (1 - ax) * ay * t(x0, y0 + 1) + ax * ay * t(x0 + 1, y0 + 1))
    return out


@pytest.fixture(scope="module")
def small_scene():
    from patchmatch_cuda_gb300 import scene
    w = scene.WORKLOADS["plane3_320x240"]
    return scene.make_views(w)


def make_engine(sv, **over):
    """The exact-gather sampler unless a test asks otherwise: the strict 1e-4 NCC bound."""
    from patchmatch_cuda_gb300 import Engine
    over.setdefault("sampler", 0)
    return Engine(sv.images, sv.ref_id, sv.workload.params(**over))


def oracle_for(eng, sv, params=None):
    from oracle import pm_oracle
    src = [eng.source_texels(v) for v in range(eng.n_src)]
    ref, si, sii = eng.ref_maps()
    return pm_oracle.from_images(sv.images, sv.ref_id, params or eng.params, source_texels=src, ref_texels=ref)


@pytest.mark.parametrize("prefilter,precision", [(0, 0), (1, 0), (1, 1)])
def test_source_sampling_exact_bilinear(small_scene, prefilter, precision):
    eng = make_engine(small_scene, prefilter=prefilter, precision=precision)
    rng = np.random.default_rng(1)
    tex = eng.source_texels(1)
    h, w = tex.shape
    xs = rng.uniform(-3, w + 2, 3000).astype(np.float32)
    ys = rng.uniform(-3, h + 2, 3000).astype(np.float32)
    xs[:50] = np.arange(50, dtype=np.float32)  # exact texel positions
    ys[:50] = 7.0
    got = eng.sample_source(1, xs, ys)
    want = bilinear_ref(tex, xs, ys)
    np.testing.assert_allclose(got, want, atol=2e-6, rtol=0)
    eng.close()


@pytest.mark.parametrize("texel_format,tol", [(4, 2e-7), (1, 2e-5)])
def test_hardware_sampler_matches_fixed_point_model(small_scene, texel_format, tol, parity_log):
    """Texture-unit bilinear filtering equals the oracle's fixed-point model: fractions and
    their product rounded half-up to 1/256 (FP32 texels exactly; u8 texels to the filter's
    output precision, about 2^-17)."""
    over = dict(sampler=1, texel_format=texel_format, prefilter=1 if texel_format == 4 else 0)
    eng = make_engine(small_scene, **over)
    orc = oracle_for(eng, small_scene, small_scene.workload.params(**over))
    rng = np.random.default_rng(5)
    h, w = eng.source_texels(2).shape
    xs = rng.uniform(-2, w + 1, 20000).astype(np.float32)
    ys = rng.uniform(-2, h + 1, 20000).astype(np.float32)
    got = eng.sample_source(2, xs, ys)
    err = np.abs(got - orc.sample(2, xs, ys))
    parity_log(f"hw_sampler_texels{texel_format}", err_max=float(err.max()))
    assert err.max() <= tol
    eng.close()


@pytest.mark.parametrize("texel_format", [4, 1])
def test_ncc_parity_hardware_sampler(small_scene, texel_format, parity_log):
    """NCC through texture-unit filtering against the oracle's fixed-point model. The GPU forms
    source coordinates in FP32, so near a 1/256 weight boundary it can round a fraction the
    other way than the FP64 oracle; the bound reflects those single-step weight flips."""
    over = dict(sampler=1, texel_format=texel_format, prefilter=1 if texel_format == 4 else 0)
    eng = make_engine(small_scene, **over)
    orc = oracle_for(eng, small_scene, small_scene.workload.params(**over))
    rng = np.random.default_rng(6)
    n = 4096
    w = small_scene.workload
    xs = rng.integers(0, w.width, n)
    ys = rng.integers(0, w.height, n)
    vs = rng.integers(0, w.n_src, n)
    gt = small_scene.gt_depth[ys, xs]
    ds = np.where(rng.random(n) < 0.5, gt, rng.uniform(w.depth_near, w.depth_far, n)).astype(np.float32)
    ax = rng.integers(0, 2, n)
    err = ncc_err(eng.eval_costs(xs, ys, vs, ds, ax), orc.ncc_batch(xs, ys, vs, ds, ax))
    parity_log(f"ncc_hw_texels{texel_format}", err_max=float(err.max()), err_q999=float(np.quantile(err, 0.999)),
               err_median=float(np.median(err)))
    assert np.quantile(err, 0.999) <= 5 * NCC_TOL and err.max() <= 20 * NCC_TOL
    eng.close()


def test_u8_texels_are_unorm(small_scene):
    eng = make_engine(small_scene, prefilter=0)
    src = [im for i, im in enumerate(small_scene.images) if i != small_scene.ref_id][0]
    np.testing.assert_array_equal(eng.source_texels(0), src.image.astype(np.float32) / np.float32(255))
    ref, _, _ = eng.ref_maps()
    np.testing.assert_array_equal(ref, small_scene.images[small_scene.ref_id].image.astype(np.float32) / np.float32(255))
    eng.close()


def test_reference_moments_and_prefilter(small_scene):
    from oracle import pm_oracle
    eng = make_engine(small_scene, prefilter=1)
    ref, si, sii = eng.ref_maps()
    raw = small_scene.images[small_scene.ref_id].image.astype(np.float32) / np.float32(255)
    want_ref = pm_oracle.prefilter(raw, 1, 1.0)
    np.testing.assert_allclose(ref, want_ref, rtol=1e-6, atol=1e-6)
    osi, osii = pm_oracle.box_moments(ref, small_scene.workload.half_window)
    np.testing.assert_allclose(si, osi, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(sii, osii, rtol=1e-5, atol=1e-5)
    eng.close()


@pytest.mark.parametrize("quirks", [1, 0])
def test_ncc_parity(small_scene, quirks, parity_log):
    eng = make_engine(small_scene, quirks=quirks)
    orc = oracle_for(eng, small_scene)
    rng = np.random.default_rng(2)
    n = 4096
    w = small_scene.workload
    xs = rng.integers(0, w.width, n)
    ys = rng.integers(0, w.height, n)
    xs[:256] = rng.integers(0, w.half_window + 1, 256)  # leading edges, where the quirk acts
    ys[256:512] = rng.integers(0, w.half_window + 1, 256)
    vs = rng.integers(0, w.n_src, n)
    gt = small_scene.gt_depth[ys, xs]
    ds = np.where(rng.random(n) < 0.5, gt, rng.uniform(w.depth_near, w.depth_far, n)).astype(np.float32)
    ax = rng.integers(0, 2, n)
    got = eng.eval_costs(xs, ys, vs, ds, ax)
    want = orc.ncc_batch(xs, ys, vs, ds, ax)
    err = ncc_err(got, want)
    parity_log(f"ncc_quirks{quirks}", n=n, err_max=float(err.max()), err_median=float(np.median(err)),
               unbounded_values=int(np.sum(np.abs(want) > 2)))
    assert np.quantile(err, 0.999) <= NCC_TOL, f"NCC error q999 {np.quantile(err, 0.999):.3g}"
    assert err.max() <= EXACT_TAIL_TOL, f"max NCC error {err.max():.3g} at {np.argmax(err)}"
    eng.close()


def kat_views(kind):
    """Reference plus one source whose principal point is shifted by half a pixel, so the
    plane-induced homography maps reference pixel centre i + 1/2 onto source texel i."""
    from patchmatch_cuda_gb300 import Image
    rng = np.random.default_rng(4)
    ref = rng.integers(0, 256, (40, 48)).astype(np.uint8)
    if kind == "identical":
        src = ref.copy()
    elif kind == "flat":
        ref = np.full_like(ref, 90)
        src = ref.copy()
    else:  # black source
        src = np.zeros_like(ref)
    K = np.array([[50.0, 0, 24], [0, 50.0, 20], [0, 0, 1]])
    Ks = K.copy()
    Ks[0, 2] -= 0.5
    Ks[1, 2] -= 0.5
    I3, z = np.eye(3), np.zeros(3)
    return [Image(K, I3, z, ref), Image(Ks, I3, z, src)]


@pytest.mark.parametrize("kind,expected", [("identical", 0.0), ("flat", 1.0), ("black", 2.0)])
def test_ncc_known_answers(kind, expected):
    from patchmatch_cuda_gb300 import Engine, default_params
    p = default_params()
    p.depth_near, p.depth_far, p.half_window = 1.0, 10.0, 3
    eng = Engine(kat_views(kind), 0, p)
    xs, ys = np.meshgrid(np.arange(3, 45), np.arange(3, 37))
    xs, ys = xs.ravel(), ys.ravel()
    got = eng.eval_costs(xs, ys, np.zeros_like(xs), np.full(xs.shape, 4.0, np.float32), 0)
    np.testing.assert_allclose(got, expected, atol=1e-5)
    eng.close()


def test_philox_matches_oracle(engine_lib):
    import ctypes as C
    from oracle import pm_oracle
    rng = np.random.default_rng(3)
    ctr = rng.integers(0, 2**32, (257, 4), dtype=np.uint64).astype(np.uint32)
    out = np.zeros_like(ctr)
    seed = 0x1234_5678_9ABC_DEF0
    assert engine_lib.pm_philox(seed, len(ctr), ctr.ctypes.data, out.ctypes.data) == 0
    key = np.array([seed & 0xFFFFFFFF, seed >> 32], np.uint32)
    for i in range(len(ctr)):
        np.testing.assert_array_equal(out[i], pm_oracle.philox(ctr[i], key))


def test_newton_reciprocal_is_correctly_rounded(engine_lib):
    """The samplers' 1/z (hardware approximation + one Newton correction) equals the correctly
    rounded reciprocal for every significand, both signs, of every binade from 2^-120 to 2^120:
    the oracle's single-precision coordinates rest on that."""
    import ctypes as C
    failing = []
    for exp_shift in range(-120, 121):
        bad = C.c_ulonglong(0)
        assert engine_lib.pm_check_reciprocal(exp_shift, C.byref(bad)) == 0
        if bad.value:
            failing.append((exp_shift, bad.value))
    assert not failing, failing


def test_initial_depth_and_costs_match_oracle(small_scene, parity_log):
    eng = make_engine(small_scene)
    orc = oracle_for(eng, small_scene)
    eng.init_depth()
    d = eng.depth()
    od = orc.init_depth()
    np.testing.assert_allclose(d, od, rtol=2e-7, atol=1e-6)
    eng.compute_costs(1)
    c = eng.costs()
    oc = orc.initial_costs(d.astype(np.float64))
    err = ncc_err(c, oc)
    i = np.unravel_index(np.argmax(err), err.shape)
    parity_log("initial_costs", n=int(err.size), err_max=float(err.max()),
               err_q9999=float(np.quantile(err, 0.9999)), worst_pixel=[int(i[1]), int(i[0])],
               worst_view=int(i[2]), worst_gpu=float(c[i]), worst_oracle=float(oc[i]),
               frac_over_tol=float(np.mean(err > NCC_TOL)))
    assert np.quantile(err, 0.9999) <= NCC_TOL, f"cost error q9999 {np.quantile(err, 0.9999):.3g}"
    assert err.max() <= 3 * NCC_TOL, f"max cost error {err.max():.3g} at {i}: {c[i]} vs {oc[i]}"
    eng.close()


@pytest.mark.parametrize("sampler", [0, 1])
@pytest.mark.parametrize("direction", [0, 1, 2, 3])
def test_sweep_lockstep(small_scene, direction, sampler, parity_log):
    """One sweep from the same state. Decisions match until an argmin or CDF near-tie flips
    (FP32 vs FP64), after which a line legitimately diverges; such events must be rare, and
    every cost before a line's first divergence matches to the NCC tolerance at the 99.9th
    percentile and within 5x it everywhere (the exact sampler's tail at source edges, see
    parity_util; the texture-filtering sampler's NCC bound is 5x too, see its NCC test)."""
    eng = make_engine(small_scene, sampler=sampler)
    orc = oracle_for(eng, small_scene)
    eng.init_depth()
    eng.compute_costs(1)
    d0 = eng.depth().astype(np.float64)
    c0 = eng.costs().astype(np.float64)
    S = small_scene.workload.num_samples
    eng.run_sweep(direction, 4 + direction, S, record_views=True)
    gd, gc, gvs = eng.depth(), eng.costs(), eng.view_selection()
    od, oc = d0.copy(), c0.copy()
    ovs = np.full(gvs.shape, 255, np.uint8)
    orc.sweep(od, oc, direction, 4 + direction, S, view_sel=ovs)
    prefix, nsteps = first_divergence(gd, od, direction)
    events, decisions = divergence_stats(prefix, nsteps)
    rate = events / decisions
    mask = matched_mask(gd.shape, prefix, nsteps, direction)
    cerr = ncc_err(gc, oc)[mask]
    vs_bad = view_selection_mismatches(gvs, ovs, mask)
    parity_log(f"sweep_lockstep_dir{direction}_sampler{sampler}", divergence_events=events, decisions=decisions,
               divergence_rate=rate, matched_fraction=float(mask.mean()),
               cost_err_max=float(cerr.max()), cost_err_q999=float(np.quantile(cerr, 0.999)),
               view_sel_checked=int(S * mask.sum()), view_sel_mismatches=vs_bad)
    assert rate <= 2e-4, f"{events} divergences in {decisions} decisions"
    assert np.quantile(cerr, 0.999) <= NCC_TOL, f"cost error q999 {np.quantile(cerr, 0.999):.3g}"
    assert cerr.max() <= EXACT_TAIL_TOL, f"cost error {cerr.max():.3g} before divergence"
    # the sampled views (usedImgsID, patchMatch.cu:1159-1163) are indices: equal entry for entry
    # but for CDF near-ties (a uniform within a rounding step of a CDF value), which leave the
    # decision unchanged
    assert vs_bad <= 5e-5 * S * mask.sum(), f"{vs_bad} view-selection entries differ before divergence"
    eng.close()


@pytest.mark.parametrize("sampler", [0, 1])
def test_full_run_matches_oracle(small_scene, sampler, parity_log):
    """The end-to-end parity bar: at least 99.5% of final depths within 0.1% of the oracle's."""
    from patchmatch_cuda_gb300 import scene
    eng = make_engine(small_scene, sampler=sampler)
    orc = oracle_for(eng, small_scene)
    eng.run()
    gd = eng.depth()
    w = small_scene.workload
    od, oc, ovs, n = orc.run(w.iterations, w.num_samples)
    rel = np.abs(gd - od) / od
    frac = float(np.mean(rel <= 1e-3))
    bad_g = scene.bad_pixel_rate(gd, small_scene.gt_depth)
    bad_o = scene.bad_pixel_rate(od.astype(np.float32), small_scene.gt_depth)
    # the last sweep's sampled views: equal wherever the lines did not diverge before
    gvs = eng.view_selection()
    vs_same = float(np.mean(np.all(gvs == ovs, axis=0)))
    parity_log(f"full_run_plane3_320x240_sampler{sampler}", within_0p1pct=frac, bad1_gpu=bad_g, bad1_oracle=bad_o,
               view_sel_equal=vs_same)
    assert abs(bad_g - bad_o) <= 0.01, (bad_g, bad_o)
    assert frac >= 0.995, f"only {frac:.4f} of depths within 0.1% of the oracle"
    assert vs_same >= 0.99, f"view selection equal on only {vs_same:.4f} of the pixels"
    st = eng.stats()
    assert st.cost_evals > 0
    eng.close()


@pytest.mark.parametrize("direction", [1, 2])
def test_sweep_lockstep_local_search(small_scene, direction, parity_log):
    """The local random search (perturbation > 0, no counterpart in the reference) against the
    oracle's restatement of it: same decisions and costs as the plain lockstep test."""
    eng = make_engine(small_scene, perturbation=0.05)
    orc = oracle_for(eng, small_scene)
    assert abs(orc.p.perturbation - 0.05) < 1e-7
    eng.init_depth()
    eng.compute_costs(1)
    d0 = eng.depth().astype(np.float64)
    c0 = eng.costs().astype(np.float64)
    S = small_scene.workload.num_samples
    eng.run_sweep(direction, 4 + direction, S)
    gd, gc = eng.depth(), eng.costs()
    od, oc = d0.copy(), c0.copy()
    orc.sweep(od, oc, direction, 4 + direction, S)
    prefix, nsteps = first_divergence(gd, od, direction)
    events, decisions = divergence_stats(prefix, nsteps)
    changed = float(np.mean(np.abs(gd - d0) > 1e-6 * d0))
    parity_log(f"sweep_lockstep_local_search_dir{direction}", divergence_events=events, decisions=decisions,
               changed_fraction=changed)
    assert events / decisions <= 2e-4, f"{events} divergences in {decisions} decisions"
    assert changed > 0.05
    eng.close()


@pytest.mark.parametrize("sampler", [0, 1])
def test_refinement_matches_oracle(small_scene, sampler, parity_log):
    """pm_refine from the same depth map and view selection as the oracle's restatement: the
    hypotheses are the same FP32 numbers, so only near-ties between FP32 and FP64 mean costs
    may pick differently; at least 99.5% of depths within 0.1% (most bit-identical)."""
    eng = make_engine(small_scene, sampler=sampler)
    orc = oracle_for(eng, small_scene)
    eng.run()
    d0 = eng.depth().astype(np.float64)
    vs = eng.view_selection()
    S = small_scene.workload.num_samples
    eng.refine(10, 0.05, 77, S, 0)
    gd = eng.depth()
    od = d0.copy()
    orc.refine(od, vs, S, 10, 0.05, 77, 0)
    rel = np.abs(gd - od) / od
    within = float(np.mean(rel <= 1e-3))
    identical = float(np.mean(gd == od.astype(np.float32)))
    changed = float(np.mean(gd != d0.astype(np.float32)))
    parity_log(f"refine_plane3_320x240_sampler{sampler}", within_0p1pct=within, bit_identical=identical,
               changed=changed)
    assert within >= 0.995 and identical >= 0.99
    assert changed > 0.02
    eng.close()


def test_texture_peak_is_plausible(engine_lib):
    """The measured texture-filtering rate the bench reports the sweep kernel against: between
    1 and 5 bilinear samples per clock per SM."""
    import ctypes as C
    import torch
    r = C.c_double(0.0)
    assert engine_lib.pm_texture_peak(C.byref(r)) == 0
    props = torch.cuda.get_device_properties(0)
    per_sm_clk = r.value / (props.multi_processor_count * 2.07e9)
    assert 1.0 <= per_sm_clk <= 5.0, per_sm_clk
