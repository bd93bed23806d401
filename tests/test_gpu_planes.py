"""Slanted-plane mode (pm_params.planes = 1; no counterpart in the reference, whose plane normal
is one constant, patchMatch.cu:32) against the oracle's restatement, stage by stage (needs a GPU).

The hypotheses are formed in the same single-precision steps on both sides (initial slopes,
the previous step's plane carried to the next pixel, the three kinds of random hypothesis), so
a sweep's decisions match until an FP32-vs-FP64 near-tie of the argmin or the CDF; costs use
the tolerances of the reference-mode tests (1e-4, with the exact sampler's tail at source edges
within 5e-4; 5e-4 texture filtering).
"""
import numpy as np
import pytest

from parity_util import EXACT_TAIL_TOL, NCC_TOL, first_divergence, ncc_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_scene():
    from patchmatch_cuda_gb300 import scene
    return scene.make_views(scene.WORKLOADS["plane3_320x240"])


def make_engine(sv, **over):
    from patchmatch_cuda_gb300 import Engine
    over.setdefault("sampler", 0)
    over.setdefault("planes", 1)
    return Engine(sv.images, sv.ref_id, sv.workload.params(**over))


def oracle_for(eng, sv):
    from oracle import pm_oracle
    src = [eng.source_texels(v) for v in range(eng.n_src)]
    ref, _, _ = eng.ref_maps()
    orc = pm_oracle.from_images(sv.images, sv.ref_id, eng.params, source_texels=src, ref_texels=ref)
    assert orc.p.planes == 1
    return orc


def test_initial_planes_match_oracle(small_scene):
    eng = make_engine(small_scene)
    orc = oracle_for(eng, small_scene)
    eng.init_depth()
    np.testing.assert_array_equal(eng.slopes(), orc.init_planes())
    np.testing.assert_allclose(eng.depth(), orc.init_depth(), rtol=2e-7, atol=1e-6)
    n = eng.normals()
    s = eng.slopes()
    want = np.concatenate([s, np.ones(s.shape[:2] + (1,), np.float32)], axis=2)
    want /= np.linalg.norm(want, axis=2, keepdims=True)
    np.testing.assert_allclose(n, want, atol=1e-6)
    eng.close()


@pytest.mark.parametrize("sampler", [0, 1])
def test_plane_ncc_parity(small_scene, sampler, parity_log):
    eng = make_engine(small_scene, sampler=sampler)
    orc = oracle_for(eng, small_scene)
    rng = np.random.default_rng(12)
    n = 4096
    w = small_scene.workload
    xs = rng.integers(0, w.width, n)
    ys = rng.integers(0, w.height, n)
    xs[:256] = rng.integers(0, w.half_window + 1, 256)  # leading edges
    vs = rng.integers(0, w.n_src, n)
    gt = small_scene.gt_depth[ys, xs]
    ds = np.where(rng.random(n) < 0.5, gt, rng.uniform(w.depth_near, w.depth_far, n)).astype(np.float32)
    sl = rng.uniform(-1.5, 1.5, (n, 2)).astype(np.float32)
    sl[:64] = 0.0
    ax = rng.integers(0, 2, n)
    got = eng.eval_costs_planes(xs, ys, vs, ds, sl, ax)
    want = orc.ncc_plane_batch(xs, ys, vs, ds, sl, ax)
    err = ncc_err(got, want)
    parity_log(f"plane_ncc_sampler{sampler}", n=n, err_max=float(err.max()), err_q999=float(np.quantile(err, 0.999)))
    if sampler == 0:
        assert err.max() <= NCC_TOL, f"max NCC error {err.max():.3g}"
    else:
        assert np.quantile(err, 0.999) <= 5 * NCC_TOL and err.max() <= 20 * NCC_TOL
    eng.close()


def test_plane_initial_costs_match_oracle(small_scene, parity_log):
    eng = make_engine(small_scene)
    orc = oracle_for(eng, small_scene)
    eng.init_depth()
    eng.compute_costs(1)
    c = eng.costs()
    oc = orc.initial_costs_planes(eng.depth().astype(np.float64), eng.slopes())
    err = ncc_err(c, oc)
    parity_log("plane_initial_costs", n=int(err.size), err_max=float(err.max()),
               err_q9999=float(np.quantile(err, 0.9999)))
    assert np.quantile(err, 0.9999) <= NCC_TOL and err.max() <= 3 * NCC_TOL
    eng.close()


def _lockstep(eng, orc, sv, direction, sweep_id):
    eng.init_depth()
    eng.compute_costs(1)
    d0 = eng.depth().astype(np.float64)
    s0 = eng.slopes()
    c0 = eng.costs().astype(np.float64)
    S = sv.workload.num_samples
    eng.run_sweep(direction, sweep_id, S)
    gd, gs, gc = eng.depth(), eng.slopes(), eng.costs()
    od, os_, oc = d0.copy(), s0.copy(), c0.copy()
    orc.sweep_planes(od, os_, oc, direction, sweep_id, S)
    prefix, nsteps = first_divergence(gd, od, direction)
    mask = np.zeros(gd.shape, bool)
    for line, p in enumerate(prefix):
        steps = np.arange(p)
        if direction in (2, 3):
            steps = nsteps - 1 - steps
        if direction in (0, 2):
            mask[line, steps] = True
        else:
            mask[steps, line] = True
    events = int(np.sum(prefix < nsteps))
    decisions = int(np.sum(np.minimum(prefix + 1, nsteps)))
    return events, decisions, mask, (gd, gs, gc), (od, os_, oc), (d0, s0)


@pytest.mark.parametrize("sampler", [0, 1])
@pytest.mark.parametrize("direction", [0, 1, 2, 3])
def test_plane_sweep_lockstep(small_scene, direction, sampler, parity_log):
    """One sweep from the same state: decisions, slopes and costs match the oracle until a
    near-tie flips a line; such events must be rare."""
    eng = make_engine(small_scene, sampler=sampler)
    orc = oracle_for(eng, small_scene)
    events, decisions, mask, (gd, gs, gc), (od, os_, oc), (d0, s0) = _lockstep(eng, orc, small_scene, direction,
                                                                             4 + direction)
    cerr = ncc_err(gc, oc)[mask]
    slopes_equal = float(np.mean(np.all(gs == os_, axis=2)[mask]))
    changed = float(np.mean(np.any(gs != s0, axis=2)))
    parity_log(f"plane_sweep_lockstep_dir{direction}_sampler{sampler}", divergence_events=events,
               decisions=decisions, matched_fraction=float(mask.mean()), cost_err_max=float(cerr.max()),
               cost_err_q999=float(np.quantile(cerr, 0.999)), slopes_equal_matched=slopes_equal,
               slopes_changed=changed)
    assert events / decisions <= 2e-4, f"{events} divergences in {decisions} decisions"
    assert np.quantile(cerr, 0.999) <= NCC_TOL and cerr.max() <= EXACT_TAIL_TOL
    assert slopes_equal == 1.0
    assert changed > 0.05  # the sweep does move planes
    eng.close()


@pytest.mark.parametrize("sampler", [0, 1])
def test_plane_full_run_matches_oracle(small_scene, sampler, parity_log):
    """12 sweeps from the same seed. The texture-filtering sampler forms its coordinates in the
    oracle's single-precision steps: at least 99.5% of depths within 0.1%. The exact sampler
    evaluates its NCC in FP32 against the oracle's FP64 (within 1e-4): a rare near-tie flips a
    decision, and with per-pixel planes the flipped plane is carried along the rest of the line
    and into later sweeps, so the bar is 99% (every single sweep matches: the lockstep test)."""
    from patchmatch_cuda_gb300 import scene
    eng = make_engine(small_scene, sampler=sampler)
    orc = oracle_for(eng, small_scene)
    eng.run()
    gd = eng.depth()
    w = small_scene.workload
    od, os_, oc, ovs, n = orc.run_planes(w.iterations, w.num_samples)
    rel = np.abs(gd - od) / od
    frac = float(np.mean(rel <= 1e-3))
    bad_g = scene.bad_pixel_rate(gd, small_scene.gt_depth)
    bad_o = scene.bad_pixel_rate(od.astype(np.float32), small_scene.gt_depth)
    parity_log(f"plane_full_run_sampler{sampler}", within_0p1pct=frac, bad1_gpu=bad_g, bad1_oracle=bad_o)
    assert abs(bad_g - bad_o) <= 0.01, (bad_g, bad_o)
    assert frac >= (0.995 if sampler == 1 else 0.99), f"only {frac:.4f} of depths within 0.1% of the oracle"
    eng.close()


def test_plane_refinement_matches_oracle(small_scene, parity_log):
    eng = make_engine(small_scene)
    orc = oracle_for(eng, small_scene)
    eng.run()
    d0 = eng.depth().astype(np.float64)
    vs = eng.view_selection()
    S = small_scene.workload.num_samples
    eng.refine(10, 0.05, 77, S, 0)
    gd = eng.depth()
    od = d0.copy()
    orc.refine_planes(od, eng.slopes(), vs, S, 10, 0.05, 77, 0)
    within = float(np.mean(np.abs(gd - od) / od <= 1e-3))
    identical = float(np.mean(gd == od.astype(np.float32)))
    parity_log("plane_refine", within_0p1pct=within, bit_identical=identical)
    assert within >= 0.995 and identical >= 0.99
    eng.close()


def test_plane_mode_sharpens_depths(small_scene, parity_log):
    """On a scene of slanted planes, per-pixel planes reach a lower median depth error than the
    reference's one fronto-parallel normal, at no worse 1 % bad-pixel rate (6 iterations)."""
    from patchmatch_cuda_gb300 import scene
    gt = small_scene.gt_depth
    res = {}
    for planes in (0, 1):
        eng = make_engine(small_scene, planes=planes, sampler=1, num_iterations=6)
        eng.run()
        d = eng.depth()
        rel = np.abs(d - gt) / gt
        res[planes] = (float(np.median(rel)), scene.bad_pixel_rate(d, gt), float(np.mean(rel > 0.002)))
        eng.close()
    parity_log("plane_mode_accuracy_plane3", reference_median=res[0][0], planes_median=res[1][0],
               reference_bad1=res[0][1], planes_bad1=res[1][1], reference_bad02=res[0][2], planes_bad02=res[1][2])
    assert res[1][0] < 0.9 * res[0][0]
    assert res[1][1] <= res[0][1] + 0.002


def test_plane_batch_equals_single_runs(small_scene):
    from patchmatch_cuda_gb300 import Batch
    a = make_engine(small_scene, sampler=1)
    a.run()
    want_d, want_s = a.depth(), a.slopes()
    b = make_engine(small_scene, sampler=1)
    c = make_engine(small_scene, sampler=1, planes=0)
    batch = Batch([b, c])
    batch.run()
    np.testing.assert_array_equal(b.depth(), want_d)
    np.testing.assert_array_equal(b.slopes(), want_s)
    single = make_engine(small_scene, sampler=1, planes=0)
    single.run()
    np.testing.assert_array_equal(c.depth(), single.depth())
    batch.close()
    for e in (a, b, c, single):
        e.close()


def test_slopes_need_plane_mode(small_scene):
    from patchmatch_cuda_gb300._native import PatchMatchError
    eng = make_engine(small_scene, planes=0)
    with pytest.raises(PatchMatchError, match="STATE"):
        eng.slopes()
    with pytest.raises(PatchMatchError, match="STATE"):
        eng.eval_costs_planes([1], [1], [0], [3.0], [[0.0, 0.0]], [0])
    eng.close()


def test_learned_initialisation_with_planes(small_scene):
    """A learned initialisation in plane mode: pixels taken from the network start
    fronto-parallel, the others exactly as the random initialisation (threshold 1: all of
    them), and a short run keeps depths in range and slopes finite."""
    from patchmatch_cuda_gb300 import INIT_PROPOSAL, proposal
    rnd = make_engine(small_scene, sampler=1)
    orc = oracle_for(rnd, small_scene)
    want_slopes = orc.init_planes()
    rnd.init_depth()
    want_depth = rnd.depth()
    all_rand = make_engine(small_scene, sampler=1, init_mode=INIT_PROPOSAL, proposal_threshold=1.0)
    all_net = make_engine(small_scene, sampler=1, init_mode=INIT_PROPOSAL, proposal_threshold=0.0, num_sweeps=2)
    hp, wp = all_rand.proposal_shape()
    net = proposal.ProposalNet(1, hp, wp, seed=3)
    all_rand.set_proposal(net)
    all_net.set_proposal(net)
    all_rand.init_depth()
    np.testing.assert_array_equal(all_rand.slopes(), want_slopes)
    np.testing.assert_array_equal(all_rand.depth(), want_depth)
    all_net.init_depth()
    assert np.all(all_net.slopes() == 0.0)
    all_net.run()
    d, s = all_net.depth(), all_net.slopes()
    w = small_scene.workload
    assert np.all(np.isfinite(d)) and d.min() >= w.depth_near and d.max() <= w.depth_far
    assert np.all(np.isfinite(s)) and np.abs(s).max() <= 2.0
    for e in (rnd, all_rand, all_net):
        e.close()
    net.close()
