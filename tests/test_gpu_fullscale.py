"""Parity at the full-scale configuration's parameters (needs a GPU): box2000_3072x2048 -- a
3072x2048 reference with 20 source views, 19x19 window (the whole-warp NCC layout, one column
per lane), numOfSamples 5, depth [0.5, 50], 60 planes + 2000 boxes, u8 texels, texture-unit
sampler (the batched full-scale workload runs eight such references).

* NCC on the full 3072x2048 reference, borders included, both samplers;
* the initial costs and the whole 5-iteration schedule on a 256x160 crop of the same reference
  (same cameras and sources, small enough for the FP64 oracle): every sweep in lockstep from the
  oracle's state, and the plain run end to end.

Bounds are those of tests/test_gpu_headline.py (the benchmarked configuration), which explains
them: NCC 1e-4 at the 99.99th percentile, special-value flips and far-from-origin low-variance
windows bounded separately, near-ties bounded per decision.
"""
import numpy as np
import pytest

from parity_util import NCC_TOL, agreement, float_floor, ncc_err, special_value_flips, whole_run_lockstep

pytestmark = pytest.mark.gpu

HW_TOL_Q999 = 5 * NCC_TOL
HW_TOL_MAX = 20 * NCC_TOL


@pytest.fixture(scope="module")
def fullscale():
    from patchmatch_cuda_gb300 import scene
    return scene.make_views(scene.WORKLOADS["box2000_3072x2048"])


@pytest.fixture(scope="module")
def fullscale_crop(fullscale):
    from patchmatch_cuda_gb300 import scene
    return scene.crop_reference(fullscale, 1408, 944, 256, 160)


def make_engine(sv, **over):
    from patchmatch_cuda_gb300 import Engine
    return Engine(sv.images, sv.ref_id, sv.workload.params(**over))


def oracle_for(eng, sv):
    from oracle import pm_oracle
    src = [eng.source_texels(v) for v in range(eng.n_src)]
    ref, _, _ = eng.ref_maps()
    return pm_oracle.from_images(sv.images, sv.ref_id, eng.params, source_texels=src, ref_texels=ref)


def test_fullscale_parameters(fullscale):
    w = fullscale.workload
    assert (w.width, w.height, w.n_src, 2 * w.half_window + 1, w.num_samples, w.depth_near, w.depth_far) == \
        (3072, 2048, 20, 19, 5, 0.5, 50.0)


@pytest.mark.parametrize("sampler", [0, 1])
def test_fullscale_ncc(fullscale, sampler, parity_log):
    eng = make_engine(fullscale, sampler=sampler)
    orc = oracle_for(eng, fullscale)
    w = fullscale.workload
    rng = np.random.default_rng(19)
    n = 4096
    xs, ys = rng.integers(0, w.width, n), rng.integers(0, w.height, n)
    hw = w.half_window
    xs[:256] = rng.integers(0, hw + 1, 256)
    ys[256:512] = rng.integers(0, hw + 1, 256)
    xs[512:768] = rng.integers(w.width - hw - 1, w.width, 256)
    ys[768:1024] = rng.integers(w.height - hw - 1, w.height, 256)
    vs = rng.integers(0, w.n_src, n)
    gt = fullscale.gt_depth[ys, xs]
    ds = np.where(rng.random(n) < 0.5, gt, rng.uniform(w.depth_near, w.depth_far, n)).astype(np.float32)
    ax = rng.integers(0, 2, n)
    got = eng.eval_costs(xs, ys, vs, ds, ax)
    want = orc.ncc_batch(xs, ys, vs, ds, ax)
    err = ncc_err(got, want)
    flips = special_value_flips(got, want)
    rest = err[~flips]
    parity_log(f"fullscale_ncc_sampler{sampler}", n=n, err_q999=float(np.quantile(err, 0.999)),
               err_max_other=float(rest.max()), special_value_flips=int(flips.sum()),
               err_median=float(np.median(err)))
    assert flips.sum() <= 1
    if sampler == 0:
        assert np.quantile(err, 0.999) <= NCC_TOL and rest.max() <= 5 * NCC_TOL
    else:
        assert np.quantile(err, 0.999) <= HW_TOL_Q999 and rest.max() <= HW_TOL_MAX
    eng.close()


def test_fullscale_initial_costs(fullscale_crop, parity_log):
    eng = make_engine(fullscale_crop)
    orc = oracle_for(eng, fullscale_crop)
    eng.init_depth()
    d = eng.depth()
    eng.compute_costs(1)
    c = eng.costs()
    oc = orc.initial_costs(d.astype(np.float64))
    err = ncc_err(c, oc)
    flips = special_value_flips(c, oc)
    rest = err[~flips]
    q = float(np.quantile(err, 0.9999))
    parity_log("fullscale_initial_costs_crop256x160", n=int(err.size), err_q9999=q,
               special_value_flips=int(flips.sum()), err_max_other=float(rest.max()))
    assert q <= NCC_TOL
    assert flips.sum() <= max(1, 1e-6 * err.size)
    assert rest.max() <= HW_TOL_MAX
    eng.close()


def test_fullscale_whole_run_lockstep(fullscale_crop, parity_log):
    """All 20 sweeps of the schedule with 20 views and a 19x19 window, each from the oracle's
    state: near-ties at most 1e-4 per decision, costs before each line's first divergence
    within the NCC bounds."""
    sv = fullscale_crop
    w = sv.workload
    eng = make_engine(sv)
    orc = oracle_for(eng, sv)
    rows = whole_run_lockstep(eng, orc, w.iterations, w.num_samples)
    events = sum(r[0] for r in rows)
    decisions = sum(r[1] for r in rows)
    cerr = np.concatenate([r[2] for r in rows])
    parity_log("fullscale_whole_run_lockstep_crop256x160", divergence_events=events, decisions=decisions,
               per_sweep_events=[r[0] for r in rows], cost_err_q9999=float(np.quantile(cerr, 0.9999)),
               cost_err_max=float(cerr.max()))
    assert events <= 1e-4 * decisions, f"{events} divergences in {decisions} decisions"
    assert np.quantile(cerr, 0.9999) <= NCC_TOL and cerr.max() <= HW_TOL_MAX
    eng.close()


def test_fullscale_full_run(fullscale_crop, parity_log):
    """The plain run end to end, with the bar of tests/test_gpu_headline.py: the agreement with
    the FP64 oracle's run may fall at most 5 points (within 1 %) and 10 points (within 0.1 %)
    under that of the oracle's own FP32 build, and the bad-pixel rates agree within half a
    point. The wide depth range makes a run more sensitive to near-ties here: the FP32 build
    itself reaches 85-99 % within 0.1 % on this crop, depending on the sampler."""
    from patchmatch_cuda_gb300 import scene
    sv = fullscale_crop
    w = sv.workload
    eng = make_engine(sv)
    orc = oracle_for(eng, sv)
    eng.run()
    gd = eng.depth()
    od, _, ovs, _ = orc.run(w.iterations, w.num_samples)
    within_01, within_1 = agreement(gd, od)
    f01, f1 = float_floor(eng, sv, od, w.iterations, w.num_samples)
    bad_g = scene.bad_pixel_rate(gd, sv.gt_depth)
    bad_o = scene.bad_pixel_rate(od.astype(np.float32), sv.gt_depth)
    parity_log("fullscale_full_run_crop256x160", within_0p1pct=within_01, within_1pct=within_1,
               fp32_oracle_within_0p1pct=f01, fp32_oracle_within_1pct=f1,
               view_sel_equal=float(np.mean(np.all(eng.view_selection() == ovs, axis=0))),
               bad1_gpu=bad_g, bad1_oracle=bad_o)
    assert within_1 >= min(f1, 0.99) - 0.05 and within_01 >= min(f01, 0.99) - 0.10, (within_1, within_01, f1, f01)
    assert abs(bad_g - bad_o) <= 0.005, (bad_g, bad_o)
    eng.close()
