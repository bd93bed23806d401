"""The oracle pinned to the reference's own code (CPU).

tests/golden/ref_box200_96x64.npz holds outputs of yhsa678/patchMatch_cuda's own kernels --
patchMatch.cu's computeNCC, computeMessageForward/Backward, findMinCost,
computeAllCostGivenDepth, topToDown and downToTop, array2d_refImg.cu's window sums,
array2d_wrapper.cu's random initial depth and GaussianBlurCUDA.cu's filter -- compiled for the
CPU and run by oracle/ref_host.cpp
(make_ref_golden.py wrote it), on a 96x64 crop of the benchmarked scene with its window, view
and sample counts (15x15, 10 sources, numOfSamples 5). Two builds of the reference wrote it:
"f32" computes as the reference is written (float, flush-to-zero as under --use_fast_math);
"f64" is the same code with its floats widened to double. The oracle (FP64) must reproduce:

* the f64 build to rounding level: window sums exactly, NCC within 1e-12, the initial depth
  and costs within float storage, every sweep decision on every line whose posterior CDF stays
  defined, with the same costs, draw counts and view selections;
* the f32 build, the reference's own float arithmetic: NCC within its float error (1.4e-4 here),
  sweep decisions equal on every line (the reference's undefined read at a NaN CDF is defined
  as the oracle's "keep the current depth", see ref_host.cpp) but for rare near-ties.

Where the reference's sources are present (this repository's development container, not the
GPU machine), the live tests rebuild the reference, reproduce the fixture bit for bit and run a
whole-run lockstep: at every sweep of a 3-iteration run both start from the oracle's state.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

from parity_util import divergence_stats, first_divergence

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import make_ref_golden as G  # noqa: E402

S = G.WORKLOAD.num_samples


@pytest.fixture(scope="module")
def golden():
    z = np.load(GOLDEN / "ref_box200_96x64.npz")
    return {k: z[k] for k in z.files}


@pytest.fixture(scope="module")
def orc(golden, oracle_lib):
    from oracle import pm_oracle
    return pm_oracle.from_images(G.stored_views(golden), int(golden["ref_id"]), G.params())


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(1.0, np.abs(b))


def test_fixture_is_the_benchmarked_configuration(golden):
    w = G.WORKLOAD
    assert (2 * w.half_window + 1, w.n_src, w.num_samples, w.depth_near, w.depth_far) == (15, 10, 5, 1.0, 20.0)
    assert golden["image_0"].dtype == np.uint8 and len(golden["K"]) == 11


def test_window_sums_match_reference(orc, golden):
    """Array2d_refImg::filterImage (array2d_refImg.cu:11-131)."""
    np.testing.assert_array_equal(orc.sum_i, golden["sum_i_f64"])
    np.testing.assert_array_equal(orc.sum_ii, golden["sum_ii_f64"])
    assert rel_err(orc.sum_i, golden["sum_i_f32"]).max() < 1e-6


def test_ncc_matches_reference(orc, golden, parity_log):
    """computeNCC (patchMatch.cu:433-611) on 1024 queries, a quarter of them at the borders."""
    q = (golden["q_x"], golden["q_y"], golden["q_view"], golden["q_depth"], golden["q_axis"])
    o = orc.ncc_batch(*q)
    e64, e32 = rel_err(o, golden["ncc_f64"]), rel_err(o, golden["ncc_f32"])
    parity_log("ref_pin_ncc", err_max_f64=float(e64.max()), err_max_f32=float(e32.max()),
               err_q99_f32=float(np.quantile(e32, 0.99)))
    assert e64.max() <= 1e-12
    # the reference's own float error: its raw window sums cancel (1.4e-4 at most here, more
    # than the engine's shifted moments lose against the same FP64 oracle)
    assert np.quantile(e32, 0.99) <= 1e-4 and e32.max() <= 5e-4


def test_ncc_fixed_point_weights_match_reference(golden, oracle_lib, parity_log):
    """The texture unit's 1/256 weights on both sides. The oracle forms coordinates in the
    engine's single-precision steps, the widened reference in double, so a coordinate near a
    1/256 step rounds a weight the other way now and then."""
    from oracle import pm_oracle
    p = G.params()
    p.sampler = 1
    o = pm_oracle.from_images(G.stored_views(golden), int(golden["ref_id"]), p).ncc_batch(
        golden["q_x"], golden["q_y"], golden["q_view"], golden["q_depth"], golden["q_axis"])
    e = rel_err(o, golden["ncc_f64_fixed"])
    parity_log("ref_pin_ncc_fixed_point", err_max=float(e.max()), err_median=float(np.median(e)),
               exact_fraction=float(np.mean(e <= 1e-12)))
    assert np.median(e) <= 1e-12 and np.quantile(e, 0.99) <= 1e-4 and e.max() <= 1e-3


def test_initial_depth_and_costs_match_reference(orc, golden):
    """randNumGen (array2d_wrapper.cu:3-20) from the per-pixel random states, then
    computeAllCostGivenDepth (patchMatch.cu:775-816)."""
    counts = np.zeros(golden["counts0"].shape, np.uint32)
    orc.set_stream(counts)
    try:
        d0 = orc.init_depth()
    finally:
        orc.set_stream(None)
    np.testing.assert_array_equal(counts, golden["counts0"])
    assert (np.abs(d0 - golden["depth0_f64"]) / d0).max() <= 1.2e-7   # the oracle rounds to float
    # (1 - U)(far - near) + near: one rounding in the oracle (the GPU build contracts it into a
    # fused multiply-add), two in the host's float build: at most one unit in the last place
    assert (np.abs(d0.astype(np.float32) - golden["depth0_f32"]) / d0).max() <= 2.4e-7
    c0 = orc.initial_costs(golden["depth0_f64"])
    assert rel_err(c0, golden["costs0_f64"]).max() <= 1.2e-7          # stored as float32


def _undefined_prefix(vrows, nsteps):
    """Per line (processing order), the first step whose every view sample found no view (a NaN
    posterior CDF); nsteps if none."""
    und = np.all(vrows == 255, axis=-1)
    und[:, 0] = False  # a line's first step is not processed
    return np.where(und.any(axis=1), np.argmax(und, axis=1), nsteps)


@pytest.mark.parametrize("direction", [0, 1, 2, 3])
def test_sweep_matches_reference(orc, golden, direction, parity_log):
    """topToDown / downToTop (patchMatch.cu:818-1209) from the same state and random states,
    on two bands of 16 lines (the border and the middle)."""
    w = G.WORKLOAD
    d0 = golden["depth0_f64"].astype(np.float32).astype(np.float64)
    c0 = golden["costs0_f64"].astype(np.float64)
    stats = {"f64": [0, 0, 0, 0], "f32": [0, 0, 0, 0]}  # events, decisions, excluded lines, lines
    for b, band in enumerate(G.bands(direction)):
        d, c, counts = d0.copy(), c0.copy(), golden["counts0"].copy()
        vs = np.full((S, w.height, w.width), 255, np.uint8)
        orc.set_stream(counts)
        try:
            orc.sweep(d, c, direction, 4 + direction, S, view_sel=vs, lines=band)
        finally:
            orc.set_stream(None)
        rev = direction in (2, 3)
        od = G.band_rows(d, direction, band)
        oc = G.band_rows(c, direction, band)
        ov = G.band_rows(np.moveaxis(vs, 0, -1), direction, band)
        oc_n = counts[band[0]:band[1], 0] if direction in (0, 2) else counts[0, band[0]:band[1]]
        if rev:
            od, oc, ov = od[:, ::-1], oc[:, ::-1], ov[:, ::-1]
        nsteps = od.shape[1]
        undefined = _undefined_prefix(ov, nsteps)
        for tag in ("f64", "f32"):
            rd = golden[f"sweep{direction}_band{b}_depth_{tag}"].astype(np.float64)
            rd = rd[:, ::-1] if rev else rd
            same = np.abs(od - rd) <= 1e-6 * np.abs(rd)
            prefix = np.where(same.all(axis=1), nsteps, np.argmin(same, axis=1))
            # the widened build has no float underflow: lines with a NaN CDF in the oracle (and
            # in the float reference) are compared up to that step only
            limit = undefined if tag == "f64" else np.full_like(prefix, nsteps)
            diverged = (prefix < nsteps) & (prefix < limit)
            ev, dec = divergence_stats(np.minimum(prefix, limit), nsteps)
            st = stats[tag]
            st[0] += int(diverged.sum())
            st[1] += dec
            st[2] += int(np.sum(limit < nsteps))
            st[3] += len(prefix)
            counts_ok = golden[f"sweep{direction}_band{b}_counts_{tag}"] == oc_n
            assert np.all(counts_ok[~diverged & (limit == nsteps)]), "random-state draw counts differ"
            if tag == "f64":
                mask = np.arange(nsteps)[None, :] < np.minimum(prefix, limit)[:, None]
                rc = golden[f"sweep{direction}_band{b}_costs_f64"].astype(np.float64)
                rc = rc[:, ::-1] if rev else rc
                # the oracle forms hypotheses in float, the widened reference in double: the
                # same decisions, costs at depths one float rounding apart
                assert rel_err(oc[mask], rc[mask]).max() <= 5e-5
                if direction == 3:
                    rv = golden[f"sweep3_band{b}_view_sel_f64"][:, ::-1]
                    np.testing.assert_array_equal(ov[mask], rv[mask])
    parity_log(f"ref_pin_sweep_dir{direction}", f64_divergences=stats["f64"][0], f64_decisions=stats["f64"][1],
               f64_lines_cut_at_nan_cdf=stats["f64"][2], f32_divergences=stats["f32"][0],
               f32_decisions=stats["f32"][1], lines=stats["f64"][3])
    assert stats["f64"][0] == 0, f"{stats['f64'][0]} decisions differ from the widened reference"
    assert stats["f32"][0] <= 2, f"{stats['f32'][0]} decisions differ from the reference as written"


def test_messages_match_reference(golden, oracle_lib):
    """computeMessageForward / computeMessageBackward (patchMatch.cu:669-715), a cost of 2
    replaced by 2 U from the pixel's random state, in the reference's order."""
    from oracle import pm_oracle
    w = G.WORKLOAD
    for fwd, name in ((1, "fwd"), (0, "bwd")):
        for i, (m, c) in enumerate(zip(golden["msg_in"], golden["msg_cost"])):
            k = 0
            got = np.empty(len(m))
            for v in range(len(m)):
                u = 0.0
                if c[v] == 2.0:
                    u = pm_oracle.load().pmo_uniform(w.seed, 1000 + i, k, 0x5EED << 16, 0)
                    k += 1
                f = pm_oracle.msg_forward if fwd else pm_oracle.msg_backward
                got[v] = f(m[v], c[v], u, w.sp_alpha)
            assert k == golden[f"msg_{name}_draws_f64"][i] == golden[f"msg_{name}_draws_f32"][i]
            np.testing.assert_allclose(got, golden[f"msg_{name}_f64"][i], rtol=1e-7, atol=1e-12)
            np.testing.assert_allclose(got, golden[f"msg_{name}_f32"][i], rtol=5e-5, atol=1e-7)


def test_find_min_cost_matches_reference(golden, oracle_lib):
    """findMinCost (patchMatch.cu:613-618): ties go to the later index."""
    from oracle import pm_oracle
    got = [pm_oracle.find_min_cost(c) for c in golden["min_cost_in"]]
    np.testing.assert_array_equal(got, golden["min_cost_idx_f64"])
    np.testing.assert_array_equal(got, golden["min_cost_idx_f32"])


def test_prefilter_matches_reference_blur(golden, oracle_lib):
    """GaussianBlurCUDA::Filter (GaussianBlurCUDA.cu:185-191) as written, the oracle's box
    prefilter: taps of 1/width, width (int)(5 sigma) made odd within [5, 45], edge pixels
    repeated outside the image (the class's texture keeps its default clamp addressing). The
    oracle's FP32 build reproduces the reference's float build bit for bit; the FP64 oracle,
    whose output is float, the widened build within that rounding."""
    from oracle import pm_oracle
    img = golden[f"image_{int(golden['ref_id'])}"].astype(np.float32) / np.float32(255)
    np.testing.assert_array_equal(golden["blur_taps"], [5, 11, 45])
    for i, sigma in enumerate(golden["blur_sigma"]):
        np.testing.assert_array_equal(pm_oracle.prefilter(img, 1, float(sigma), fp32=True), golden[f"blur{i}_f32"])
        assert np.abs(pm_oracle.prefilter(img, 1, float(sigma)) - golden[f"blur{i}_f64"]).max() <= 6e-8
        # the same filter over the image padded with its edge pixels
        kw = int(golden["blur_taps"][i])
        pad = np.pad(img.astype(np.float64), kw // 2, mode="edge")
        rows = np.stack([pad[:, k:k + img.shape[1]] for k in range(kw)]).sum(0) / kw
        box = np.stack([rows[k:k + img.shape[0]] for k in range(kw)]).sum(0) / kw
        assert np.abs(box - golden[f"blur{i}_f64"]).max() <= 1e-12


def test_full_run_matches_reference(orc, golden, parity_log):
    """PatchMatch::run<15> (patchMatch.cu:307-394), 3 iterations from the random initial depth,
    random states drawn in the reference's order: the final depths of the reference as written
    and of the oracle agree within 0.1 % on at least 99 % of the pixels (a near-tie anywhere
    changes the rest of a line's random stream), and their bad-pixel rates agree."""
    from patchmatch_cuda_gb300 import scene
    w = G.WORKLOAD
    counts = np.zeros(golden["counts0"].shape, np.uint32)
    orc.set_stream(counts)
    try:
        od, _, ovs, _ = orc.run(w.iterations, S)
    finally:
        orc.set_stream(None)
    rd = golden["run_depth_f32"].astype(np.float64)
    within = float(np.mean(np.abs(od - rd) / rd <= 1e-3))
    vs_same = float(np.mean(np.all(ovs == golden["run_view_sel_f32"], axis=0)))
    bad_o = scene.bad_pixel_rate(od.astype(np.float32), golden["gt_depth"])
    bad_r = scene.bad_pixel_rate(golden["run_depth_f32"], golden["gt_depth"])
    parity_log("ref_pin_full_run", within_0p1pct=within, view_sel_equal=vs_same, bad1_oracle=bad_o,
               bad1_reference=bad_r)
    assert within >= 0.99 and vs_same >= 0.99
    assert abs(bad_o - bad_r) <= 0.005


# ---- live: the reference's own code, where its sources are present ------------------------------
needs_reference = pytest.mark.skipif(not __import__("oracle.pm_ref", fromlist=["x"]).sources_present(),
                                     reason="the reference's sources are not on this machine")


@needs_reference
def test_reference_run_reproduces_fixture(golden):
    """Rebuilding the reference from its sources and running it again gives the fixture bit for
    bit (the fixture is what the reference's code computes, nothing else)."""
    sv = G.views()
    for i, im in enumerate(sv.images):
        np.testing.assert_array_equal(im.image, golden[f"image_{i}"])
    wide = G.compute(sv, True)
    got = dict(wide)
    got.update(G.compute(sv, False, G.start_state(wide)))
    for k, v in got.items():
        np.testing.assert_array_equal(v, golden[k], err_msg=k)


@needs_reference
@pytest.mark.parametrize("wide", [False, True])
def test_whole_run_lockstep_against_reference(golden, orc, wide, parity_log):
    """Every sweep of a 3-iteration run, the reference and the oracle each from the oracle's
    state: decisions equal but for rare near-ties (as written) and none on defined lines
    (widened)."""
    from oracle import pm_ref
    w = G.WORKLOAD
    rp = pm_ref.RefProblem.from_images(G.stored_views(golden), int(golden["ref_id"]), G.params(), wide=wide)
    counts = np.zeros(golden["counts0"].shape, np.uint32)
    orc.set_stream(counts)
    try:
        d = orc.init_depth()
        c = orc.initial_costs(d)
        events = decisions = 0
        for it in range(w.iterations):
            s = 1 if it == 0 else S
            for direction in range(4):
                rd, rc, rcount = d.copy(), c.copy(), counts.copy()
                rp.sweep(rd, rc, rcount, direction, s)
                vs = np.full((s, w.height, w.width), 255, np.uint8)
                orc.sweep(d, c, direction, 4 * it + direction, s, view_sel=vs)
                prefix, nsteps = first_divergence(rd, d, direction)
                if wide:  # compare up to the first NaN-CDF step (no float underflow when widened)
                    rows = np.moveaxis(vs, 0, -1) if direction in (0, 2) else np.moveaxis(vs, 0, -1).swapaxes(0, 1)
                    rows = rows[:, ::-1] if direction in (2, 3) else rows
                    prefix = np.where(_undefined_prefix(rows, nsteps) <= prefix, nsteps, prefix)
                ev, dec = divergence_stats(prefix, nsteps)
                events += ev
                decisions += dec
    finally:
        orc.set_stream(None)
    parity_log(f"ref_pin_whole_run_lockstep_{'f64' if wide else 'f32'}", divergences=events, decisions=decisions)
    assert events <= (0 if wide else 2e-4 * decisions), f"{events} divergences in {decisions} decisions"


@needs_reference
@pytest.mark.parametrize("shape", [(1, 1), (5, 7), (64, 3), (37, 53)])
def test_blur_against_reference(shape, oracle_lib):
    """The reference's blur on images smaller than its filter and on ragged shapes, for widths
    at and beyond both clamps (sigma 0.1 -> 5 taps, 1.4 -> 7, 20 -> 45): the oracle's FP32
    build equal bit for bit, its filter width the reference's."""
    from oracle import pm_oracle, pm_ref
    rng = np.random.default_rng(sum(shape))
    img = rng.integers(0, 256, shape).astype(np.float32) / np.float32(255)
    for sigma, taps in [(0.1, 5), (1.0, 5), (1.4, 7), (3.0, 15), (20.0, 45)]:
        r32, kw = pm_ref.blur(img, sigma)
        r64, kw64 = pm_ref.blur(img, sigma, wide=True)
        assert kw == kw64 == taps
        np.testing.assert_array_equal(pm_oracle.prefilter(img, 1, sigma, fp32=True), r32.astype(np.float32))
        assert np.abs(pm_oracle.prefilter(img, 1, sigma) - r64).max() <= 6e-8


@needs_reference
@pytest.mark.parametrize("half_window", [1, 4, 9, 11])
def test_window_sums_and_ncc_against_reference_at_other_windows(golden, half_window, oracle_lib, parity_log):
    """The reference instantiates its kernels for every odd window (PatchMatch::run<W>,
    patchMatch.cu:276-296); the fixture holds its 15x15 outputs. At other windows, on the
    fixture's views: the window sums of the widened build equal the oracle's, and computeNCC
    (patchMatch.cu:433-611) agrees to FP64 rounding on queries at every border and inside
    (1e-11: a 3x3 window's nine samples make the NCC far worse conditioned than 15x15's), and
    with the texture unit's weights as closely as at 15x15 (bounds scaled by the window side)."""
    from oracle import pm_oracle, pm_ref
    p = G.params()
    p.half_window = half_window
    views = G.stored_views(golden)
    ref_id = int(golden["ref_id"])
    rp = pm_ref.RefProblem.from_images(views, ref_id, p, wide=True, fixed_point_weights=False)
    orc = pm_oracle.from_images(views, ref_id, p)
    _, si, sii = rp.box_moments()
    np.testing.assert_array_equal(orc.sum_i, si)
    np.testing.assert_array_equal(orc.sum_ii, sii)
    w = G.WORKLOAD
    rng = np.random.default_rng(100 + half_window)
    n = 512
    xs, ys = rng.integers(0, w.width, n), rng.integers(0, w.height, n)
    xs[:64] = rng.integers(0, half_window + 1, 64)
    ys[64:128] = rng.integers(0, half_window + 1, 64)
    xs[128:192] = rng.integers(w.width - half_window - 1, w.width, 64)
    ys[192:256] = rng.integers(w.height - half_window - 1, w.height, 64)
    vs = rng.integers(0, w.n_src, n)
    ds = rng.uniform(w.depth_near, w.depth_far, n).astype(np.float32).astype(np.float64)
    ax = rng.integers(0, 2, n)
    want = rp.ncc(xs, ys, vs, ds, ax)
    got = orc.ncc_batch(xs.astype(np.int32), ys.astype(np.int32), vs.astype(np.int32), ds, ax.astype(np.int32))
    err = rel_err(got, want)
    # the texture unit's 1/256 weights on both sides (coordinates in the engine's float steps
    # against the widened build's double ones: now and then a weight rounds the other way)
    p.sampler = 1
    rpf = pm_ref.RefProblem.from_images(views, ref_id, p, wide=True, fixed_point_weights=True)
    orcf = pm_oracle.from_images(views, ref_id, p)
    ef = rel_err(orcf.ncc_batch(xs.astype(np.int32), ys.astype(np.int32), vs.astype(np.int32), ds,
                                ax.astype(np.int32)), rpf.ncc(xs, ys, vs, ds, ax))
    parity_log(f"ref_pin_ncc_half_window{half_window}", n=n, err_max=float(err.max()),
               fixed_point_err_median=float(np.median(ef)), fixed_point_err_q99=float(np.quantile(ef, 0.99)),
               fixed_point_err_max=float(ef.max()))
    assert err.max() <= 1e-11
    # one weight rounded the other way moves one sample by a 1/256 step of the texel gradient;
    # its effect on the NCC grows as the window shrinks (3x3: nine samples), so the 15x15 bounds
    # scale with 15 / side
    k = max(1.0, 15.0 / (2 * half_window + 1))
    assert np.median(ef) <= 1e-12 and np.quantile(ef, 0.99) <= 1e-4 * k and ef.max() <= 1e-3 * k


@needs_reference
@pytest.mark.parametrize("half_window", [4, 9])
def test_sweeps_against_reference_at_other_windows(golden, half_window, oracle_lib, parity_log):
    """topToDown / downToTop (patchMatch.cu:818-1209) at windows other than the fixture's:
    every line of one sweep per direction with S = 5, the widened build and the oracle each from
    the oracle's initial depth and costs with the same random streams; every decision equal up
    to a line's first step whose posterior CDF is NaN (where the widened build has no float
    underflow)."""
    from oracle import pm_oracle, pm_ref
    p = G.params()
    p.half_window = half_window
    views = G.stored_views(golden)
    ref_id = int(golden["ref_id"])
    rp = pm_ref.RefProblem.from_images(views, ref_id, p, wide=True, fixed_point_weights=False)
    orc = pm_oracle.from_images(views, ref_id, p)
    w = G.WORKLOAD
    counts0 = np.zeros(golden["counts0"].shape, np.uint32)
    orc.set_stream(counts0)
    try:
        d0 = orc.init_depth()
        c0 = orc.initial_costs(d0)
        events = decisions = cut = 0
        for direction in range(4):
            rd, rc, rcount = d0.copy(), c0.copy(), counts0.copy()
            rp.sweep(rd, rc, rcount, direction, S)
            od, oc, ocount = d0.copy(), c0.copy(), counts0.copy()
            vs = np.full((S, w.height, w.width), 255, np.uint8)
            orc.set_stream(ocount)
            orc.sweep(od, oc, direction, 4 + direction, S, view_sel=vs)
            prefix, nsteps = first_divergence(rd, od, direction)
            rows = np.moveaxis(vs, 0, -1) if direction in (0, 2) else np.moveaxis(vs, 0, -1).swapaxes(0, 1)
            rows = rows[:, ::-1] if direction in (2, 3) else rows
            limit = _undefined_prefix(rows, nsteps)
            events += int(np.sum((prefix < nsteps) & (prefix < limit)))
            ev, dec = divergence_stats(np.minimum(prefix, limit), nsteps)
            decisions += dec
            cut += int(np.sum(limit < nsteps))
    finally:
        orc.set_stream(None)
    parity_log(f"ref_pin_sweeps_half_window{half_window}", divergences=events, decisions=decisions,
               lines_cut_at_nan_cdf=cut)
    assert decisions > 0 and events == 0, f"{events} decisions differ from the widened reference"


@needs_reference
@pytest.mark.parametrize("n_views", [1, 2, 20, 32])
def test_messages_against_reference_at_other_view_counts(n_views, oracle_lib):
    """computeMessageForward / computeMessageBackward (patchMatch.cu:669-715) for view counts
    other than the fixture's 10, up to the 32 a warp's lanes hold, and three SPMAlpha values:
    the oracle's messages and replacement-draw counts equal the widened build's."""
    from oracle import pm_oracle, pm_ref
    rng = np.random.default_rng(n_views)
    n = 24
    msg = rng.uniform(0.0, 1.0, (n, n_views))
    cost = rng.uniform(0.0, 2.0, (n, n_views))
    cost[rng.random((n, n_views)) < 0.15] = 2.0      # the cost-2 replacement draws
    cost[:4] = rng.uniform(2.0, 12.0, (4, n_views))   # leading-edge values beyond [0, 2]
    msg[4:8] = rng.choice([0.0, 1.0, 0.5], (4, n_views))
    seed = 2024
    for sp_alpha in (0.2, 0.45, 1.0):
        for fwd in (True, False):
            f = pm_oracle.msg_forward if fwd else pm_oracle.msg_backward
            for i in range(n):
                want, draws = pm_ref.messages(fwd, msg[i], cost[i], sp_alpha, seed, 1000 + i, 0, wide=True)
                k = 0
                got = np.empty(n_views)
                for v in range(n_views):
                    u = 0.0
                    if cost[i, v] == 2.0:
                        u = pm_oracle.load().pmo_uniform(seed, 1000 + i, k, 0x5EED << 16, 0)
                        k += 1
                    got[v] = f(msg[i, v], cost[i, v], u, sp_alpha)
                assert k == draws
                np.testing.assert_allclose(got, want, rtol=1e-7, atol=1e-12)
