"""The C ABI end to end on a GPU: outputs and file formats, determinism, batched runs, the
direction-flip utility, the CLI, the Python mirror of the reference class, FP16 texels."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small():
    from patchmatch_cuda_gb300 import scene
    w = scene.Workload("api_192x144", 192, 144, 3, 4, 2, 2.0, 8.0, 3, 0, seed=21)
    return scene.make_views(w)


def _engine(sv, **over):
    from patchmatch_cuda_gb300 import Engine
    return Engine(sv.images, sv.ref_id, sv.workload.params(**over))


def test_depth_outputs_file_format_and_view_selection(small, tmp_path):
    from patchmatch_cuda_gb300 import PatchMatchError, load_depth_file
    eng = _engine(small)
    with pytest.raises(PatchMatchError, match="STATE"):
        eng.view_selection()                        # nothing recorded before a run
    eng.run()
    d = eng.depth()
    w = small.workload
    assert d.shape == (w.height, w.width)
    assert d.min() >= w.depth_near and d.max() <= w.depth_far
    eng.save_depth(tmp_path / "d.bin")
    raw = (tmp_path / "d.bin").read_bytes()
    assert raw.startswith(f"{w.width}&{w.height}&1&".encode())
    np.testing.assert_array_equal(load_depth_file(tmp_path / "d.bin"), d)
    vs = eng.view_selection()
    assert vs.shape == (w.num_samples, w.height, w.width)
    assert np.all(vs[:, -1, :] == 255)              # the final sweep's first processed row
    body = vs[:, :-1, :]
    assert np.all((body < w.n_src) | (body == 255))
    # 255: no view (every emission of the step underflowed, a NaN posterior). That happens only
    # at the final bottom-to-top sweep's leading edge, the top half-window rows whose cut
    # windows give costs beyond ~6
    assert not np.any(body[:, w.half_window + 1:, :] == 255)
    assert np.mean(body == 255) < 0.02
    st = eng.stats()
    assert st.cost_evals >= st.cost_evals_done > 0 and st.ms_total > 0
    eng.close()


def test_warps_per_line_reported(small):
    """The tuner's counts (vertical interior, vertical edge lines, horizontal interior, horizontal
    edge lines) are reported in the stats; a caller's threads_per_line sets all four, and the
    depth map does not depend on them."""
    tuned = _engine(small)
    tuned.run()
    st = tuned.stats()
    wpl = list(st.warps_per_line)
    assert all(1 <= w <= 6 for w in wpl), wpl
    assert st.threads_per_line == 32 * max(wpl[0], wpl[2])
    fixed = _engine(small, threads_per_line=64)
    fixed.run()
    assert list(fixed.stats().warps_per_line) == [2, 2, 2, 2]
    np.testing.assert_array_equal(fixed.depth(), tuned.depth())
    np.testing.assert_array_equal(fixed.view_selection(), tuned.view_selection())
    tuned.close()
    fixed.close()


def test_runs_are_deterministic_and_async_matches_sync(small):
    eng = _engine(small)
    eng.run()
    a = eng.depth()
    eng.run_async()
    eng.synchronize()
    np.testing.assert_array_equal(eng.depth(), a)
    eng.close()
    e2 = _engine(small)
    e2.run()
    np.testing.assert_array_equal(e2.depth(), a)
    e2.close()


def test_batched_run_equals_single_runs(small):
    from patchmatch_cuda_gb300 import run_batch, scene
    w2 = scene.Workload("api_b", 160, 120, 4, 4, 3, 2.0, 8.0, 3, 0, seed=22)
    sv2 = scene.make_views(w2)
    singles = []
    for sv in (small, sv2):
        e = _engine(sv)
        e.run()
        singles.append((e.depth(), e.costs(), e.view_selection()))
        e.close()
    engines = [_engine(small), _engine(sv2)]
    run_batch(engines)
    for e, (d, c, vs) in zip(engines, singles):
        np.testing.assert_array_equal(e.depth(), d)
        np.testing.assert_array_equal(e.costs(), c)
        np.testing.assert_array_equal(e.view_selection(), vs)     # each reference's last sweep
        e.close()


def test_transpose_layers(engine_lib):
    torch = pytest.importorskip("torch")
    import ctypes as C
    layers, h, w = 3, 37, 70
    x = torch.arange(layers * h * w, dtype=torch.float32, device="cuda").reshape(layers * h, w)
    y = torch.full((layers * w, h), -1.0, device="cuda")
    st = engine_lib.pm_transpose_layers(C.c_void_p(x.data_ptr()), w * 4, C.c_void_p(y.data_ptr()), h * 4,
                                        w, h, layers, None)
    assert st == 0
    torch.cuda.synchronize()
    want = x.reshape(layers, h, w).transpose(1, 2).reshape(layers * w, h)
    assert torch.equal(y, want)


@pytest.mark.parametrize("planes", [0, 1])
def test_cli_matches_the_library(small, tmp_path, planes):
    from patchmatch_cuda_gb300 import _native, load_depth_file, write_middlebury, write_pgm
    names = []
    for i, im in enumerate(small.images):
        write_pgm(tmp_path / f"v{i}.pgm", im.image)
        names.append(f"v{i}.pgm")
    write_middlebury(tmp_path / "scene_par.txt", names, small.images)
    w = small.workload
    (tmp_path / "run.ini").write_text(
        "[params]\n"
        f"imageInfoFileName = {tmp_path / 'scene_par.txt'}\n"
        f"refImageId = {small.ref_id}\nhalfWindowSize = {w.half_window}\nnumOfSamples = {w.num_samples}\n"
        f"SPMAlpha = {w.sp_alpha}\ngaussianSigma = {w.gaussian_sigma}\nnumOfIterations = {w.iterations}\n"
        f"depthRangeNear = {w.depth_near}\ndepthRangeFar = {w.depth_far}\n"
        f"outputFileName = {tmp_path / 'depth.bin'}\nprefilter = {w.prefilter}\nseed = {w.seed}\n"
        f"planes = {planes}\n")
    r = subprocess.run([str(_native.LIB_DIR / "pm_cli"), str(tmp_path / "run.ini")], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    eng = _engine(small, planes=planes)
    eng.run()
    np.testing.assert_array_equal(load_depth_file(tmp_path / "depth.bin"), eng.depth())
    eng.close()


def test_cli_on_an_nvm_model_matches_the_library(small, tmp_path):
    """An NVM_V3 model through the CLI (cameras and the reference's depth range from the file)
    gives the depth map of the library run on read_nvm's views and range."""
    from patchmatch_cuda_gb300 import Engine, _native, load_depth_file, read_nvm, scene, write_pgm
    names = []
    for i, im in enumerate(small.images):
        write_pgm(tmp_path / f"v{i}.pgm", im.image)
        names.append(f"v{i}.pgm")
    scene.write_nvm(tmp_path / "model.nvm", names, small.images, scene.nvm_points(small, step=6))
    w = small.workload
    (tmp_path / "run.ini").write_text(
        "[params]\n"
        f"imageInfoFileName = {tmp_path / 'model.nvm'}\n"
        f"refImageId = {small.ref_id}\nhalfWindowSize = {w.half_window}\nnumOfSamples = {w.num_samples}\n"
        f"SPMAlpha = {w.sp_alpha}\ngaussianSigma = {w.gaussian_sigma}\nnumOfIterations = {w.iterations}\n"
        f"outputFileName = {tmp_path / 'depth.bin'}\nprefilter = {w.prefilter}\nseed = {w.seed}\n")
    r = subprocess.run([str(_native.LIB_DIR / "pm_cli"), str(tmp_path / "run.ini")], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    imgs, ranges = read_nvm(tmp_path / "model.nvm")
    near, far = ranges[small.ref_id]
    eng = Engine(imgs, small.ref_id, w.params(depth_near=near, depth_far=far))
    eng.run()
    d = eng.depth()
    np.testing.assert_array_equal(load_depth_file(tmp_path / "depth.bin"), d)
    eng.close()
    gt = small.gt_depth
    assert scene.bad_pixel_rate(d, gt, 0.05) < 0.5             # the NVM cameras reconstruct the scene


def test_refinement_in_the_schedule(small):
    """refine_trials > 0 appends the refinement to the run: the same as a plain run followed by
    pm_refine on the last sweep's views (keyed by the sweep count), in singles and batches; a
    depth changes only to one with a lower mean cost over the pixel's sampled views."""
    from patchmatch_cuda_gb300 import Batch
    w = small.workload
    plain = _engine(small)
    plain.run()
    before = plain.depth()
    plain.refine(10, 0.05, 4 * w.iterations, w.num_samples, 0)       # last sweep: bottom to top
    want = plain.depth()
    views = plain.view_selection()
    eng = _engine(small, refine_trials=10, refine_sigma=0.05)
    eng.run()
    np.testing.assert_array_equal(eng.depth(), want)
    b = Batch([eng])
    b.run()
    np.testing.assert_array_equal(eng.depth(), want)
    np.testing.assert_array_equal(eng.view_selection(), views)    # the last sweep's, as a single run
    b.close()
    # where a depth changed, the mean cost over the pixel's sampled views fell (pm_eval_costs)
    ys, xs = np.nonzero(want != before)
    assert len(ys) > 0.02 * want.size
    sel = np.random.default_rng(0).choice(len(ys), min(2000, len(ys)), replace=False)
    qx, qy, qv, qd0, qd1, owner = [], [], [], [], [], []
    for k in sel:
        y, x = ys[k], xs[k]
        for v in views[:, y, x]:
            if v < plain.n_src:
                qx.append(x); qy.append(y); qv.append(v); qd0.append(before[y, x]); qd1.append(want[y, x])
                owner.append(k)
    axes = np.zeros(len(qx), np.int32)
    c0 = plain.eval_costs(qx, qy, qv, qd0, axes)
    c1 = plain.eval_costs(qx, qy, qv, qd1, axes)
    owner = np.array(owner)
    for k in np.unique(owner):
        m = owner == k
        assert c1[m].mean() < c0[m].mean() + 1e-6
    plain.close()
    eng.close()


def test_reference_mirror_class(small):
    from patchmatch_cuda_gb300 import PatchMatch
    w = small.workload
    pm = PatchMatch(small.images, w.depth_near, w.depth_far, w.half_window, 32, 16, small.ref_id,
                    w.num_samples, w.sp_alpha, w.gaussian_sigma, w.iterations, 0.0, 1.0,
                    prefilter=w.prefilter, seed=w.seed)
    pm.runPatchMatch()
    eng = _engine(small)
    eng.run()
    np.testing.assert_array_equal(pm.depth_map, eng.depth())
    pm.close()
    eng.close()


def test_fp16_texels_parity(small, parity_log):
    """Mixed precision stores FP16 texels; NCC against the oracle on the same (FP16-rounded)
    texels stays within the NCC tolerance."""
    from oracle import pm_oracle
    eng = _engine(small, precision=1, sampler=0)  # FP16 texels are always gathered exactly
    assert eng.stats().texel_bytes == 2
    src = [eng.source_texels(v) for v in range(eng.n_src)]
    ref, _, _ = eng.ref_maps()
    orc = pm_oracle.from_images(small.images, small.ref_id, eng.params, source_texels=src, ref_texels=ref)
    rng = np.random.default_rng(8)
    n = 2048
    w = small.workload
    xs, ys = rng.integers(0, w.width, n), rng.integers(0, w.height, n)
    vs, ax = rng.integers(0, w.n_src, n), rng.integers(0, 2, n)
    ds = rng.uniform(w.depth_near, w.depth_far, n).astype(np.float32)
    got, want = eng.eval_costs(xs, ys, vs, ds, ax), orc.ncc_batch(xs, ys, vs, ds, ax)
    err = np.abs(got - want) / np.maximum(1.0, np.abs(want))
    parity_log("ncc_fp16_texels", err_max=float(err.max()))
    assert err.max() <= 1e-4
    eng.close()


def test_ground_truth_accuracy_small_scene(parity_log):
    """The engine reproduces the 320x240 three-plane workload's accuracy against ground truth."""
    from patchmatch_cuda_gb300 import scene
    w = scene.WORKLOADS["plane3_320x240"]
    sv = scene.make_views(w)
    eng = _engine(sv)
    eng.run()
    d = eng.depth()
    bad1, bad5 = scene.bad_pixel_rate(d, sv.gt_depth), scene.bad_pixel_rate(d, sv.gt_depth, 0.05)
    parity_log("gt_plane3_320x240", bad1=bad1, bad5=bad5)
    assert bad1 < 0.15 and bad5 < 0.05
    eng.close()


def test_graph_batch_equals_single_runs(small):
    """pm_batch: tuned warps per line and one CUDA graph for the whole schedule; two launches of
    the graph reproduce the single runs exactly."""
    from patchmatch_cuda_gb300 import Batch, scene
    w2 = scene.Workload("api_g", 160, 120, 4, 4, 3, 2.0, 8.0, 3, 0, seed=23)
    sv2 = scene.make_views(w2)
    singles = []
    for sv in (small, sv2):
        e = _engine(sv)
        e.run()
        singles.append(e.depth())
        e.close()
    engines = [_engine(small), _engine(sv2)]
    b = Batch(engines)
    info = b.info()
    assert info["groups"] >= 1 and info["launches"] > 0
    assert all(1 <= v <= 6 for pair in info["warps_per_line"] for v in pair)
    for _ in range(2):
        b.run()
        for e, d in zip(engines, singles):
            np.testing.assert_array_equal(e.depth(), d)
    b.close()
    for e in engines:
        e.close()
