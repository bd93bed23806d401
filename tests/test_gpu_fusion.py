"""Consistency filtering and fusion on the GPU (pm_fusion) against the CPU oracle: bit-exact
fused depths, counts and points from the same FP32 matrices; geometry within FP32 rounding of
the oracle's FP64; engines read in place; fusion removes wrong depths of PatchMatch output."""
import numpy as np
import pytest

from oracle import pm_fuse_oracle as fo

pytestmark = pytest.mark.gpu

SPECS = [(-6.0, 0.0, 160, 120, 150.0), (0.0, 1.0, 160, 120, 150.0), (6.0, -1.0, 200, 136, 180.0),
         (3.0, 0.5, 96, 64, 90.0)]


@pytest.fixture(scope="module")
def views():
    from patchmatch_cuda_gb300 import scene
    return scene.scene_views(SPECS, seed=9, n_planes=5, n_boxes=10)


def _noisy(views, seed=1):
    rng = np.random.default_rng(seed)
    out = []
    for _, gt in views:
        d = gt * rng.normal(1.0, 0.004, gt.shape).astype(np.float32)
        bad = rng.random(gt.shape) < 0.1
        d[bad] = rng.uniform(2.0, 8.0, int(bad.sum())).astype(np.float32)
        d[rng.random(gt.shape) < 0.02] = 0.0
        d[rng.random(gt.shape) < 0.01] = np.nan
        d[rng.random(gt.shape) < 0.01] = -1.0
        d[rng.random(gt.shape) < 0.005] = np.inf
        out.append(d.astype(np.float32))
    return out


def _compare(fus, depths, grays, params, parity_log=None, name=None):
    pairs, bp = fus.geometry()
    n = fus.run(params)
    fused, count, pts = fo.fuse(depths, pairs, bp, params.max_reproj_px, params.max_rel_depth,
                                params.min_consistent, grays=grays)
    assert n == len(pts)
    for i in range(len(depths)):
        f, c = fus.depth(i)
        np.testing.assert_array_equal(c, count[i])
        np.testing.assert_array_equal(f.view(np.uint32), fused[i].view(np.uint32))
    got = fus.points()
    np.testing.assert_array_equal(got.view(np.uint32), pts.view(np.uint32))
    if parity_log is not None:
        parity_log(name, points=int(n), pixels=int(sum(d.size for d in depths)), mismatches=0)
    return n


def test_fusion_matches_the_oracle_bit_for_bit(views, parity_log):
    from patchmatch_cuda_gb300 import Fusion, default_fuse_params
    depths = _noisy(views)
    images = [im for im, _ in views]
    fus = Fusion.from_depth_maps(depths, images)
    pairs, bp = fus.geometry()
    p64, b64 = fo.geometry([(im.K, im.R, im.T) for im in images])
    np.testing.assert_allclose(pairs, p64, rtol=1e-6, atol=1e-6 * np.abs(p64).max())
    np.testing.assert_allclose(bp, b64, rtol=1e-6, atol=1e-9)
    grays = [im.image for im in images]
    for params in (default_fuse_params(), default_fuse_params(min_consistent=1, max_reproj_px=0.5),
                   default_fuse_params(min_consistent=0), default_fuse_params(min_consistent=3, max_rel_depth=0.002)):
        _compare(fus, depths, grays, params, parity_log, f"fusion_min{params.min_consistent}")
    info = fus.info()
    assert info["launches"] == 4 and info["ms_total"] >= info["ms_check"] > 0
    fus.close()


def test_fusion_edge_cases(views, tmp_path):
    from patchmatch_cuda_gb300 import Fusion, PatchMatchError, default_fuse_params
    images = [im for im, _ in views]
    one = Fusion.from_depth_maps([views[0][1]], images[:1])
    assert one.run(default_fuse_params(min_consistent=1)) == 0           # nothing to agree with
    assert one.run(default_fuse_params(min_consistent=0)) == int((views[0][1] > 0).sum())
    one.close()
    empty = [np.zeros_like(gt) for _, gt in views]
    fus = Fusion.from_depth_maps(empty, images)
    with pytest.raises(PatchMatchError, match="STATE"):
        fus.points()
    assert fus.run() == 0
    assert fus.points().shape == (0, 4)
    with pytest.raises(PatchMatchError, match="INVALID"):
        fus.run(default_fuse_params(max_reproj_px=float("nan")))
    with pytest.raises(PatchMatchError, match="INVALID"):
        fus.run(default_fuse_params(min_consistent=-1))
    fus.close()
    gt = [g for _, g in views]
    fus = Fusion.from_depth_maps(gt, images)
    n = fus.run(default_fuse_params(min_consistent=1))
    fus.write_ply(tmp_path / "cloud.ply")
    raw = (tmp_path / "cloud.ply").read_bytes()
    head, body = raw.split(b"end_header\n", 1)
    assert f"element vertex {n}".encode() in head and len(body) == 15 * n
    xyz = np.frombuffer(body, np.dtype([("p", "<f4", 3), ("c", "u1", 3)]))
    np.testing.assert_array_equal(xyz["p"], fus.points()[:, :3])
    fus.close()
    bad = images[0].__class__(np.zeros((3, 3)), images[0].R, images[0].T, images[0].image)
    with pytest.raises(PatchMatchError, match="CAMERA"):
        Fusion.from_depth_maps(gt[:2], [bad, images[1]])


def test_fusion_reads_engines_in_place(views):
    """Fusion over engines equals fusion over host copies of their depth maps (reference texels
    as intensity), and a second engine run is picked up by the same fusion object."""
    from patchmatch_cuda_gb300 import (Engine, Fusion, PatchMatchError, default_fuse_params, default_params,
                                       run_batch, scene)
    sets = []
    for r, (yaw, pitch) in enumerate([(-4.0, 0.0), (0.0, 0.5), (4.0, -0.5)]):
        specs = [(yaw + dy, pitch, 160, 120, 150.0) for dy in (-4.0, -2.0, 0.0, 2.0, 4.0)]
        vs = scene.scene_views(specs, seed=9, n_planes=5, n_boxes=10)
        sets.append([im for im, _ in vs])
    p = default_params()
    p.depth_near, p.depth_far, p.half_window, p.num_iterations, p.num_samples = 2.0, 8.0, 3, 3, 3
    engines = [Engine(ims, 2, p) for ims in sets]
    with pytest.raises(PatchMatchError, match="STATE"):
        Fusion(engines)                                                  # no depth map yet
    run_batch(engines)
    fus = Fusion(engines)
    params = default_fuse_params(min_consistent=1)
    n1 = fus.run(params)
    depths = [e.depth() for e in engines]
    host = Fusion.from_depth_maps(depths, [s[2] for s in sets])
    assert host.run(params) == n1
    np.testing.assert_array_equal(host.points()[:, :3], fus.points()[:, :3])
    np.testing.assert_array_equal(host.points()[:, 3], fus.points()[:, 3])   # u8 / 255 either way
    host.close()
    engines[0].set_depth(np.zeros_like(depths[0]))
    n2 = fus.run(params)
    assert n2 < n1
    fus.close()
    for e in engines:
        e.close()


def test_fusion_removes_wrong_depths(parity_log):
    """PatchMatch depth maps of three overlapping references: the pixels fusion keeps have a far
    lower bad-pixel rate than the raw maps."""
    from patchmatch_cuda_gb300 import Engine, Fusion, default_fuse_params, default_params, run_batch, scene
    engines, gts, refs = [], [], []
    p = default_params()
    p.depth_near, p.depth_far, p.half_window, p.num_iterations, p.num_samples = 2.0, 8.0, 4, 3, 3
    for yaw in (-5.0, 0.0, 5.0):
        specs = [(yaw + dy, 0.0, 256, 192, 240.0) for dy in (-4.0, -2.0, 0.0, 2.0, 4.0)]
        vs = scene.scene_views(specs, seed=13, n_planes=5, n_boxes=12)
        engines.append(Engine([im for im, _ in vs], 2, p))
        gts.append(vs[2][1])
    run_batch(engines)
    fus = Fusion(engines)
    fus.run(default_fuse_params(min_consistent=2))
    raw_bad, kept_bad, kept_share = [], [], []
    for i, (e, gt) in enumerate(zip(engines, gts)):
        d = e.depth()
        f, _ = fus.depth(i)
        valid = gt > 0
        raw_bad.append(scene.bad_pixel_rate(d, gt, 0.01))
        k = (f > 0) & valid
        kept_share.append(k.sum() / valid.sum())
        kept_bad.append(float(np.mean(np.abs(f[k] - gt[k]) / gt[k] > 0.01)))
    parity_log("fusion_filtering", raw_bad=raw_bad, kept_bad=kept_bad, kept_share=kept_share)
    assert np.mean(kept_bad) < 0.5 * np.mean(raw_bad)
    assert np.mean(kept_share) > 0.25
    fus.close()
    for e in engines:
        e.close()


def test_fusion_over_several_scan_tiles(parity_log):
    """Four 640x480 maps (4800 blocks of 256 pixels: five scan tiles of 1024 blocks), bit-exact."""
    from patchmatch_cuda_gb300 import Fusion, default_fuse_params, scene
    specs = [(yaw, 0.0, 640, 480, 600.0) for yaw in (-6.0, -2.0, 2.0, 6.0)]
    vs = scene.scene_views(specs, seed=4, n_planes=6, n_boxes=20)
    depths = _noisy(vs, seed=5)
    images = [im for im, _ in vs]
    fus = Fusion.from_depth_maps(depths, images)
    n = _compare(fus, depths, [im.image for im in images], default_fuse_params(), parity_log, "fusion_640x480x4")
    assert n > 100000
    fus.close()
