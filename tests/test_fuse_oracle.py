"""The fusion oracle on exact geometry (CPU): ground-truth depth maps of one scene agree with
each other, a corrupted map stops agreeing, and fused points lie on the scene."""
import numpy as np
import pytest

from oracle import pm_fuse_oracle as fo

SPECS = [(-6.0, 0.0, 96, 72, 90.0), (0.0, 1.0, 96, 72, 90.0), (6.0, -1.0, 120, 80, 110.0)]


@pytest.fixture(scope="module")
def views():
    from patchmatch_cuda_gb300 import scene
    return scene.scene_views(SPECS, seed=3)


def _geom(views):
    pairs, bp = fo.geometry([(im.K, im.R, im.T) for im, _ in views])
    return pairs.astype(np.float32), bp.astype(np.float32)


def test_geometry_round_trips(views):
    pairs, bp = fo.geometry([(im.K, im.R, im.T) for im, _ in views])
    for i in range(3):
        A = pairs[i, i, :9].reshape(3, 3)
        np.testing.assert_allclose(A, np.eye(3), atol=1e-5)   # float32 R is orthonormal to ~1e-7
        np.testing.assert_allclose(pairs[i, i, 9:], 0, atol=1e-4)
        np.testing.assert_allclose(bp[i, 9:], views[i][0].C, rtol=1e-6, atol=1e-6)


def test_ground_truth_maps_agree(views):
    pairs, bp = _geom(views)
    depths = [gt for _, gt in views]
    fused, count, pts = fo.fuse(depths, pairs, bp, min_consistent=1, grays=[im.image for im, _ in views])
    for (im, gt), f, c in zip(views, fused, count):
        valid = gt > 0
        kept = f > 0
        assert kept.sum() > 0.6 * valid.sum()
        assert np.all(c <= 2)
        np.testing.assert_allclose(f[kept], gt[kept], rtol=0.01)
    assert len(pts) == sum(int((f > 0).sum()) for f in fused)
    # the first reference's points project back onto its pixels at their fused depth
    im0 = views[0][0]
    k0 = int((fused[0] > 0).sum())
    cam = (im0.R.astype(np.float64) @ pts[:k0, :3].T.astype(np.float64)).T + im0.T
    np.testing.assert_allclose(cam[:, 2], fused[0][fused[0] > 0], rtol=1e-5)
    assert np.all((pts[:, 3] >= 0) & (pts[:, 3] <= 1))


def test_corrupted_map_stops_agreeing(views):
    pairs, bp = _geom(views)
    depths = [gt.copy() for _, gt in views]
    rng = np.random.default_rng(0)
    depths[2] = depths[2] * rng.uniform(1.2, 1.5, depths[2].shape).astype(np.float32)
    _, count, _ = fo.fuse(depths, pairs, bp, min_consistent=1)
    _, count_ok, _ = fo.fuse([gt for _, gt in views], pairs, bp, min_consistent=1)
    assert (count[0] == 2).sum() < 0.05 * (count_ok[0] == 2).sum()
    assert (count[2] > 0).sum() < 0.05 * (count_ok[2] > 0).sum()


def test_missing_depths_and_thresholds(views):
    pairs, bp = _geom(views)
    depths = [gt.copy() for _, gt in views]
    depths[1][:10] = 0.0
    depths[1][10:20] = np.nan
    depths[1][20:30] = -1.0
    depths[1][30:32] = np.inf
    fused, count, _ = fo.fuse(depths, pairs, bp, min_consistent=0)
    assert np.all(fused[1][:32] == 0) and np.all(count[1][:32] == 0)
    assert np.all(fused[0][depths[0] > 0] > 0)           # min_consistent 0 keeps every valid depth
    f2, _, p2 = fo.fuse(depths, pairs, bp, min_consistent=3)
    assert all(np.all(f == 0) for f in f2) and len(p2) == 0
