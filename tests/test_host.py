"""Host-side logic without a GPU: scene generator, file formats, the CLI's configuration
handling, and the replica aggregation bench.py uses across ranks (gloo, world size 2)."""
import hashlib
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_scene_is_deterministic_and_in_range():
    from patchmatch_cuda_gb300 import scene
    w = scene.Workload("t", 160, 120, 2, 3, 1, 2.0, 8.0, 3, 5, seed=42)
    a, b = scene.make_views(w), scene.make_views(w)
    for ia, ib in zip(a.images, b.images):
        np.testing.assert_array_equal(ia.image, ib.image)
    np.testing.assert_array_equal(a.gt_depth, b.gt_depth)
    assert a.gt_depth.min() > w.depth_near and a.gt_depth.max() < w.depth_far
    ref = a.images[a.ref_id]
    np.testing.assert_allclose(ref.R, np.eye(3), atol=1e-7)  # reference camera at the origin
    np.testing.assert_allclose(ref.T, 0, atol=1e-6)
    assert ref.image.std() > 10  # textured


def test_scene_ground_truth_is_consistent_with_projection():
    """A reference pixel's ground-truth point projects into a source view where that view's own
    ground truth sees the same depth (up to occlusion and pixel rounding)."""
    from patchmatch_cuda_gb300 import scene
    w = scene.Workload("t", 160, 120, 2, 3, 1, 2.0, 8.0, 3, 0, seed=3)
    sc = scene.Scene(w.seed, w.n_planes, w.n_boxes, w.depth_near, w.depth_far, w.width, w.height, w.focal)
    K, R, t = sc.camera(0, 0, w.width, w.height, w.focal)
    _, d0 = sc.render(K, R, t, w.width, w.height)
    Ks, Rs, ts = sc.camera(5.0, 0, w.width, w.height, w.focal)
    _, d1 = sc.render(Ks, Rs, ts, w.width, w.height)
    rng = np.random.default_rng(0)
    ok = 0
    for _ in range(200):
        x, y = rng.integers(10, w.width - 10), rng.integers(10, w.height - 10)
        X = d0[y, x] * np.linalg.inv(K) @ np.array([x + 0.5, y + 0.5, 1.0])
        Xs = Rs @ X + ts
        p = Ks @ Xs
        u, v = p[0] / p[2] - 0.5, p[1] / p[2] - 0.5
        if 0 <= u < w.width - 1 and 0 <= v < w.height - 1:
            ok += abs(d1[int(round(v)), int(round(u))] - Xs[2]) < 0.02 * Xs[2]
    assert ok > 150


def test_pnm_roundtrip_and_ppm_luma(tmp_path):
    from patchmatch_cuda_gb300 import read_pnm, write_pgm
    img = np.arange(12 * 7, dtype=np.uint8).reshape(7, 12)
    write_pgm(tmp_path / "a.pgm", img)
    np.testing.assert_array_equal(read_pnm(tmp_path / "a.pgm"), img)
    rgb = np.stack([np.full((2, 3), 200), np.full((2, 3), 100), np.full((2, 3), 50)], -1).astype(np.uint8)
    (tmp_path / "b.ppm").write_bytes(b"P6\n# comment\n3 2\n255\n" + rgb.tobytes())
    expected = (200 * 4899 + 100 * 9617 + 50 * 1868 + 8192) >> 14
    assert np.all(read_pnm(tmp_path / "b.ppm") == expected)


def test_middlebury_list_roundtrip(tmp_path):
    from patchmatch_cuda_gb300 import Image, read_middlebury, write_middlebury, write_pgm
    imgs = []
    for i in range(3):
        im = np.full((4, 5), 10 * i, np.uint8)
        write_pgm(tmp_path / f"v{i}.pgm", im)
        imgs.append(Image(np.diag([100.0 + i, 101.0, 1.0]), np.eye(3), np.array([0.1 * i, 0.2, 0.3]), im))
    write_middlebury(tmp_path / "list_par.txt", [f"v{i}.pgm" for i in range(3)], imgs)
    back = read_middlebury(tmp_path / "list_par.txt")
    for a, b in zip(imgs, back):
        np.testing.assert_array_equal(a.image, b.image)
        np.testing.assert_allclose(a.K, b.K)
        np.testing.assert_allclose(a.T, b.T)


def test_depth_file_format(tmp_path):
    """'<W>&<H>&<D>&' then raw float32 (array2d_wrapper.h:51-70)."""
    from patchmatch_cuda_gb300 import load_depth_file
    d = np.arange(6, dtype=np.float32).reshape(2, 3)
    (tmp_path / "d.bin").write_bytes(b"3&2&1&" + d.tobytes())
    np.testing.assert_array_equal(load_depth_file(tmp_path / "d.bin"), d)


def _cli():
    from patchmatch_cuda_gb300 import _native
    return _native.LIB_DIR / "pm_cli"


@pytest.mark.parametrize("ini,message", [
    ("[params]\nimageInfoFileName = x\n", "No such node (params.refImageId)"),
    ("[params]\nimageInfoFileName = /nonexistent/list.txt\nrefImageId = 0\nhalfWindowSize = 2\n"
     "numOfSamples = 1\nSPMAlpha = 0.45\ngaussianSigma = 1\nnumOfIterations = 1\noutputFileName = o\n",
     "cannot parse image files"),
    ("not an ini line\n", "Problems with config file"),
])
def test_cli_configuration_errors(tmp_path, ini, message):
    cli = _cli()
    if not cli.exists():
        pytest.skip("CLI not built")
    (tmp_path / "c.ini").write_text(ini)
    r = subprocess.run([str(cli), str(tmp_path / "c.ini")], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0
    assert message in r.stdout


def _gloo_worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t, n = bench.allreduce_max_sum(world, 10.0 + rank, 100.0 * (rank + 1))
    bench.barrier(world)
    out.put((rank, t, n))
    dist.destroy_process_group()


def test_replica_aggregation_over_gloo():
    """bench.py's whole-job value for N replicas: evaluations summed over ranks, time the
    maximum over ranks."""
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_gloo_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [r[1] for r in res] == [11.0, 11.0]
    assert [r[2] for r in res] == [300.0, 300.0]


def _nvm_scene(tmp_path, n_views=3):
    from patchmatch_cuda_gb300 import scene, write_pgm
    w = scene.Workload("nvm_96x64", 96, 64, n_views - 1, 2, 1, 2.0, 8.0, 3, 0, seed=5)
    sv = scene.make_views(w)
    names = []
    for i, im in enumerate(sv.images):
        write_pgm(tmp_path / f"c{i}.pgm", im.image)
        names.append(f"c{i}.pgm")
    return sv, names


def _loosened(lo, hi):
    """The widening rule of image.cpp:222-235 in float32."""
    lo, hi = np.float32(lo), np.float32(hi)
    size = np.float32(hi - lo)
    ratio = np.float32(0.25)
    near = np.float32(lo - ratio * size)
    while near <= 0:
        ratio = np.float32(ratio / np.float32(1.1))
        near = np.float32(lo - ratio * size)
    return float(near), float(np.float32(hi + np.float32(0.25) * size))


def test_nvm_reader_cameras_and_depth_ranges(tmp_path):
    from patchmatch_cuda_gb300 import read_nvm, scene
    sv, names = _nvm_scene(tmp_path)
    pts = scene.nvm_points(sv)
    behind = sv.images[0].C.astype(np.float64) - 3.0 * sv.images[0].R[2].astype(np.float64)
    pts_all = np.concatenate([pts, behind[None]], axis=0)          # one point behind camera 0
    vis = [list(range(3))] * len(pts) + [[0]]
    scene.write_nvm(tmp_path / "model.nvm", names, sv.images, pts_all, visible=vis)
    imgs, ranges = read_nvm(tmp_path / "model.nvm")
    assert len(imgs) == 3 and len(ranges) == 3
    for a, b in zip(imgs, sv.images):
        h, w = b.image.shape
        np.testing.assert_array_equal(a.image, b.image)
        np.testing.assert_allclose(a.R, b.R, atol=1e-6)
        np.testing.assert_allclose(a.T, b.T, rtol=1e-6, atol=1e-6)
        np.testing.assert_array_equal(a.K, np.array([[b.K[0, 0], 0, w / 2], [0, b.K[0, 0], h / 2], [0, 0, 1]],
                                                     np.float32))
    for a, im in zip(ranges, imgs):
        z = (pts.astype(np.float32).astype(np.float64) @ im.R[2].astype(np.float64)) + float(im.T[2])
        want = _loosened(np.float32(z.min()), np.float32(z.max()))
        np.testing.assert_allclose(a, want, rtol=2e-7)
        assert 0 < a[0] < z.min() and a[1] > z.max()


def test_nvm_reader_edge_cases(tmp_path):
    from patchmatch_cuda_gb300 import read_nvm, scene
    sv, names = _nvm_scene(tmp_path)
    pts = scene.nvm_points(sv, step=16)
    scene.write_nvm(tmp_path / "m.nvm", names, sv.images, pts, visible=[[0, 1]] * len(pts))
    _, ranges = read_nvm(tmp_path / "m.nvm")
    assert ranges[2] is None and ranges[0] is not None           # camera 2 sees no point
    # the near side shrinks its margin while it would reach zero
    lo, hi = 1.0, 9.0
    near, far = _loosened(lo, hi)
    assert 0 < near < lo and far == 11.0
    (tmp_path / "one.nvm").write_text("NVM_V3\n1\nc0.pgm 100 1 0 0 0 0 0 0 0 0\n1\n0 0 5 1 1 1 1 0 0 1 1\n")
    with pytest.raises(ValueError, match="two cameras"):
        read_nvm(tmp_path / "one.nvm")
    (tmp_path / "mb.txt").write_text("1\nc0.pgm" + " 0" * 21 + "\n")
    with pytest.raises(ValueError, match="not an NVM_V3"):
        read_nvm(tmp_path / "mb.txt")


def test_cli_reads_nvm_and_uses_its_depth_range(tmp_path):
    """main.cpp:98-121: the list is tried as NVM first, and the reference image's NVM range
    replaces the configured one. Without a GPU the run stops at engine creation, after the
    range is printed."""
    import re
    from patchmatch_cuda_gb300 import read_nvm, scene
    cli = _cli()
    if not cli.exists():
        pytest.skip("CLI not built")
    sv, names = _nvm_scene(tmp_path)
    pts = scene.nvm_points(sv)
    scene.write_nvm(tmp_path / "model.nvm", names, sv.images, pts, visible=[[0, 1, 2]] * (len(pts) - 1) + [[0, 1]])
    _, ranges = read_nvm(tmp_path / "model.nvm")
    ini = ("[params]\nimageInfoFileName = {}\nrefImageId = {}\nhalfWindowSize = 2\nnumOfSamples = 1\n"
           "SPMAlpha = 0.45\ngaussianSigma = 1\nnumOfIterations = 1\noutputFileName = {}\n")
    for ref in (1, 2):
        (tmp_path / "c.ini").write_text(ini.format(tmp_path / "model.nvm", ref, tmp_path / "d.bin"))
        r = subprocess.run([str(cli), str(tmp_path / "c.ini")], capture_output=True, text=True, timeout=60)
        m = re.search(r"using NVM files: depth range \[([^,]+), ([^\]]+)\] for image (\d+)", r.stdout)
        assert m, r.stdout
        assert int(m.group(3)) == ref
        assert (np.float32(m.group(1)), np.float32(m.group(2))) == (np.float32(ranges[ref][0]),
                                                                    np.float32(ranges[ref][1]))
    scene.write_nvm(tmp_path / "m2.nvm", names, sv.images, pts, visible=[[0, 1]] * len(pts))
    (tmp_path / "c.ini").write_text(ini.format(tmp_path / "m2.nvm", 2, tmp_path / "d.bin"))
    r = subprocess.run([str(cli), str(tmp_path / "c.ini")], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "no 3D point seen by image 2" in r.stdout
