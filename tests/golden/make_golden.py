"""Writes tests/golden/plane3_128x96.npz: a small seeded scene (reference + 3 sources) and the
FP64 oracle's outputs on it (initial depth and costs, 256 NCC queries on both pairing axes, the
depth and view selection after a full 2-iteration run). The engine is compared against these
outputs on the GPU; the oracle is re-checked against them on the CPU.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import pm_oracle  # noqa: E402
from patchmatch_cuda_gb300 import PmParams, scene  # noqa: E402

OUT = Path(__file__).resolve().parent / "plane3_128x96.npz"
WORKLOAD = scene.Workload("plane3_128x96", 128, 96, 3, 3, 2, 2.0, 8.0, 3, 0, seed=77)


def params(w=WORKLOAD):
    p = PmParams()
    p.depth_near, p.depth_far, p.half_window = w.depth_near, w.depth_far, w.half_window
    p.num_samples, p.sp_alpha, p.gaussian_sigma = w.num_samples, w.sp_alpha, w.gaussian_sigma
    p.prefilter, p.num_iterations, p.orientation_x, p.orientation_z = w.prefilter, w.iterations, 0.0, 1.0
    p.seed, p.quirks = w.seed, 1
    return p


def queries(w=WORKLOAD, n=256):
    rng = np.random.default_rng(1234)
    xs = rng.integers(0, w.width, n)
    ys = rng.integers(0, w.height, n)
    vs = rng.integers(0, w.n_src, n)
    ds = rng.uniform(w.depth_near, w.depth_far, n).astype(np.float32).astype(np.float64)
    ax = rng.integers(0, 2, n)
    return xs, ys, vs, ds, ax


def compute(sv):
    p = params()
    orc = pm_oracle.from_images(sv.images, sv.ref_id, p)
    d0 = orc.init_depth()
    c0 = orc.initial_costs(d0)
    q = queries()
    ncc = orc.ncc_batch(*q)
    depth, cost, vsel, n = orc.run(WORKLOAD.iterations, WORKLOAD.num_samples)
    return dict(init_depth=d0.astype(np.float32), init_costs=c0.astype(np.float32), ncc=ncc,
                depth=depth.astype(np.float32), view_sel=vsel, evals=np.int64(n))


def main():
    sv = scene.make_views(WORKLOAD)
    out = dict(images=np.stack([im.image for im in sv.images]),
               K=np.stack([im.K for im in sv.images]), R=np.stack([im.R for im in sv.images]),
               T=np.stack([im.T for im in sv.images]), ref_id=np.int64(sv.ref_id), gt_depth=sv.gt_depth)
    out.update(compute(sv))
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
