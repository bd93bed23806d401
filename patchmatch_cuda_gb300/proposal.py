"""Learned depth proposal: the network (pm_net through the C ABI), its training data and its
training loop.

The network maps the reference image and two source images warped onto 8 fronto-parallel
depths (17 channels at a quarter of the reference resolution) to a normalised inverse depth
and a confidence per quarter pixel; the engine turns that into the initial depth map
(init_mode = INIT_PROPOSAL), keeping the uniform random initialisation wherever the confidence
is below the threshold. It is trained here, on the GPU, by the engine's own forward and
backward kernels, on depth maps that plain PatchMatch itself produces on seeded synthetic
scenes.

    python -m patchmatch_cuda_gb300.proposal train --scenes 2000 --epochs 30 --out weights.npz

Device memory for inputs and targets comes from torch (plumbing only: no torch operator runs
on the data path).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import multiprocessing as mp
import os
import time
import warnings
from pathlib import Path

import numpy as np

from . import INIT_PROPOSAL, PREFILTER_NONE, Engine, _native

WEIGHTS = Path(__file__).resolve().parent / "weights" / "proposal.npz"
IN_CH = 17
TRAIN_SIZE = (640, 480)
TRAIN_SOURCES = 6


class ProposalNet:
    """One pm_net: a batch size and a level-0 size (multiples of 16)."""

    def __init__(self, batch: int, height: int, width: int, seed: int = 1):
        self._lib = _native.load_engine()
        self.h = C.c_void_p()
        _native.check(self._lib.pm_net_create(batch, height, width, seed, C.byref(self.h)))
        n = C.c_size_t()
        _native.check(self._lib.pm_net_num_params(self.h, C.byref(n)))
        self.n_params = n.value
        self.batch, self.height, self.width = batch, height, width

    def close(self) -> None:
        if getattr(self, "h", None):
            self._lib.pm_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        p = np.empty(self.n_params, np.float32)
        _native.check(self._lib.pm_net_get_params(self.h, p.ctypes.data, self.n_params))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {p.size}")
        _native.check(self._lib.pm_net_set_params(self.h, p.ctypes.data, self.n_params))

    def forward(self, d_input: int, d_out: int, stream: int = 0) -> None:
        _native.check(self._lib.pm_net_forward(self.h, C.c_void_p(d_input), C.c_void_p(d_out), C.c_void_p(stream)))

    def train_step(self, d_input: int, d_target: int, inv_far: float, inv_range: float, lr: float):
        loss = np.zeros(3, np.float32)
        _native.check(self._lib.pm_net_train_step(self.h, C.c_void_p(d_input), C.c_void_p(d_target), inv_far,
                                                  inv_range, lr, loss.ctypes.data))
        return float(loss[0]), float(loss[1]), int(loss[2])

    def loss(self, d_input: int, d_target: int, inv_far: float, inv_range: float):
        loss = np.zeros(3, np.float32)
        _native.check(self._lib.pm_net_gradients(self.h, C.c_void_p(d_input), C.c_void_p(d_target), inv_far,
                                                 inv_range, None, 0, loss.ctypes.data))
        return float(loss[0]), float(loss[1]), int(loss[2])

    def save(self, path, **meta) -> None:
        np.savez_compressed(path, params=self.params(), meta=json.dumps(meta))


WIDTHS = (32, 64, 96, 128, 128)


def layer_table():
    """(cin, cout, ksize, stride, relu, input level) of the network's convolutions in execution
    order, as pm_net.cu builds them."""
    c = WIDTHS
    up = (c[1], c[2], c[3], c[4])
    t = [(IN_CH, c[0], 3, 1, 1, 0), (c[0], c[0], 3, 1, 1, 0)]
    for lv in range(1, 4):
        t += [(c[lv - 1], c[lv], 3, 2, 1, lv - 1), (c[lv], c[lv], 3, 1, 1, lv)]
    t += [(c[3], c[4], 3, 2, 1, 3), (c[4], c[4], 3, 1, 1, 4)]
    for lv in range(3, -1, -1):
        t += [(up[lv] + c[lv], c[lv], 3, 1, 1, lv), (c[lv], c[lv], 3, 1, 1, lv)]
    t.append((c[0], 2, 1, 1, 0, 0))
    return t


def forward_flops(height: int, width: int, batch: int = 1) -> float:
    """2 x multiply-accumulates of one forward pass (unpadded channels and taps)."""
    total = 0.0
    for cin, cout, k, stride, relu, level in layer_table():
        h_in, w_in = height >> level, width >> level
        total += 2.0 * batch * (h_in // stride) * (w_in // stride) * k * k * cin * cout
    return total


def load_params(path=WEIGHTS) -> np.ndarray:
    with np.load(path) as z:
        return z["params"].astype(np.float32)


def for_engine(engine: Engine, params: np.ndarray | None = None) -> ProposalNet:
    """A batch-1 network sized for `engine`'s reference, with the given (default: the
    committed) weights, attached to the engine."""
    hp, wp = engine.proposal_shape()
    net = ProposalNet(1, hp, wp)
    net.set_params(load_params() if params is None else params)
    engine.set_proposal(net)
    return net


def quarter_target_mean(depth: np.ndarray, near: float, far: float, hp: int, wp: int) -> np.ndarray:
    """Normalised inverse depth (1/d - 1/far) / (1/near - 1/far) of each 4x4 block as the mean
    of 1/d over all its pixels; -1 on the padding."""
    H, W = depth.shape
    h4, w4 = H // 4, W // 4
    inv = 1.0 / depth[:4 * h4, :4 * w4].astype(np.float64)
    blk = inv.reshape(h4, 4, w4, 4).mean(axis=(1, 3))
    out = np.full((hp, wp), -1.0, np.float32)
    out[:h4, :w4] = np.clip((blk - 1.0 / far) / (1.0 / near - 1.0 / far), 0.0, 1.0)
    return out


def quarter_target(depth: np.ndarray, near: float, far: float, hp: int, wp: int,
                   cost: np.ndarray | None = None, max_cost: float = 0.35, min_valid: int = 8) -> np.ndarray:
    """Normalised inverse depth (1/d - 1/far) / (1/near - 1/far) of each 4x4 block: the median
    of 1/d over the block's pixels whose best PatchMatch cost (1 - NCC, over the source views)
    is at most max_cost; -1 (masked) where fewer than min_valid pixels qualify and on the
    padding. PatchMatch's own costs judge which of its depths to learn from."""
    H, W = depth.shape
    h4, w4 = H // 4, W // 4
    inv = 1.0 / depth[:4 * h4, :4 * w4].astype(np.float64)
    blocks = inv.reshape(h4, 4, w4, 4).transpose(0, 2, 1, 3).reshape(h4, w4, 16)
    if cost is not None:
        ok = cost[:4 * h4, :4 * w4].min(axis=2) <= max_cost
        ok = ok.reshape(h4, 4, w4, 4).transpose(0, 2, 1, 3).reshape(h4, w4, 16)
    else:
        ok = np.ones_like(blocks, bool)
    vals = np.where(ok, blocks, np.nan)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)   # blocks without a qualifying pixel
        med = np.nanmedian(vals, axis=2)
    t = np.clip((med - 1.0 / far) / (1.0 / near - 1.0 / far), 0.0, 1.0)
    t[ok.sum(axis=2) < min_valid] = -1.0
    out = np.full((hp, wp), -1.0, np.float32)
    out[:h4, :w4] = np.nan_to_num(t, nan=-1.0)
    return out


def training_workload(i: int):
    from . import scene
    w, h = TRAIN_SIZE
    return scene.Workload(f"train{i}", w, h, TRAIN_SOURCES, 7, 5, 1.0, 20.0, 12, 200,
                          prefilter=PREFILTER_NONE, seed=100000 + i)


def _worker_init():
    os.environ["OMP_NUM_THREADS"] = "2"


def _make_scene(i: int):
    from . import scene
    wl = training_workload(i)
    sv = scene.make_views(wl)
    return i, [(im.K, im.R, im.T, im.image) for im in sv.images], sv.ref_id


def make_dataset(n_scenes: int, workers: int = 8, target: str = "mean", log=print):
    """Inputs [n, hp, wp, 17] and targets [n, hp, wp] (torch CUDA tensors): the proposal input
    of each seeded 640x480 scene and its plain-PatchMatch depth map (5 iterations), as the mean
    inverse depth of each 4x4 block ("mean", the committed weights' recipe) or the median over
    the pixels PatchMatch's own costs deem reliable ("confident")."""
    import torch
    from . import Image
    ctx = mp.get_context("spawn")
    inputs = targets = None
    t0 = time.time()
    with ctx.Pool(workers, initializer=_worker_init) as pool:
        for k, (i, views, ref_id) in enumerate(pool.imap(_make_scene, range(n_scenes), chunksize=2)):
            images = [Image(K, R, T, img) for K, R, T, img in views]
            wl = training_workload(i)
            eng = Engine(images, ref_id, wl.params())
            eng.run()
            depth = eng.depth()
            cost = eng.costs()
            hp, wp = eng.proposal_shape()
            if inputs is None:
                inputs = torch.empty((n_scenes, hp, wp, IN_CH), device="cuda")
                targets = torch.empty((n_scenes, hp, wp), device="cuda")
            eng.proposal_input(inputs[k].data_ptr())
            if target == "mean":
                tq = quarter_target_mean(depth, wl.depth_near, wl.depth_far, hp, wp)
            else:
                tq = quarter_target(depth, wl.depth_near, wl.depth_far, hp, wp, cost)
            targets[k] = torch.from_numpy(tq)
            eng.close()
            if (k + 1) % 200 == 0:
                log(f"dataset {k + 1}/{n_scenes} ({time.time() - t0:.0f} s)")
    return inputs, targets


def train(inputs, targets, epochs: int, batch: int, lr: float, near: float = 1.0, far: float = 20.0,
          val_frac: float = 0.05, seed: int = 1, log=print):
    """Adam on the engine's kernels; returns the network and a history of losses."""
    import torch
    n, hp, wp = targets.shape
    n_val = max(batch, int(n * val_frac))
    n_tr = n - n_val
    net = ProposalNet(batch, hp, wp, seed=seed)
    inv_far, inv_range = 1.0 / far, 1.0 / near - 1.0 / far
    xb = torch.empty((batch, hp, wp, IN_CH), device="cuda")
    tb = torch.empty((batch, hp, wp), device="cuda")
    g = torch.Generator().manual_seed(seed)
    steps = epochs * (n_tr // batch)
    hist = []
    step = 0
    t0 = time.time()
    for ep in range(epochs):
        perm = torch.randperm(n_tr, generator=g)
        run = [0.0, 0.0]
        for b in range(n_tr // batch):
            idx = perm[b * batch:(b + 1) * batch].cuda()
            xb.copy_(inputs.index_select(0, idx))
            tb.copy_(targets.index_select(0, idx))
            warm = min(1.0, (step + 1) / 100.0)                       # linear warm-up
            cur = lr * warm * 0.5 * (1 + np.cos(np.pi * step / steps))  # cosine decay
            l1, bce, _ = net.train_step(xb.data_ptr(), tb.data_ptr(), inv_far, inv_range, cur)
            run[0] += l1
            run[1] += bce
            step += 1
        nb = max(1, n_tr // batch)
        vl = [0.0, 0.0, 0]
        for b in range(0, n_val - batch + 1, batch):
            xb.copy_(inputs[n_tr + b:n_tr + b + batch])
            tb.copy_(targets[n_tr + b:n_tr + b + batch])
            l1, bce, _ = net.loss(xb.data_ptr(), tb.data_ptr(), inv_far, inv_range)
            vl[0] += l1
            vl[1] += bce
            vl[2] += 1
        rec = {"epoch": ep, "train_l1": run[0] / nb, "train_bce": run[1] / nb,
               "val_l1": vl[0] / max(1, vl[2]), "val_bce": vl[1] / max(1, vl[2]), "s": round(time.time() - t0, 1)}
        hist.append(rec)
        log(json.dumps(rec))
    return net, hist


def main(argv=None):
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    tr = sub.add_parser("train")
    tr.add_argument("--scenes", type=int, default=2000)
    tr.add_argument("--epochs", type=int, default=30)
    tr.add_argument("--batch", type=int, default=16)
    tr.add_argument("--lr", type=float, default=5e-4)
    tr.add_argument("--workers", type=int, default=12)
    tr.add_argument("--target", choices=["mean", "confident"], default="mean")
    tr.add_argument("--out", default=str(WEIGHTS))
    a = ap.parse_args(argv)
    if a.cmd == "train":
        t0 = time.time()
        x, t = make_dataset(a.scenes, a.workers, a.target)
        t1 = time.time()
        print(f"dataset: {a.scenes} scenes in {t1 - t0:.0f} s", flush=True)
        net, hist = train(x, t, a.epochs, a.batch, a.lr)
        net.save(a.out, scenes=a.scenes, epochs=a.epochs, batch=a.batch, lr=a.lr, target=a.target, history=hist,
                 dataset_s=round(t1 - t0, 1), train_s=round(time.time() - t1, 1),
                 workload="seeded 640x480 scenes of 12 planes + 200 boxes, 1 ref + 6 sources, depth [1, 20]")
        print(f"saved {a.out}", flush=True)


if __name__ == "__main__":
    main()
