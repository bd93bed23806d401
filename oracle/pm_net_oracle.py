"""CPU oracle of the learned depth proposal's network (test infrastructure).

A float64 numpy restatement of the encoder-decoder that patchmatch_cuda_gb300/csrc/pm_net.cu
trains on the GPU: the same layers, the same parameter layout (per layer: weights
[cout][ky][kx][cin], then the bias), the same loss (L1 of the relative inverse-depth error,
the inverse depth read from the sigmoid of output 0, plus 0.1 x binary cross-entropy of the
sigmoid of output 1 against "predicted depth within 2 % of the target's"), and its gradients
by hand-written backward passes. With bf16=True it rounds to bfloat16 exactly where the GPU stores bfloat16 (the
input, the weights, every activation and the convolution output gradients), so the remaining
difference is the order of FP32 accumulation. The reference project has no learned part:
this oracle checks the engine's own kernels, and the tests only use it as the checker.
"""
from __future__ import annotations

import numpy as np

IN_CH = 17
WIDTHS = (32, 64, 96, 128, 128)


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest, ties to even), returned as float64."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def layers():
    """(cin, cout, ksize, stride, relu, level_in) in execution order, as pm_net.cu builds them."""
    c = WIDTHS
    up = (c[1], c[2], c[3], c[4])
    out = [(IN_CH, c[0], 3, 1, 1, 0), (c[0], c[0], 3, 1, 1, 0)]
    for l in range(1, 4):
        out += [(c[l - 1], c[l], 3, 2, 1, l - 1), (c[l], c[l], 3, 1, 1, l)]
    out += [(c[3], c[4], 3, 2, 1, 3), (c[4], c[4], 3, 1, 1, 4)]
    for l in range(3, -1, -1):
        out += [(up[l] + c[l], c[l], 3, 1, 1, l), (c[l], c[l], 3, 1, 1, l)]
    out.append((c[0], 2, 1, 1, 0, 0))
    return out


def param_offsets():
    offs, n = [], 0
    for cin, cout, k, _, _, _ in layers():
        offs.append(n)
        n += cout * k * k * cin + cout
    return offs, n


def _im2col(x, k, s):
    B, H, W, C = x.shape
    p = (k - 1) // 2
    xp = np.pad(x, ((0, 0), (p, p), (p, p), (0, 0)))
    Ho, Wo = H // s, W // s
    cols = np.empty((B, Ho, Wo, k * k * C))
    for ky in range(k):
        for kx in range(k):
            t = ky * k + kx
            cols[..., t * C:(t + 1) * C] = xp[:, ky:ky + s * Ho:s, kx:kx + s * Wo:s, :]
    return cols.reshape(B * Ho * Wo, k * k * C), (B, Ho, Wo)


def _col2im(dcol, shape, k, s):
    B, H, W, C = shape
    p = (k - 1) // 2
    Ho, Wo = H // s, W // s
    dxp = np.zeros((B, H + 2 * p, W + 2 * p, C))
    d = dcol.reshape(B, Ho, Wo, k * k * C)
    for ky in range(k):
        for kx in range(k):
            t = ky * k + kx
            dxp[:, ky:ky + s * Ho:s, kx:kx + s * Wo:s, :] += d[..., t * C:(t + 1) * C]
    return dxp[:, p:p + H, p:p + W, :]


def _up2(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def _up2_back(g):
    B, H, W, C = g.shape
    return g.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def forward_backward(params, x, target, inv_far, inv_range, use_bf16=True):
    """Loss terms and d(loss)/d(params) for input x [B, H, W, 17] and target [B, H, W]
    (normalised inverse depth, < 0 masked). Returns (grad, (mean_l1, mean_bce, count), out)."""
    rnd = bf16 if use_bf16 else (lambda a: np.asarray(a, np.float64))
    offs, n = param_offsets()
    params = np.asarray(params, np.float64)
    L = layers()
    W_, b_ = [], []
    for (cin, cout, k, s, relu, lv), o in zip(L, offs):
        K = k * k * cin
        W_.append(rnd(params[o:o + cout * K].reshape(cout, K)))
        b_.append(params[o + cout * K:o + cout * K + cout])
    cache = []

    def conv(i, a):
        cin, cout, k, s, relu, lv = L[i]
        col, (B, Ho, Wo) = _im2col(a, k, s)
        z = col @ W_[i].T + b_[i]
        y = np.maximum(z, 0.0) if relu else z
        y = rnd(y) if relu else y                       # the head's output stays FP32
        cache.append((i, col, a.shape, y))
        return y.reshape(B, Ho, Wo, cout)

    a = rnd(x)
    h = conv(0, a)
    skip = [None] * 5
    skip[0] = conv(1, h)
    i = 2
    for l in range(1, 4):
        h = conv(i, skip[l - 1]); i += 1
        skip[l] = conv(i, h); i += 1
    h = conv(i, skip[3]); i += 1
    h = conv(i, h); i += 1
    for l in range(3, -1, -1):
        cat = np.concatenate([_up2(h), skip[l]], axis=3)
        h = conv(i, cat); i += 1
        h = conv(i, h); i += 1
    o = conv(i, h)                                       # [B, H, W, 2]
    B, H, W, _ = o.shape
    P0 = B * H * W
    o = o.reshape(P0, 2)
    t = np.asarray(target, np.float64).reshape(P0)
    valid = t >= 0
    sg = 1.0 / (1.0 + np.exp(-o[:, 0]))
    q = 1.0 / (1.0 + np.exp(-o[:, 1]))
    inv_p = inv_far + sg * inv_range
    inv_t = inv_far + t * inv_range
    yl = (np.abs(inv_p - inv_t) <= 0.02 * inv_t).astype(np.float64)
    l1 = np.abs(inv_p - inv_t) / inv_t
    bce = -(yl * np.log(np.maximum(q, 1e-7)) + (1 - yl) * np.log(np.maximum(1 - q, 1e-7)))
    go = np.zeros((P0, 2))
    go[:, 0] = np.sign(sg - t) * inv_range / inv_t * sg * (1 - sg) / P0
    go[:, 1] = 0.1 * (q - yl) / P0
    go[~valid] = 0.0
    cnt = float(valid.sum())
    stats = (float(l1[valid].sum() / max(cnt, 1)), float(bce[valid].sum() / max(cnt, 1)), cnt)

    grad = np.zeros(n)
    # backward through the layers in reverse, with the same routing of gradients as the GPU
    g_head = go.reshape(B, H, W, 2)

    def conv_back(i, gy):
        cin, cout, k, s, relu, lv = L[i]
        _, col, shape, y = cache[i]
        gz = gy.reshape(-1, cout)
        if relu:
            gz = gz * (y.reshape(-1, cout) > 0)
        gz_r = rnd(gz)
        o_ = offs[i]
        K = k * k * cin
        grad[o_:o_ + cout * K] = (gz_r.T @ col).reshape(-1)
        grad[o_ + cout * K:o_ + cout * K + cout] = gz.sum(axis=0)
        return _col2im(gz_r @ W_[i], shape, k, s)

    nl = len(L)
    g = conv_back(nl - 1, g_head)                    # head -> D0b output
    i = nl - 2
    gskip = [None] * 5
    for l in range(0, 4):
        g = conv_back(i, g); i -= 1                  # Dlb -> Dla output
        g = conv_back(i, g); i -= 1                  # Dla -> concat
        up = (WIDTHS[1], WIDTHS[2], WIDTHS[3], WIDTHS[4])[l]
        gskip[l] = g[..., up:]
        g = _up2_back(g[..., :up])                   # -> output of the level below
    g = conv_back(i, g); i -= 1                      # L4b
    g = conv_back(i, g); i -= 1                      # L4a -> skip3
    gs = gskip[3] + g
    for l in range(3, 0, -1):
        g = conv_back(i, gs); i -= 1                 # Llb -> Lla output
        g = conv_back(i, g); i -= 1                  # Lla -> skip(l-1)
        gs = gskip[l - 1] + g
    g = conv_back(i, gs); i -= 1                     # L0b
    conv_back(i, g)                                  # L0a (input gradient unused)
    return grad, stats, np.stack([sg, q], axis=1).reshape(B, H, W, 2)
