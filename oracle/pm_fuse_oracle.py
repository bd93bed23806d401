"""CPU oracle of the consistency filter and fusion (test infrastructure).

A numpy restatement of patchmatch_cuda_gb300/csrc/pm_fuse.cu used only as the checker. The
reference project has no fusion step (its output stops at one depth map per run,
patchMatch.cu:263-407, main.cpp:124-128), so this oracle pins the engine's own specification:

  * geometry(cams): the pair matrices K_j R_j R_i^T K_i^-1, K_j (t_j - R_j R_i^T t_i) and the
    back-projections R_i^T K_i^-1, -R_i^T t_i in float64 from the float32 cameras;
  * fuse(depths, pairs, bp, ...): the per-pixel round trip, counts, fused depths and points in
    float32, every operation rounded to nearest in the kernel's order (numpy's float32
    elementwise arithmetic does not contract; 1 / z is correctly rounded as the kernel's
    reciprocal is on (1e-30, 1e30)), so the same float32 matrices give the same bits.
"""
from __future__ import annotations

import numpy as np

F = np.float32
RCP_MIN, RCP_MAX = F(1e-30), F(1e30)


def geometry(cams):
    """cams: list of (K, R, t). Returns (pairs [n, n, 12], bp [n, 12]) in float64."""
    n = len(cams)
    K = [np.asarray(c[0], np.float32).astype(np.float64).reshape(3, 3) for c in cams]
    R = [np.asarray(c[1], np.float32).astype(np.float64).reshape(3, 3) for c in cams]
    t = [np.asarray(c[2], np.float32).astype(np.float64).reshape(3) for c in cams]
    Ki = [np.linalg.inv(k) for k in K]
    pairs = np.zeros((n, n, 12))
    bp = np.zeros((n, 12))
    for i in range(n):
        bp[i, :9] = (R[i].T @ Ki[i]).ravel()
        bp[i, 9:] = -(R[i].T @ t[i])
        for j in range(n):
            RR = R[j] @ R[i].T
            pairs[i, j, :9] = (K[j] @ RR @ Ki[i]).ravel()
            pairs[i, j, 9:] = K[j] @ (t[j] - RR @ t[i])
    return pairs, bp


def _apply(m, k, u, v, d):
    """depth * (m[3k] u + m[3k+1] v + m[3k+2]) + m[9+k] in float32, the kernel's order."""
    r = (F(m[3 * k]) * u + F(m[3 * k + 1]) * v) + F(m[3 * k + 2])
    return d * r + F(m[9 + k])


def fuse(depths, pairs, bp, max_reproj_px=1.0, max_rel_depth=0.01, min_consistent=2, grays=None):
    """depths: list of [H_i, W_i] float32; pairs [n, n, 12] and bp [n, 12] float32 (the matrices
    the kernels use). Returns (fused depths, counts, points [m, 4]) as the kernels do."""
    n = len(depths)
    pairs = np.asarray(pairs, np.float32)
    bp = np.asarray(bp, np.float32)
    max_err2 = F(max_reproj_px) * F(max_reproj_px)
    max_rel = F(max_rel_depth)
    fused_all, count_all, pts = [], [], []
    with np.errstate(all="ignore"):
        for i in range(n):
            D = np.asarray(depths[i], np.float32)
            H, W = D.shape
            ys, xs = np.mgrid[0:H, 0:W]
            u = xs.astype(np.float32) + F(0.5)
            v = ys.astype(np.float32) + F(0.5)
            d = D.copy()
            valid = (d > 0) & (d < np.inf)
            count = np.zeros((H, W), np.int32)
            acc = d.copy()
            tol = max_rel * d
            for j in range(n):
                if j == i:
                    continue
                A, B = pairs[i, j], pairs[j, i]
                Dj = np.asarray(depths[j], np.float32)
                Hj, Wj = Dj.shape
                pz = _apply(A, 2, u, v, d)
                ok = valid & (pz > RCP_MIN) & (pz < RCP_MAX)
                rz = F(1) / pz                      # the kernel's correctly rounded reciprocal
                uj = _apply(A, 0, u, v, d) * rz
                vj = _apply(A, 1, u, v, d) * rz
                ok &= (uj >= 0) & (uj < F(Wj)) & (vj >= 0) & (vj < F(Hj))
                ix = np.minimum(np.where(ok, uj, 0).astype(np.int64), Wj - 1)
                iy = np.minimum(np.where(ok, vj, 0).astype(np.int64), Hj - 1)
                dj = np.where(ok, Dj[iy, ix], F(0))
                ok &= (dj > 0) & (dj < np.inf)
                uc = ix.astype(np.float32) + F(0.5)
                vc = iy.astype(np.float32) + F(0.5)
                qz = _apply(B, 2, uc, vc, dj)
                ok &= qz > 0
                ex = _apply(B, 0, uc, vc, dj) - u * qz
                ey = _apply(B, 1, uc, vc, dj) - v * qz
                err2 = ex * ex + ey * ey
                ok &= (err2 < max_err2 * (qz * qz)) & (np.abs(qz - d) < tol)
                count += ok
                acc = np.where(ok, acc + qz, acc)
            fused = np.zeros((H, W), np.float32)
            cand = valid & (count >= min_consistent)
            f = acc / (count + 1).astype(np.float32)
            keep = cand & (f > 0) & (f < np.inf)
            fused[keep] = f[keep]
            fused_all.append(fused)
            count_all.append(np.minimum(count, 255).astype(np.uint8))
            m = bp[i]
            dk, uk, vk = fused[keep], u[keep], v[keep]
            if grays is not None and grays[i] is not None:
                inten = np.asarray(grays[i], np.uint8)[keep].astype(np.float32) / F(255)
            else:
                inten = np.zeros(dk.shape, np.float32)
            pts.append(np.stack([_apply(m, 0, uk, vk, dk), _apply(m, 1, uk, vk, dk),
                                 _apply(m, 2, uk, vk, dk), inten], axis=1))
    points = np.concatenate(pts, axis=0) if pts else np.zeros((0, 4), np.float32)
    return fused_all, count_all, points.astype(np.float32)
