"""CPU restatement of the per-pixel cubic depth calibration (test
infrastructure only): JSLAB_StereoCalib_V2::computePixelwiseDepthCalibration,
src/JSLAB_StereoCalib_V2.cpp:113-240.

FP64 throughout, as the reference: points reprojected through Q
(:131-140, :186-190), plane by PCA (cv::PCA, DATA_AS_ROW: the eigenvector of
the smallest eigenvalue of the scatter about the mean, :153-158), samples moved
along the normal onto their plane (:195-199), and per pixel with >= 4 samples
the Vandermonde system [1 d d^2 d^3] solved by SVD least squares
(cv::solve(DECOMP_SVD): the minimum-norm least-squares solution, here
numpy.linalg.lstsq), stored as float32 (:208-235).  Parity with OpenCV's own
PCA/SVD is unpinned (no OpenCV here); the eigenvector sign is arbitrary in
both and does not affect the samples.
"""
from __future__ import annotations

import numpy as np


def q_points(Q, d, r, c):
    Q = np.asarray(Q, np.float64).reshape(4, 4)
    w = Q[3, 2] * d + Q[3, 3]
    return (c + Q[0, 3]) / w, (r + Q[1, 3]) / w, Q[2, 3] / w


def plane_pca(Q, disp, mask):
    r, c = np.nonzero((mask != 0) & (disp > 0))
    x, y, z = q_points(Q, disp[r, c].astype(np.float64), r, c)
    P = np.stack([x, y, z], axis=1)
    mean = P.mean(axis=0)
    S = (P - mean).T @ (P - mean)
    w, V = np.linalg.eigh(S)
    n = V[:, 0] / np.linalg.norm(V[:, 0])
    return np.array([n[0], n[1], n[2], -(n @ mean)])


def fit(Q, disps, masks):
    """Returns (cx, cy, cz) float32 (rows, cols, 4) and the plane equations."""
    eqs = [plane_pca(Q, d, m) for d, m in zip(disps, masks)]
    H, W = disps[0].shape
    out = np.zeros((3, H, W, 4), np.float32)
    D = np.stack([d.astype(np.float64) for d in disps])
    M = np.stack([(m != 0) & (d > 0) for d, m in zip(disps, masks)])
    for r in range(H):
        for c in range(W):
            ks = np.nonzero(M[:, r, c])[0]
            if ks.size < 4:
                continue
            d = D[ks, r, c]
            x, y, z = q_points(Q, d, r, c)
            tgt = []
            for k, xi, yi, zi in zip(ks, x, y, z):
                A, B, Cc, Dd = eqs[k]
                dist = A * xi + B * yi + Cc * zi + Dd
                tgt.append((xi - A * dist, yi - B * dist, zi - Cc * dist))
            V = np.stack([np.ones_like(d), d, d * d, d * d * d], axis=1)
            sol = np.linalg.lstsq(V, np.array(tgt), rcond=None)[0]
            out[:, r, c, :] = sol.T.astype(np.float32)
    return out[0], out[1], out[2], np.array(eqs)


def evaluate(coef, d):
    """The fitted cubic at disparity d (FP64)."""
    c = coef.astype(np.float64)
    return c[..., 0] + c[..., 1] * d + c[..., 2] * d * d + c[..., 3] * d * d * d


def synthetic_planes(Q, rows, cols, n_planes=6, seed=0, noise=0.02, dropout=0.05, z0=600.0, z1=1200.0):
    """Seeded planar targets in the rectified frame (tilt up to 30 degrees, depth
    z0..z1): disparity maps from Q with Gaussian noise (px) and random
    dropouts, as float32 maps and uint8 masks."""
    rng = np.random.default_rng(seed)
    Q = np.asarray(Q, np.float64).reshape(4, 4)
    r, c = np.mgrid[0:rows, 0:cols].astype(np.float64)
    disps, masks = [], []
    for k in range(n_planes):
        depth = z0 + (z1 - z0) * k / max(n_planes - 1, 1) + rng.uniform(-0.03, 0.03) * (z1 - z0)
        tx, ty = np.radians(rng.uniform(-30, 30, 2))
        n = np.array([np.sin(tx), np.sin(ty), 1.0])
        n /= np.linalg.norm(n)
        # plane n . X = n . (0, 0, depth); X = (c + Q03, r + Q13, Q23) / w
        num = n[0] * (c + Q[0, 3]) + n[1] * (r + Q[1, 3]) + n[2] * Q[2, 3]
        w = num / (n[2] * depth)
        d = (w - Q[3, 3]) / Q[3, 2]
        d = d + rng.normal(0, noise, d.shape)
        m = (rng.random(d.shape) > dropout) & (d > 0)
        disps.append(d.astype(np.float32))
        masks.append(m.astype(np.uint8))
    return disps, masks
