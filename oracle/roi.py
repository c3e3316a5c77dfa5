"""CPU restatement of the ROI-restricted path (test infrastructure only):
prepareRectifiedROI and startCalculate_v2_roi,
src/JSLAB_PhaseEpipolarReconstructor_V2.cpp:595-914.

The source-image ROI mask follows cv::RotatedRect::points (single precision)
and cv::fillConvexPoly on the rounded corners.  Without OpenCV here, the fill
is restated from its documented behaviour: every pixel inside or on the closed
convex polygon plus the pixels of its 8-connected outline.  This module tests
containment per pixel with exact integer cross products -- a different method
from the library's per-row span computation -- so the two pin each other;
parity with OpenCV's own rasteriser stays unpinned.
"""
from __future__ import annotations

import math

import numpy as np

from . import oracle as O

f32 = np.float32


def rotated_rect_points(cx, cy, w, h, angle):
    """cv::RotatedRect::points in float arithmetic, one rounding per operation."""
    ang = float(angle) * math.pi / 180.0
    b = f32(f32(math.cos(ang)) * f32(0.5))
    a = f32(f32(math.sin(ang)) * f32(0.5))
    cx, cy, w, h = f32(cx), f32(cy), f32(w), f32(h)
    p0 = (f32(f32(cx - f32(a * h)) - f32(b * w)), f32(f32(cy + f32(b * h)) - f32(a * w)))
    p1 = (f32(f32(cx + f32(a * h)) - f32(b * w)), f32(f32(cy - f32(b * h)) - f32(a * w)))
    p2 = (f32(f32(2) * cx - p0[0]), f32(f32(2) * cy - p0[1]))
    p3 = (f32(f32(2) * cx - p1[0]), f32(f32(2) * cy - p1[1]))
    return [p0, p1, p2, p3]


def _bresenham(x0, y0, x1, y1):
    pts = []
    dx, dy = abs(x1 - x0), -abs(y1 - y0)
    sx, sy = (1 if x0 < x1 else -1), (1 if y0 < y1 else -1)
    err = dx + dy
    while True:
        pts.append((x0, y0))
        if x0 == x1 and y0 == y1:
            return pts
        e2 = 2 * err
        if e2 >= dy:
            err += dy
            x0 += sx
        if e2 <= dx:
            err += dx
            y0 += sy


def fill_rotated_rect(rows, cols, roi):
    """0/255 source mask of ((cx, cy), (w, h), angle)."""
    (cx, cy), (w, h), ang = roi
    v = [(int(np.rint(p[0])), int(np.rint(p[1]))) for p in rotated_rect_points(cx, cy, w, h, ang)]
    m = np.zeros((rows, cols), np.uint8)
    xs = [p[0] for p in v]
    ys = [p[1] for p in v]
    area2 = sum(v[i][0] * v[(i + 1) % 4][1] - v[(i + 1) % 4][0] * v[i][1] for i in range(4))
    if area2 != 0:
        y0, y1 = max(min(ys), 0), min(max(ys), rows - 1)
        x0, x1 = max(min(xs), 0), min(max(xs), cols - 1)
        if y0 <= y1 and x0 <= x1:
            Y, X = np.mgrid[y0:y1 + 1, x0:x1 + 1].astype(np.int64)
            inside = np.ones(X.shape, bool)
            s = 1 if area2 > 0 else -1
            for i in range(4):
                (px, py), (qx, qy) = v[i], v[(i + 1) % 4]
                inside &= s * ((qx - px) * (Y - py) - (qy - py) * (X - px)) >= 0
            m[y0:y1 + 1, x0:x1 + 1][inside] = 255
    for i in range(4):
        for x, y in _bresenham(*v[i], *v[(i + 1) % 4]):
            if 0 <= x < cols and 0 <= y < rows:
                m[y, x] = 255
    return m


def dilate5(m):
    p = np.pad(m, 2)
    out = np.zeros_like(m)
    for dy in range(5):
        for dx in range(5):
            out = np.maximum(out, p[dy:dy + m.shape[0], dx:dx + m.shape[1]])
    return out


def prepare(roi, src_shape, mapx, mapy, l_order, r_order, pha_f, pad=32):
    """prepareRectifiedROI: (left_rect, right_rect, mask) or None."""
    src = fill_rotated_rect(*src_shape, roi)
    lin = O.remap_u8(src, mapx, mapy)
    mask = dilate5(np.where(lin > 0, 255, 0).astype(np.uint8))
    ys, xs = np.nonzero(mask)
    if ys.size == 0:
        return None
    L = (int(xs.min()), int(ys.min()), int(xs.max() - xs.min() + 1), int(ys.max() - ys.min() + 1))
    lx, ly, lw, lh = L
    win_m = mask[ly:ly + lh, lx:lx + lw] > 0
    k = l_order[ly:ly + lh, lx:lx + lw][win_m]
    needed = np.zeros(max(pha_f + 1, 1), bool)
    needed[k[(k > 0) & (k <= pha_f)]] = True
    rk = r_order[ly:ly + lh]
    ok = (rk > 0) & (rk <= pha_f)
    hit = np.zeros(rk.shape, bool)
    hit[ok] = needed[rk[ok]]
    cols_hit = np.nonzero(hit.any(axis=0))[0]
    W = r_order.shape[1]
    if cols_hit.size:
        x0 = max(0, int(cols_hit.min()) - pad)
        x1 = min(W - 1, int(cols_hit.max()) + pad)
        R = (x0, ly, x1 - x0 + 1, lh)
    else:
        R = (0, ly, W, lh)
    return L, R, mask


def reconstruct(roi_rects, mask, lph, lk, rph, rk, pha_f, R1, *, poly=None, Q=None, grad_threshold=1.0,
                use_median=True, min_depth=0.0, max_depth=1000.0, use_px_gaussian=True, use_ror=True,
                ror=(0.7, 10, 10), mls=None):
    """startCalculate_v2_roi on full-frame rectified phase/order maps (FP64 phase)."""
    (lx, ly, lw, lh), (rx, ry, rw, rh) = roi_rects
    sl = (slice(ly, ly + lh), slice(lx, lx + lw))
    sr = (slice(ly, ly + lh), slice(rx, rx + rw))
    m = (mask[sl] > 0).astype(np.uint8)
    disp, best, near = O.stereo_match_roi(lph[sl], lk[sl], m, rph[sr], rk[sr], lx - rx, pha_f, grad_threshold)
    d32 = disp.astype(np.float32)
    dm = O.median5(d32) if use_median else d32
    if poly is not None:
        maps = [np.ascontiguousarray(c[sl]) for c in poly]
        xyz, pm = O.poly_reproject(dm, maps, R1, min_depth, max_depth, True)
    else:
        Qr = np.array(Q, np.float64).copy()
        Qr[0, 3] += lx
        Qr[1, 3] += ly
        xyz, pm, _ = O.reproject(dm, Qr, R1, min_depth, max_depth, True)
    xyz[m == 0] = 0
    pm = pm * m
    p_raw = pm.copy()
    if use_px_gaussian:
        xyz, _, _ = O.px_gaussian(xyz, pm, False)
    if use_ror:
        xr, mr, _ = O.ror(xyz, pm, *ror)
        raw, kept = int(p_raw.sum()), int(mr.sum())
        if not (raw > 0 and kept < raw * 0.1):
            xyz, pm = xr, mr
    if mls is not None:
        xyz, _ = O.mls(xyz, pm, *mls)
    return xyz, pm, dm, near
