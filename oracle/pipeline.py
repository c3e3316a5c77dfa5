"""The whole reconstruction path on the CPU, composed from the FP64 oracle.

Test infrastructure and CPU baseline only.  ``run_pair`` processes a full
stereo pair; ``run_band`` processes the rectified rows [y0, y1) (plus the halos
its stencils need), which bounds the CPU work of one benchmark step while
keeping every stage of the path.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import oracle as O


@dataclass
class Filters:
    use_median: bool = True
    use_px_gaussian: bool = False
    px_gaussian_updates_mask: bool = False
    use_ror: bool = False
    ror: tuple = (0.7, 10, 10)
    use_sor: bool = False
    sor_k: int = 30
    sor_std_mul: float = 1.0
    use_mls: bool = False
    mls: tuple = (7, 2.0 / math.sqrt(2.0), 2, 2.0, 1)  # window, sigma, order, max_radius, iterations
    use_metric_gaussian: bool = False
    mg_sigma: float = 0.5
    min_depth: float = 0.0
    max_depth: float = 1000.0


CONFIG1_FILTERS = Filters(use_sor=True, use_mls=True, use_metric_gaussian=True)


class Rectification:
    def __init__(self, rig: dict, full_left: bool = True):
        self.rig = rig
        c = O.make_calib(rig["K"], rig["D"], rig["R"], rig["t"], rig["width"], rig["height"])
        self.R1, self.R2, self.P1, self.P2, self.Q, self.w, self.h = O.rectification(c, full_left)
        self.maps = []
        for cam, (Rk, Pk) in enumerate(((self.R1, self.P1), (self.R2, self.P2))):
            self.maps.append(O.init_rectify_map(rig["K"][cam], rig["D"][cam], Rk, Pk, self.w, self.h))


def _filters(xyz, mask, f: Filters):
    if f.use_px_gaussian:
        xyz, mask, _ = O.px_gaussian(xyz, mask, f.px_gaussian_updates_mask)
    if f.use_ror:
        xyz, mask, _ = O.ror(xyz, mask, *f.ror)
    if f.use_sor:
        mask, _, _, _ = O.sor(xyz, mask, f.sor_k, f.sor_std_mul)
        xyz = xyz * mask[..., None]
    if f.use_mls:
        w, s, o, r, it = f.mls
        xyz, _ = O.mls(xyz, mask, w, s, o, r, it)
    if f.use_metric_gaussian:
        xyz, _ = O.metric_gaussian(xyz, mask, f.mg_sigma)
    return xyz, mask


def run_pair(decode_kwargs, pha_f, L, R, rect: Rectification, f: Filters = Filters(), poly=None):
    """poly: (cx, cy, cz) coefficient maps for startCalculate_v2's reprojection."""
    cfg = O.make_decode_cfg(**decode_kwargs)
    r = []
    for cam, fr in enumerate((L, R)):
        ph, k, _, valid, _ = O.decode(cfg, fr)
        r.append(O.rectify_decoded(ph, k, *rect.maps[cam], bool(cfg.post_smooth),
                                   valid if cfg.enable_hdr else None))
    disp, _, _ = O.stereo_match(r[0][0], r[1][0], r[0][1], r[1][1], pha_f)
    d32 = disp.astype(np.float32)
    dm = O.median5(d32) if f.use_median else d32
    if poly is not None:
        xyz, mask = O.poly_reproject(dm, poly, rect.R1, f.min_depth, f.max_depth, True)
    else:
        xyz, mask, _ = O.reproject(dm, rect.Q, rect.R1, f.min_depth, f.max_depth, True)
    return _filters(xyz, mask, f)


def run_band(decode_kwargs, pha_f, L, R, rect: Rectification, y0: int, y1: int, f: Filters = Filters()):
    """Rectified rows [y0, y1): decodes only the source rows they sample."""
    halo = 2 + (f.mls[0] if f.use_mls else 0) + (1 if f.use_px_gaussian else 0) + (f.ror[2] // 2 if f.use_ror else 0)
    ya, yb = max(0, y0 - halo), min(rect.h, y1 + halo)
    cfg = O.make_decode_cfg(**decode_kwargs)
    r = []
    for cam, fr in enumerate((L, R)):
        mx, my = rect.maps[cam]
        mxb, myb = mx[ya:yb], my[ya:yb]
        lo = int(max(0, math.floor(np.nanmin(myb)) - 3))
        hi = int(min(fr.shape[1], math.ceil(np.nanmax(myb)) + 4))
        ph, k, _, valid, _ = O.decode(cfg, np.ascontiguousarray(fr[:, lo:hi]))
        r.append(O.rectify_decoded(ph, k, mxb, myb - lo, bool(cfg.post_smooth), valid if cfg.enable_hdr else None))
    disp, _, _ = O.stereo_match(r[0][0], r[1][0], r[0][1], r[1][1], pha_f)
    d32 = disp.astype(np.float32)
    dm = O.median5(d32) if f.use_median else d32
    Q = rect.Q.copy()
    Q[1, 3] += ya  # band row i is rectified row ya + i
    xyz, mask, _ = O.reproject(dm, Q, rect.R1, f.min_depth, f.max_depth, True)
    xyz, mask = _filters(xyz, mask, f)
    s = slice(y0 - ya, y1 - ya)
    return xyz[s], mask[s]
