"""Planar-target views and calibration refinement on the differentiable path.

* ``decode_views``: decodes the frame stacks of several poses of a planar
  target on the GPU and keeps the phase resident (order + residual, both
  cameras), with each pose's plane in the rectified left frame.
* ``refine``: Gauss-Newton / Levenberg-Marquardt refinement of the 16
  calibration parameters.  Each iteration re-derives the integer match columns
  of every view at the current parameters (zim_diff_rectify + zim_match; the
  decisions are then held fixed for the adjoint), runs one batched
  forward/adjoint launch over all views (zim_diff_backward) and takes a host
  step in FP64.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import api, diff


@dataclass
class PoseData:
    order: List[torch.Tensor]
    residual: List[torch.Tensor]
    plane: np.ndarray  # (n, d) in the rectified left frame of the context's calibration
    best: Optional[torch.Tensor] = None


def decode_views(ctx: api.Context, dcfg, frames: Sequence, planes_world: Sequence) -> List[PoseData]:
    """frames: per pose (left, right) host or device stacks; planes_world: per
    pose (n, d) with n . X = d in left-camera coordinates.  The context's
    calibration defines the rectified frame the planes are expressed in."""
    out = []
    R1 = np.asarray(ctx.R1)
    for (L, R), (n, d) in zip(frames, planes_world):
        ords, ress = [], []
        for F in (L, R):
            t = F if isinstance(F, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(F))
            dec = api.decode(ctx, dcfg, t.cuda(), want_mod=False, want_valid=False)
            ords.append(dec["order"])
            ress.append(dec["residual"])
        n = np.asarray(n, np.float64)
        out.append(PoseData(ords, ress, np.concatenate([R1 @ n, [-float(d)]])))
    return out


def update_matches(ctx: api.Context, theta, poses: Sequence[PoseData], pha_f: int, grad_threshold: float = 1.0):
    for p in poses:
        p.best = diff.match_columns(ctx, theta, p.order[0], p.residual[0], p.order[1], p.residual[1], pha_f,
                                    grad_threshold)


def views_of(poses: Sequence[PoseData]) -> List[diff.View]:
    return [diff.View(p.order, p.residual, p.best, tuple(p.plane)) for p in poses]


@dataclass
class RefineLog:
    losses: List[float] = field(default_factory=list)
    thetas: List[np.ndarray] = field(default_factory=list)
    seconds: float = 0.0
    iterations: int = 0


def refine(ctx: api.Context, poses: Sequence[PoseData], theta0, pha_f: int, iterations: int = 200,
           free: Optional[Sequence[int]] = None, damping: float = 1e-3, z_min: float = 0.0,
           z_max: float = 1e4) -> tuple:
    """Levenberg-Marquardt over the views; the damping adapts (x0.3 on an
    accepted step, x10 and retry on a rejected one).  Returns (theta, log)."""
    th = np.asarray(theta0, np.float64).copy()
    log = RefineLog()
    lam = damping
    t0 = time.perf_counter()
    update_matches(ctx, th, poses, pha_f)
    cur = diff.backward(ctx, th, views_of(poses), 1.0, z_min, z_max)
    for it in range(iterations):
        cand = diff.gauss_newton_step(th, cur, damping=lam, free=free)
        update_matches(ctx, cand, poses, pha_f)
        nxt = diff.backward(ctx, cand, views_of(poses), 1.0, z_min, z_max)
        # compare mean squared distances: the point set moves with the matches
        if nxt["loss"] / max(nxt["n_points"], 1) <= cur["loss"] / max(cur["n_points"], 1):
            th, cur = cand, nxt
            lam = max(lam * 0.3, 1e-9)
        else:
            lam = min(lam * 10.0, 1e6)
            update_matches(ctx, th, poses, pha_f)
        log.losses.append(cur["loss"] / max(cur["n_points"], 1))
        log.thetas.append(th.copy())
    torch.cuda.synchronize()
    log.seconds = time.perf_counter() - t0
    log.iterations = iterations
    return th, log
