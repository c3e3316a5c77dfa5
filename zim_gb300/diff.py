"""Differentiable sub-pixel matching + reprojection (``zim_diff_*`` in include/zim.h).

The forward restates the reference's sub-pixel refinement and rectified
reprojection (PhaseShiftGrayCode3D/src/JSLAB_PhaseEpipolarReconstructor_V2.cpp
:985-1000, :414-461) on phase sampled with exact bilinear weights; the adjoint
is a hand-written CUDA kernel.  Integer decisions (fringe orders, match
columns) are inputs and stay fixed.

* ``forward`` / ``backward``: the C-ABI pair over a batch of views (one launch
  each), with a point-to-plane loss per view; FP64 totals on the host.
* ``Reconstruct``: the same pair as a ``torch.autograd.Function`` (points out,
  gradients of any downstream loss back to the 16 calibration parameters and
  the per-pixel phase).
* ``gauss_newton_step`` / ``compose_rotation``: the host side of calibration
  refinement (FP64).

Parameter vector order (``PARAM_NAMES``): per camera fx, fy, cx, cy, k1, k2;
then the baseline and the three components of a right-multiplied rotation
update of the right camera's rectifying rotation.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib
from .api import Context, _p, _stream, match

PARAM_NAMES = ["fx0", "fy0", "cx0", "cy0", "k1_0", "k2_0", "fx1", "fy1", "cx1", "cy1", "k1_1", "k2_1", "baseline",
               "rot0", "rot1", "rot2"]
NP = _lib.DIFF_NPARAMS


def params_struct(theta) -> _lib.DiffParams:
    th = np.asarray(theta, np.float64).reshape(NP)
    p = _lib.DiffParams()
    for c in range(2):
        for k in range(6):
            p.cam[c][k] = float(th[6 * c + k])
    p.baseline = float(th[12])
    for k in range(3):
        p.rot[k] = float(th[13 + k])
    return p


def theta_of(p: _lib.DiffParams) -> np.ndarray:
    return np.array([p.cam[c][k] for c in range(2) for k in range(6)] + [p.baseline] + list(p.rot), np.float64)


def nominal(ctx: Context) -> np.ndarray:
    """The parameters of the context's calibration (rotation update 0)."""
    p = _lib.DiffParams()
    ctx.check(ctx._L.zim_diff_params_nominal(ctx.h, C.byref(p)))
    return theta_of(p)


def rectify(ctx: Context, theta, cam: int, order: torch.Tensor, residual: torch.Tensor):
    """Exact-bilinear rectification of one camera under theta: (base, res, order)."""
    rh, rw = ctx.rect_h, ctx.rect_w
    dev = order.device
    base = torch.empty((rh, rw), dtype=torch.int32, device=dev)
    res = torch.empty((rh, rw), dtype=torch.float32, device=dev)
    ordr = torch.empty((rh, rw), dtype=torch.int32, device=dev)
    p = params_struct(theta)
    rows, cols = order.shape
    ctx.check(ctx._L.zim_diff_rectify(ctx.h, C.byref(p), cam, _p(order), _p(residual), rows, cols, _p(base), _p(res),
                                      _p(ordr), _stream()))
    return base, res, ordr


def match_columns(ctx: Context, theta, order_l, res_l, order_r, res_r, pha_f: int, grad_threshold: float = 1.0):
    """The integer match columns (rect_h x rect_w, -1 = none) under theta."""
    left = rectify(ctx, theta, 0, order_l, res_l)
    right = rectify(ctx, theta, 1, order_r, res_r)
    _, best = match(ctx, left, right, pha_f, grad_threshold, want_best=True)
    return best


@dataclass
class View:
    """One view: decoded phase of both cameras, match columns, target plane
    (n, d: distance n . P + d, P in the rectified left frame)."""
    order: Sequence[torch.Tensor]
    residual: Sequence[torch.Tensor]
    best_col: torch.Tensor
    plane: Sequence[float] = (0.0, 0.0, 0.0, 0.0)
    xyz: Optional[torch.Tensor] = None
    mask: Optional[torch.Tensor] = None
    grad_xyz: Optional[torch.Tensor] = None
    grad_phase: Optional[Sequence[torch.Tensor]] = None

    def struct(self) -> _lib.DiffView:
        v = _lib.DiffView()
        for c in range(2):
            v.order[c] = _p(self.order[c]).value
            v.residual[c] = _p(self.residual[c]).value
            v.grad_phase[c] = _p(self.grad_phase[c]).value if self.grad_phase is not None else None
        v.best_col = _p(self.best_col).value
        for k in range(4):
            v.plane[k] = float(self.plane[k])
        v.xyz = _p(self.xyz).value if self.xyz is not None else None
        v.mask = _p(self.mask).value if self.mask is not None else None
        v.grad_xyz = _p(self.grad_xyz).value if self.grad_xyz is not None else None
        return v


def _views(views: Sequence[View]):
    arr = (_lib.DiffView * len(views))()
    for i, v in enumerate(views):
        arr[i] = v.struct()
    return arr


def _result(r: _lib.DiffResult) -> dict:
    return {"loss": r.loss, "n_points": r.n_points, "grad": np.array(list(r.grad)),
            "jtj": np.array(list(r.jtj)).reshape(NP, NP)}


def forward(ctx: Context, theta, views: Sequence[View], z_min: float = 0.0, z_max: float = 1e4) -> dict:
    rows, cols = views[0].order[0].shape
    r = _lib.DiffResult()
    p = params_struct(theta)
    ctx.check(ctx._L.zim_diff_forward(ctx.h, C.byref(p), _views(views), len(views), rows, cols, z_min, z_max,
                                      C.byref(r), _stream()))
    return _result(r)


def backward(ctx: Context, theta, views: Sequence[View], loss_weight: float = 1.0, z_min: float = 0.0,
             z_max: float = 1e4) -> dict:
    rows, cols = views[0].order[0].shape
    r = _lib.DiffResult()
    p = params_struct(theta)
    ctx.check(ctx._L.zim_diff_backward(ctx.h, C.byref(p), _views(views), len(views), rows, cols, z_min, z_max,
                                       loss_weight, C.byref(r), _stream()))
    return _result(r)


class Reconstruct(torch.autograd.Function):
    """points, mask = Reconstruct.apply(theta, residual_l, residual_r, ctx, order_l, order_r, best_col, z_min, z_max)

    theta: (16,) float64 CPU tensor; residuals: device float32 phase residuals
    (phase = 2 pi order + residual).  points: (rect_h, rect_w, 3) float32 on the
    device, 0 where excluded.  The backward takes dLoss/dpoints and returns the
    gradient for theta (FP64 reduction) and for both residual maps."""

    @staticmethod
    def forward(fctx, theta, residual_l, residual_r, ctx, order_l, order_r, best_col, z_min=0.0, z_max=1e4):
        rh, rw = ctx.rect_h, ctx.rect_w
        xyz = torch.empty((rh, rw, 3), dtype=torch.float32, device=residual_l.device)
        mask = torch.empty((rh, rw), dtype=torch.uint8, device=residual_l.device)
        th = theta.detach().cpu().numpy()
        v = View((order_l, order_r), (residual_l, residual_r), best_col, xyz=xyz, mask=mask)
        forward(ctx, th, [v], z_min, z_max)
        fctx.zim = (ctx, th, order_l, order_r, best_col, z_min, z_max)
        fctx.save_for_backward(residual_l, residual_r)
        fctx.mark_non_differentiable(mask)
        return xyz, mask

    @staticmethod
    def backward(fctx, grad_xyz, grad_mask):
        ctx, th, order_l, order_r, best_col, z_min, z_max = fctx.zim
        residual_l, residual_r = fctx.saved_tensors
        gl = torch.zeros_like(residual_l)
        gr = torch.zeros_like(residual_r)
        v = View((order_l, order_r), (residual_l, residual_r), best_col, grad_xyz=grad_xyz.contiguous(),
                 grad_phase=(gl, gr))
        r = backward(ctx, th, [v], loss_weight=0.0, z_min=z_min, z_max=z_max)
        return (torch.from_numpy(r["grad"]), gl, gr, None, None, None, None, None, None)


# ---- host side of calibration refinement (FP64) ----

def rotation_matrix(v) -> np.ndarray:
    """Rotation matrix of a rotation vector (Rodrigues' formula)."""
    v = np.asarray(v, np.float64)
    th = float(np.linalg.norm(v))
    if th == 0.0:
        return np.eye(3)
    k = v / th
    Kx = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(th) * Kx + (1 - np.cos(th)) * Kx @ Kx


def rotation_vector(R) -> np.ndarray:
    """Inverse of rotation_matrix for rotations below pi."""
    R = np.asarray(R, np.float64)
    c = np.clip((np.trace(R) - 1) / 2, -1.0, 1.0)
    th = np.arccos(c)
    w = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    if th < 1e-12:
        return w / 2
    return w * th / (2 * np.sin(th))


def compose_rotation(rot, delta) -> np.ndarray:
    """rot' with exp(rot') = exp(rot) exp(delta): the update the rotation
    gradient refers to (a right-multiplied perturbation at the current value)."""
    return rotation_vector(rotation_matrix(rot) @ rotation_matrix(delta))


def gauss_newton_step(theta, result: dict, damping: float = 1e-6, free: Optional[Sequence[int]] = None) -> np.ndarray:
    """One Levenberg-Marquardt-damped Gauss-Newton step on sum of squared
    distances from a backward result (grad = J^T 2r, jtj = J^T J), over the
    parameter indices in `free` (default: all).  Returns the new theta."""
    th = np.asarray(theta, np.float64).copy()
    idx = np.arange(NP) if free is None else np.asarray(free)
    H = result["jtj"][np.ix_(idx, idx)]
    g = 0.5 * result["grad"][idx]
    H = H + damping * np.diag(np.diag(H) + 1e-30)
    step = -np.linalg.solve(H, g)
    full = np.zeros(NP)
    full[idx] = step
    th[:13] += full[:13]
    th[13:] = compose_rotation(th[13:], full[13:])
    return th
