"""GPU differentiable matching + reprojection against the FP64 oracle.

Both sides get identical inputs: the oracle's decoded phase (FP32 residuals),
the same match columns and the same plane.  The kernel works in FP32 (FP64 for
w, the plane distance and the reductions), so the loss, points and gradients
agree to FP32 accuracy; the errors are printed so the test log records them.
Gradients are compared at a perturbed calibration (baseline +0.5 %, cx +3 px,
k1 +0.02: the refinement start point), where they are systematic; at the true
calibration they are sums of zero-mean noise terms that cancel to ~1e-3 of
their magnitude, which no FP32 per-point arithmetic resolves."""
import math

import numpy as np
import pytest
import torch

from diffcase import DiffCase, fd_step

pytestmark = pytest.mark.gpu

PARAMS = ["fx0", "fy0", "cx0", "cy0", "k1_0", "k2_0", "fx1", "fy1", "cx1", "cy1", "k1_1", "k2_1", "baseline",
          "rot0", "rot1", "rot2"]


@pytest.fixture(scope="module")
def cases():
    return [DiffCase(width=480, height=400, pose=p) for p in (0, 1)]


@pytest.fixture(scope="module")
def gctx(native, cases):
    from zim_gb300 import api
    c = api.Context(0)
    c.set_calibration(cases[0].spec.rig.as_dict(), True)
    return c


def _view(case, with_points=False, with_phase_grad=False):
    from zim_gb300 import diff
    dev = "cuda"
    order = [torch.from_numpy(o).to(dev) for o in case.order]
    res = [torch.from_numpy(r.astype(np.float32)).to(dev) for r in case.residual]
    best = torch.from_numpy(case.best.astype(np.int32)).to(dev)
    v = diff.View(order, res, best, tuple(case.plane))
    if with_points:
        v.xyz = torch.empty((case.rect_h, case.rect_w, 3), dtype=torch.float32, device=dev)
        v.mask = torch.empty((case.rect_h, case.rect_w), dtype=torch.uint8, device=dev)
    if with_phase_grad:
        v.grad_phase = [torch.zeros_like(res[0]), torch.zeros_like(res[1])]
    return v


def _oracle(case, theta=None, best=None, **kw):
    from oracle import oracle as O
    r32 = [r.astype(np.float32).astype(np.float64) for r in case.residual]
    th = case.theta0 if theta is None else theta
    bc = case.best if best is None else best
    return O.diff_eval(case.geom, th, case.order[0], r32[0], case.order[1], r32[1], bc, case.plane, **kw)


def perturbed(theta0):
    th = np.array(theta0, np.float64)
    th[12] *= 1.005
    th[2] += 3.0
    th[4] += 0.02
    return th


@pytest.fixture(scope="module")
def pert(gctx, cases):
    """Perturbed parameters and the match columns they give on the GPU."""
    from zim_gb300 import diff
    c = cases[0]
    th = perturbed(c.theta0)
    v = _view(c)
    best = diff.match_columns(gctx, th, v.order[0], v.residual[0], v.order[1], v.residual[1], c.spec.pha_f)
    return th, best


def test_geometry_matches_oracle(gctx, cases):
    c = cases[0]
    assert (gctx.rect_w, gctx.rect_h) == (c.rect_w, c.rect_h)
    assert np.allclose(gctx.Q, c.Q, rtol=1e-12, atol=1e-9)


def test_forward_matches_oracle(gctx, cases):
    from zim_gb300 import diff
    c = cases[0]
    th = diff.nominal(gctx)
    assert np.allclose(th, c.theta0, rtol=1e-15, atol=0)
    v = _view(c, with_points=True)
    r = diff.forward(gctx, th, [v])
    o = _oracle(c, want_grad=False, want_points=True)
    m = v.mask.cpu().numpy() > 0
    both = m & (o["mask"] > 0)
    assert (m != (o["mask"] > 0)).sum() <= 1e-4 * m.sum() + 2
    xg, xo = v.xyz.cpu().numpy()[both], o["xyz"][both]
    rel = np.abs(xg - xo).max() / np.abs(xo).max()
    lrel = abs(r["loss"] - o["loss"]) / o["loss"]
    print("forward: points max rel %.2e, loss rel %.2e, n %d vs %d" % (rel, lrel, r["n_points"], o["n_points"]))
    assert rel < 2e-6
    assert lrel < 1e-3


def test_backward_matches_oracle(gctx, cases, pert):
    from zim_gb300 import diff
    c = cases[0]
    th, best = pert
    v = _view(c, with_phase_grad=True)
    v.best_col = best
    r = diff.backward(gctx, th, [v])
    o = _oracle(c, theta=th, best=best.cpu().numpy(), want_phase_grad=True)
    assert abs(r["n_points"] - o["n_points"]) <= 1e-4 * o["n_points"] + 2
    g, go = r["grad"], o["grad"]
    rel = np.abs(g - go) / np.abs(go)
    for k in range(16):
        print("  %-8s gpu % .9e  fp64 % .9e  rel %.2e" % (PARAMS[k], g[k], go[k], rel[k]))
    nrm = np.linalg.norm(g - go) / np.linalg.norm(go)
    print("backward: gradient rel err: norm-wise %.2e, worst component %.2e" % (nrm, rel.max()))
    # FP32 per-point terms, FP64 sums: measured 3.3e-6 norm-wise and 2.5e-4 on
    # the worst component (fy1, whose phase slope is near zero for vertical
    # fringes); FP32 sample positions alone move the FP64 gradient by as much
    # (test_oracle_diff.py).  Bounds: about twice the measured values.
    assert nrm < 6e-6
    assert rel.max() < 5e-4
    H, Ho = r["jtj"], o["jtj"]
    assert np.linalg.norm(H - Ho) / np.linalg.norm(Ho) < 1e-4
    for cam in (0, 1):
        gp = v.grad_phase[cam].cpu().numpy().astype(np.float64)
        gpo = o["grad_phase"][cam]
        e = np.linalg.norm(gp - gpo) / np.linalg.norm(gpo)
        print("  phase gradient cam %d: rel L2 err %.2e" % (cam, e))
        assert e < 5e-5  # measured 1.6e-5, 1.7e-5


def test_gpu_gradient_against_finite_differences(gctx, cases, pert):
    """GPU gradient vs Richardson central differences (h = 1e-4 relative) of
    the FP64 oracle loss with the bilinear cells frozen: the check of the
    differentiation itself."""
    from zim_gb300 import diff
    c = cases[0]
    th0, best_t = pert
    best = best_t.cpu().numpy()
    v = _view(c)
    v.best_col = best_t
    r = diff.backward(gctx, th0, [v])
    cells = np.zeros(c.rect_w * c.rect_h * 8, np.int32)
    _oracle(c, theta=th0, best=best, want_grad=False, cells=cells, cells_mode=1)
    h = fd_step(th0)

    def central(k, step):
        out = []
        for s in (step, -step):
            th = th0.copy()
            th[k] += s
            out.append(_oracle(c, theta=th, best=best, want_grad=False, cells=cells, cells_mode=2)["loss"])
        return (out[0] - out[1]) / (2 * step)

    fd = np.array([(4 * central(k, h[k] / 2) - central(k, h[k])) / 3 for k in range(16)])
    rel = np.abs(r["grad"] - fd) / np.abs(fd)
    nrm = np.linalg.norm(r["grad"] - fd) / np.linalg.norm(fd)
    print("GPU gradient vs FP64 central differences: norm-wise %.2e, worst component %.2e" % (nrm, rel.max()))
    assert nrm < 6e-6  # measured 3.3e-6
    assert rel.max() < 5e-4  # measured 2.5e-4


def test_batched_views_sum(gctx, cases):
    from zim_gb300 import diff
    v0, v1 = _view(cases[0]), _view(cases[1])
    both = diff.backward(gctx, cases[0].theta0, [v0, v1])
    a = diff.backward(gctx, cases[0].theta0, [v0])
    b = diff.backward(gctx, cases[0].theta0, [v1])
    assert both["n_points"] == a["n_points"] + b["n_points"]
    assert np.allclose(both["grad"], a["grad"] + b["grad"], rtol=1e-9, atol=0)
    again = diff.backward(gctx, cases[0].theta0, [v0, v1])
    assert np.array_equal(both["grad"], again["grad"]) and both["loss"] == again["loss"]


def test_autograd_function(gctx, cases, pert):
    from zim_gb300 import diff
    c = cases[0]
    th, best = pert
    v = _view(c)
    v.best_col = best
    theta = torch.tensor(th, dtype=torch.float64, requires_grad=True)
    res_l = v.residual[0].clone().requires_grad_(True)
    xyz, mask = diff.Reconstruct.apply(theta, res_l, v.residual[1], gctx, v.order[0], v.order[1], v.best_col)
    n = torch.tensor(c.plane[:3], dtype=torch.float32, device="cuda")
    dist = (xyz @ n + float(c.plane[3])) * mask
    loss = (dist * dist).sum()
    loss.backward()
    ref = diff.backward(gctx, th, [v])
    rel = (theta.grad.numpy() - ref["grad"]) / np.abs(ref["grad"])
    print("autograd vs backward: worst rel %.2e" % np.abs(rel).max())
    assert np.abs(rel).max() < 1e-3  # the torch side forms the distance from FP32 points
    assert res_l.grad is not None and torch.isfinite(res_l.grad).all()


def test_rectify_and_match_decisions(gctx, cases):
    """zim_diff_rectify + zim_match agree with the oracle's match columns on
    almost every pixel (exact bilinear vs 1/32-quantised remap)."""
    from zim_gb300 import diff
    c = cases[0]
    v = _view(c)
    best = diff.match_columns(gctx, c.theta0, v.order[0], v.residual[0], v.order[1], v.residual[1], c.spec.pha_f)
    b = best.cpu().numpy()
    both = (b >= 0) & (c.best >= 0)
    assert both.sum() > 0.9 * (c.best >= 0).sum()
    assert np.mean(np.abs(b[both] - c.best[both]) <= 1) > 0.999
