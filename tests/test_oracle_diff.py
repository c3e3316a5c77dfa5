"""The FP64 oracle of the differentiable path, pinned against its own central
finite differences (CPU).  With every sample's bilinear cell frozen (an
integer decision, like the fringe orders and match columns) the loss is smooth
in the parameters, so the analytic gradient must match to ~1e-7 relative."""
import math

import numpy as np
import pytest

from diffcase import DiffCase, fd_step

PARAMS = ["fx0", "fy0", "cx0", "cy0", "k1_0", "k2_0", "fx1", "fy1", "cx1", "cy1", "k1_1", "k2_1", "baseline",
          "rot0", "rot1", "rot2"]


@pytest.fixture(scope="module")
def case():
    return DiffCase(width=320, height=256, pose=0)


def test_view_reconstructs_the_plane(case):
    r = case.eval(case.theta0, want_grad=False, want_points=True)
    assert r["n_points"] > 0.3 * case.rect_w * case.rect_h
    # at the true calibration only the phase noise remains: at 320 px width one
    # pixel of disparity is ~13 mm of depth, so a few tenths of a mm, unbiased
    rms = math.sqrt(r["loss"] / r["n_points"])
    assert rms < 1.5, rms
    m = r["mask"] > 0
    dist = r["xyz"][m] @ case.plane[:3] + case.plane[3]
    assert abs(dist.mean()) < 0.05, dist.mean()


def test_gradient_matches_central_differences(case):
    cells = np.zeros(case.rect_w * case.rect_h * 8, np.int32)
    th = case.theta0
    r0 = case.eval(th, cells=cells, cells_mode=1)
    r_free = case.eval(th, want_grad=False)
    assert r0["loss"] == r_free["loss"]  # recording the cells changes nothing
    g = r0["grad"]
    h = fd_step(th)

    def central(k, step):
        tp, tm = th.copy(), th.copy()
        tp[k] += step
        tm[k] -= step
        lp = case.eval(tp, want_grad=False, cells=cells, cells_mode=2)["loss"]
        lm = case.eval(tm, want_grad=False, cells=cells, cells_mode=2)["loss"]
        return (lp - lm) / (2 * step)

    worst = 0.0
    for k in range(16):
        # h = 1e-4 relative leaves an O(h^2) truncation term of up to ~1e-2
        # (pixels whose sub-pixel parabola is nearly flat are strongly curved);
        # Richardson's combination of h and h/2 cancels it
        fd = (4 * central(k, h[k] / 2) - central(k, h[k])) / 3
        floor = 1e-13 * r0["loss"] / h[k]  # what FP64 loss sums can resolve
        err = abs(fd - g[k])
        assert err <= 1e-6 * abs(g[k]) + floor, (PARAMS[k], g[k], fd)
        worst = max(worst, err / max(abs(g[k]), floor))
    print("oracle gradient vs central differences: worst relative error %.2e" % worst)


def test_jtj_is_a_gram_matrix(case):
    r = case.eval(case.theta0)
    H = r["jtj"]
    assert np.allclose(H, H.T, rtol=0, atol=1e-12 * np.abs(H).max())
    ev = np.linalg.eigvalsh(H / np.abs(H).max())
    assert ev.min() > -1e-9


def test_phase_gradient_matches_central_differences(case):
    rg = case.eval(case.theta0, want_grad=False, want_phase_grad=True)
    cells = np.zeros(case.rect_w * case.rect_h * 8, np.int32)
    case.eval(case.theta0, want_grad=False, cells=cells, cells_mode=1)
    for cam in (0, 1):
        gph = rg["grad_phase"][cam]
        idx = np.argsort(np.abs(gph).ravel())[-3:]
        for flat in idx:
            y, x = divmod(int(flat), gph.shape[1])
            h = 1e-6
            res = [case.residual[0].copy(), case.residual[1].copy()]
            losses = []
            for s in (h, -h):
                rr = [res[0].copy(), res[1].copy()]
                rr[cam][y, x] += s
                from oracle import oracle as O
                losses.append(O.diff_eval(case.geom, case.theta0, case.order[0], rr[0], case.order[1], rr[1],
                                          case.best, case.plane, want_grad=False, cells=cells, cells_mode=2)["loss"])
            fd = (losses[0] - losses[1]) / (2 * h)
            assert abs(fd - gph[y, x]) <= 1e-5 * abs(gph[y, x]) + 1e-13 * rg["loss"] / h, (cam, y, x, gph[y, x], fd)


def test_gauss_newton_recovers_a_perturbed_baseline(case):
    # one plane of known offset fixes the depth scale, hence the baseline (the
    # full calibration needs many poses; see the refinement bench leg)
    from zim_gb300.diff import gauss_newton_step
    th = case.theta0.copy()
    th[12] *= 1.005
    l0 = case.eval(th, want_grad=False)["loss"]
    for _ in range(3):
        th = gauss_newton_step(th, case.eval(th), damping=1e-6, free=[12])
    l1 = case.eval(th, want_grad=False)["loss"]
    assert l1 < 0.5 * l0
    assert abs(th[12] / case.theta0[12] - 1) < 2e-4


def test_fp32_sample_positions_set_a_floor_above_1e6():
    """The per-component floor an FP32 forward cannot pass: the FP64 oracle's
    gradient moves by more than 1e-6 relative on some components when only
    its sample positions (u, v, hundreds of pixels) are rounded to FP32.  The
    GPU path computes positions in FP32 (as its specification asks), so its
    per-component agreement is bounded by this, not by the reductions."""
    from diffcase import DiffCase
    from oracle import oracle as O
    c = DiffCase(width=640, height=512)
    th = c.theta0.copy()
    th[12] *= 1.005
    th[2] += 3.0
    th[4] += 0.02
    g0 = c.eval(th)["grad"]
    O.diff_round_positions(True)
    try:
        g1 = c.eval(th)["grad"]
    finally:
        O.diff_round_positions(False)
    rel = np.abs(g1 - g0) / np.abs(g0)
    assert rel.max() > 1e-6
    assert np.linalg.norm(g1 - g0) / np.linalg.norm(g0) < 1e-4
    assert np.array_equal(c.eval(th)["grad"], g0)  # the switch is off again
