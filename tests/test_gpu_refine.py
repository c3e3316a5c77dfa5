"""Calibration refinement (the benchmark spec's batched forward/adjoint use):
Levenberg-Marquardt over the differentiable matching + reprojection from a
perturbed calibration (baseline +0.5 %, cx0 +3 px, k1_0 +0.02), on planar
target poses decoded on the GPU.

The perturbed calibration defines the rectified frame of the views; the
truth is the true calibration's parameters in that frame (as in bench.py's
refinement leg).  Checked: the loss falls, and baseline, cx0 and k1_0 come
back to within a small fraction of their starting errors."""
import numpy as np
import pytest


@pytest.mark.gpu
def test_refinement_recovers_the_perturbed_parameters(native):
    import torch
    from zim_gb300 import api, calib_refine as CR, diff, synth

    n_poses, iterations = 6, 40
    specs = [synth.pose_plane(seed=3, width=1224, height=1024, pose=p) for p in range(n_poses)]
    rig = specs[0].rig.as_dict()
    truth = api.Context(0)
    truth.set_calibration(rig, True)
    theta_true = diff.nominal(truth)
    pert = dict(rig)
    pert["K"] = [k.copy() for k in rig["K"]]
    pert["D"] = [d.copy() for d in rig["D"]]
    pert["K"][0][0, 2] += 3.0
    pert["D"][0][0] += 0.02
    pert["t"] = rig["t"] * 1.005
    ctx = api.Context(0)
    ctx.set_calibration(pert, True)
    dcfg = api.decode_config(**specs[0].decode_kwargs())
    poses = []
    for s in specs:
        poses += CR.decode_views(ctx, dcfg, [(s.render(0), s.render(1))], [(s.plane_n, s.plane_d)])
    th0 = diff.nominal(ctx)
    th, log = CR.refine(ctx, poses, th0, specs[0].pha_f, iterations=iterations)
    torch.cuda.synchronize()
    e0, e1 = th0 - theta_true, th - theta_true
    names = diff.PARAM_NAMES
    print("refine: %d poses, %d iterations in %.2f s (%.1f it/s); loss %.4g -> %.4g" % (
        n_poses, iterations, log.seconds, iterations / log.seconds, log.losses[0], log.losses[-1]))
    for k in (2, 4, 12):
        print("  %s: start error %.4g, final error %.4g" % (names[k], e0[k], e1[k]))
    assert log.losses[-1] < 0.5 * log.losses[0]
    for k in (2, 4, 12):  # cx0, k1_0, baseline
        assert abs(e1[k]) < 0.1 * abs(e0[k]), (names[k], e0[k], e1[k])
