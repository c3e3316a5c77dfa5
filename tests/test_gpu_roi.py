"""ROI-restricted reconstruction on the GPU (prepareRectifiedROI /
startCalculate_v2_roi, JSLAB_PhaseEpipolarReconstructor_V2.cpp:595-914).

Stages are fed the GPU's own rectified maps, so each comparison isolates the
ROI arithmetic.  Tolerances:
* prepare: ROI mask bit-exact and both rectangles equal (integer work);
* reconstruct: median disparity, mask and points as the whole-pair test
  (FP32 matching against the FP64 oracle: decisions within 1e-5 rad of a
  threshold or a tie may differ; at most 2e-3 of the ROI);
* deep inside the ROI, where the right window holds every candidate, the ROI
  disparity equals the whole-frame disparity bit for bit.
"""
import math

import numpy as np
import pytest
import torch

from conftest import scene_data
from polycase import q_maps

ROIS = [((306, 256), (180, 120), 0.0), ((280, 240), (150, 90), 27.5), ((330, 270), (120, 160), -41.0)]


@pytest.fixture(scope="module")
def rectified(ctx):
    from zim_gb300 import api
    spec, L, R, _ = scene_data("config1", width=612, height=512)
    ctx.set_calibration(spec.rig.as_dict(), True)
    ctx.set_poly_calib(*q_maps(ctx.Q, ctx.rect_h, ctx.rect_w, "inv"))
    dcfg = api.decode_config(**spec.decode_kwargs())
    cams = []
    for fr in (L, R):
        d = api.decode(ctx, dcfg, torch.from_numpy(fr).cuda())
        cams.append(api.rectify(ctx, len(cams), d["order"], d["residual"], True))
    yield ctx, spec, cams
    ctx.set_poly_calib()


def f64_phase(base, res):
    return 2 * math.pi * base.cpu().numpy().astype(np.float64) + res.cpu().numpy().astype(np.float64)


@pytest.mark.gpu
@pytest.mark.parametrize("roi", ROIS)
def test_prepare_roi_matches_oracle(rectified, roi):
    from oracle import roi as R
    from zim_gb300 import api
    ctx, spec, (lc, rc) = rectified
    g = api.prepare_roi(ctx, roi, lc[2], rc[2], spec.pha_f)
    mx, my = (t.cpu().numpy() for t in ctx.rectify_maps(0))
    o = R.prepare(roi, (ctx.src_h, ctx.src_w), mx, my, lc[2].cpu().numpy(), rc[2].cpu().numpy(), spec.pha_f)
    assert g is not None and o is not None
    assert g.left_rect == o[0] and g.right_rect == o[1], (g.left_rect, g.right_rect, o[:2])
    assert np.array_equal(g.mask.cpu().numpy(), o[2])
    # the window narrows the search: fewer columns than the full row
    assert g.right_rect[2] < ctx.rect_w


@pytest.mark.gpu
def test_empty_roi(rectified):
    from zim_gb300 import api
    ctx, spec, (lc, rc) = rectified
    assert api.prepare_roi(ctx, ((-500, -500), (20, 20), 0.0), lc[2], rc[2], spec.pha_f) is None


@pytest.mark.gpu
@pytest.mark.parametrize("roi", ROIS)
@pytest.mark.parametrize("model", [1, 0])
def test_reconstruct_roi_matches_oracle(rectified, oracle_lib, roi, model):
    from oracle import roi as R
    from zim_gb300 import api
    ctx, spec, (lc, rc) = rectified
    g = api.prepare_roi(ctx, roi, lc[2], rc[2], spec.pha_f)
    # ROR radius 5 mm: the test scene's pixel spacing is 1-1.5 mm
    rcfg = api.recon_config(reproject_model=model, radius_search=5.0)
    xyz, mask, disp = api.reconstruct_roi(ctx, rcfg, g, lc, rc, spec.pha_f, want_disp=True)
    poly = q_maps(ctx.Q, ctx.rect_h, ctx.rect_w, "inv") if model == 1 else None
    ox, om, od, near = R.reconstruct((g.left_rect, g.right_rect), g.mask.cpu().numpy(), f64_phase(lc[0], lc[1]),
                                     lc[2].cpu().numpy(), f64_phase(rc[0], rc[1]), rc[2].cpu().numpy(), spec.pha_f,
                                     ctx.R1, poly=poly, Q=ctx.Q, ror=(5.0, 10, 10))
    gx, gm, gd = xyz.cpu().numpy(), mask.cpu().numpy(), disp.cpu().numpy()
    n = gm.size
    assert om.sum() > 0.3 * n
    assert (np.abs(gd - od) > 2e-4).sum() <= 2e-3 * n + (near > 0).sum()
    assert (gm != om).sum() <= 2e-3 * n
    both = (gm > 0) & (om > 0)
    rel = np.abs(gx[both] - ox[both]) / np.maximum(1.0, np.abs(ox[both]))
    assert (rel > 1e-4).any(axis=1).mean() <= 2e-3


@pytest.mark.gpu
def test_roi_interior_equals_whole_frame(rectified):
    from zim_gb300 import api
    ctx, spec, (lc, rc) = rectified
    roi = ROIS[0]
    g = api.prepare_roi(ctx, roi, lc[2], rc[2], spec.pha_f)
    rcfg = api.recon_config(reproject_model=1, use_px_gaussian=0, use_ror=0)
    _, _, rd = api.reconstruct_roi(ctx, rcfg, g, lc, rc, spec.pha_f, want_disp=True)
    full, best = api.match(ctx, lc, rc, spec.pha_f)
    fd, _, _ = api.median_reproject(ctx, rcfg, full)
    lx, ly, lw, lh = g.left_rect
    rx, _, rw, _ = g.right_rect
    m = g.mask.cpu().numpy()[ly:ly + lh, lx:lx + lw] > 0
    # interior: the 5x5 median sees only matched mask pixels whose whole-frame
    # match lies inside the window, away from its edges
    b = best.cpu().numpy()[ly:ly + lh, lx:lx + lw]
    ok = m & (b >= rx + 2) & (b < rx + rw - 1)
    inner = np.zeros_like(ok)
    inner[2:-2, 2:-2] = np.all([ok[2 + dy:lh - 2 + dy, 2 + dx:lw - 2 + dx] for dy in range(-2, 3)
                                for dx in range(-2, 3)], axis=0)
    assert inner.sum() > 0.5 * m.sum()
    a = rd.cpu().numpy()[inner]
    f = fd.cpu().numpy()[ly:ly + lh, lx:lx + lw][inner]
    assert np.array_equal(a, f)


@pytest.mark.gpu
def test_reconstructor_class_roi(rectified):
    from zim_gb300 import api
    ctx, spec, (lc, rc) = rectified
    rec = api.JSLAB_PhaseEpipolarReconstructor_V2(api.JSLAB_PhaseEpipolarReconstructor_V2.Config(radius_search=5.0),
                                                  ctx=ctx)
    rec._rect, rec._pha_f, rec._use_v2 = [lc, rc], spec.pha_f, True
    xyz, P = rec.startCalculate_v2_roi(ROIS[1])
    g = api.prepare_roi(ctx, ROIS[1], lc[2], rc[2], spec.pha_f)
    gx, gm, _ = api.reconstruct_roi(ctx, api.recon_config(reproject_model=1, radius_search=5.0), g, lc, rc,
                                    spec.pha_f)
    assert torch.equal(P, gm) and torch.equal(xyz, gx)
    assert rec.getDisparityMap().shape == (g.left_rect[3], g.left_rect[2])
    assert rec.startCalculate_v2_roi(((-500, -500), (20, 20), 0.0)) == (None, None)
