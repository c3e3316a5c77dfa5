"""Per-pixel polynomial reprojection on the GPU (startCalculate_v2 /
evaluateV2CalibPoint, JSLAB_PhaseEpipolarReconstructor_V2.cpp:13-76,482-593).

* zim_median_reproject with reproject_model 1 against the oracle on maps that
  mix every model branch and rejection: points and mask bit-exact (both sides
  evaluate in FP64 in the reference's order without contraction), with and
  without the 5x5 median, rectified and R1-rotated output.
* The whole pair with maps equivalent to the rig's Q matrix against the Q path:
  the same cloud within 1e-5 relative (float rounding of the coefficients).
* Error behaviour: model 1 without maps, maps of the wrong size, unknown model.
"""
import numpy as np
import pytest
import torch

from conftest import scene_data
from polycase import BRANCHES, q_maps, random_disparity, random_maps


@pytest.fixture()
def calibrated(ctx):
    spec, L, R, _ = scene_data("config0")
    ctx.set_calibration(spec.rig.as_dict(), True)
    yield ctx, spec, L, R
    ctx.set_poly_calib()


@pytest.mark.gpu
@pytest.mark.parametrize("rectified", [1, 0])
@pytest.mark.parametrize("median", [0, 1])
def test_poly_reproject_bit_exact(calibrated, oracle_lib, rectified, median):
    from zim_gb300 import api
    ctx, *_ = calibrated
    H, W = ctx.rect_h, ctx.rect_w
    cx, cy, cz, br = random_maps(H, W, seed=11)
    d = random_disparity(H, W, br, seed=12)
    ctx.set_poly_calib(cx, cy, cz)
    rc = api.recon_config(reproject_model=1, use_rectified_coords=rectified, use_disp_median_filter=median)
    dout, xyz, mask = api.median_reproject(ctx, rc, torch.from_numpy(d).cuda())
    dm = oracle_lib.median5(d) if median else d
    assert np.array_equal(dout.cpu().numpy(), dm)
    ox, om = oracle_lib.poly_reproject(dm, (cx, cy, cz), ctx.R1, 0.0, 1000.0, bool(rectified))
    gx, gm = xyz.cpu().numpy(), mask.cpu().numpy()
    assert np.array_equal(gm, om)
    assert np.array_equal(gx.view(np.uint32), ox.view(np.uint32))
    if not median:
        hit = {BRANCHES[b] for b in np.unique(br[om > 0])}
        assert {"inv_cubic", "ray_inv", "ray_cubic", "lin_rational", "lin_cubic", "z_inv", "cubic"} <= hit


@pytest.mark.gpu
@pytest.mark.parametrize("model", ["inv", "ray", "rational"])
def test_pair_with_q_equivalent_maps_matches_q_path(calibrated, model):
    from zim_gb300 import api
    ctx, spec, L, R = calibrated
    H, W = ctx.rect_h, ctx.rect_w
    if model == "rational" and abs(ctx.Q[3, 3]) < 1e-12:
        pytest.skip("Q33 = 0: no rational form")
    dcfg = api.decode_config(**spec.decode_kwargs())
    lt, rt = torch.from_numpy(L).cuda(), torch.from_numpy(R).cuda()
    rq = api.recon_config(use_px_gaussian=1, use_ror=1, radius_search=5.0, max_depth=1e6)
    qx, qm, qd = api.reconstruct_pair(ctx, dcfg, rq, lt, rt, want_disp=True)
    ctx.set_poly_calib(*q_maps(ctx.Q, H, W, model))
    rp = api.recon_config(use_px_gaussian=1, use_ror=1, radius_search=5.0, max_depth=1e6, reproject_model=1)
    px, pm, pd = api.reconstruct_pair(ctx, dcfg, rp, lt, rt, want_disp=True)
    assert torch.equal(pd, qd)
    qm, pm = qm.cpu().numpy(), pm.cpu().numpy()
    both = (qm > 0) & (pm > 0)
    assert both.sum() > 0.5 * qm.size
    # ROR decisions on a radius boundary may flip with the last float bit
    assert (qm != pm).mean() < 1e-4
    rel = np.abs(px.cpu().numpy()[both] - qx.cpu().numpy()[both]) / (np.abs(qx.cpu().numpy()[both]) + 1.0)
    assert rel.max() < 1e-5, rel.max()


@pytest.mark.gpu
def test_reconstructor_class_v2_matches_pair_path(ctx):
    from zim_gb300 import api
    spec, L, R, _ = scene_data("ref_heterodyne", width=612, height=512)
    conf = api.JSLAB_PhaseShiftDecoder.Config(freq=spec.freq, shift_num=spec.shift_num,
                                              modulation_threshold=spec.modulation_threshold)
    dec = api.JSLAB_PhaseShiftDecoder.create(conf, api.JSLAB_PhaseShiftDecoder.Version.V2, ctx=ctx)
    dec.setImages(L); dec.startCalculate(); dl = dec.getDecoded()
    dec.setImages(R); dec.startCalculate(); dr = dec.getDecoded()
    rig = spec.rig.as_dict()
    params = api.JSLAB_StereoCalibParams_V2(rig["K"], rig["D"], rig["R"], rig["t"], (rig["width"], rig["height"]))
    ctx.set_calibration(rig, True)
    params.xyz_calib_coeffs = list(q_maps(ctx.Q, ctx.rect_h, ctx.rect_w, "inv"))
    rec = api.JSLAB_PhaseEpipolarReconstructor_V2(ctx=ctx)
    rec.setCalibrationParamsV2(params)
    rec.setData(dl, dr, pha_f=int(conf.freq[0]))
    vx, vm = rec.startCalculate_v2()
    rcfg = api.recon_config(reproject_model=1)
    dcfg = api.decode_config(**spec.decode_kwargs())
    px, pm, _ = api.reconstruct_pair(ctx, dcfg, rcfg, torch.from_numpy(L).cuda(), torch.from_numpy(R).cuda(),
                                     pha_f=int(conf.freq[0]))
    assert vm.any() and torch.equal(vm, pm) and torch.equal(vx, px)
    # without maps startCalculate_v2 writes no point, like the reference
    params.xyz_calib_coeffs = [np.zeros((0, 0, 4), np.float32)] * 3
    rec.setCalibrationParamsV2(params)
    rec.setData(dl, dr, pha_f=int(conf.freq[0]))
    ex, em = rec.startCalculate_v2()
    assert not em.any() and not ex.any()


@pytest.mark.gpu
def test_poly_errors(calibrated):
    from zim_gb300 import _lib, api
    ctx, *_ = calibrated
    H, W = ctx.rect_h, ctx.rect_w
    d = torch.zeros((H, W), dtype=torch.float32, device="cuda")
    ctx.set_poly_calib()
    with pytest.raises(_lib.ZimError) as e:
        api.median_reproject(ctx, api.recon_config(reproject_model=1), d)
    assert e.value.status == _lib.ERR_NOT_CALIBRATED
    with pytest.raises(_lib.ZimError) as e:
        api.median_reproject(ctx, api.recon_config(reproject_model=2), d)
    assert e.value.status == _lib.ERR_INVALID_ARG
    m = np.zeros((H, W + 1, 4), np.float32)
    with pytest.raises(_lib.ZimError) as e:
        ctx.set_poly_calib(m, m, m)
    assert e.value.status == _lib.ERR_INVALID_ARG
