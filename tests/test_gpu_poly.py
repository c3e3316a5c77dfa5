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


# ------------------------------------------------- cubic calibration fit ----

def _fit_case(ctx, n_planes=6, seed=3, noise=0.02):
    from oracle import calib_fit as F
    spec, *_ = scene_data("config0")
    ctx.set_calibration(spec.rig.as_dict(), False)
    H, W = 48, 64  # a corner of the rectified frame keeps the FP64 oracle fast
    disps, masks = F.synthetic_planes(ctx.Q, H, W, n_planes=n_planes, seed=seed, noise=noise, dropout=0.1)
    return F, disps, masks, H, W


@pytest.mark.gpu
def test_fit_poly_calib_matches_oracle(ctx):
    from zim_gb300 import api
    F, disps, masks, H, W = _fit_case(ctx)
    g = api.fit_poly_calib(ctx, ctx.Q, [torch.from_numpy(d).cuda() for d in disps],
                           [torch.from_numpy(m).cuda() for m in masks])
    gx, gy, gz = (t.cpu().numpy() for t in g[:3])
    ox, oy, oz, oeq = F.fit(ctx.Q, disps, masks)
    # planes: the same up to the eigenvector's sign
    for a, b in zip(g[3], oeq):
        s = 1.0 if a[:3] @ b[:3] > 0 else -1.0
        assert np.allclose(a, s * b, rtol=0, atol=1e-9 * max(1.0, abs(b[3])))
    fitted = np.count_nonzero(np.stack([(m > 0) & (d > 0) for d, m in zip(disps, masks)]).sum(0) >= 4)
    assert np.count_nonzero(gz.any(-1)) == np.count_nonzero(oz.any(-1)) == fitted
    # the two least-squares cubics agree at every sample disparity to the
    # float32 rounding of their coefficients
    for d, m in zip(disps, masks):
        r, c = np.nonzero((m > 0) & (d > 0))
        dv = d[r, c].astype(np.float64)
        for gc, oc in ((gx, ox), (gy, oy), (gz, oz)):
            a, b = F.evaluate(gc[r, c], dv), F.evaluate(oc[r, c], dv)
            scale = sum(np.abs(oc[r, c, k].astype(np.float64) * dv ** k) for k in range(4))
            live = oc[r, c].any(-1)
            assert np.all(np.abs(a - b)[live] <= 4e-7 * scale[live] + 1e-6)


@pytest.mark.gpu
def test_fitted_maps_reconstruct_the_planes(ctx):
    """Fit on the whole rectified frame, then reproject one plane's disparity
    through the maps (reproject_model 1): the points lie on that plane."""
    from oracle import calib_fit as F
    from zim_gb300 import api
    spec, *_ = scene_data("config0")
    ctx.set_calibration(spec.rig.as_dict(), False)
    H, W = ctx.rect_h, ctx.rect_w
    # 800-1000 mm: over a 1.25:1 depth range a cubic in d follows z = Q23 / (Q32 d + Q33)
    # to ~1e-4 relative
    disps, masks = F.synthetic_planes(ctx.Q, H, W, n_planes=6, seed=4, noise=0.0, dropout=0.0, z0=800.0, z1=1000.0)
    cx, cy, cz, eqs = api.fit_poly_calib(ctx, ctx.Q, [torch.from_numpy(d).cuda() for d in disps],
                                         [torch.from_numpy(m).cuda() for m in masks])
    ctx.set_poly_calib(cx.cpu().numpy(), cy.cpu().numpy(), cz.cpu().numpy())
    try:
        rc = api.recon_config(reproject_model=1, use_disp_median_filter=0, max_depth=1e4)
        _, xyz, mask = api.median_reproject(ctx, rc, torch.from_numpy(disps[2]).cuda())
        p = xyz.cpu().numpy()[mask.cpu().numpy() > 0].astype(np.float64)
        assert p.shape[0] > 0.9 * H * W
        dist = p @ eqs[2, :3] + eqs[2, 3]
        assert np.abs(dist).max() < 5e-4 * np.abs(p[:, 2]).max()
    finally:
        ctx.set_poly_calib()
        ctx.set_calibration(spec.rig.as_dict(), True)


@pytest.mark.gpu
def test_stereo_calib_v2_class_roundtrip(ctx, tmp_path):
    from oracle import calib_fit as F
    from zim_gb300 import api, calib_io
    spec, *_ = scene_data("config0")
    rig = spec.rig.as_dict()
    base = api.JSLAB_StereoCalibParams_V1(rig["K"], rig["D"], rig["R"], rig["t"], (rig["width"], rig["height"]))
    cal = api.JSLAB_StereoCalib_V2((rig["width"], rig["height"]), base, ctx=api.Context(0))
    cal._ctx.set_calibration(rig, False)
    disps, masks = F.synthetic_planes(cal._ctx.Q, rig["height"], rig["width"], n_planes=5, seed=6)
    for d, m in zip(disps, masks):
        cal.addPlaneReferenceData(d, m)
    cal.computePixelwiseDepthCalibration()
    fn = str(tmp_path / "stereo_v2.xml")
    assert cal.saveCalibResult(fn)
    back = api.JSLAB_StereoCalibParams_V2()
    assert calib_io.loadStereoCalibParams_V2(fn, back)
    for a, b in zip(cal.getParams().xyz_calib_coeffs, back.xyz_calib_coeffs):
        assert np.array_equal(a, b) and a.shape == (rig["height"], rig["width"], 4)
    cal.clearPlaneReferenceData()
    assert cal._disps == []
