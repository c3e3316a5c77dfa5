"""Whole-pair path (zim_reconstruct_pair) against the oracle run end to end on
the same frames, the host-buffer entry against the device entry, and the
reference-shaped Python classes against the C ABI."""
import math

import numpy as np
import pytest
import torch

from conftest import SMALL_SCENES, scene_data


def oracle_pair(oracle, spec, L, R, rc):
    cfg = oracle.make_decode_cfg(**spec.decode_kwargs())
    rig = spec.rig.as_dict()
    c = oracle.make_calib(rig["K"], rig["D"], rig["R"], rig["t"], rig["width"], rig["height"])
    R1, R2, P1, P2, Q, w, h = oracle.rectification(c, True)
    rect = []
    for cam, fr in enumerate((L, R)):
        ph, k, _, _, _ = oracle.decode(cfg, fr)
        mx, my = oracle.init_rectify_map(rig["K"][cam], rig["D"][cam], R1 if cam == 0 else R2,
                                         P1 if cam == 0 else P2, w, h)
        rect.append(oracle.rectify_decoded(ph, k, mx, my, True))
    disp, _, _ = oracle.stereo_match(rect[0][0], rect[1][0], rect[0][1], rect[1][1], spec.pha_f)
    dm = oracle.median5(disp.astype(np.float32))
    xyz, mask, _ = oracle.reproject(dm, Q, R1, rc["min_depth"], rc["max_depth"], True)
    if rc.get("use_px_gaussian"):
        xyz, mask, _ = oracle.px_gaussian(xyz, mask, False)
    if rc.get("use_ror"):
        xyz, mask, _ = oracle.ror(xyz, mask, rc["radius_search"], rc["radius_min_neighbors"],
                                  rc["radius_window_size"])
    return xyz, mask


def compare_clouds(g_xyz, g_mask, o_xyz, o_mask):
    both = (g_mask > 0) & (o_mask > 0)
    diff = (g_mask != o_mask).sum()
    rel = np.abs(g_xyz[both] - o_xyz[both]) / np.maximum(1.0, np.abs(o_xyz[both]))
    big = (rel > 1e-4).any(axis=1)
    return dict(points=int(both.sum()), mask_diff=int(diff), frac_mask_diff=float(diff / g_mask.size),
                frac_beyond_1e4=float(big.mean()) if both.any() else 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("name,kw", SMALL_SCENES)
def test_pair_matches_oracle_end_to_end(ctx, oracle_lib, name, kw):
    from zim_gb300 import api
    spec, L, R, _ = scene_data(name, **kw)
    ctx.set_calibration(spec.rig.as_dict(), True)
    # ROR radius 5 mm: the test scenes' pixel spacing is 1-1.5 mm
    rc = dict(use_px_gaussian=1, use_ror=1, radius_search=5.0, radius_min_neighbors=10, radius_window_size=10,
              min_depth=0.0, max_depth=1000.0)
    dcfg = api.decode_config(**spec.decode_kwargs())
    rcfg = api.recon_config(**rc)
    xyz, mask, _ = api.reconstruct_pair(ctx, dcfg, rcfg, torch.from_numpy(L).cuda(), torch.from_numpy(R).cuda())
    ox, om = oracle_pair(oracle_lib, spec, L, R, rc)
    s = compare_clouds(xyz.cpu().numpy(), mask.cpu().numpy(), ox, om)
    print(name, s)
    assert s["points"] > 0.5 * om.size, s
    # end to end, FP32-vs-FP64 decisions near their thresholds propagate through
    # matching and the filters; they stay a tiny fraction of the image
    assert s["frac_mask_diff"] <= 2e-3, s
    assert s["frac_beyond_1e4"] <= 2e-3, s


@pytest.mark.gpu
@pytest.mark.parametrize("pinned", [False, True])
def test_host_entry_equals_device_entry(ctx, oracle_lib, pinned):
    """Pageable outputs are copied back; a pinned cloud buffer takes the last
    stage's writes directly.  Both equal the device entry bit for bit."""
    from zim_gb300 import api
    spec, L, R, _ = scene_data("config1", width=612, height=512)
    ctx.set_calibration(spec.rig.as_dict(), True)
    dcfg = api.decode_config(**spec.decode_kwargs())
    rcfg = api.recon_config(use_px_gaussian=0, use_ror=0, use_mls=1, mls_window_size=7, mls_spatial_sigma=1.4142135,
                            mls_polynomial_order=2, mls_max_radius=2.0, mls_iterations=1)
    xyz, mask, disp = api.reconstruct_pair(ctx, dcfg, rcfg, torch.from_numpy(L).cuda(), torch.from_numpy(R).cuda(),
                                           want_disp=True)
    kw = {}
    if pinned:
        kw = dict(xyz=torch.empty((ctx.rect_h, ctx.rect_w, 3), dtype=torch.float32).pin_memory(),
                  mask=torch.empty((ctx.rect_h, ctx.rect_w), dtype=torch.uint8).pin_memory())
    hx, hm, hd = api.reconstruct_pair_host(ctx, dcfg, rcfg, L, R,
                                           disp=np.empty((ctx.rect_h, ctx.rect_w), np.float32), **kw)
    hx, hm = np.asarray(hx), np.asarray(hm)
    assert np.array_equal(hm, mask.cpu().numpy())
    assert np.array_equal(hx, xyz.cpu().numpy())
    assert np.array_equal(hd, disp.cpu().numpy())


@pytest.mark.gpu
def test_async_host_entry_two_pairs_in_flight(ctx, oracle_lib):
    """Two contexts on two streams, the asynchronous host entry alternating
    between them over four pairs of two different scenes (each context sees
    both scenes, so its scratch is reused while the other context's pair is in
    flight): every output equals the synchronous entry's, bit for bit."""
    from zim_gb300 import api
    spec, L1, R1, _ = scene_data("config1", width=612, height=512)
    _, L2, R2, _ = scene_data("config1", seed=5, width=612, height=512)
    rig = spec.rig.as_dict()
    dcfg = api.decode_config(**spec.decode_kwargs())
    rcfg = api.recon_config(use_px_gaussian=0, use_ror=0, use_sor=1, sor_mean_k=30, use_mls=1, mls_window_size=7,
                            mls_spatial_sigma=1.4142135, mls_polynomial_order=2, mls_max_radius=2.0,
                            mls_iterations=1, use_metric_gaussian=1, metric_gaussian_sigma=0.5)
    ctx.set_calibration(rig, True)
    want = [api.reconstruct_pair_host(ctx, dcfg, rcfg, L, R)[:2] for (L, R) in ((L1, R1), (L2, R2))]
    ctxs = [api.Context(0), api.Context(0)]
    for c in ctxs:
        c.set_calibration(rig, True)
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    frames = [(torch.from_numpy(L).pin_memory(), torch.from_numpy(R).pin_memory()) for (L, R) in ((L1, R1), (L2, R2))]
    outs = [(torch.empty((ctx.rect_h, ctx.rect_w, 3), dtype=torch.float32).pin_memory(),
             torch.empty((ctx.rect_h, ctx.rect_w), dtype=torch.uint8).pin_memory()) for _ in range(4)]
    for i in range(4):
        hl, hr = frames[(i // 2) % 2] if i % 2 == 0 else frames[(i // 2 + 1) % 2]
        api.reconstruct_pair_host(ctxs[i % 2], dcfg, rcfg, hl, hr, xyz=outs[i][0], mask=outs[i][1],
                                  stream=streams[i % 2], asynchronous=True)
    for s in streams:
        s.synchronize()
    for i in range(4):
        k = (i // 2) % 2 if i % 2 == 0 else (i // 2 + 1) % 2
        assert np.array_equal(outs[i][1].numpy(), want[k][1]), i
        assert np.array_equal(outs[i][0].numpy(), want[k][0]), i


@pytest.mark.gpu
def test_reference_classes_match_c_abi(ctx, oracle_lib):
    from zim_gb300 import api
    spec, L, R, _ = scene_data("ref_heterodyne", width=612, height=512)
    conf = api.JSLAB_PhaseShiftDecoder.Config(freq=spec.freq, shift_num=spec.shift_num,
                                              modulation_threshold=spec.modulation_threshold)
    dec = api.JSLAB_PhaseShiftDecoder.create(conf, api.JSLAB_PhaseShiftDecoder.Version.V2, ctx=ctx)
    dec.setImages([L[i] for i in range(L.shape[0])])
    lphase = dec.startCalculate()
    lk = dec.getOrderMap()
    lmod = dec.getModulationMap()
    ldec = dec.getDecoded()
    dec.setImages(R)
    dec.startCalculate()
    rdec = dec.getDecoded()
    assert lphase.dtype == torch.float64 and lk.dtype == torch.int32 and lmod.dtype == torch.float64
    rig = spec.rig.as_dict()
    params = api.JSLAB_StereoCalibParams_V1(rig["K"], rig["D"], rig["R"], rig["t"], (rig["width"], rig["height"]))
    rcon = api.JSLAB_PhaseEpipolarReconstructor_V2(ctx=ctx)
    rcon.setCalibrationParams(params)
    rcon.setData(ldec, rdec, pha_f=int(conf.freq[0]))
    xyz, P = rcon.startCalculate()
    dcfg = api.decode_config(**spec.decode_kwargs())
    gx, gm, _ = api.reconstruct_pair(ctx, dcfg, api.recon_config(), torch.from_numpy(L).cuda(),
                                     torch.from_numpy(R).cuda())
    assert torch.equal(P, gm) and torch.equal(xyz, gx)
    assert rcon.getDisparityMap().shape == (ctx.rect_h, ctx.rect_w)
    # the reference-style f64 entry (already smoothed phase + order) reproduces the exact path closely
    rcon2 = api.JSLAB_PhaseEpipolarReconstructor_V2(ctx=ctx)
    rcon2.setCalibrationParams(params)
    rphase = api.decode_phase_f64(ctx, rdec.order, rdec.residual, True)
    rcon2.setData(lphase, rphase, lk, rdec.order, lmod, int(conf.freq[0]))
    xyz2, P2 = rcon2.startCalculate()
    agree = (P2 == P).float().mean().item()
    assert agree > 0.999, agree


@pytest.mark.gpu
def test_pair_errors_are_reported_not_thrown(ctx, oracle_lib):
    from zim_gb300 import api, _lib
    spec, L, R, _ = scene_data("config0")
    ctx.set_calibration(spec.rig.as_dict(), True)
    dcfg = api.decode_config(**spec.decode_kwargs())
    bad = torch.from_numpy(L[:, :100, :100].copy()).cuda()
    with pytest.raises(api.ZimError) as e:
        api.reconstruct_pair(ctx, dcfg, api.recon_config(), bad, bad)
    assert e.value.status == _lib.ERR_INVALID_ARG
    dz = api.decode_config(freq=(0, 1, 2))
    with pytest.raises(api.ZimError):
        api.decode(ctx, dz, torch.from_numpy(L).cuda())
