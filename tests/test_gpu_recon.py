"""Rectification, matching and reprojection parity against the FP64 oracle.

Each stage is fed the GPU's own previous-stage output, so the comparison
isolates that stage's arithmetic.  Tolerances:
* calibration products (R1, R2, P1, P2, Q): 1e-9 relative;
* rectification maps: equal within 1 float ulp, 1/32-pixel sample positions equal;
* rectified order: bit-exact; rectified phase: 2e-5 rad;
* match column: bit-exact except argmin ties / threshold costs within 1e-5 rad
  (counted); disparity: 2e-4 px (about 2 float ulps at 600 px);
* median: bit-exact; reprojected points: 1e-5 relative (the target is 1e-4);
  mask bit-exact except depth-gate decisions within 1e-5 relative (counted).
"""
import math

import numpy as np
import pytest
import torch

from conftest import SMALL_SCENES, scene_data

EPS = 1e-5


def setup(ctx, oracle, spec):
    rig = spec.rig.as_dict()
    ctx.set_calibration(rig, True)
    c = oracle.make_calib(rig["K"], rig["D"], rig["R"], rig["t"], rig["width"], rig["height"])
    return rig, oracle.rectification(c, True)


def decode_both(ctx, spec):
    from zim_gb300 import api
    cfg = api.decode_config(**spec.decode_kwargs())
    _, L, R, _ = scene_data(spec.name if spec.name != "ref_heterodyne" else "ref_heterodyne",
                            **({} if spec.name == "config0" else {"width": spec.rig.width, "height": spec.rig.height}))
    out = []
    for fr in (L, R):
        d = api.decode(ctx, cfg, torch.from_numpy(fr).cuda())
        out.append(d)
    return out


def f64_phase(base, res):
    return 2 * math.pi * base.cpu().numpy().astype(np.float64) + res.cpu().numpy().astype(np.float64)


@pytest.mark.gpu
@pytest.mark.parametrize("name,kw", SMALL_SCENES)
def test_calibration_and_maps(ctx, oracle_lib, name, kw):
    spec, *_ = scene_data(name, **kw)
    rig, (R1, R2, P1, P2, Q, w, h) = setup(ctx, oracle_lib, spec)
    assert (ctx.rect_w, ctx.rect_h) == (w, h)
    for a, b in ((ctx.R1, R1), (ctx.R2, R2), (ctx.P1, P1), (ctx.P2, P2), (ctx.Q, Q)):
        assert np.allclose(a, b, rtol=1e-9, atol=1e-9), (a, b)
    for cam, (Rk, Pk) in enumerate(((R1, P1), (R2, P2))):
        mx, my = ctx.rectify_maps(cam)
        ox, oy = oracle_lib.init_rectify_map(rig["K"][cam], rig["D"][cam], Rk, Pk, w, h)
        gx, gy = mx.cpu().numpy(), my.cpu().numpy()
        ulp = lambda a: np.spacing(np.abs(a).astype(np.float32))
        assert (np.abs(gx - ox) <= ulp(ox)).all() and (np.abs(gy - oy) <= ulp(oy)).all()
        qg = np.rint(gx * 32), np.rint(gy * 32)
        qo = np.rint(ox * 32), np.rint(oy * 32)
        assert np.array_equal(qg[0], qo[0]) and np.array_equal(qg[1], qo[1])


@pytest.mark.gpu
@pytest.mark.parametrize("name,kw", SMALL_SCENES)
def test_rectify_parity(ctx, oracle_lib, name, kw):
    from zim_gb300 import api
    spec, L, R, _ = scene_data(name, **kw)
    setup(ctx, oracle_lib, spec)
    cfg = api.decode_config(**spec.decode_kwargs())
    for cam, fr in enumerate((L, R)):
        d = api.decode(ctx, cfg, torch.from_numpy(fr).cuda())
        base, res, rord = api.rectify(ctx, cam, d["order"], d["residual"], True)
        mx, my = ctx.rectify_maps(cam)
        raw = f64_phase(d["order"], d["residual"])
        oph, ok = oracle_lib.rectify_decoded(raw, d["order"].cpu().numpy(), mx.cpu().numpy(), my.cpu().numpy(), True)
        assert np.array_equal(rord.cpu().numpy(), ok)
        err = np.abs(f64_phase(base, res) - oph)
        print(name, cam, "rectified phase max err", err.max())
        assert err.max() <= 2e-5
        # the residual stays small: base carries the integer cycles
        assert np.abs(res.cpu().numpy()).max() < 4 * math.pi


def rectified_pair(ctx, oracle, spec, L, R):
    from zim_gb300 import api
    setup(ctx, oracle, spec)
    cfg = api.decode_config(**spec.decode_kwargs())
    rects = []
    for cam, fr in enumerate((L, R)):
        d = api.decode(ctx, cfg, torch.from_numpy(fr).cuda())
        rects.append(api.rectify(ctx, cam, d["order"], d["residual"], True))
    return rects


@pytest.mark.gpu
@pytest.mark.parametrize("name,kw", SMALL_SCENES)
def test_match_parity(ctx, oracle_lib, name, kw):
    from zim_gb300 import api
    spec, L, R, _ = scene_data(name, **kw)
    rl, rr = rectified_pair(ctx, oracle_lib, spec, L, R)
    disp, best = api.match(ctx, rl, rr, spec.pha_f, 1.0)
    od, ob, near = oracle_lib.stereo_match(f64_phase(rl[0], rl[1]), f64_phase(rr[0], rr[1]), rl[2].cpu().numpy(),
                                           rr[2].cpu().numpy(), spec.pha_f, 1.0, eps=EPS)
    gb, gd = best.cpu().numpy(), disp.cpu().numpy()
    mis = gb != ob
    nearm = near != 0
    print(name, "match: valid", int((ob >= 0).sum()), "mismatch", int(mis.sum()), "near", int(nearm.sum()))
    assert (mis & ~nearm).sum() == 0
    assert mis.sum() <= 1e-4 * gb.size + 2
    same = ~mis & (ob >= 0)
    derr = np.abs(gd[same].astype(np.float64) - od[same])
    assert derr.max() <= 2e-4, derr.max()
    assert (gd[ob < 0] == 0).all() and (od[ob < 0] == 0).all()


@pytest.mark.gpu
@pytest.mark.parametrize("name,kw", SMALL_SCENES)
@pytest.mark.parametrize("rectified", [True, False])
def test_median_reproject_parity(ctx, oracle_lib, name, kw, rectified):
    from zim_gb300 import api
    spec, L, R, _ = scene_data(name, **kw)
    rl, rr = rectified_pair(ctx, oracle_lib, spec, L, R)
    disp, _ = api.match(ctx, rl, rr, spec.pha_f, 1.0, want_best=False)
    rc = api.recon_config(use_rectified_coords=int(rectified))
    dmed, xyz, mask = api.median_reproject(ctx, rc, disp)
    om = oracle_lib.median5(disp.cpu().numpy())
    assert np.array_equal(dmed.cpu().numpy(), om)
    oxyz, omask, near = oracle_lib.reproject(om, ctx.Q, ctx.R1, 0.0, 1000.0, rectified, eps=EPS)
    gm, gx = mask.cpu().numpy(), xyz.cpu().numpy()
    mis = gm != omask
    assert (mis & (near == 0)).sum() == 0
    both = (gm > 0) & (omask > 0)
    rel = np.abs(gx[both] - oxyz[both]) / np.maximum(1.0, np.abs(oxyz[both]))
    print(name, rectified, "reproject max rel err", rel.max(), "points", int(both.sum()))
    assert rel.max() <= 1e-5
    assert (gx[gm == 0] == 0).all()


def _rows_case(rows=64, cols=512, pha_f=16, seed=11):
    """Rectified phase rows that exercise both matching paths: rising spans
    (binary search), noisy spans that fall back to the scan, foreign orders
    inside spans, and plateaus of equal phase (ties)."""
    rng = np.random.default_rng(seed)
    c = np.arange(cols, dtype=np.float64)
    rph = np.zeros((rows, cols)); lph = np.zeros((rows, cols))
    for i in range(rows):
        off = rng.uniform(0.0, 1.0)
        r = off + 0.2 * c
        kind = i % 4
        if kind == 1:
            r = r + rng.uniform(-0.15, 0.15, cols)
        elif kind == 3:
            r = np.floor(r / 0.4) * 0.4 + off  # pairs of equal values
        disp = rng.uniform(5.0, 40.0)
        lph[i] = off + 0.2 * (c - disp) + rng.normal(0, 0.01, cols)
        rph[i] = r
    rk = np.clip(np.floor(rph / TWO_PI).astype(np.int32) + 1, 0, pha_f)
    lk = np.clip(np.floor(lph / TWO_PI).astype(np.int32) + 1, 0, pha_f)
    for i in range(2, rows, 4):  # foreign orders inside the spans
        j = rng.integers(0, cols, 12)
        rk[i, j] = rng.integers(1, pha_f + 1, 12)
    return lph, lk, rph, rk, pha_f


TWO_PI = 2 * math.pi


@pytest.mark.gpu
def test_match_fast_path_and_scan_agree_with_oracle(ctx, oracle_lib):
    from zim_gb300 import api
    lph, lk, rph, rk, pha_f = _rows_case()

    def split(ph, k):
        base = np.floor(ph / TWO_PI + 0.5).astype(np.int32)
        res = (ph - TWO_PI * base).astype(np.float32)
        f64 = TWO_PI * base.astype(np.float64) + res.astype(np.float64)
        return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (base, res, k.astype(np.int32))], f64

    L, lf = split(lph, lk)
    R, rf = split(rph, rk)
    disp, best = api.match(ctx, L, R, pha_f, 1.0)
    od, ob, near = oracle_lib.stereo_match(lf, rf, lk, rk, pha_f, 1.0, eps=EPS)
    gb, gd = best.cpu().numpy(), disp.cpu().numpy()
    ok = near == 0
    assert np.array_equal(gb[ok], ob[ok])
    # the sub-pixel step divides by 2 (c0 - c1)(c1 - c2): on the plateau rows
    # that product nearly vanishes and FP32 against FP64 differs there by more
    # than the tolerance, so disparities are compared where it is >= 1e-2
    m = ok & (ob >= 0)
    rr, cc = np.nonzero(m)
    b = ob[rr, cc]
    c0 = rf[rr, b - 1] - lf[rr, cc]
    c1 = rf[rr, b] - lf[rr, cc]
    c2 = rf[rr, b + 1] - lf[rr, cc]
    well = np.abs(2 * (c0 - c1) * (c1 - c2)) >= 1e-2
    assert well.mean() > 0.5
    assert np.abs(gd[rr, cc][well].astype(np.float64) - od[rr, cc][well]).max() <= 2e-4
    for kind in range(4):  # every row kind matches something
        assert (ob[kind::4] >= 0).mean() > 0.3, kind


@pytest.mark.gpu
@pytest.mark.parametrize("name,kw", SMALL_SCENES)
def test_rectify_match_equals_rectify_then_match(ctx, oracle_lib, name, kw):
    """zim_rectify_match (the whole-pair path's fused setData + stereoMatch)
    gives the disparity of zim_rectify on both cameras then zim_match, bit for
    bit, with and without the post-smooth."""
    from zim_gb300 import api
    spec, L, R, _ = scene_data(name, **kw)
    setup(ctx, oracle_lib, spec)
    cfg = api.decode_config(**spec.decode_kwargs())
    dl = api.decode(ctx, cfg, torch.from_numpy(L).cuda())
    dr = api.decode(ctx, cfg, torch.from_numpy(R).cuda())
    for smooth in (True, False):
        rl = api.rectify(ctx, 0, dl["order"], dl["residual"], smooth)
        rr = api.rectify(ctx, 1, dr["order"], dr["residual"], smooth)
        disp, _ = api.match(ctx, rl, rr, spec.pha_f, 1.0, want_best=False)
        fused = api.rectify_match(ctx, (dl["order"], dl["residual"]), (dr["order"], dr["residual"]), spec.pha_f,
                                  post_smooth=smooth)
        assert torch.equal(disp, fused), smooth
        assert (fused != 0).float().mean().item() > 0.3
