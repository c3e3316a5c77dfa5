"""The CUDA path against the committed golden fixtures (tests/golden/), with
the decode and matching tolerances of the stage tests: orders and validity
exact except pixels the oracle flagged near a decision, phase within 1e-5 rad,
match columns exact except flagged near ties/thresholds, disparity 2e-4 px;
polynomial reprojection bit-exact is covered by test_gpu_poly.py."""
import json
import math
from pathlib import Path

import numpy as np
import pytest
import torch

GOLDEN = Path(__file__).resolve().parent / "golden"
DECODES = sorted(p.name for p in GOLDEN.glob("decode_*.npz"))
TWO_PI = 2 * math.pi


@pytest.mark.gpu
@pytest.mark.parametrize("name", DECODES)
def test_decode_matches_fixture(ctx, name):
    from zim_gb300 import api
    d = np.load(GOLDEN / name)
    kw = json.loads(str(d["cfg"]))
    g = api.decode(ctx, api.decode_config(**kw), torch.from_numpy(d["frames"]).cuda())
    order, res, valid = (g[k].cpu().numpy() for k in ("order", "residual", "valid"))
    near = d["near"] > 0
    ok = ~near
    assert np.array_equal(valid[ok], d["valid"][ok])
    both = ok & (valid > 0) & (d["valid"] > 0)
    assert np.array_equal(order[both], d["order"][both])
    phase = TWO_PI * order.astype(np.float64) + res.astype(np.float64)
    assert np.abs(phase[both] - d["phase"][both]).max() <= 1e-5
    assert both.mean() > 0.5


@pytest.mark.gpu
def test_match_matches_fixture(ctx):
    from zim_gb300 import api
    d = np.load(GOLDEN / "match_config0_rows.npz")

    def split(ph, k):
        base = np.floor(ph / TWO_PI + 0.5).astype(np.int32)
        res = (ph - TWO_PI * base).astype(np.float32)
        return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (base, res, k.astype(np.int32))]

    disp, best = api.match(ctx, split(d["lph"], d["lk"]), split(d["rph"], d["rk"]), int(d["pha_f"]))
    disp, best = disp.cpu().numpy(), best.cpu().numpy()
    ok = d["near"] == 0
    assert np.array_equal(best[ok], d["best"][ok])
    m = ok & (d["best"] >= 0)
    assert np.abs(disp[m] - d["disp"][m]).max() <= 2e-4


def _rig(d):
    rig = json.loads(str(d["rig"]))
    for k in ("K", "D"):
        rig[k] = [np.asarray(v, np.float64) for v in rig[k]]
    for k in ("R", "t"):
        rig[k] = np.asarray(rig[k], np.float64)
    return rig


def _dilate(m, r):
    out = m.copy()
    for dy in range(-r, r + 1):
        for dx in range(-r, r + 1):
            out |= np.roll(np.roll(m, dy, 0), dx, 1)
    return out


@pytest.mark.gpu
def test_pair_matches_reference_fixture(ctx, oracle_lib):
    """The whole pair against the REFERENCE's own outputs (its decoder and
    startCalculate compiled from its sources, tests/golden/make_golden.py):
    median disparity within 2e-4 px and the reprojected mask identical except
    within the median window of a match the oracle flags as a near tie; points
    within 1e-5 relative; after the pixel Gaussian and radius outlier filter,
    the mask identical except where a flagged match or a radius decision
    within 1e-5 of the radius reaches, and points within 1e-5 mm + 2 ulps."""
    from zim_gb300 import api
    d = np.load(GOLDEN / "recon_ref_pair.npz")
    assert str(d["source"]) == "reference"
    ctx.set_calibration(_rig(d), True)
    assert (ctx.rect_h, ctx.rect_w) == d["mask"].shape
    dcfg = api.decode_config(**json.loads(str(d["decode_cfg"])))
    rects = []
    for cam, fr in enumerate((d["left"], d["right"])):
        g = api.decode(ctx, dcfg, torch.from_numpy(fr).cuda())
        rects.append(api.rectify(ctx, cam, g["order"], g["residual"], True))
    disp, _ = api.match(ctx, rects[0], rects[1], int(d["pha_f"]), 1.0, want_best=False)
    dmed, xyz, mask = api.median_reproject(ctx, api.recon_config(), disp)
    gd, gm, gx = dmed.cpu().numpy(), mask.cpu().numpy(), xyz.cpu().numpy()
    flagged = _dilate(d["match_near"] > 0, 2)
    ok = ~flagged
    assert np.abs(gd[ok].astype(np.float64) - d["disp"][ok]).max() <= 2e-4
    assert np.array_equal(gm[ok], d["raw_mask"][ok])
    both = (gm > 0) & (d["raw_mask"] > 0)
    rel = np.abs(gx[both] - d["raw_xyz"][both]) / np.maximum(1.0, np.abs(d["raw_xyz"][both]))
    assert rel.max() <= 1e-5
    cfg = json.loads(str(d["recon_cfg"]))
    prm = (cfg["radius_search"], cfg["radius_min_neighbors"], cfg["radius_window_size"])
    gg, _ = api.filter_px_gaussian(ctx, xyz, mask, False)
    fx, fm = api.filter_ror(ctx, gg, mask, *prm)
    _, _, rnear = oracle_lib.ror(gg.cpu().numpy(), gm, *prm, eps=1e-5)
    reach = _dilate(flagged, 1 + prm[2] // 2) | (rnear > 0)
    fm, fx = fm.cpu().numpy(), fx.cpu().numpy()
    print("pair vs reference: points", int(d["mask"].sum()), "flagged", int(reach.sum()))
    assert np.array_equal(fm[~reach], d["mask"][~reach])
    sel = ~reach & (fm > 0)
    big = np.abs(d["xyz"][sel]).max(axis=-1, keepdims=True).astype(np.float32)
    assert (np.abs(fx[sel] - d["xyz"][sel]) <= 1e-5 + 2 * np.spacing(big)).all()
    assert sel.sum() > 0.9 * d["mask"].sum()


@pytest.mark.gpu
@pytest.mark.parametrize("run", ["w7_s1.414_o2_r2", "w7_s2.83_o1_r4"])
def test_mls_matches_reference_fixture(ctx, run):
    """MLS against the reference's MLS source evaluated in double
    (oracle/ref_mls_f64.cpp): points the oracle flags (a neighbour at the
    cut-off, or an ill-conditioned frame) are counted, the rest agree within
    1e-5 mm + 2 float ulps."""
    from zim_gb300 import api
    d = np.load(GOLDEN / "mls_ref_cloud.npz")
    w, s, o, r, it = json.loads(str(d["runs"]))[run]
    out = api.filter_mls(ctx, torch.from_numpy(d["xyz"]).cuda(), torch.from_numpy(d["mask"]).cuda(), w, s, o, r, it)
    g, ref = out.cpu().numpy(), d[f"ref_f64_{run}"]
    m = d["mask"] > 0
    sel = m & (d[f"near_{run}"] == 0)
    big = np.abs(ref[sel]).max(axis=-1, keepdims=True).astype(np.float32)
    err = np.abs(g[sel].astype(np.float64) - ref[sel])
    print(run, "points", int(m.sum()), "flagged", int((m & ~sel).sum()), "max err mm", float(err.max()))
    assert (err <= 1e-5 + 2 * np.spacing(big)).all()
    assert (m & ~sel).sum() <= 0.01 * m.sum()
