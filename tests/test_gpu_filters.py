"""Point-cloud filter parity (pixel Gaussian, ROR, MLS, SOR, metric Gaussian).

Every filter gets the same input cloud (the GPU's reprojected config-1-geometry
cloud) on both sides.  Tolerances: masks bit-exact except decisions within 1e-5
of their threshold (counted); smoothed points within POINT_TOL_MM plus 2 float
ulps of the coordinate (an absolute 1e-5 mm cannot be represented at 900 mm,
where one float ulp is 6.1e-5 mm).
"""
import numpy as np
import pytest
import torch

from conftest import scene_data

EPS = 1e-5
POINT_TOL_MM = 1e-5


def cloud(ctx, oracle, name="config1", width=612, height=512):
    from zim_gb300 import api
    spec, L, R, _ = scene_data(name, width=width, height=height)
    rig = spec.rig.as_dict()
    ctx.set_calibration(rig, True)
    cfg = api.decode_config(**spec.decode_kwargs())
    rects = []
    for cam, fr in enumerate((L, R)):
        d = api.decode(ctx, cfg, torch.from_numpy(fr).cuda())
        rects.append(api.rectify(ctx, cam, d["order"], d["residual"], True))
    disp, _ = api.match(ctx, rects[0], rects[1], spec.pha_f, 1.0, want_best=False)
    _, xyz, mask = api.median_reproject(ctx, api.recon_config(), disp)
    return xyz, mask


def point_tol(ref, iterations=1):
    """Per-point tolerance (N, 1): POINT_TOL_MM plus 2 float ulps of the
    point's largest coordinate per pass (a pass feeds FP32-rounded points into
    the next, so one ulp at 900 mm can move every coordinate of the next pass)."""
    big = np.abs(ref).max(axis=-1, keepdims=True).astype(np.float32)
    return POINT_TOL_MM + 2 * iterations * np.spacing(big)


def report(tag, got, ref, sel):
    err = np.abs(got[sel].astype(np.float64) - ref[sel].astype(np.float64))
    print(tag, "points", int(sel.sum()), "max err mm", float(err.max()) if err.size else 0.0,
          "rms", float(np.sqrt((err ** 2).mean())) if err.size else 0.0)
    return err


@pytest.mark.gpu
@pytest.mark.parametrize("update_mask", [False, True])
def test_px_gaussian_parity(ctx, oracle_lib, update_mask):
    from zim_gb300 import api
    xyz, mask = cloud(ctx, oracle_lib)
    out, mo = api.filter_px_gaussian(ctx, xyz, mask, update_mask)
    ox, om, near = oracle_lib.px_gaussian(xyz.cpu().numpy(), mask.cpu().numpy(), update_mask, eps=EPS)
    g, gm = out.cpu().numpy(), mo.cpu().numpy()
    assert ((gm != om) & (near == 0)).sum() == 0
    sel = (near == 0)
    err = report("px_gaussian", g, ox, sel)
    assert (err <= point_tol(ox[sel])).all()


@pytest.mark.gpu
def test_ror_parity(ctx, oracle_lib):
    from zim_gb300 import api
    xyz, mask = cloud(ctx, oracle_lib)
    for (r, mn, win) in ((5.0, 10, 10), (3.0, 5, 5), (8.0, 30, 15)):
        out, mo = api.filter_ror(ctx, xyz, mask, r, mn, win)
        ox, om, near = oracle_lib.ror(xyz.cpu().numpy(), mask.cpu().numpy(), r, mn, win, eps=EPS)
        gm = mo.cpu().numpy()
        mis = gm != om
        print("ror", r, mn, win, "kept", int(om.sum()), "mismatch", int(mis.sum()), "near", int(near.sum()))
        assert (mis & (near == 0)).sum() == 0
        assert 0.5 * mask.sum().item() < om.sum()
        assert np.array_equal(out.cpu().numpy()[~mis], ox[~mis])


@pytest.mark.gpu
# The test scene is 612 px wide (1.5 mm pixel spacing, 4x the 5 MP scene's), so
# the 5 MP settings (radius 2 mm, sigma 2/sqrt(2)) are scaled by 4 here.
# flag_max: the flagged fraction measured on this cloud by the oracle alone
# (2.50 %, 0.26 %, 0.22 %) plus a margin.
@pytest.mark.parametrize("order,window,sigma,radius,iters,flag_max", [(2, 7, 5.656854, 8.0, 1, 0.030),
                                                                        (1, 7, 5.656854, 8.0, 1, 0.030),
                                                                        (0, 7, 5.656854, 8.0, 2, 0.030),
                                                                        (1, 5, 2.4, 0.0, 2, 0.004),
                                                                        (0, 4, 2.0, 0.0, 1, 0.0035)])
def test_mls_parity(ctx, oracle_lib, order, window, sigma, radius, iters, flag_max):
    """Points the oracle flags (a neighbour within 1e-6 of the cut-off, or a
    frame / normal-equation conditioning at which FP32 rounding alone moves the
    result by more than 1e-5 mm) are counted and bounded by flag_max; all
    others must agree."""
    from zim_gb300 import api
    xyz, mask = cloud(ctx, oracle_lib)
    out = api.filter_mls(ctx, xyz, mask, window, sigma, order, radius, iters)
    ox, near = oracle_lib.mls(xyz.cpu().numpy(), mask.cpu().numpy(), window, sigma, order, radius, iters, eps=EPS)
    g = out.cpu().numpy()
    m = mask.cpu().numpy() > 0
    sel = m & (near == 0)
    err = report(f"mls o{order} w{window}", g, ox, sel)
    tol = point_tol(ox[sel], iters)
    bad = (err > tol).any(axis=1)
    allerr = np.abs(g[m].astype(np.float64) - ox[m]).max(axis=1)
    print("  flagged:", int((m & (near > 0)).sum()), "of", int(m.sum()), " beyond tolerance:", int(bad.sum()),
          " all-points max/rms err mm:", float(allerr.max()), float(np.sqrt((allerr ** 2).mean())))
    assert bad.sum() == 0
    assert (m & (near > 0)).sum() <= flag_max * m.sum()
    assert np.array_equal(g[~m], xyz.cpu().numpy()[~m])


@pytest.mark.gpu
@pytest.mark.parametrize("k", [30, 50])
def test_sor_parity(ctx, oracle_lib, k):
    from zim_gb300 import api
    xyz, mask = cloud(ctx, oracle_lib)
    mo, md = api.filter_sor(ctx, xyz, mask, k, 1.0, want_mean_dist=True)
    om, omd, thr, near = oracle_lib.sor(xyz.cpu().numpy(), mask.cpu().numpy(), k, 1.0, eps=EPS)
    gm, gmd = mo.cpu().numpy(), md.cpu().numpy()
    m = mask.cpu().numpy() > 0
    rel = np.abs(gmd[m] - omd[m]) / np.maximum(omd[m], 1e-6)
    mis = gm != om
    print("sor k", k, "threshold", thr, "kept", int(om.sum()), "of", int(m.sum()), "mismatch", int(mis.sum()),
          "mean-dist max rel err", float(rel.max()))
    assert rel.max() <= 1e-5
    assert (mis & (near == 0)).sum() == 0
    assert ctx.check_device() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("k", [30, 50])
def test_sor_window_path_equals_grid_path(ctx, oracle_lib, k):
    """The window fast path (certified by the ray bound) gives the same bits as
    the grid search: the same cloud padded by one invalid column has no pixel
    rays (its size is not the calibrated one), so every query takes the grid."""
    from zim_gb300 import api
    xyz, mask = cloud(ctx, oracle_lib)
    H, W = mask.shape
    xp = torch.zeros((H, W + 1, 3), dtype=torch.float32, device="cuda")
    mp = torch.zeros((H, W + 1), dtype=torch.uint8, device="cuda")
    xp[:, :W] = xyz
    mp[:, :W] = mask
    m1, md1 = api.filter_sor(ctx, xyz, mask, k, 1.0, want_mean_dist=True)
    s1 = api.sor_stats(ctx)
    m2, md2 = api.filter_sor(ctx, xp.contiguous(), mp.contiguous(), k, 1.0, want_mean_dist=True)
    s2 = api.sor_stats(ctx)
    assert torch.equal(md1, md2[:, :W].contiguous()) and torch.equal(m1, m2[:, :W].contiguous())
    assert s1["threshold"] == s2["threshold"]
    print("sor k", k, "far searches: window path", s1["n_far_search"], "grid path", s2["n_far_search"])


@pytest.mark.gpu
@pytest.mark.parametrize("k", [30, 63])
def test_sor_isolated_and_duplicate_points(ctx, oracle_lib, k):
    """Far-isolated points (their k + 1 nearest lie hundreds of mm away: the
    CTA-per-query coarse search) and a pile of 150 identical points (ties at
    distance 0 beyond any list's room) against the oracle, on both search
    paths."""
    from zim_gb300 import api
    xyz, mask = cloud(ctx, oracle_lib)
    H, W = mask.shape
    x = xyz.cpu().numpy().copy()
    m = mask.cpu().numpy().copy()
    rng = np.random.default_rng(7)
    idx = np.flatnonzero(m.reshape(-1))
    pick = rng.choice(idx, 190, replace=False)
    flat = x.reshape(-1, 3)
    # 40 outliers pushed 150-600 mm along random directions
    d = rng.normal(size=(40, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    flat[pick[:40]] += (d * rng.uniform(150, 600, (40, 1))).astype(np.float32)
    # 150 copies of one surface point
    flat[pick[40:]] = flat[pick[40]]
    xt = torch.from_numpy(x).cuda()
    mt = torch.from_numpy(m).cuda()
    mo, md = api.filter_sor(ctx, xt, mt, k, 1.0, want_mean_dist=True)
    om, omd, thr, near = oracle_lib.sor(x, m, k, 1.0, eps=EPS)
    gmd = md.cpu().numpy()
    v = m > 0
    rel = np.abs(gmd[v] - omd[v]) / np.maximum(omd[v], 1e-6)
    assert rel.max() <= 1e-5, float(rel.max())
    assert (gmd.reshape(-1)[pick[40:]] == 0).all()
    assert ((mo.cpu().numpy() != om) & (near == 0)).sum() == 0
    assert ctx.check_device() == 0
    # the grid-only path (no pixel rays) gives the same bits
    xp = torch.zeros((H, W + 1, 3), dtype=torch.float32, device="cuda")
    mp = torch.zeros((H, W + 1), dtype=torch.uint8, device="cuda")
    xp[:, :W] = xt
    mp[:, :W] = mt
    m2, md2 = api.filter_sor(ctx, xp.contiguous(), mp.contiguous(), k, 1.0, want_mean_dist=True)
    assert torch.equal(md, md2[:, :W].contiguous()) and torch.equal(mo, m2[:, :W].contiguous())
    assert ctx.check_device() == 0


@pytest.mark.gpu
def test_mls_ray_disk_equals_full_window(ctx, oracle_lib):
    """The ray bound only skips window pixels beyond the cut-off: with pixel
    rays (the calibrated size) and without (the cloud padded by one invalid
    column) the MLS output is bit-identical."""
    import math
    from zim_gb300 import api
    xyz, mask = cloud(ctx, oracle_lib)
    H, W = mask.shape
    xp = torch.zeros((H, W + 1, 3), dtype=torch.float32, device="cuda")
    mp = torch.zeros((H, W + 1), dtype=torch.uint8, device="cuda")
    xp[:, :W] = xyz
    mp[:, :W] = mask
    args = (7, 2.0 / math.sqrt(2.0), 2, 2.0, 2)
    a = api.filter_mls(ctx, xyz, mask, *args)
    b = api.filter_mls(ctx, xp.contiguous(), mp.contiguous(), *args)[:, :W].contiguous()
    assert torch.equal(a, b)


@pytest.mark.gpu
def test_metric_gaussian_window_path_matches_grid_path(ctx, oracle_lib):
    """Window-certified points against the grid path (the padded cloud has no
    pixel rays): the same neighbours, summed in another order, so equal to a
    few float ulps."""
    from zim_gb300 import api
    xyz, mask = cloud(ctx, oracle_lib)
    H, W = mask.shape
    xp = torch.zeros((H, W + 1, 3), dtype=torch.float32, device="cuda")
    mp = torch.zeros((H, W + 1), dtype=torch.uint8, device="cuda")
    xp[:, :W] = xyz
    mp[:, :W] = mask
    a = api.filter_metric_gaussian(ctx, xyz, mask, 0.5).cpu().numpy()
    b = api.filter_metric_gaussian(ctx, xp.contiguous(), mp.contiguous(), 0.5)[:, :W].cpu().numpy()
    m = mask.cpu().numpy() > 0
    assert np.array_equal(a[~m], b[~m])
    err = np.abs(a[m].astype(np.float64) - b[m]).max(axis=1)
    scale = np.abs(b[m]).max(axis=1)
    assert (err <= 4 * np.spacing(scale.astype(np.float32))).all(), float(err.max())


@pytest.mark.gpu
def test_metric_gaussian_pending_queries_take_the_grid(ctx, oracle_lib):
    """Points moved 30 mm off their pixel rays make the ray bound useless for
    every query, so with pixel rays the window pass leaves them all to the
    grid (built on demand): the same bits as the grid-only path (the cloud
    padded by an invalid column has no rays), and the oracle's values."""
    from zim_gb300 import api
    xyz, mask = cloud(ctx, oracle_lib)
    H, W = mask.shape
    x = xyz.cpu().numpy().copy()
    m = mask.cpu().numpy()
    idx = np.flatnonzero(m.reshape(-1))[::9973][:20]
    x.reshape(-1, 3)[idx, 0] += 30.0
    xt = torch.from_numpy(x).cuda()
    out = api.filter_metric_gaussian(ctx, xt, mask, 0.5)
    xp = torch.zeros((H, W + 1, 3), dtype=torch.float32, device="cuda")
    mp = torch.zeros((H, W + 1), dtype=torch.uint8, device="cuda")
    xp[:, :W] = xt
    mp[:, :W] = mask
    out2 = api.filter_metric_gaussian(ctx, xp.contiguous(), mp.contiguous(), 0.5)
    assert torch.equal(out, out2[:, :W].contiguous())
    ox, near = oracle_lib.metric_gaussian(x, m, 0.5, eps=EPS)
    g = out.cpu().numpy()
    sel = (m > 0) & (near == 0)
    err = report("metric_gaussian pending", g, ox, sel)
    assert ((err > point_tol(ox[sel])).any(axis=1)).mean() <= 1e-3
    assert ctx.check_device() == 0


@pytest.mark.gpu
def test_metric_gaussian_parity(ctx, oracle_lib):
    from zim_gb300 import api
    xyz, mask = cloud(ctx, oracle_lib)
    out = api.filter_metric_gaussian(ctx, xyz, mask, 0.5)
    ox, near = oracle_lib.metric_gaussian(xyz.cpu().numpy(), mask.cpu().numpy(), 0.5, eps=EPS)
    g = out.cpu().numpy()
    m = mask.cpu().numpy() > 0
    sel = m & (near == 0)
    err = report("metric_gaussian", g, ox, sel)
    bad = (err > point_tol(ox[sel])).any(axis=1)
    assert bad.mean() <= 1e-3
    assert np.array_equal(g[~m], xyz.cpu().numpy()[~m])


@pytest.mark.gpu
def test_compact_points_layout(ctx, oracle_lib):
    from zim_gb300 import api
    xyz, mask = cloud(ctx, oracle_lib)
    pts = api.compact_points(ctx, xyz, mask).cpu().numpy()
    m = mask.cpu().numpy() > 0
    ref = xyz.cpu().numpy()[m]
    assert pts.shape == (int(m.sum()), 4)
    assert np.array_equal(pts[:, :3], ref)
