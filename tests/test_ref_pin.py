"""The oracle pinned to the reference itself.

oracle/_ref/libzim_ref.so is the reference's own decoder V2, reconstructor V2
and CPU MLS, compiled from its sources (oracle/ref_build.py) against a small
OpenCV stand-in whose image primitives are the oracle's restatements.  These
tests run both on the same seeded inputs and require:

* decode (heterodyne 121/110/120 and 107/100/94, option variants): phase
  before and after the post-smooth, fringe order, modulation and validity
  bit-identical; HDR (the reference's cached pseudo-inverses against the
  oracle's per-pixel normal equations) within 1e-9 rad;
* calibration: R1, Q, rectified size and both rectification maps identical;
* setData + startCalculate: the rectified maps, the disparity (stereoMatch +
  5x5 median) and the reprojected cloud identical, for the reference defaults
  and variants; its pixel Gaussian + radius outlier filter identical when the
  oracle's filter is fed the reference's Gaussian output (the Gaussian itself
  is compared to float rounding below); stereoMatch alone identical;
* startCalculate_v2 (per-pixel polynomial reprojection): identical;
* pixel Gaussian: the same output support, values within 4 float ulps (the
  reference sums in float, the oracle in double); radius outlier filter
  identical;
* MLS: the reference source evaluated in double (oracle/ref_mls_f64.cpp)
  within one float ulp of the oracle for orders 0/1/2 (two passes of
  rounding in between with 3 iterations: 4 ulps); the reference's FP32 build
  is reported against it (its own rounding).

Skipped where the reference sources are not present (they are needed to build
the library)."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from oracle import pipeline as P
from oracle import ref as Z


@pytest.fixture(scope="module")
def ref():
    if not Z.available():
        pytest.skip("reference sources not available to build oracle/_ref")
    O.build()
    return Z


def _scene(**kw):
    from zim_gb300 import synth
    return synth.ref_heterodyne(**kw)


def test_factory_rejects_a_zero_frequency(ref):
    frames = np.zeros((24, 8, 8), np.uint8)
    with pytest.raises(ValueError):
        ref.decode(ref.decode_cfg(freq=(121, 0, 120)), frames)


DECODE_CASES = {
    "121_110_120": dict(seed=2, freq=(121, 110, 120), steps=8),
    "107_100_94": dict(seed=4, freq=(107, 100, 94), steps=8),  # f1 > f2: the other phase23 branch
    "4step": dict(seed=5, freq=(121, 110, 120), steps=4),
}
DECODE_OPTIONS = {
    "defaults": {},
    "uphase1_only": dict(avg_three_phase=False),
    "no_post_smooth": dict(post_smooth=False),
    "preblur_sigma0": dict(preblur_sigma=0.0),
    "threshold_0.5": dict(modulation_threshold=0.5),
}


# every scene with the defaults, every option on the first scene
DECODE_RUNS = [(c, "defaults") for c in sorted(DECODE_CASES)] + \
    [("121_110_120", o) for o in sorted(DECODE_OPTIONS) if o != "defaults"]


@pytest.mark.parametrize("case,opt", DECODE_RUNS)
def test_decode_bit_identical(ref, case, opt):
    spec = _scene(width=640, height=512, **DECODE_CASES[case])
    frames = spec.render(0)
    kw = dict(spec.decode_kwargs(), **DECODE_OPTIONS[opt])
    ph, raw, k, mod, valid = ref.decode(ref.decode_cfg(**kw), frames)
    oph, ok, omod, ov, _ = O.decode(O.make_decode_cfg(**kw), frames)
    assert np.array_equal(raw, oph)
    assert np.array_equal(k, ok)
    assert np.array_equal(mod, omod)
    assert np.array_equal(valid, ov)
    smoothed = O.post_smooth(oph) if kw.get("post_smooth", True) else oph
    assert np.array_equal(ph, smoothed)
    assert valid.mean() > 0.5


def test_decode_hdr_within_round_off(ref):
    spec = _scene(seed=21, width=320, height=256)
    spec.A, spec.B = (170.0, 220.0), (80.0, 120.0)  # 8-bit peaks clip
    frames = spec.render(0)
    kw = dict(spec.decode_kwargs(), enable_hdr=True, hdr_saturation_gray=255.0, hdr_min_amplitude=2.0)
    ph, raw, k, mod, valid = ref.decode(ref.decode_cfg(**kw), frames)
    oph, ok, omod, ov, near = O.decode(O.make_decode_cfg(**kw), frames)
    assert np.array_equal(valid, ov)
    assert np.array_equal(k, ok)  # -1 where invalid, as the reference's HDR mode
    assert np.abs(raw - oph).max() < 1e-9
    assert np.abs(mod - omod).max() < 1e-12
    assert np.abs(ph - O.post_smooth_hdr(oph, ov)).max() < 1e-9
    assert (frames >= 255).any() and valid.mean() > 0.5


RIGS = {"config1_distorted": dict(seed=2, width=640, height=512)}


@pytest.mark.parametrize("full_left", [True, False])
def test_rectification_identical(ref, full_left):
    spec = _scene(**RIGS["config1_distorted"])
    rig = spec.rig.as_dict()
    rec = ref.Reconstructor(ref.recon_cfg(use_full_left_rectification=full_left), rig)
    R1, Q, lm, rm = rec.rectification()
    r = P.Rectification(rig, full_left)
    assert (rec.w, rec.h) == (r.w, r.h)
    assert np.array_equal(R1, r.R1) and np.array_equal(Q, r.Q)
    for a, b in zip(lm + rm, r.maps[0] + r.maps[1]):
        assert np.array_equal(a, b)


def _decoded_pair(ref, spec):
    kw = spec.decode_kwargs()
    return [ref.decode(ref.decode_cfg(**kw), spec.render(cam)) for cam in (0, 1)]


RECON_VARIANTS = {
    "reference_defaults": dict(),
    "ror_2mm_8_of_7x7": dict(radius_search=2.0, radius_min_neighbors=8, radius_window_size=7),
    "camera_coords": dict(use_rectified_coords=False, radius_search=2.0, radius_min_neighbors=8, radius_window_size=7),
    "no_median": dict(use_disp_median_filter=False, radius_search=2.0, radius_min_neighbors=8, radius_window_size=7),
}


@pytest.mark.parametrize("variant", sorted(RECON_VARIANTS))
def test_reconstruct_identical(ref, variant):
    spec = _scene(**RIGS["config1_distorted"])
    rig = spec.rig.as_dict()
    v = RECON_VARIANTS[variant]
    rec = ref.Reconstructor(ref.recon_cfg(**v), rig)
    (lph, _, lk, lmod, _), (rph, _, rk, _, _) = _decoded_pair(ref, spec)
    xyz, mask, disp, rmaps, (raw_xyz, raw_mask) = rec.run(lph, rph, lk, rk, lmod, spec.pha_f)

    rect = P.Rectification(rig, True)
    f = P.Filters(use_median=v.get("use_disp_median_filter", True), use_px_gaussian=True, use_ror=True,
                  ror=(v.get("radius_search", 0.7), v.get("radius_min_neighbors", 10), v.get("radius_window_size", 10)))
    cfg = O.make_decode_cfg(**spec.decode_kwargs())
    r = []
    for cam in (0, 1):
        ph, k, _, _, _ = O.decode(cfg, spec.render(cam))
        r.append(O.rectify_decoded(ph, k, *rect.maps[cam], True))
    assert np.array_equal(rmaps[0], r[0][0]) and np.array_equal(rmaps[1], r[1][0])
    assert np.array_equal(rmaps[2], r[0][1]) and np.array_equal(rmaps[3], r[1][1])
    od, _, _ = O.stereo_match(r[0][0], r[1][0], r[0][1], r[1][1], spec.pha_f)
    dm = O.median5(od.astype(np.float32)) if f.use_median else od
    assert np.array_equal(disp, dm.astype(np.float64) if f.use_median else od)
    use_rect = v.get("use_rectified_coords", True)
    oxyz, omask, _ = O.reproject(dm.astype(np.float32), rect.Q, rect.R1, 0.0, 1000.0, use_rect)
    assert np.array_equal(raw_mask, omask)
    if f.use_median:
        assert np.array_equal(raw_xyz, oxyz)
    else:
        # Without the median the reference's CPU path reprojects its FP64
        # disparity; the oracle (like the reference's GPU path and this
        # library) reprojects the FP32 one: points agree to that rounding.
        rel = np.abs(raw_xyz.astype(np.float64) - oxyz) / np.maximum(np.abs(oxyz).max(-1, keepdims=True), 1.0)
        assert rel.max() < 1e-6
        oxyz = raw_xyz
    # the filters: the reference's float Gaussian, then the oracle's radius filter on it
    g = ref.px_gaussian(oxyz, omask)
    fx, fm, near = O.ror(g, omask, *f.ror)
    ok = near == 0  # a neighbour distance within 1e-6 relative of the radius: the decision may go either way
    assert near.sum() <= 5
    assert np.array_equal(mask[ok], fm[ok]) and np.array_equal(xyz[ok], fx[ok])
    if variant != "reference_defaults":
        assert mask.sum() > 10000


def test_stereo_match_identical(ref):
    spec = _scene(seed=3, width=480, height=384)
    rect = P.Rectification(spec.rig.as_dict(), True)
    cfg = O.make_decode_cfg(**spec.decode_kwargs())
    r = []
    for cam in (0, 1):
        ph, k, _, _, _ = O.decode(cfg, spec.render(cam))
        r.append(O.rectify_decoded(ph, k, *rect.maps[cam], True))
    for thr in (1.0, 0.05):
        od, ob, _ = O.stereo_match(r[0][0], r[1][0], r[0][1], r[1][1], spec.pha_f, thr)
        zd = ref.stereo_match(r[0][0], r[1][0], r[0][1], r[1][1], spec.pha_f, thr)
        assert np.array_equal(od, zd)
        assert (ob >= 0).mean() > (0.3 if thr == 1.0 else 0.05)


def test_startcalculate_v2_identical(ref):
    from polycase import q_maps
    spec = _scene(seed=6, width=480, height=384)
    rig = spec.rig.as_dict()
    rect = P.Rectification(rig, True)
    maps = q_maps(rect.Q, rect.h, rect.w, "inv")
    rec = ref.Reconstructor(ref.recon_cfg(radius_search=2.5, radius_min_neighbors=8, radius_window_size=7), rig,
                            poly=maps)
    (lph, _, lk, lmod, _), (rph, _, rk, _, _) = _decoded_pair(ref, spec)
    xyz, mask, _, _, (raw_xyz, raw_mask) = rec.run(lph, rph, lk, rk, lmod, spec.pha_f, v2=True)
    oxyz, omask = P.run_pair(spec.decode_kwargs(), spec.pha_f, spec.render(0), spec.render(1), rect, P.Filters(),
                             poly=maps)
    assert np.array_equal(raw_mask, omask) and np.array_equal(raw_xyz, oxyz)
    fx, fm, _ = O.ror(ref.px_gaussian(oxyz, omask), omask, 2.5, 8, 7)
    assert np.array_equal(mask, fm) and np.array_equal(xyz, fx)
    assert mask.sum() > 5000


@pytest.fixture(scope="module")
def cloud(ref):
    from zim_gb300 import synth
    spec = synth.config1(1, 612, 512)
    rect = P.Rectification(spec.rig.as_dict(), True)
    return P.run_pair(spec.decode_kwargs(), spec.pha_f, spec.render(0), spec.render(1), rect, P.Filters())


def _ulps(x):
    return np.spacing(np.abs(x).max(axis=-1).astype(np.float32)).astype(np.float64)


def test_px_gaussian_within_float_rounding(ref, cloud):
    xyz, mask = cloud
    zg = ref.px_gaussian(xyz, mask)
    og, _, near = O.px_gaussian(xyz, mask)
    ok = near == 0
    assert np.array_equal((zg != 0).any(-1)[ok], (og != 0).any(-1)[ok])
    d = np.abs(zg.astype(np.float64) - og).max(axis=-1)
    assert (d[ok] <= 4 * _ulps(og)[ok]).all()
    assert (og != 0).any(-1).sum() > 100000


@pytest.mark.parametrize("prm", [(0.7, 10, 10), (2.0, 8, 7), (1.2, 3, 5)])
def test_ror_identical(ref, cloud, prm):
    xyz, mask = cloud
    zx, zp = ref.ror(xyz, mask, *prm)
    ox, op, near = O.ror(xyz, mask, *prm)
    assert near.sum() == 0
    assert np.array_equal(zp, op) and np.array_equal(zx, ox)


MLS_CASES = {  # window, sigma, order, max_radius, iterations
    "o2_r8": (7, 4 * 2 / math.sqrt(2), 2, 8.0, 1),
    "o1_r8": (7, 4 * 2 / math.sqrt(2), 1, 8.0, 1),
    "o0_r8": (7, 4 * 2 / math.sqrt(2), 0, 8.0, 1),
    "o2_r2": (7, 2 / math.sqrt(2), 2, 2.0, 1),
    "o2_auto_3it": (5, 2.0, 2, 0.0, 3),
}


@pytest.mark.parametrize("case", sorted(MLS_CASES))
def test_mls_pinned_to_reference_source(ref, cloud, case):
    xyz, mask = cloud
    w, s, o, r, it = MLS_CASES[case]
    z64 = ref.mls_f64(xyz, mask, w, s, o, r, it)
    oo, _ = O.mls(xyz, mask, w, s, o, r, it)
    m = mask > 0
    d = np.abs(z64.astype(np.float64) - oo).max(axis=-1)[m]
    tol = (1.0 if it == 1 else 4.0) * _ulps(oo)[m]
    assert (d <= tol).all(), (d / _ulps(oo)[m]).max()
    # the reference's own FP32 arithmetic: most points agree to a few um, a
    # few carry its float accumulation of absolute coordinates
    z32 = ref.mls(xyz, mask, w, s, o, r, it)
    d32 = np.abs(z32.astype(np.float64) - oo).max(axis=-1)[m]
    assert np.quantile(d32, 0.99) < 2e-3


def test_polynomial_point_model_identical(ref):
    """evaluateV2CalibPoint over every model branch (tags -1..-4, rejections,
    non-finite values) against the oracle's per-pixel model."""
    from polycase import random_disparity, random_maps
    H, W = 24, 32
    cx, cy, cz, br = random_maps(H, W, seed=31)
    d = random_disparity(H, W, br, seed=32)
    xyz, mask = O.poly_reproject(d, (cx, cy, cz), np.eye(3), -1e30, 1e30, True)
    n_ok = 0
    for i in range(H):
        for j in range(W):
            if abs(float(d[i, j])) < 1e-5:
                assert mask[i, j] == 0
                continue
            ok, p = ref.poly_point(cx[i, j], cy[i, j], cz[i, j], float(d[i, j]))
            assert bool(mask[i, j]) == ok, (i, j)
            if ok:
                n_ok += 1
                assert np.array_equal(p.astype(np.float32), xyz[i, j]), (i, j)
    assert n_ok > H * W // 3
