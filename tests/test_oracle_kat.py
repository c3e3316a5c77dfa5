"""Known-answer tests of the FP64 oracle (CPU).

The reference ships no golden vectors, so the oracle is pinned against
analytic answers (exact phase-shift sums, single-pixel unwrapping, linear
rows with a known sub-pixel shift, plane depth, identity rectification, exact
planes and quadrics for MLS) and against independent implementations (numpy
median, scipy's KD-tree for the k-nearest-neighbour statistics).
"""
import math

import numpy as np
import pytest

from oracle import oracle as O

TWO_PI = 2 * math.pi


def test_gaussian_kernel3():
    assert np.array_equal(O.gaussian_kernel3(0.0), [0.25, 0.5, 0.25])
    for s in (0.7, 3.0):
        k = O.gaussian_kernel3(s)
        t = math.exp(-0.5 / (s * s))
        assert np.allclose(k, np.array([t, 1, t]) / (2 * t + 1), rtol=0, atol=1e-16)
        assert abs(k.sum() - 1) < 1e-15


def test_blur3_replicate_border():
    img = np.arange(20, dtype=float).reshape(4, 5)
    k = np.array([0.25, 0.5, 0.25])
    pad = np.pad(img, 1, mode="edge")
    ref = sum(k[a] * k[b] * pad[a:a + 4, b:b + 5] for a in range(3) for b in range(3))
    assert np.allclose(O.blur3(img, k), ref, atol=1e-12)


def frames_for(x, A, B, freqs, steps, offset):
    """Phase-shift frames of one pixel row for projector coordinates x in [0, 1)."""
    out = []
    for f, n in zip(freqs, steps):
        th = TWO_PI * f * x - offset
        for k in range(n):
            out.append(A + B * np.cos(th + TWO_PI * k / n))
    return np.array(out)[:, None, :]


def test_four_step_exact_sums_and_modulation():
    x = np.linspace(0.01, 0.99, 97)
    fr = frames_for(x, 100.0, 50.0, [121, 110, 120], [4, 4, 4], 0.0)
    cfg = O.make_decode_cfg(O.ENC_HETERODYNE3, (121, 110, 120), (4, 4, 4), modulation_threshold=0.1, preblur_sigma=0)
    # a one-row image: the 3x3 replicate blur along the row mixes neighbours, so use a constant row per pixel
    for i in range(len(x)):
        img = np.repeat(np.repeat(fr[:, :, i:i + 1], 3, axis=1), 3, axis=2)
        ph, k, mod, valid, _ = O.decode(cfg, img)
        assert valid[1, 1] == 1
        assert abs(mod[1, 1] - 0.5) < 1e-12
        assert k[1, 1] == round(121 * x[i])
        assert abs(ph[1, 1] - TWO_PI * 121 * x[i]) < 1e-9


@pytest.mark.parametrize("freqs", [(121, 110, 120), (107, 100, 94)])
def test_single_pixel_heterodyne(freqs):
    rng = np.random.default_rng(0)
    for x in rng.uniform(0.002, 0.998, 200):
        img = np.repeat(np.repeat(frames_for(np.array([x]), 120.0, 80.0, freqs, (8, 8, 8), 0.0), 3, 1), 3, 2)
        cfg = O.make_decode_cfg(O.ENC_HETERODYNE3, freqs, (8, 8, 8), modulation_threshold=0.3)
        ph, k, _, valid, _ = O.decode(cfg, img)
        assert valid[1, 1] == 1
        assert k[1, 1] == round(freqs[0] * x)
        assert abs(ph[1, 1] - TWO_PI * freqs[0] * x) < 1e-9


def test_hdr_least_squares_recovers_clipped_pixels():
    """JSLAB_HDRPhaseFit semantics: samples at or above the saturation grey are
    dropped and A + C cos d - S sin d is fitted to the rest, so a bright pixel
    whose peaks clip still decodes exactly, where the plain sums are biased."""
    rng = np.random.default_rng(1)
    freqs = (121, 110, 120)
    n_exact = 0
    for x in rng.uniform(0.002, 0.998, 100):
        raw = frames_for(np.array([x]), 200.0, 100.0, freqs, (8, 8, 8), 0.0)
        clipped = np.minimum(raw, 255.0)  # 8-bit sensor: peaks saturate
        img = np.repeat(np.repeat(clipped, 3, 1), 3, 2)
        cfg = O.make_decode_cfg(O.ENC_HETERODYNE3, freqs, (8, 8, 8), modulation_threshold=0.3, enable_hdr=True,
                                hdr_saturation_gray=255.0, hdr_min_amplitude=2.0)
        ph, k, mod, valid, _ = O.decode(cfg, img)
        assert valid[1, 1] == 1
        assert k[1, 1] == round(121 * x)
        assert abs(ph[1, 1] - TWO_PI * 121 * x) < 1e-9
        assert abs(mod[1, 1] - 0.5) < 1e-9
        n_exact += 1
    assert n_exact == 100


def test_hdr_rejects_and_marks_invalid_orders():
    # all samples saturated -> fewer than three usable: invalid, order -1
    img = np.full((24, 3, 3), 255.0)
    cfg = O.make_decode_cfg(O.ENC_HETERODYNE3, (121, 110, 120), (8, 8, 8), modulation_threshold=0.3,
                            enable_hdr=True, hdr_saturation_gray=255.0)
    ph, k, mod, valid, _ = O.decode(cfg, img)
    assert (valid == 0).all() and (k == -1).all() and (ph == 0).all()
    # amplitude at the threshold is rejected (hypot(C, S) <= min_amp)
    x = np.array([0.3])
    img = np.repeat(np.repeat(frames_for(x, 100.0, 2.0, (121, 110, 120), (8, 8, 8), 0.0), 3, 1), 3, 2)
    cfg = O.make_decode_cfg(O.ENC_HETERODYNE3, (121, 110, 120), (8, 8, 8), modulation_threshold=0.0,
                            enable_hdr=True, hdr_min_amplitude=2.0 + 1e-9)
    _, k, _, valid, _ = O.decode(cfg, img)
    assert valid[1, 1] == 0 and k[1, 1] == -1


def test_hdr_post_smooth_normalises_by_validity():
    ph = np.arange(25, dtype=float).reshape(5, 5) + 100.0
    valid = np.ones((5, 5), np.uint8)
    valid[2, 3] = 0
    ph[2, 3] = 0.0
    out = O.post_smooth_hdr(ph, valid)
    k = np.array([0.25, 0.5, 0.25])
    pad = np.pad(ph, 1, mode="edge")
    padv = np.pad(valid.astype(float), 1, mode="edge")
    num = sum(k[a] * k[b] * pad[a:a + 5, b:b + 5] for a in range(3) for b in range(3))
    den = sum(k[a] * k[b] * padv[a:a + 5, b:b + 5] for a in range(3) for b in range(3))
    ref = np.where(valid > 0, num / den, 0.0)
    assert np.allclose(out, ref, rtol=0, atol=1e-12)


def test_hierarchical_1_8_64():
    for x in np.linspace(0.001, 0.999, 301):
        img = np.repeat(np.repeat(frames_for(np.array([x]), 2000.0, 1500.0, (1, 8, 64), (4, 4, 4), math.pi), 3, 1), 3,
                        2)
        cfg = O.make_decode_cfg(O.ENC_HIERARCHICAL, (1, 8, 64), (4, 4, 4), modulation_threshold=0.3)
        ph, k, _, valid, _ = O.decode(cfg, img)
        assert k[1, 1] == math.floor(64 * x)
        assert abs(ph[1, 1] - (TWO_PI * 64 * x - math.pi)) < 1e-9


@pytest.mark.parametrize("complementary", [False, True])
def test_gray_code_orders(complementary):
    P, nb = 32, 5
    xs = (np.arange(640) + 0.37) / 640  # avoids exact period boundaries, where the wrap is +-pi
    A, B = 100.0, 60.0
    for x in xs:
        fr = list(frames_for(np.array([x]), A, B, (P,), (4,), math.pi)[:, 0, 0])
        period, half = int(math.floor(P * x)), int(math.floor(2 * P * x))
        g1, g2 = period ^ (period >> 1), half ^ (half >> 1)
        for b in range(nb):
            fr.append(A + B * (2 * ((g1 >> (nb - 1 - b)) & 1) - 1))
        if complementary:
            fr.append(A + B * (2 * (g2 & 1) - 1))
        img = np.repeat(np.repeat(np.array(fr)[:, None, None], 3, 1), 3, 2)
        enc = O.ENC_GRAYCODE_COMPLEMENTARY if complementary else O.ENC_GRAYCODE
        cfg = O.make_decode_cfg(enc, (P,), (4,), gray_bits=nb, modulation_threshold=0.3)
        ph, k, _, valid, _ = O.decode(cfg, img)
        assert valid[1, 1] == 1
        assert k[1, 1] == period
        assert abs(ph[1, 1] - (TWO_PI * P * x - math.pi)) < 1e-9


def test_match_linear_rows_known_subpixel_shift():
    W = 200
    a = 0.3
    for d in (3.0, 17.25, 40.6, 55.999):
        j = np.arange(W, dtype=float)
        rph = (a * j)[None, :].repeat(4, 0)
        lph = (a * (j - d))[None, :].repeat(4, 0)
        rk = np.ones((4, W), np.int32)
        lk = np.ones((4, W), np.int32)
        disp, best, _ = O.stereo_match(lph, rph, lk, rk, pha_f=1, grad_threshold=1.0)
        ok = best >= 0
        assert ok[:, int(d) + 3:W - 3].all()
        assert np.allclose(disp[ok], d, atol=1e-9)
        # first-column tie-break and order 0 never matched
        disp0, best0, _ = O.stereo_match(lph, rph, lk * 0, rk * 0, pha_f=1)
        assert (best0 < 0).all()


def test_median5_matches_numpy():
    rng = np.random.default_rng(1)
    img = rng.normal(size=(23, 31)).astype(np.float32)
    img[rng.random(img.shape) < 0.3] = 0
    pad = np.pad(img, 2, mode="edge")
    ref = np.median(np.stack([pad[a:a + 23, b:b + 31] for a in range(5) for b in range(5)]), axis=0)
    assert np.array_equal(O.median5(img), ref.astype(np.float32))


def test_reproject_plane_depth():
    f, B, Z = 800.0, 120.0, 800.0
    K = np.array([[f, 0, 320], [0, f, 240], [0, 0, 1]])
    c = O.make_calib([K, K], [np.zeros(5)] * 2, np.eye(3), [-B, 0, 0], 640, 480)
    R1, R2, P1, P2, Q, w, h = O.rectification(c, True)
    assert (w, h) == (640, 480)
    assert np.allclose(R1, np.eye(3)) and np.allclose(R2, np.eye(3))
    d = np.full((480, 640), f * B / Z, np.float32)
    xyz, mask, _ = O.reproject(d, Q, R1)
    assert mask.all()
    assert np.allclose(xyz[..., 2], Z, rtol=1e-6)
    assert np.allclose(xyz[240, 320, :2], 0, atol=1e-3)


def test_identity_rectification_maps_and_remap():
    K = np.array([[800.0, 0, 319.5], [0, 800.0, 239.5], [0, 0, 1]])
    c = O.make_calib([K, K], [np.zeros(5)] * 2, np.eye(3), [-100, 0, 0], 64, 48)
    R1, R2, P1, P2, Q, w, h = O.rectification(c, False)
    mx, my = O.init_rectify_map(K, np.zeros(5), R1, P1, w, h)
    jj, ii = np.meshgrid(np.arange(w), np.arange(h))
    assert np.abs(mx - jj).max() < 1e-4 and np.abs(my - ii).max() < 1e-4
    src = np.random.default_rng(2).normal(size=(h, w))
    assert np.allclose(O.remap_linear(src, np.rint(mx), np.rint(my)), src)
    # half-pixel shift averages neighbours; positions quantise to 1/32 px
    sh = O.remap_linear(src, np.rint(mx) + 0.5, np.rint(my))
    assert np.allclose(sh[:, :-1], 0.5 * (src[:, :-1] + src[:, 1:]))
    q = O.remap_linear(src, np.rint(mx) + np.float32(0.51), np.rint(my))
    assert np.allclose(q[:, :-1], 0.5 * (src[:, :-1] + src[:, 1:]))  # 0.51 -> 16/32
    # outside the source: BORDER_CONSTANT 0; nearest rounds half to even
    assert (O.remap_linear(src, mx - 1000, my) == 0).all()
    k = np.arange(h * w, dtype=np.int32).reshape(h, w)
    assert np.array_equal(O.remap_nearest(k, np.rint(mx) + np.float32(0.5), np.rint(my))[:, 1:-1:2],
                          k[:, 2:-1:2])


def test_undistort_roundtrip():
    K = np.array([[2400.0, 0, 1223.5], [0, 2400.0, 1023.5], [0, 0, 1]])
    D = np.array([-0.05, 0.01, 0.001, -0.0005, 0.0])
    rng = np.random.default_rng(3)
    pts = rng.uniform([0, 0], [2447, 2047], size=(200, 2)).astype(np.float32)
    und = O.undistort_points(K, D, pts)  # normalised coordinates
    x, y = und[:, 0].astype(float), und[:, 1].astype(float)
    r2 = x * x + y * y
    kr = 1 + (D[1] + D[4] * r2) * r2 * r2 + D[0] * r2
    xd = x * kr + 2 * D[2] * x * y + D[3] * (r2 + 2 * x * x)
    yd = y * kr + D[2] * (r2 + 2 * y * y) + 2 * D[3] * x * y
    back = np.stack([K[0, 0] * xd + K[0, 2], K[1, 1] * yd + K[1, 2]], 1)
    # five fixed-point iterations (OpenCV's default) converge to ~1e-3 px here
    assert np.abs(back - pts).max() < 5e-3


def test_mls_reproduces_plane_and_quadric():
    H, W = 21, 21
    jj, ii = np.meshgrid(np.arange(W, dtype=float), np.arange(H, dtype=float))
    X, Y = jj * 0.4, ii * 0.4
    mask = np.ones((H, W), np.uint8)
    plane = np.stack([X, Y, 900 + 0.2 * X - 0.1 * Y], -1).astype(np.float32)
    for order in (0, 1, 2):
        out, _ = O.mls(plane, mask, 4, 1.0, order, 0.0, 1)
        assert np.abs(out - plane).max() < 1e-9 + 1e-4  # plane points are fixed points
    quad = np.stack([X, Y, 900 + 0.01 * (X - 4) ** 2 + 0.02 * (Y - 4) ** 2], -1).astype(np.float32)
    out, _ = O.mls(quad, mask, 5, 2.0, 2, 0.0, 1)
    inner = (slice(6, 15), slice(6, 15))
    assert np.abs(out[inner] - quad[inner]).max() < 2e-4  # order 2 reproduces a quadric up to frame tilt


def test_sor_matches_kdtree_and_pcl_statistics():
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(4)
    H, W = 40, 50
    jj, ii = np.meshgrid(np.arange(W, dtype=float), np.arange(H, dtype=float))
    xyz = np.stack([jj * 0.5, ii * 0.5, 900 + rng.normal(0, 0.05, (H, W))], -1).astype(np.float32)
    out = rng.random((H, W)) < 0.02
    xyz[out, 2] += rng.uniform(5, 50, out.sum())
    mask = (rng.random((H, W)) < 0.95).astype(np.uint8)
    k = 30
    mo, md, thr, _ = O.sor(xyz, mask, k, 1.0)
    pts = xyz[mask > 0].astype(np.float64)
    d, _ = cKDTree(pts).query(pts, k=k + 1)
    ref = (np.sqrt(d[:, 1:] ** 2).sum(1) / k).astype(np.float32)
    assert np.allclose(md[mask > 0], ref, rtol=1e-6)
    # PCL: float mean distances, float squares, double sums, sample variance
    m32 = md[mask > 0].astype(np.float32)
    s1, s2 = m32.astype(np.float64).sum(), (m32 * m32).astype(np.float64).sum()
    mean = s1 / len(m32)
    sd = np.sqrt((s2 - s1 * s1 / len(m32)) / (len(m32) - 1))
    assert abs(thr - (mean + sd)) < 1e-12 * thr
    assert np.array_equal(mo[mask > 0], (ref <= thr).astype(np.uint8))
    assert (mo[mask == 0] == 0).all()


def test_metric_gaussian_bruteforce():
    rng = np.random.default_rng(5)
    xyz = rng.uniform(0, 3, size=(12, 14, 3)).astype(np.float32)
    mask = (rng.random((12, 14)) < 0.8).astype(np.uint8)
    s = 0.4
    out, _ = O.metric_gaussian(xyz, mask, s)
    P = xyz[mask > 0].astype(np.float64)
    for p, o in zip(P, out[mask > 0]):
        d2 = ((P - p) ** 2).sum(1)
        w = np.exp(-d2 / (2 * s * s)) * (d2 <= 9 * s * s)
        ref = p + (w[:, None] * (P - p)).sum(0) / w.sum()
        assert np.allclose(o, ref, atol=1e-5)
