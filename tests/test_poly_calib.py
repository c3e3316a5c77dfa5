"""V2 polynomial calibration on the CPU: the oracle's restatement of
evaluateV2CalibPoint / startCalculate_v2 (JSLAB_PhaseEpipolarReconstructor_V2.cpp:13-76,
482-593), pinned by hand-computed answers and by an independent pure-Python
evaluation in the reference's operation order (Python floats are IEEE
doubles with no contraction, numpy float32 scalars are IEEE floats); and the
calibration file formats (JSLAB_StereoCalibParams_V1/V2.cpp, saveMatBinary in
JSLAB_StereoCalib_V2.cpp:22-30).
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from polycase import BRANCHES, q_maps, random_disparity, random_maps

f32 = np.float32


def tag(c, t):
    return abs(f32(c) - f32(t)) < f32(1e-6)


def ref_point(cx, cy, cz, d):
    """evaluateV2CalibPoint written out term by term (None = rejected)."""
    cx = [float(f32(v)) for v in cx]
    cy = [float(f32(v)) for v in cy]
    z = [float(f32(v)) for v in cz]
    if all(abs(v) <= 1e-9 for v in z):
        return None
    fin = math.isfinite
    if tag(cx[3], -1):
        d2 = d * d
        iz = z[0] + z[1] * d + z[2] * d2 + z[3] * d2 * d
        if not fin(iz) or abs(iz) < 1e-12:
            return None
        Z = 1.0 / iz
        X, Y = cx[0] * Z, cy[0] * Z
    elif tag(cx[3], -2):
        d2 = d * d
        if tag(cz[3], -1):
            iz = z[0] + z[1] * d + z[2] * d2
            if not fin(iz) or abs(iz) < 1e-12:
                return None
            Z = 1.0 / iz
        else:
            Z = z[0] + z[1] * d + z[2] * d2 + z[3] * d2 * d
        X, Y = cx[0] * Z, cy[0] * Z
    elif tag(cx[3], -3):
        if tag(cz[3], -4):
            den = z[1] * d + 1.0
            if not fin(den) or abs(den) < 1e-12:
                return None
            Z = z[0] / den
        else:
            d2 = d * d
            d3 = d2 * d
            Z = z[0] + z[1] * d + z[2] * d2 + z[3] * d3
        X, Y = cx[0] * Z + cx[1], cy[0] * Z + cy[1]
    elif tag(cz[3], -1):
        iz = z[0] + z[1] * d + z[2] * d * d
        if not fin(iz) or abs(iz) < 1e-12:
            return None
        Z = 1.0 / iz
        X, Y = cx[0] * Z, cy[0] * Z
    else:
        d2 = d * d
        d3 = d2 * d
        X = cx[0] + cx[1] * d + cx[2] * d2 + cx[3] * d3
        Y = cy[0] + cy[1] * d + cy[2] * d2 + cy[3] * d3
        Z = z[0] + z[1] * d + z[2] * d2 + z[3] * d3
    if not (fin(X) and fin(Y) and fin(Z)):
        return None
    return X, Y, Z


def one(cx, cy, cz, d, R1=np.eye(3), rectified=True, lo=0.0, hi=1e9):
    m = [np.asarray(v, np.float32).reshape(1, 1, 4) for v in (cx, cy, cz)]
    xyz, mask = O.poly_reproject(np.array([[d]], np.float32), m, R1, lo, hi, rectified)
    return xyz[0, 0], mask[0, 0]


def test_hand_computed_models():
    # inverse depth: 1/z = 0.001 + 2e-5 * 50 = 0.002 -> z = 500, x = 0.5 z, y = -0.25 z
    xyz, m = one([0.5, 0, 0, -1], [-0.25, 0, 0, 0], [0.001, 2e-5, 0, 0], 50.0)
    assert m == 1 and np.allclose(xyz, [250, -125, 500], rtol=1e-6)
    # fitted ray, quadratic inverse depth (z-map tag -1): 1/z = 0.5 + 0.25 * 2 + 0.125 * 4 = 1.5
    xyz, m = one([3, 0, 0, -2], [6, 0, 0, 0], [0.5, 0.25, 0.125, -1], 2.0)
    assert m == 1 and np.allclose(xyz, [2, 4, 1 / 1.5], rtol=1e-6)
    # fitted ray, cubic depth: z = 1 + 2 * 2 + 3 * 4 + 4 * 8 = 49
    xyz, m = one([1, 0, 0, -2], [2, 0, 0, 0], [1, 2, 3, 4], 2.0)
    assert m == 1 and np.allclose(xyz, [49, 98, 49])
    # z-linear x/y, rational depth: z = 600 / (0.5 * 2 + 1) = 300; x = 0.1 z + 5
    xyz, m = one([0.1, 5, 0, -3], [0.2, -7, 0, 0], [600, 0.5, 0, -4], 2.0)
    assert m == 1 and np.allclose(xyz, [35, 53, 300])
    # z-linear x/y, cubic depth: z = 10 + 1 * 3 = 13
    xyz, m = one([2, 1, 0, -3], [1, 0, 0, 0], [10, 1, 0, 0], 3.0)
    assert m == 1 and np.allclose(xyz, [27, 13, 13])
    # z-map tag only: 1/z = 0.25 + 0.125 * 2 + 0.0625 * 2 * 2 = 0.75
    xyz, m = one([3, 0, 0, 0.5], [-3, 0, 0, 0], [0.25, 0.125, 0.0625, -1], 2.0)
    assert m == 1 and np.allclose(xyz, [4, -4, 4 / 3], rtol=1e-6)
    # plain cubics in d
    xyz, m = one([1, 1, 1, 1], [0, 1, 0, 0], [100, 0, 0, 1], 2.0)
    assert m == 1 and np.allclose(xyz, [15, 2, 108])


def test_rejections_and_gates():
    assert one([1, 0, 0, -1], [1, 0, 0, 0], [0, 0, 5e-10, -5e-10], 10.0)[1] == 0      # all-zero z map
    assert one([1, 0, 0, -1], [1, 0, 0, 0], [1, -1, 0, 0], 1.0)[1] == 0                 # 1/z = 0
    assert one([1, 0, 0, -3], [1, 0, 0, 0], [1, -1, 0, -4], 1.0)[1] == 0                # rational den = 0
    assert one([1, 0, 0, -1], [1, 0, 0, 0], [1, np.inf, 0, 0], 1.0)[1] == 0             # 1/z infinite
    assert one([np.nan, 0, 0, 0], [1, 0, 0, 0], [500, 0, 0, 0], 1.0)[1] == 0            # x not finite
    assert one([1, 0, 0, -1], [1, 0, 0, 0], [0.001, 2e-5, 0, 0], 9e-6)[1] == 0          # |d| < 1e-5
    # 1/z = 2^-10 + 2^-14 * 16 = 2^-9 exactly: z = 512 sits on the open gate
    assert one([1, 0, 0, -1], [1, 0, 0, 0], [2.0 ** -10, 2.0 ** -14, 0, 0], 16.0, lo=0, hi=512)[1] == 0
    assert one([1, 0, 0, -1], [1, 0, 0, 0], [2.0 ** -10, 2.0 ** -14, 0, 0], 16.0, lo=0, hi=513)[1] == 1
    assert one([1, 0, 0, -1], [1, 0, 0, 0], [2.0 ** -10, 2.0 ** -14, 0, 0], 16.0, lo=512, hi=600)[1] == 0
    # tag tolerance is float 1e-6: -1 + 2e-6 is not a tag (plain cubic: z = 0.001 + 2e-5 d)
    xyz, m = one([1, 0, 0, -1 + 2e-6], [1, 0, 0, 0], [0.001, 2e-5, 0, 0], 50.0, hi=1e9)
    assert m == 1 and abs(xyz[2] - 0.002) < 1e-9


def test_rotated_output_uses_r1_transpose():
    a = 0.3
    R1 = np.array([[math.cos(a), -math.sin(a), 0], [math.sin(a), math.cos(a), 0], [0, 0, 1]])
    xyz, m = one([0.5, 0, 0, -1], [-0.25, 0, 0, 0], [0.001, 2e-5, 0, 0], 50.0, R1=R1, rectified=False)
    assert m == 1 and np.allclose(xyz, R1.T @ np.array([250, -125, 500]), rtol=1e-6)


@pytest.mark.parametrize("rectified", [True, False])
def test_oracle_matches_term_by_term_evaluation(rectified):
    H, W = 24, 40
    cx, cy, cz, br = random_maps(H, W, seed=3)
    d = random_disparity(H, W, br, seed=4)
    R1 = np.array([[0.99, -0.1, 0.05], [0.1, 0.99, 0.0], [-0.05, 0.0, 0.998]])
    xyz, mask = O.poly_reproject(d, (cx, cy, cz), R1, 0.0, 1000.0, rectified)
    seen = set()
    for i in range(H):
        for j in range(W):
            dv = float(d[i, j])
            p = None if abs(dv) < 1e-5 else ref_point(cx[i, j], cy[i, j], cz[i, j], dv)
            want, wm = np.zeros(3, np.float32), 0
            if p is not None:
                X, Y, Z = p
                rx = R1[0, 0] * X + R1[1, 0] * Y + R1[2, 0] * Z
                ry = R1[0, 1] * X + R1[1, 1] * Y + R1[2, 1] * Z
                rz = R1[0, 2] * X + R1[1, 2] * Y + R1[2, 2] * Z
                g = (X, Y, Z) if rectified else (rx, ry, rz)
                if 0.0 < g[2] < 1000.0:
                    want, wm = np.array(g, np.float32), 1
                seen.add(BRANCHES[br[i, j]])
            assert mask[i, j] == wm, (i, j, BRANCHES[br[i, j]])
            assert np.array_equal(xyz[i, j], want), (i, j, BRANCHES[br[i, j]], xyz[i, j], want)
    assert {"inv_cubic", "ray_inv", "ray_cubic", "lin_rational", "lin_cubic", "z_inv", "cubic"} <= seen


@pytest.mark.parametrize("model", ["inv", "ray", "zinv", "rational"])
def test_q_equivalent_maps_reproduce_q_reprojection(model):
    f, B, Z = 800.0, 120.0, 800.0
    K0 = np.array([[f, 0, 320], [0, f, 240], [0, 0, 1]])
    K1 = np.array([[f, 0, 300], [0, f, 240], [0, 0, 1]])  # cx differs: Q33 != 0 for the rational model
    c = O.make_calib([K0, K1], [np.zeros(5)] * 2, np.eye(3), [-B, 0, 0], 640, 480)
    R1, R2, P1, P2, Q, w, h = O.rectification(c, False)
    rng = np.random.default_rng(7)
    d = rng.uniform(60, 200, (h, w)).astype(np.float32)
    ref, rm, _ = O.reproject(d, Q, R1, 0.0, 1e6, True)
    xyz, mask = O.poly_reproject(d, q_maps(Q, h, w, model), R1, 0.0, 1e6, True)
    assert np.array_equal(mask, rm) and rm.all()
    assert np.max(np.abs(xyz - ref) / (np.abs(ref) + 1.0)) < 1e-5


# ------------------------------------------------------------ file formats ----

def test_mat_binary_layout_and_roundtrip(tmp_path):
    from zim_gb300 import calib_io
    a = np.arange(2 * 3 * 4, dtype=np.float32).reshape(2, 3, 4) * 0.5
    p = tmp_path / "m_rx.bin"
    calib_io.save_mat_binary(str(p), a)
    raw = p.read_bytes()
    # header: CV_32FC4 = 5 + (3 << 3) = 29, rows 2, cols 3; then the 24 floats
    assert np.frombuffer(raw[:12], "<i4").tolist() == [29, 2, 3] and len(raw) == 12 + a.nbytes
    assert np.array_equal(calib_io.load_mat_binary(str(p)), a)
    b = np.arange(6, dtype=np.float64).reshape(2, 3)
    calib_io.save_mat_binary(str(p), b)
    assert np.frombuffer(p.read_bytes()[:4], "<i4")[0] == 6  # CV_64FC1
    assert np.array_equal(calib_io.load_mat_binary(str(p)), b)
    p.write_bytes(raw[:40])  # shorter than the header says
    assert calib_io.load_mat_binary(str(p)) is None
    assert calib_io.load_mat_binary(str(tmp_path / "absent.bin")) is None


def _params_v2(h=4, w=5):
    from zim_gb300 import api
    p = api.JSLAB_StereoCalibParams_V2()
    p.camera_matrix = [np.array([[2400.0, 0, 1224.5], [0, 2401.0, 1023.25], [0, 0, 1]]),
                       np.array([[2399.0, 0, 1220.0], [0, 2398.5, 1025.0], [0, 0, 1]])]
    p.dist_coeffs = [np.array([-0.05, 0.01, 1e-4, -2e-4, 0.0]), np.array([-0.04, 0.008, 0.0, 1e-4, 1e-3])]
    p.R = np.array([[0.9998, -0.01, 0.017], [0.0101, 0.99994, -0.005], [-0.01695, 0.00517, 0.99984]])
    p.t = np.array([-200.0, 0.5, 1.25])
    p.image_size = (2448, 2048)
    rng = np.random.default_rng(0)
    p.xyz_calib_coeffs = [rng.normal(size=(h, w, 4)).astype(np.float32) for _ in range(3)]
    return p


def test_calib_xml_and_bins_roundtrip(tmp_path):
    from zim_gb300 import api, calib_io
    p = _params_v2()
    fn = str(tmp_path / "stereo_calib.xml")
    assert calib_io.saveStereoCalibParams(fn, p)
    for s in ("_rx.bin", "_ry.bin", "_rz.bin"):
        assert (tmp_path / ("stereo_calib" + s)).exists()
    q = api.JSLAB_StereoCalibParams_V2()
    assert calib_io.loadStereoCalibParams_V2(fn, q)
    for a, b in zip(p.camera_matrix + p.dist_coeffs + [p.R, p.t], q.camera_matrix + q.dist_coeffs + [q.R, q.t]):
        assert np.array_equal(np.asarray(a, np.float64), b)
    assert q.image_size == (2448, 2048)
    for a, b in zip(p.xyz_calib_coeffs, q.xyz_calib_coeffs):
        assert np.array_equal(a, b)
    v1 = api.JSLAB_StereoCalibParams_V1()
    assert calib_io.loadStereoCalibParams_V1(fn, v1) and np.array_equal(v1.R, q.R)
    (tmp_path / "stereo_calib_rz.bin").unlink()
    assert not calib_io.loadStereoCalibParams_V2(fn, api.JSLAB_StereoCalibParams_V2())
    assert not calib_io.loadStereoCalibParams_V1(str(tmp_path / "none.xml"), v1)


def test_file_storage_yaml_and_opencv_xml_text(tmp_path):
    from zim_gb300 import api, calib_io
    yml = tmp_path / "c.yml"
    yml.write_text("%YAML:1.0\n---\nLeftCameraMatrix: !!opencv-matrix\n   rows: 3\n   cols: 3\n   dt: d\n"
                   "   data: [ 800., 0., 320., 0., 800., 240., 0., 0., 1. ]\n"
                   "TranslationVector: !!opencv-matrix\n   rows: 3\n   cols: 1\n   dt: d\n"
                   "   data: [ -120., 0., 0. ]\nImageSize: [ 640, 480 ]\n")
    p = api.JSLAB_StereoCalibParams_V1()
    assert calib_io.loadStereoCalibParams_V1(str(yml), p)
    assert p.camera_matrix[0][0, 2] == 320 and p.t[0] == -120 and p.image_size == (640, 480)
    xml = tmp_path / "c.xml"
    xml.write_text('<?xml version="1.0"?>\n<opencv_storage>\n<RotationMatrix type_id="opencv-matrix">\n'
                   "  <rows>3</rows>\n  <cols>3</cols>\n  <dt>d</dt>\n  <data>\n    1. 0. 0. 0. 1. 0. 0. 0. 1.</data>"
                   "</RotationMatrix>\n<ImageSize>\n  2448 2048</ImageSize>\n</opencv_storage>\n")
    p = api.JSLAB_StereoCalibParams_V1()
    assert calib_io.loadStereoCalibParams_V1(str(xml), p)
    assert np.array_equal(p.R, np.eye(3)) and p.image_size == (2448, 2048)


def test_recon_config_reproject_model_default(native):
    from zim_gb300 import api
    assert api.recon_config().reproject_model == 0


# ------------------------------------------------- cubic calibration fit ----

def _small_rig_q():
    f, B = 600.0, 150.0
    K0 = np.array([[f, 0, 47.5], [0, f, 31.5], [0, 0, 1]])
    K1 = np.array([[f, 0, 45.0], [0, f, 31.5], [0, 0, 1]])
    c = O.make_calib([K0, K1], [np.zeros(5)] * 2, np.eye(3), [-B, 0, 0], 96, 64)
    return O.rectification(c, False)


def test_fit_oracle_recovers_planes_and_points():
    from oracle import calib_fit as F
    R1, R2, P1, P2, Q, w, h = _small_rig_q()
    disps, masks = F.synthetic_planes(Q, h, w, n_planes=6, seed=1, noise=0.0, dropout=0.0)
    cx, cy, cz, eqs = F.fit(Q, disps, masks)
    # the PCA plane of noise-free samples holds every sample
    for k, (d, m) in enumerate(zip(disps, masks)):
        r, c = np.nonzero(m)
        x, y, z = F.q_points(Q, d[r, c].astype(np.float64), r, c)
        dist = eqs[k, 0] * x + eqs[k, 1] * y + eqs[k, 2] * z + eqs[k, 3]
        assert np.abs(dist).max() < 1e-6 * np.abs(z).max()
    # a cubic in d approximates z = Q23 / (Q32 d + Q33) over a 2:1 depth range
    # (600-1200 mm) to about 0.2 % -- the model's own limit
    for d, m in zip(disps, masks):
        r, c = np.nonzero(m)
        dv = d[r, c].astype(np.float64)
        x, y, z = F.q_points(Q, dv, r, c)
        zf = F.evaluate(cz[r, c], dv)
        assert np.max(np.abs(zf - z) / z) < 3e-3


def test_fit_oracle_needs_four_samples():
    from oracle import calib_fit as F
    R1, R2, P1, P2, Q, w, h = _small_rig_q()
    disps, masks = F.synthetic_planes(Q, h, w, n_planes=4, seed=2, noise=0.0, dropout=0.0)
    masks[0][10, 20] = 0
    cx, cy, cz, _ = F.fit(Q, disps, masks)
    assert not cz[10, 20].any() and cz[11, 20].any()
