"""On-disk outputs on the CPU: the .raw phase/disparity dump with its info text
(JSLAB_PhaseDisparityExporter.cpp:115-141), the Matlab text dump with its depth
filter (main.cpp:162-184) and the PLY header (main.cpp:85-160)."""
import numpy as np

from zim_gb300 import export


def test_raw64f_roundtrip_and_info(tmp_path):
    a = np.random.default_rng(0).normal(size=(7, 5))
    raw, info = str(tmp_path / "d.raw"), str(tmp_path / "d.info.txt")
    assert export.saveRaw64F(a, raw, info)
    assert (tmp_path / "d.raw").stat().st_size == 7 * 5 * 8
    assert np.array_equal(export.loadRaw64F(raw, 7, 5), a)
    lines = (tmp_path / "d.info.txt").read_text().splitlines()
    assert lines[:3] == ["rows 7", "cols 5", "type CV_64FC1 (double)"]
    assert not export.saveRaw64F(a.astype(np.float32), raw, info)  # CV_64FC1 only
    assert not export.saveRaw64F(np.zeros((0, 3)), raw, info)


def test_txt_filter_and_format(tmp_path):
    xyz = np.array([[[1.5, -2.25, 800.0], [0.0, 0.0, 0.0], [1.0, 2.0, 20000.0]],
                    [[0.1234567, 1e6, 0.00005], [3.0, 4.0, -500.125], [1.0, 1.0, np.nan]]], np.float32)
    fn = tmp_path / "p.txt"
    assert export.saveToTxt(xyz, str(fn))
    # z = 0, |z| <= 1e-4, |z| >= 1e4 and NaN are dropped; %g-style six digits
    assert fn.read_text().splitlines() == ["1.5 -2.25 800", "3 4 -500.125"]


def test_ply_header():
    h = export._ply_header(3, True).decode()
    assert h == ("ply\nformat binary_little_endian 1.0\nelement vertex 3\nproperty float x\nproperty float y\n"
                 "property float z\nproperty uchar red\nproperty uchar green\nproperty uchar blue\nend_header\n")
    assert "red" not in export._ply_header(3, False).decode()
