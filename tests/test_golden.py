"""The committed golden fixtures (tests/golden/, written by make_golden.py):
the oracle reproduces each one byte for byte, and the library's host
rasteriser reproduces the ROI masks."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
DECODES = sorted(p.name for p in GOLDEN.glob("decode_*.npz"))


def test_fixtures_present():
    assert len(DECODES) >= 4
    for n in ("match_config0_rows.npz", "poly_reproject.npz", "roi_fill.npz"):
        assert (GOLDEN / n).exists(), n


@pytest.mark.parametrize("name", DECODES)
def test_oracle_decode_reproduces_fixture(oracle_lib, name):
    d = np.load(GOLDEN / name)
    kw = json.loads(str(d["cfg"]))
    ph, k, mod, valid, near = oracle_lib.decode(oracle_lib.make_decode_cfg(**kw), d["frames"])
    for a, b in ((ph, d["phase"]), (k, d["order"]), (mod, d["mod"]), (valid, d["valid"]), (near, d["near"])):
        assert np.array_equal(a, b)


def test_oracle_match_reproduces_fixture(oracle_lib):
    d = np.load(GOLDEN / "match_config0_rows.npz")
    disp, best, near = oracle_lib.stereo_match(d["lph"], d["rph"], d["lk"], d["rk"], int(d["pha_f"]))
    assert np.array_equal(disp, d["disp"]) and np.array_equal(best, d["best"]) and np.array_equal(near, d["near"])
    assert (d["best"] >= 0).mean() > 0.5


def test_oracle_poly_reproduces_fixture(oracle_lib):
    d = np.load(GOLDEN / "poly_reproject.npz")
    for rectified in (1, 0):
        xyz, mask = oracle_lib.poly_reproject(d["disp"], (d["cx"], d["cy"], d["cz"]), d["R1"], 0.0, 1000.0,
                                              bool(rectified))
        assert np.array_equal(xyz.view(np.uint32), d[f"xyz_{rectified}"].view(np.uint32))
        assert np.array_equal(mask, d[f"mask_{rectified}"])


def test_roi_fill_fixture(native):
    from oracle import roi as R
    from zim_gb300 import api
    d = np.load(GOLDEN / "roi_fill.npz")
    for r, m in zip(d["rects"], d["masks"]):
        roi = ((r[0], r[1]), (r[2], r[3]), r[4])
        assert np.array_equal(R.fill_rotated_rect(m.shape[0], m.shape[1], roi), m)
        lo, hi = api.roi_source_spans(roi, m.shape[0], m.shape[1])
        cols = np.arange(m.shape[1])
        lib = ((cols[None, :] >= lo[:, None]) & (cols[None, :] <= hi[:, None])).astype(np.uint8) * 255
        assert np.array_equal(lib, m)
