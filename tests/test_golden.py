"""The committed golden fixtures (tests/golden/, written by make_golden.py).

Fixtures with source "reference" hold the reference's own outputs (its
sources compiled here as oracle/_ref); the oracle reproduces them byte for
byte (decode, matching, the whole pair up to the reprojected cloud), within
float rounding of the reference's float sums (its pixel Gaussian), and within
one float ulp for MLS (against the reference's MLS source evaluated in
double).  Fixtures with source "oracle" (Gray code, hierarchical unwrapping,
polynomial branch mix, ROI rasteriser: computations the reference does not
have) are reproduced byte for byte.  These tests need no reference tree: they
read the committed fixtures only."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
DECODES = sorted(p.name for p in GOLDEN.glob("decode_*.npz"))


REFERENCE_SOURCED = ("decode_heterodyne.npz", "decode_heterodyne_hdr.npz", "match_config0_rows.npz",
                     "recon_ref_pair.npz", "mls_ref_cloud.npz")


def test_fixtures_present():
    assert len(DECODES) >= 4
    for n in ("match_config0_rows.npz", "poly_reproject.npz", "roi_fill.npz", "recon_ref_pair.npz",
              "mls_ref_cloud.npz"):
        assert (GOLDEN / n).exists(), n
    for p in sorted(GOLDEN.glob("*.npz")):
        src = str(np.load(p)["source"])
        assert src == ("reference" if p.name in REFERENCE_SOURCED else "oracle"), (p.name, src)


def _rig(d):
    rig = json.loads(str(d["rig"]))
    for k in ("K", "D"):
        rig[k] = [np.asarray(v, np.float64) for v in rig[k]]
    for k in ("R", "t"):
        rig[k] = np.asarray(rig[k], np.float64)
    return rig


def test_oracle_reproduces_reference_pair(oracle_lib):
    from oracle import pipeline as P
    d = np.load(GOLDEN / "recon_ref_pair.npz")
    rect = P.Rectification(_rig(d), True)
    kw = json.loads(str(d["decode_cfg"]))
    cfg = oracle_lib.make_decode_cfg(**kw)
    r = []
    for cam, fr in enumerate((d["left"], d["right"])):
        ph, k, _, _, _ = oracle_lib.decode(cfg, fr)
        r.append(oracle_lib.rectify_decoded(ph, k, *rect.maps[cam], True))
    od, _, _ = oracle_lib.stereo_match(r[0][0], r[1][0], r[0][1], r[1][1], int(d["pha_f"]))
    dm = oracle_lib.median5(od.astype(np.float32))
    assert np.array_equal(dm, d["disp"])
    xyz, mask, _ = oracle_lib.reproject(dm, rect.Q, rect.R1, 0.0, 1000.0, True)
    assert np.array_equal(mask, d["raw_mask"]) and np.array_equal(xyz, d["raw_xyz"])
    c = json.loads(str(d["recon_cfg"]))
    g, _, gnear = oracle_lib.px_gaussian(xyz, mask)
    fx, fm, rnear = oracle_lib.ror(g, mask, c["radius_search"], c["radius_min_neighbors"], c["radius_window_size"])
    ok = (rnear == 0)
    assert np.array_equal(fm[ok], d["mask"][ok]) and rnear.sum() <= 3
    sel = ok & (fm > 0)
    big = np.abs(d["xyz"][sel]).max(axis=-1, keepdims=True).astype(np.float32)
    assert (np.abs(fx[sel] - d["xyz"][sel]) <= 4 * np.spacing(big)).all()
    assert d["mask"].sum() > 0.5 * d["mask"].size


def test_oracle_mls_reproduces_reference_fixture(oracle_lib):
    d = np.load(GOLDEN / "mls_ref_cloud.npz")
    m = d["mask"] > 0
    for run, (w, s, o, r, it) in json.loads(str(d["runs"])).items():
        oo, _ = oracle_lib.mls(d["xyz"], d["mask"], w, s, o, r, it)
        ref = d[f"ref_f64_{run}"]
        ulp = np.spacing(np.abs(oo).max(axis=-1).astype(np.float32))
        assert (np.abs(ref.astype(np.float64) - oo).max(axis=-1)[m] <= ulp[m]).all(), run


@pytest.mark.parametrize("name", DECODES)
def test_oracle_decode_reproduces_fixture(oracle_lib, name):
    d = np.load(GOLDEN / name)
    kw = json.loads(str(d["cfg"]))
    ph, k, mod, valid, near = oracle_lib.decode(oracle_lib.make_decode_cfg(**kw), d["frames"])
    for a, b in ((k, d["order"]), (valid, d["valid"]), (near, d["near"])):
        assert np.array_equal(a, b)
    if kw.get("enable_hdr"):
        # the reference's cached SVD pseudo-inverses against per-pixel normal equations
        assert np.abs(ph - d["phase"]).max() <= 1e-9 and np.abs(mod - d["mod"]).max() <= 1e-12
    else:
        assert np.array_equal(ph, d["phase"]) and np.array_equal(mod, d["mod"])


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
