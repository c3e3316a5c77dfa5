"""Writes the golden fixtures of this directory.

    python tests/golden/make_golden.py

Where the reference has the computation, a fixture holds the REFERENCE's own
outputs, computed by its sources compiled here (oracle/_ref, built by
oracle/ref_build.py); every such fixture records `source = "reference"` and
the script first checks that the oracle reproduces it (it stops otherwise):

* decode_heterodyne.npz, decode_heterodyne_hdr.npz: the reference decoder V2
  (JSLAB_PhaseShiftDecoder_V2.cpp) on 8-bit heterodyne 121/110/120 frames,
  plain and HDR: phase before the post-smooth, order, modulation, validity;
* match_config0_rows.npz: the reference stereoMatch
  (JSLAB_PhaseEpipolarReconstructor_V2.cpp:933-1006) on rectified phase rows;
* recon_ref_pair.npz: a whole 160x128 stereo pair (heterodyne 25/20/24, 3
  steps) through the reference decoder and setCalibrationParams / setData /
  startCalculate: the median disparity, the reprojected cloud and the cloud
  after its pixel Gaussian and radius outlier filter;
* mls_ref_cloud.npz: a 64x96 cloud through the reference MLS source
  evaluated in double (oracle/ref_mls_f64.cpp), at the
  5 MP workload's parameters (half-window 7, sigma 2/sqrt(2), order 2,
  cut-off 2 mm) and at order 1 with a 4 mm cut-off.

Where the reference has no such computation (Gray code, hierarchical
unwrapping, the per-pixel polynomial maps' random branch mix, the ROI
rasteriser), the fixture holds the FP64 oracle's outputs and records
`source = "oracle"`.  `near` arrays are always the oracle's decision-margin
flags (the reference has no such notion).  Deterministic: rerunning rewrites
identical arrays.
"""
import json
import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from oracle import oracle as O  # noqa: E402
from oracle import pipeline as P  # noqa: E402
from oracle import ref as Z  # noqa: E402
from oracle import roi as OR  # noqa: E402
from polycase import random_disparity, random_maps  # noqa: E402
from zim_gb300 import synth  # noqa: E402

CROP = (slice(200, 264), slice(272, 368))  # 64 x 96 pixels

RECON_PAIR = dict(seed=8, width=160, height=128, freq=(25, 20, 24), steps=3)
RECON_CFG = dict(radius_search=4.0, radius_min_neighbors=6, radius_window_size=5)


def oracle_decode_case(name, spec, **extra):
    frames = np.ascontiguousarray(spec.render(0)[(slice(None),) + CROP])
    kw = dict(spec.decode_kwargs(), **extra)
    ph, k, mod, valid, near = O.decode(O.make_decode_cfg(**kw), frames)
    np.savez_compressed(HERE / f"decode_{name}.npz", frames=frames, cfg=json.dumps(kw), phase=ph, order=k,
                        mod=mod, valid=valid, near=near, source="oracle")


def reference_decode_case(name, spec, phase_tol=0.0, **extra):
    frames = np.ascontiguousarray(spec.render(0)[(slice(None),) + CROP])
    kw = dict(spec.decode_kwargs(), **extra)
    _, raw, k, mod, valid = Z.decode(Z.decode_cfg(**kw), frames)
    oph, ok, omod, ov, near = O.decode(O.make_decode_cfg(**kw), frames)
    assert np.array_equal(k, ok) and np.array_equal(valid, ov), name
    assert np.abs(raw - oph).max() <= phase_tol and np.abs(mod - omod).max() <= max(phase_tol, 0.0) * 1e-3, name
    np.savez_compressed(HERE / f"decode_{name}.npz", frames=frames, cfg=json.dumps(kw), phase=raw, order=k,
                        mod=mod, valid=valid, near=near, source="reference")


def match_case():
    spec = synth.config0()
    rig = spec.rig.as_dict()
    c = O.make_calib(rig["K"], rig["D"], rig["R"], rig["t"], rig["width"], rig["height"])
    R1, R2, P1, P2, Q, w, h = O.rectification(c, True)
    cfg = O.make_decode_cfg(**spec.decode_kwargs())
    rect = []
    for cam, (Rk, Pk) in enumerate(((R1, P1), (R2, P2))):
        ph, k, _, _, _ = O.decode(cfg, spec.render(cam))
        mx, my = O.init_rectify_map(rig["K"][cam], rig["D"][cam], Rk, Pk, w, h)
        rect.append(O.rectify_decoded(ph, k, mx, my, True))
    rows = slice(h // 2 - 8, h // 2 + 8)
    lph, lk = rect[0][0][rows], rect[0][1][rows]
    rph, rk = rect[1][0][rows], rect[1][1][rows]
    disp = Z.stereo_match(lph, rph, lk, rk, spec.pha_f)
    odisp, best, near = O.stereo_match(lph, rph, lk, rk, spec.pha_f)
    assert np.array_equal(disp, odisp)
    np.savez_compressed(HERE / "match_config0_rows.npz", lph=lph, lk=lk, rph=rph, rk=rk, pha_f=spec.pha_f,
                        disp=disp, best=best, near=near, source="reference")


def recon_pair_case():
    spec = synth.ref_heterodyne(**RECON_PAIR)
    rig = spec.rig.as_dict()
    L, R = spec.render(0), spec.render(1)
    kw = spec.decode_kwargs()
    dl, dr = Z.decode(Z.decode_cfg(**kw), L), Z.decode(Z.decode_cfg(**kw), R)
    rec = Z.Reconstructor(Z.recon_cfg(**RECON_CFG), rig)
    xyz, mask, disp, _, (raw_xyz, raw_mask) = rec.run(dl[0], dr[0], dl[2], dr[2], dl[3], spec.pha_f)
    # the oracle: same disparity and reprojection bit for bit
    rect = P.Rectification(rig, True)
    oxyz, omask = P.run_pair(kw, spec.pha_f, L, R, rect, P.Filters())
    assert np.array_equal(raw_mask, omask) and np.array_equal(raw_xyz, oxyz)
    assert np.array_equal(disp.astype(np.float32).astype(np.float64), disp)
    # near flags of the matching (the oracle's, on the same rectified inputs)
    cfg = O.make_decode_cfg(**kw)
    r = []
    for cam, fr in enumerate((L, R)):
        ph, k, _, _, _ = O.decode(cfg, fr)
        r.append(O.rectify_decoded(ph, k, *rect.maps[cam], True))
    _, _, match_near = O.stereo_match(r[0][0], r[1][0], r[0][1], r[1][1], spec.pha_f)
    np.savez_compressed(HERE / "recon_ref_pair.npz", left=L, right=R, rig=json.dumps(
        {k: (np.asarray(v).tolist() if not isinstance(v, (int, float)) else v) for k, v in rig.items()}),
        decode_cfg=json.dumps(kw), recon_cfg=json.dumps(RECON_CFG), pha_f=spec.pha_f,
        disp=disp.astype(np.float32), raw_xyz=raw_xyz, raw_mask=raw_mask, xyz=xyz, mask=mask,
        match_near=match_near, source="reference")


MLS_RUNS = {"w7_s1.414_o2_r2": (7, 2.0 / math.sqrt(2.0), 2, 2.0, 1), "w7_s2.83_o1_r4": (7, 2.0 * math.sqrt(2.0), 1, 4.0, 1)}


def mls_case():
    spec = synth.config1(1, 1224, 1024)
    rect = P.Rectification(spec.rig.as_dict(), True)
    xyz, mask = P.run_pair(spec.decode_kwargs(), spec.pha_f, spec.render(0), spec.render(1), rect, P.Filters())
    y0, x0 = rect.h // 2 - 32, rect.w // 2 - 48
    cx, cm = np.ascontiguousarray(xyz[y0:y0 + 64, x0:x0 + 96]), np.ascontiguousarray(mask[y0:y0 + 64, x0:x0 + 96])
    out = {"xyz": cx, "mask": cm, "runs": json.dumps(MLS_RUNS), "source": "reference"}
    for name, (w, s, o, r, it) in MLS_RUNS.items():
        f64 = Z.mls_f64(cx, cm, w, s, o, r, it)
        oo, near = O.mls(cx, cm, w, s, o, r, it)
        d = np.abs(f64.astype(np.float64) - oo).max(axis=-1)[cm > 0]
        ulp = np.spacing(np.abs(oo).max(axis=-1).astype(np.float32))[cm > 0]
        assert (d <= ulp).all(), name
        out[f"ref_f64_{name}"] = f64
        out[f"near_{name}"] = near
    np.savez_compressed(HERE / "mls_ref_cloud.npz", **out)


def poly_case():
    H, W = 16, 24
    cx, cy, cz, br = random_maps(H, W, seed=21)
    d = random_disparity(H, W, br, seed=22)
    a = 0.2
    R1 = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
    out = {}
    for rectified in (1, 0):
        xyz, mask = O.poly_reproject(d, (cx, cy, cz), R1, 0.0, 1000.0, bool(rectified))
        out[f"xyz_{rectified}"], out[f"mask_{rectified}"] = xyz, mask
    np.savez_compressed(HERE / "poly_reproject.npz", cx=cx, cy=cy, cz=cz, branch=br, disp=d, R1=R1, **out,
                        source="oracle")


def roi_case():
    rng = np.random.default_rng(5)
    rows, cols = 120, 160
    rects, masks = [], []
    for _ in range(12):
        roi = ((float(rng.uniform(0, cols)), float(rng.uniform(0, rows))),
               (float(rng.uniform(5, 80)), float(rng.uniform(5, 80))), float(rng.uniform(-90, 90)))
        rects.append([roi[0][0], roi[0][1], roi[1][0], roi[1][1], roi[2]])
        masks.append(OR.fill_rotated_rect(rows, cols, roi))
    np.savez_compressed(HERE / "roi_fill.npz", rects=np.array(rects), masks=np.array(masks), source="oracle")


def main():
    O.build()
    if not Z.available():
        sys.exit("the reference sources are needed (oracle/_ref): run where they are mounted")
    oracle_decode_case("graycode_complementary", synth.config0())
    oracle_decode_case("hierarchical_u16", synth.config1())
    reference_decode_case("heterodyne", synth.ref_heterodyne())
    bright = synth.ref_heterodyne(21, 612, 512)  # 8-bit peaks clip
    bright.A, bright.B = (170.0, 220.0), (80.0, 120.0)
    reference_decode_case("heterodyne_hdr", bright, phase_tol=1e-9, enable_hdr=True, hdr_saturation_gray=255.0,
                          hdr_min_amplitude=2.0)
    match_case()
    recon_pair_case()
    mls_case()
    poly_case()
    roi_case()
    for p in sorted(HERE.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
