"""Writes the golden fixtures of this directory from the FP64 oracle.

    python tests/golden/make_golden.py

Small seeded cases (frames cropped from the synthetic scenes, rectified phase
rows, polynomial maps, rotated rectangles) with the oracle's outputs.  The
reference ships no golden vectors; these pin the oracle and the CUDA path to
fixed bytes so a later change to either shows up as a diff.  Deterministic:
rerunning rewrites identical files.
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
from oracle import roi as OR  # noqa: E402
from polycase import random_disparity, random_maps  # noqa: E402
from zim_gb300 import synth  # noqa: E402

CROP = (slice(200, 264), slice(272, 368))  # 64 x 96 pixels


def decode_case(name, spec, **extra):
    frames = np.ascontiguousarray(spec.render(0)[(slice(None),) + CROP])
    kw = dict(spec.decode_kwargs(), **extra)
    ph, k, mod, valid, near = O.decode(O.make_decode_cfg(**kw), frames)
    np.savez_compressed(HERE / f"decode_{name}.npz", frames=frames, cfg=json.dumps(kw), phase=ph, order=k,
                        mod=mod, valid=valid, near=near)


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
    disp, best, near = O.stereo_match(lph, rph, lk, rk, spec.pha_f)
    np.savez_compressed(HERE / "match_config0_rows.npz", lph=lph, lk=lk, rph=rph, rk=rk, pha_f=spec.pha_f,
                        disp=disp, best=best, near=near)


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
    np.savez_compressed(HERE / "poly_reproject.npz", cx=cx, cy=cy, cz=cz, branch=br, disp=d, R1=R1, **out)


def roi_case():
    rng = np.random.default_rng(5)
    rows, cols = 120, 160
    rects, masks = [], []
    for _ in range(12):
        roi = ((float(rng.uniform(0, cols)), float(rng.uniform(0, rows))),
               (float(rng.uniform(5, 80)), float(rng.uniform(5, 80))), float(rng.uniform(-90, 90)))
        rects.append([roi[0][0], roi[0][1], roi[1][0], roi[1][1], roi[2]])
        masks.append(OR.fill_rotated_rect(rows, cols, roi))
    np.savez_compressed(HERE / "roi_fill.npz", rects=np.array(rects), masks=np.array(masks))


def main():
    O.build()
    decode_case("graycode_complementary", synth.config0())
    decode_case("hierarchical_u16", synth.config1())
    decode_case("heterodyne", synth.ref_heterodyne())
    bright = synth.ref_heterodyne(21, 612, 512)  # 8-bit peaks clip
    bright.A, bright.B = (170.0, 220.0), (80.0, 120.0)
    decode_case("heterodyne_hdr", bright, enable_hdr=True, hdr_saturation_gray=255.0, hdr_min_amplitude=2.0)
    match_case()
    poly_case()
    roi_case()
    for p in sorted(HERE.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
