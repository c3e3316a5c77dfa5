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
