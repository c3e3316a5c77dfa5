"""The decode's wrapped-phase arctangent (`phase_atan2`, zim_tiles.cuh): its
coefficients are read from the source and evaluated with FP32 roundings on the
CPU (the same operation sequence as the device code), then checked against
numpy's FP64 arctan2: the accuracy bound the decode's parity margins assume,
and atan2's quadrant and signed-zero rules.  No GPU needed."""
import re
from pathlib import Path

import numpy as np

SRC = Path(__file__).resolve().parents[1] / "zim_gb300" / "csrc" / "zim_tiles.cuh"
PI = np.float32(3.14159265358979323846)


def coefficients():
    text = SRC.read_text()
    body = text[text.index("float phase_atan2(float y, float x)"):]
    body = body[:body.index("\n}\n")]
    first = re.search(r"float p = (-?[0-9.e-]+)f;", body)
    rest = re.findall(r"p = fmaf\(p, s, (-?[0-9.e-]+)f\);", body)
    assert first and len(rest) == 7
    return [np.float32(float(first.group(1)))] + [np.float32(float(c)) for c in rest]


def fma32(a, b, c):
    # one rounding of the exact a * b + c (the FP64 product of two floats is exact)
    return np.float32(np.float64(a) * np.float64(b) + np.float64(c))


def phase_atan2(y, x, coef):
    y, x = np.float32(y), np.float32(x)
    ax, ay = abs(x), abs(y)
    hi, lo = max(ax, ay), min(ax, ay)
    t = np.float32(lo / hi) if hi > 0 else np.float32(0.0)
    s = np.float32(t * t)
    p = coef[0]
    for c in coef[1:]:
        p = fma32(p, s, c)
    r = np.float32(t * p)
    if ay > ax:
        r = np.float32(np.float32(0.5) * PI - r)
    if np.signbit(x):
        r = np.float32(PI - r)
    return np.copysign(r, y)


def test_accuracy_against_fp64():
    coef = coefficients()
    rng = np.random.default_rng(3)
    n = 20000
    ys = (rng.normal(size=n) * 10 ** rng.uniform(-2, 6, n)).astype(np.float32)
    xs = (rng.normal(size=n) * 10 ** rng.uniform(-2, 6, n)).astype(np.float32)
    err = max(abs(float(phase_atan2(y, x, coef)) - float(np.arctan2(np.float64(y), np.float64(x))))
              for y, x in zip(ys, xs))
    # the device divides with __fdividef (2 ulp of the ratio): 4e-7 rad covers both
    assert err < 3e-7, err


def test_quadrants_and_signed_zeros():
    coef = coefficients()
    cases = [(0.0, 1.0), (-0.0, 1.0), (0.0, -1.0), (-0.0, -1.0), (0.0, 0.0), (-0.0, 0.0), (0.0, -0.0),
             (-0.0, -0.0), (1.0, 0.0), (-1.0, 0.0), (1.0, -0.0), (3.0, 3.0), (-3.0, -3.0), (5.0, -5.0),
             (-2.0, 7.0), (7.0, -2.0)]
    for y, x in cases:
        a = phase_atan2(y, x, coef)
        b = np.arctan2(np.float32(y), np.float32(x))
        assert np.signbit(a) == np.signbit(b), (y, x)
        assert abs(float(a) - float(b)) < 4e-7, (y, x, a, b)
