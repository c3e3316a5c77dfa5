"""ROI rasterisation on the CPU: zim_roi_source_spans (the library's per-row
span fill of a rotated rectangle) against the oracle's per-pixel containment
test plus outline, over random rectangles on and off the image."""
import numpy as np
import pytest

from oracle import roi as R


def spans_of(mask):
    rows = mask.shape[0]
    lo = np.full(rows, np.iinfo(np.int32).max, np.int64)
    hi = np.full(rows, np.iinfo(np.int32).min, np.int64)
    for y in range(rows):
        xs = np.nonzero(mask[y])[0]
        if xs.size:
            assert xs.size == xs[-1] - xs[0] + 1, "a convex fill is one run per row"
            lo[y], hi[y] = xs[0], xs[-1]
    return lo, hi


def test_rotated_rect_points_axis_aligned():
    p = R.rotated_rect_points(50, 40, 20, 10, 0)
    assert [(float(a), float(b)) for a, b in p] == [(40, 45), (40, 35), (60, 35), (60, 45)]
    p = R.rotated_rect_points(50, 40, 20, 10, 90)
    assert np.allclose([(float(a), float(b)) for a, b in p], [(45, 30), (55, 30), (55, 50), (45, 50)], atol=1e-5)


def test_axis_aligned_fill_is_inclusive(native):
    from zim_gb300 import api
    lo, hi = api.roi_source_spans(((50, 40), (20, 10), 0), 100, 120)
    rows = np.nonzero(lo <= hi)[0]
    assert rows.min() == 35 and rows.max() == 45
    assert (lo[35:46] == 40).all() and (hi[35:46] == 60).all()


@pytest.mark.parametrize("seed", range(6))
def test_spans_match_containment_fill(native, seed):
    from zim_gb300 import api
    rng = np.random.default_rng(seed)
    rows, cols = 120, 160
    for _ in range(40):
        roi = ((rng.uniform(-20, cols + 20), rng.uniform(-20, rows + 20)),
               (rng.uniform(0, 90), rng.uniform(0, 90)), rng.uniform(-180, 180))
        lo, hi = api.roi_source_spans(roi, rows, cols)
        olo, ohi = spans_of(R.fill_rotated_rect(rows, cols, roi))
        empty = lo > hi
        assert np.array_equal(empty, olo > ohi), roi
        assert np.array_equal(lo[~empty], olo[~empty]) and np.array_equal(hi[~empty], ohi[~empty]), roi
