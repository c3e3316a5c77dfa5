"""The batched path against the plain per-pair path: bit-identical outputs for
mixed sizes, encodings, sample types and calibrations, for any tuning."""
import numpy as np
import pytest
import torch

from conftest import scene_data

pytestmark = pytest.mark.gpu

PAIRS = [("config0", {}), ("config1", {"width": 612, "height": 512}),
         ("ref_heterodyne", {"width": 612, "height": 512}), ("config0", {"seed": 5})]


@pytest.fixture(scope="module")
def setup(native):
    from zim_gb300 import api
    ctx = api.Context(0)
    scenes = [scene_data(n, **kw) for n, kw in PAIRS]
    calib_of, calibs = [], []
    for spec, *_ in scenes:
        rig = spec.rig.as_dict()
        key = (spec.rig.width, spec.rig.height, float(rig["K"][0][0, 0]), float(rig["D"][0][0]))
        keys = [k for k, _ in calibs]
        if key not in keys:
            calibs.append((key, rig))
            keys.append(key)
        calib_of.append(keys.index(key))
    return ctx, scenes, calib_of, [r for _, r in calibs]


def _plain(ctx_cache, spec, L, R, rcfg):
    from zim_gb300 import api
    key = id(spec.rig)
    if key not in ctx_cache:
        c = api.Context(0)
        c.set_calibration(spec.rig.as_dict(), True)
        ctx_cache[key] = c
    c = ctx_cache[key]
    dcfg = api.decode_config(**spec.decode_kwargs())
    xyz, mask, disp = api.reconstruct_pair(c, dcfg, rcfg, torch.from_numpy(L).cuda(), torch.from_numpy(R).cuda(),
                                           want_disp=True)
    return xyz.cpu().numpy(), mask.cpu().numpy(), disp.cpu().numpy()


def _batch_pairs(scenes, calib_of):
    from zim_gb300 import api
    from zim_gb300.batch import BatchPair
    out = []
    for (spec, L, R, _), ci in zip(scenes, calib_of):
        dcfg = api.decode_config(**spec.decode_kwargs())
        out.append(BatchPair(dcfg, torch.from_numpy(L).cuda(), torch.from_numpy(R).cuda(), calib=ci))
    return out


@pytest.mark.parametrize("filters", ["default", "median_only", "pxg_updates_mask"])
def test_batch_matches_plain_path(setup, filters):
    from zim_gb300 import api
    from zim_gb300.batch import Batch
    ctx, scenes, calib_of, calibs = setup
    kw = {}
    if filters == "median_only":
        kw = dict(use_px_gaussian=0, use_ror=0)
    elif filters == "pxg_updates_mask":
        kw = dict(px_gaussian_updates_mask=1, radius_search=5.0, radius_min_neighbors=5, radius_window_size=5)
    rcfg = api.recon_config(**kw)
    b = Batch(ctx, calibs)
    pairs = _batch_pairs(scenes, calib_of)
    for p in pairs:
        w, h = b.rect_size(p.calib)
        p.disp = torch.empty((h, w), dtype=torch.float32, device="cuda")
    b.submit(pairs, rcfg)
    b.run()
    torch.cuda.synchronize()
    cache = {}
    for (spec, L, R, _), p in zip(scenes, pairs):
        xyz, mask, disp = _plain(cache, spec, L, R, rcfg)
        assert np.array_equal(p.disp.cpu().numpy(), disp)
        assert np.array_equal(p.mask.cpu().numpy(), mask)
        assert np.array_equal(p.xyz.cpu().numpy(), xyz)
        assert mask.sum() > 1000


def test_batch_grid_filters_match_plain_path(setup):
    """Per-pair grid filters (SOR; SOR + MLS + metric Gaussian; MLS of order
    1 + metric Gaussian; and the submission's own SOR for a pair without a
    filter config) run on the lanes after the batched pixel stages: every
    output equals the whole-pair path's with the pair's full config."""
    from zim_gb300 import api
    from zim_gb300.batch import Batch
    ctx, scenes, calib_of, calibs = setup
    base = dict(use_ror=0)  # pixel Gaussian on: the pixel stages end in it
    sub = api.recon_config(**base, use_sor=1, sor_mean_k=30, sor_std_mul=1.0)
    per_pair = [api.recon_config(**base, use_sor=1, sor_mean_k=50, sor_std_mul=1.0),
                api.recon_config(**base, use_sor=1, sor_mean_k=30, sor_std_mul=1.0, use_mls=1, mls_window_size=7,
                                 mls_spatial_sigma=5.656854, mls_polynomial_order=2, mls_max_radius=8.0,
                                 mls_iterations=1, use_metric_gaussian=1, metric_gaussian_sigma=2.0),
                api.recon_config(**base, use_mls=1, mls_window_size=5, mls_spatial_sigma=2.4, mls_polynomial_order=1,
                                 mls_max_radius=0.0, mls_iterations=3, use_metric_gaussian=1,
                                 metric_gaussian_sigma=1.5),
                None]
    b = Batch(ctx, calibs)
    pairs = _batch_pairs(scenes, calib_of)
    for p, f in zip(pairs, per_pair):
        p.filters = f
    b.submit(pairs, sub)
    b.run()
    torch.cuda.synchronize()
    cache = {}
    for (spec, L, R, _), p, f in zip(scenes, pairs, per_pair):
        xyz, mask, _ = _plain(cache, spec, L, R, f if f is not None else sub)
        assert np.array_equal(p.mask.cpu().numpy(), mask)
        assert np.array_equal(p.xyz.cpu().numpy(), xyz)
        assert mask.sum() > 1000
    # replays are repeatable
    ref = [(p.xyz.clone(), p.mask.clone()) for p in pairs]
    for p in pairs:
        p.xyz.zero_()
    b.run()
    torch.cuda.synchronize()
    for (x, m), p in zip(ref, pairs):
        assert torch.equal(p.xyz, x) and torch.equal(p.mask, m)


def test_batch_tunings_and_autotune_agree(setup):
    from zim_gb300 import api
    from zim_gb300.batch import Batch
    ctx, scenes, calib_of, calibs = setup
    rcfg = api.recon_config()
    b = Batch(ctx, calibs)
    pairs = _batch_pairs(scenes, calib_of)
    b.submit(pairs, rcfg, tuning={"decode_rows": 1, "match_rows": 3, "filter_rows": 2, "ctas_per_sm": 1})
    b.run()
    torch.cuda.synchronize()
    ref = [(p.xyz.clone(), p.mask.clone()) for p in pairs]
    tuning, ms = b.autotune()
    assert ms > 0 and all(v >= 1 for v in tuning.values())
    assert b.tuning() == tuning
    for p in pairs:
        p.xyz.zero_()
        p.mask.zero_()
    b.run()
    b.run()  # replays are repeatable
    torch.cuda.synchronize()
    for (x, m), p in zip(ref, pairs):
        assert torch.equal(p.xyz, x) and torch.equal(p.mask, m)


def test_batch_rejects_bad_submissions(setup):
    from zim_gb300 import api
    from zim_gb300._lib import ZimError
    from zim_gb300.batch import Batch
    ctx, scenes, calib_of, calibs = setup
    b = Batch(ctx, calibs)
    pairs = _batch_pairs(scenes[:1], calib_of[:1])
    with pytest.raises(ZimError) as e:
        b.submit(pairs, api.recon_config(use_sor=1, sor_mean_k=64))
    assert e.value.status == 1  # INVALID_ARG: k + 1 above 64
    bad = _batch_pairs(scenes[1:2], [0])  # 612x512 frames against the 640x480 calibration
    if calibs[0]["width"] != 612:
        with pytest.raises(ZimError):
            b.submit(bad, api.recon_config())
    with pytest.raises(ZimError):
        b.run()  # nothing submitted successfully


def test_batch_destroyed_after_its_context_leaves_no_error(setup):
    """A garbage collector may destroy a context before a batch made on it:
    the batch's destruction must not read the context, nor leave an error
    behind for the thread's next call (a launch check would report it)."""
    from zim_gb300 import api
    from zim_gb300.batch import Batch
    _, scenes, calib_of, calibs = setup
    ctx = api.Context(0)
    b = Batch(ctx, calibs[:1])
    ctx.close()
    b.close()
    spec, L, _, _ = scenes[0]
    c2 = api.Context(0)
    c2.set_calibration(spec.rig.as_dict(), True)
    d = api.decode(c2, api.decode_config(**spec.decode_kwargs()), torch.from_numpy(L).cuda())
    assert int(d["valid"].sum().item()) > 0
