"""The reference's own CUDA kernels as a second witness on the GPU.

oracle/ref_build.py compiles the reference's JSLAB_PhaseShiftDecoder_V2_GPU.cu,
JSLAB_PhaseEpipolarReconstructor_V2_GPU.cu and JSLAB_MLS_Filter.cu (device code
only) into cubins; oracle/ref_cuda.py launches their kernels here, as the
reference's launchers do.  Each stage gets the same input three ways -- the
reference's kernel, this library's kernel and the FP64 oracle -- so the tests
show both that the oracle restates the reference's GPU code and that the
library matches the reference's GPU code directly.  Tolerances are those of
the oracle parity tests (decisions bit-exact except the pixels the oracle flags
within 1e-5 of a threshold; phase 1e-5 rad; points 1e-5 relative), except MLS:
the reference's kernel accumulates absolute coordinates (~900 mm) in FP32, so
its own rounding reaches ~0.1 mm; there the test bounds the reference kernel's
distance from the FP64 evaluation and shows the library's is smaller.
The cubins exist where the reference's sources were present when build() ran;
elsewhere these tests skip.
"""
import math

import numpy as np
import pytest
import torch

from conftest import scene_data

EPS = 1e-5
SCENE = ("ref_heterodyne", {"width": 612, "height": 512})


@pytest.fixture(scope="module")
def rc():
    from oracle import ref_cuda
    if not ref_cuda.available():
        pytest.skip("the reference's CUDA kernels were not built here (no reference sources at build time)")
    return ref_cuda.RefCuda()


def f64_phase(base, res):
    return 2 * math.pi * base.cpu().numpy().astype(np.float64) + res.cpu().numpy().astype(np.float64)


@pytest.mark.gpu
def test_decode_kernel_witness(ctx, oracle_lib, rc):
    """decodeKernel (double precision, fused 3x3 pre-blur, heterodyne unwrap)
    against zim_decode and the oracle, on both cameras' u8 stacks."""
    from oracle import ref_cuda
    from zim_gb300 import api
    spec, L, R, _ = scene_data(SCENE[0], **SCENE[1])
    kw = spec.decode_kwargs()
    cfg = api.decode_config(**kw)
    ocfg = oracle_lib.make_decode_cfg(**kw)
    for frames in (L, R):
        # the decoder's default (Config::avg_three_phase = true, JSLAB_PhaseShiftDecoder.h:42)
        # averages the three unwrapped phases, as this scene's configs do
        rp, rk, rmod = ref_cuda.decode(rc, torch.from_numpy(frames).cuda(), kw["shift_num"], kw["freq"],
                                       kw["modulation_threshold"], kw["preblur_sigma"],
                                       avg_three=kw.get("avg_three_phase", True))
        rp, rk, rmod = rp.cpu().numpy(), rk.cpu().numpy(), rmod.cpu().numpy()
        ph, k, mod, valid, near = oracle_lib.decode(ocfg, frames, eps=EPS)
        d = api.decode(ctx, cfg, torch.from_numpy(frames).cuda())
        gk, gv, gr = d["order"].cpu().numpy(), d["valid"].cpu().numpy(), d["residual"].cpu().numpy()
        nearb = near != 0
        # the reference kernel writes phase and order only where all three
        # modulations pass: its validity is where it wrote a non-zero phase
        rv = (rp != 0).astype(np.uint8)
        # 1. the oracle restates the reference's GPU decoder
        assert ((rv != valid) & ~nearb).sum() == 0
        both = (valid > 0) & (rv > 0)
        assert ((rk != k) & both & ~nearb).sum() == 0
        okp = both & ~nearb & (rk == k)
        assert np.abs(rp - ph)[okp].max() <= 1e-9
        assert np.abs(rmod - mod)[~nearb].max() <= 1e-9
        # 2. this library against the reference's GPU decoder directly
        vmis = (gv != rv) & ~nearb
        kmis = (gk != rk) & (gv > 0) & (rv > 0) & ~nearb
        print("decode witness: valid", int(rv.sum()), "near", int(nearb.sum()), "valid mismatch", int(vmis.sum()),
              "order mismatch", int(kmis.sum()))
        assert vmis.sum() == 0 and kmis.sum() == 0
        sel = (gv > 0) & (rv > 0) & ~nearb & (gk == rk)
        err = np.abs(gr.astype(np.float64) - (rp - 2 * math.pi * rk))[sel]
        print("  phase max err vs reference kernel", float(err.max()))
        assert err.max() <= 1e-5
        gm = d["mod"].cpu().numpy().astype(np.float64)
        assert (np.abs(gm - rmod)[~nearb] / np.maximum(1.0, np.abs(rmod[~nearb]))).max() <= 1e-5


def rectified(ctx, oracle, spec, L, R):
    from zim_gb300 import api
    rig = spec.rig.as_dict()
    ctx.set_calibration(rig, True)
    cfg = api.decode_config(**spec.decode_kwargs())
    out = []
    for cam, fr in enumerate((L, R)):
        d = api.decode(ctx, cfg, torch.from_numpy(fr).cuda())
        out.append(api.rectify(ctx, cam, d["order"], d["residual"], True))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("rect", [True, False])
def test_reconstruct_kernels_witness(ctx, oracle_lib, rc, rect):
    """buildOrderRangeKernel + stereoMatchKernel, medianFilter5x5Kernel,
    reprojectTo3DKernel, gaussianFilterKernel and radiusOutlierKernel, each
    fed the same input as this library's stage and the oracle's."""
    from oracle import ref_cuda
    from zim_gb300 import api
    spec, L, R, _ = scene_data(SCENE[0], **SCENE[1])
    rl, rr = rectified(ctx, oracle_lib, spec, L, R)
    lph, rph = f64_phase(rl[0], rl[1]), f64_phase(rr[0], rr[1])
    lk, rk = rl[2], rr[2]
    # matching
    rdisp = ref_cuda.stereo_match(rc, torch.from_numpy(lph).cuda(), torch.from_numpy(rph).cuda(), lk.contiguous(),
                                  rk.contiguous(), spec.pha_f, 1.0).cpu().numpy()
    od, ob, near = oracle_lib.stereo_match(lph, rph, lk.cpu().numpy(), rk.cpu().numpy(), spec.pha_f, 1.0, eps=EPS)
    gd, gb = api.match(ctx, rl, rr, spec.pha_f, 1.0)
    gd, gb = gd.cpu().numpy(), gb.cpu().numpy()
    nearm = near != 0
    # the reference kernel and the oracle: both double; same matches, the
    # kernel's disparity the oracle's rounded to float (within one float ulp)
    assert (((rdisp == 0) != (od == 0)) & ~nearm).sum() == 0
    both = (rdisp != 0) & (od != 0) & ~nearm
    assert (np.abs(rdisp.astype(np.float64) - od)[both] <= np.spacing(np.abs(od[both]).astype(np.float32))).all()
    # the library against the reference kernel: same matches; a different
    # column is only possible at a tie the oracle flags
    dmis = ((rdisp == 0) != (gd == 0)) & ~nearm
    valid = (rdisp != 0) & (gd != 0) & ~nearm
    derr = np.abs(gd.astype(np.float64) - rdisp)[valid]
    print("match witness: matched", int((rdisp != 0).sum()), "near", int(nearm.sum()), "presence mismatch",
          int(dmis.sum()), "disp max err", float(derr.max()))
    assert dmis.sum() == 0
    assert derr.max() <= 2e-4
    # median + reprojection on the reference kernel's disparity
    rdisp_t = torch.from_numpy(rdisp).cuda()
    rmed = ref_cuda.median5(rc, rdisp_t)
    rcfg = api.recon_config(use_rectified_coords=int(rect))
    gmed, gxyz, gmask = api.median_reproject(ctx, rcfg, rdisp_t)
    assert torch.equal(gmed, rmed)
    rxyz, rP = ref_cuda.reproject(rc, rmed, ctx.Q.ravel(), ctx.R1.ravel(), 0.0, 1000.0, rect)
    oxyz, omask, rnear = oracle_lib.reproject(rmed.cpu().numpy(), ctx.Q, ctx.R1, 0.0, 1000.0, rect, eps=EPS)
    rxn, rPn, gxn, gmn = rxyz.cpu().numpy(), rP.cpu().numpy(), gxyz.cpu().numpy(), gmask.cpu().numpy()
    # the reference kernel and the oracle (double, rounded to float; the
    # kernel's products may fuse): masks equal except flagged depth-gate
    # decisions, points within one float ulp
    assert ((rPn != omask) & (rnear == 0)).sum() == 0
    bo = (rPn > 0) & (omask > 0)
    assert (np.abs(rxn[bo] - oxyz[bo]) <= np.spacing(np.abs(oxyz[bo]))).all()
    assert ((gmn != rPn) & (rnear == 0)).sum() == 0
    both = (gmn > 0) & (rPn > 0)
    rel = np.abs(gxn[both] - rxn[both]) / np.maximum(1.0, np.abs(rxn[both]))
    print("reproject witness: points", int(both.sum()), "max rel err", float(rel.max()))
    assert rel.max() <= 1e-5
    # point-cloud Gaussian (the GPU launcher's semantics: the mask is updated)
    gx2, gm2 = api.filter_px_gaussian(ctx, rxyz, rP, True)
    rx2, rm2 = ref_cuda.px_gaussian(rc, rxyz, rP)
    ox2, om2, gnear = oracle_lib.px_gaussian(rxn, rPn, True, eps=EPS)
    gm2n, rm2n = gm2.cpu().numpy(), rm2.cpu().numpy()
    assert ((gm2n != rm2n) & (gnear == 0)).sum() == 0
    sel = (gm2n > 0) & (rm2n > 0) & (gnear == 0)
    e2 = np.abs(gx2.cpu().numpy()[sel].astype(np.float64) - rx2.cpu().numpy()[sel])
    ulps = np.spacing(np.abs(rx2.cpu().numpy()[sel]).astype(np.float32))
    print("gaussian witness: points", int(sel.sum()), "max err mm", float(e2.max()))
    assert (e2 <= 4 * ulps + 1e-6).all()
    # radius outlier filter on the reference kernel's Gaussian output
    for (r, mn, win) in ((5.0, 10, 10), (3.0, 5, 5)):
        gx3, gm3 = api.filter_ror(ctx, rx2, rm2, r, mn, win)
        rx3, rm3 = ref_cuda.ror(rc, rx2, rm2, r, mn, win)
        _, om3, rnr = oracle_lib.ror(rx2.cpu().numpy(), rm2n, r, mn, win, eps=EPS)
        gm3n, rm3n = gm3.cpu().numpy(), rm3.cpu().numpy()
        # the kernel's squared distances may fuse: decisions equal except flagged ones
        assert ((rm3n != om3) & (rnr == 0)).sum() == 0
        mis = gm3n != rm3n
        print("ror witness", r, mn, win, "kept", int(rm3n.sum()), "mismatch", int(mis.sum()))
        assert (mis & (rnr == 0)).sum() == 0
        keep = (gm3n > 0) & (rm3n > 0)
        assert np.array_equal(gx3.cpu().numpy()[keep], rx3.cpu().numpy()[keep])


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 1, 0])
def test_mls_kernel_witness(ctx, oracle_lib, rc, order):
    """mlsKernel (the reference's GPU MLS, FP32 about absolute coordinates)
    against the library's MLS and the reference's MLS evaluated in FP64 (the
    oracle, pinned to it on the CPU): the reference kernel's own FP32 rounding
    stays within 0.25 mm of the FP64 evaluation; the library's stays within
    1e-5 mm + 2 ulps (flagged points aside) and below the reference kernel's
    error on the bulk of the cloud."""
    from oracle import ref_cuda
    from zim_gb300 import api
    spec, L, R, _ = scene_data(SCENE[0], **SCENE[1])
    rl, rr = rectified(ctx, oracle_lib, spec, L, R)
    disp, _ = api.match(ctx, rl, rr, spec.pha_f, 1.0, want_best=False)
    _, xyz, mask = api.median_reproject(ctx, api.recon_config(), disp)
    w, sig, rad = 7, 5.656854, 8.0  # the 5 MP settings scaled to this 612 px scene (4x the pixel spacing)
    rout = ref_cuda.mls(rc, xyz, mask, w, sig, order, rad).cpu().numpy().astype(np.float64)
    gout = api.filter_mls(ctx, xyz, mask, w, sig, order, rad, 1).cpu().numpy().astype(np.float64)
    ox, near = oracle_lib.mls(xyz.cpu().numpy(), mask.cpu().numpy(), w, sig, order, rad, 1, eps=EPS)
    m = mask.cpu().numpy() > 0
    sel = m & (near == 0)
    er = np.abs(rout - ox).max(axis=-1)
    eg = np.abs(gout - ox).max(axis=-1)
    big = np.abs(ox).max(axis=-1).astype(np.float32)
    print(f"mls o{order} witness: points {int(m.sum())}, reference kernel vs FP64 max {er[sel].max():.3e} "
          f"rms {np.sqrt((er[sel] ** 2).mean()):.3e} mm; library vs FP64 max {eg[sel].max():.3e} "
          f"rms {np.sqrt((eg[sel] ** 2).mean()):.3e} mm")
    assert er[sel].max() <= 0.25
    assert (eg[sel] <= 1e-5 + 2 * np.spacing(big[sel])).all()
    assert np.sqrt((eg[sel] ** 2).mean()) < np.sqrt((er[sel] ** 2).mean())
    # invalid points pass through unchanged in both
    assert np.array_equal(rout[~m], xyz.cpu().numpy()[~m].astype(np.float64))
