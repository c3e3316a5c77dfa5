"""Python host API over the zim_gb300 C ABI.

Two layers:

* thin functions (``decode``, ``rectify``, ``match``, ...) that call one C-ABI
  entry point on torch CUDA tensors, on the current torch stream;
* mirrors of the reference's classes with the same names, argument meaning and
  error behaviour (PhaseShiftGrayCode3D/src/): ``JSLAB_PhaseShiftDecoder``
  (JSLAB_PhaseShiftDecoder.h:10-92), ``JSLAB_StereoCalibParams_V1``
  (JSLAB_StereoCalibParams_V1.h:9-20) and ``JSLAB_PhaseEpipolarReconstructor_V2``
  (JSLAB_PhaseEpipolarReconstructor_V2.h:11-171).

Everything runs on the GPU through libzim_gb300.so; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
import enum
import math
from dataclasses import dataclass, field, fields
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib
from ._lib import (ENC_GRAYCODE, ENC_GRAYCODE_COMPLEMENTARY, ENC_HETERODYNE3, ENC_HIERARCHICAL, SAMPLE_U8,
                   SAMPLE_U16, ZimError, check)

__all__ = ["Context", "decode_config", "recon_config", "calib_struct", "decode", "decode_phase_f64",
           "rectify", "match", "median_reproject", "filter_px_gaussian", "filter_ror", "filter_mls", "filter_sor",
           "filter_metric_gaussian", "compact_points", "pack_ply", "rectify_image", "rotated_rect",
           "roi_source_spans", "RectifiedROI", "prepare_roi", "reconstruct_roi", "fit_poly_calib",
           "JSLAB_StereoCalib_V2", "reconstruct_pair", "reconstruct_pair_host", "DecodedPhase",
           "JSLAB_PhaseShiftDecoder", "JSLAB_PhaseShiftDecoderV2_GPU", "JSLAB_StereoCalibParams_V1",
           "JSLAB_StereoCalibParams_V2",
           "JSLAB_PhaseEpipolarReconstructor_V2", "ZimError", "ENC_HETERODYNE3", "ENC_HIERARCHICAL",
           "ENC_GRAYCODE", "ENC_GRAYCODE_COMPLEMENTARY"]


def _p(t) -> Optional[C.c_void_p]:
    if t is None:
        return None
    if isinstance(t, torch.Tensor):
        if not t.is_cuda:
            raise ValueError("device tensor expected")
        if not t.is_contiguous():
            raise ValueError("contiguous tensor expected")
        return C.c_void_p(t.data_ptr())
    if isinstance(t, np.ndarray):
        return t.ctypes.data_as(C.c_void_p)
    return t


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class Context:
    """Owns a zim_ctx: calibration, rectification maps and scratch on one GPU."""

    def __init__(self, device: int = 0):
        self._L = _lib.load()
        h = C.c_void_p()
        st = self._L.zim_create(int(device), C.byref(h))
        if st != _lib.OK:
            raise ZimError(st, "zim_create failed")
        self.h = h
        self.device = device
        self.rect_w = self.rect_h = 0
        self.src_w = self.src_h = 0

    def close(self):
        if getattr(self, "h", None):
            self._L.zim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st):
        check(st, self.h)

    def set_calibration(self, calib, full_left: bool = True):
        cs = calib if isinstance(calib, _lib.StereoCalib) else calib_struct(**calib)
        self.check(self._L.zim_set_calibration(self.h, C.byref(cs), int(bool(full_left))))
        R1 = np.zeros(9); R2 = np.zeros(9); P1 = np.zeros(12); P2 = np.zeros(12); Q = np.zeros(16)
        w = C.c_int(); h = C.c_int()
        self.check(self._L.zim_get_rectification(self.h, _p(R1), _p(R2), _p(P1), _p(P2), _p(Q), C.byref(w),
                                                 C.byref(h)))
        self.R1, self.R2 = R1.reshape(3, 3), R2.reshape(3, 3)
        self.P1, self.P2, self.Q = P1.reshape(3, 4), P2.reshape(3, 4), Q.reshape(4, 4)
        self.rect_w, self.rect_h = w.value, h.value
        self.src_w, self.src_h = cs.width, cs.height
        return self

    def set_poly_calib(self, cx=None, cy=None, cz=None):
        """setCalibrationParamsV2's coefficient maps: three (rect_h, rect_w, 4)
        float32 arrays (X, Y, Z), or None to drop them."""
        if cx is None and cy is None and cz is None:
            self.check(self._L.zim_set_poly_calib(self.h, None, None, None, 0, 0))
            return self
        maps = [np.ascontiguousarray(m, dtype=np.float32) for m in (cx, cy, cz)]
        for m in maps:
            if m.ndim != 3 or m.shape[2] != 4 or m.shape[:2] != maps[0].shape[:2]:
                raise ZimError(_lib.ERR_INVALID_ARG, "coefficient maps are rows x cols x 4 float32")
        H, W = maps[0].shape[:2]
        self.check(self._L.zim_set_poly_calib(self.h, *(_p(m) for m in maps), H, W))
        return self

    def rectify_maps(self, cam: int):
        mx = torch.empty((self.rect_h, self.rect_w), dtype=torch.float32, device="cuda")
        my = torch.empty_like(mx)
        self.check(self._L.zim_get_rectify_maps(self.h, cam, _p(mx), _p(my), _stream()))
        return mx, my

    def scratch_bytes(self) -> int:
        return int(self._L.zim_scratch_bytes(self.h))

    def launch_count(self) -> int:
        return int(self._L.zim_launch_count(self.h))

    def check_device(self) -> int:
        w = C.c_uint32()
        self.check(self._L.zim_check_device(self.h, C.byref(w)))
        return w.value


def decode_config(encoding=ENC_HETERODYNE3, freq=(121, 110, 120), shift_num=(8, 8, 8), gray_bits=0,
                  modulation_threshold=1.0, preblur_sigma=3.0, avg_three_phase=True, post_smooth=True,
                  enable_hdr=False, hdr_saturation_gray=255.0, hdr_min_amplitude=2.0, n_freq=None):
    c = _lib.DecodeConfig()
    _lib.load().zim_decode_config_default(C.byref(c))
    for i in range(4):
        c.freq[i] = 0.0
        c.shift_num[i] = 0
    for i, f in enumerate(list(freq)[:4]):
        c.freq[i] = float(f)
    for i, s in enumerate(list(shift_num)[:4]):
        c.shift_num[i] = int(s)
    c.encoding = int(encoding)
    c.n_freq = int(n_freq) if n_freq is not None else (
        3 if encoding == ENC_HETERODYNE3 else (len(freq) if encoding == ENC_HIERARCHICAL else 1))
    c.gray_bits = int(gray_bits)
    c.modulation_threshold = float(modulation_threshold)
    c.preblur_sigma = float(preblur_sigma)
    c.avg_three_phase = int(bool(avg_three_phase))
    c.post_smooth = int(bool(post_smooth))
    c.enable_hdr = int(bool(enable_hdr))
    c.hdr_saturation_gray = float(hdr_saturation_gray)
    c.hdr_min_amplitude = float(hdr_min_amplitude)
    return c


def recon_config(**kw):
    c = _lib.ReconConfig()
    _lib.load().zim_recon_config_default(C.byref(c))
    names = {f[0] for f in _lib.ReconConfig._fields_}
    for k, v in kw.items():
        if k not in names:
            raise KeyError(k)
        setattr(c, k, v)
    return c


def calib_struct(K, D, R, t, width, height) -> _lib.StereoCalib:
    c = _lib.StereoCalib()
    for k in range(2):
        for i, v in enumerate(np.asarray(K[k], float).reshape(9)):
            c.camera_matrix[k][i] = v
        for i, v in enumerate(np.asarray(D[k], float).reshape(5)):
            c.dist_coeffs[k][i] = v
    for i, v in enumerate(np.asarray(R, float).reshape(9)):
        c.R[i] = v
    for i, v in enumerate(np.asarray(t, float).reshape(3)):
        c.t[i] = v
    c.width, c.height = int(width), int(height)
    return c


def _sample_type(t: torch.Tensor) -> int:
    if t.dtype == torch.uint8:
        return SAMPLE_U8
    if t.dtype in (torch.uint16, torch.int16):
        return SAMPLE_U16
    raise ValueError("frames must be uint8 or uint16")


def frame_count(cfg) -> int:
    return _lib.load().zim_decode_frame_count(C.byref(cfg))


def decode(ctx: Context, cfg, frames: torch.Tensor, want_mod=True, want_valid=True):
    """zim_decode: frames (F, H, W) u8/u16 on the device -> dict of maps."""
    F, H, W = frames.shape
    dev = frames.device
    order = torch.empty((H, W), dtype=torch.int32, device=dev)
    res = torch.empty((H, W), dtype=torch.float32, device=dev)
    mod = torch.empty((H, W), dtype=torch.float32, device=dev) if want_mod else None
    valid = torch.empty((H, W), dtype=torch.uint8, device=dev) if want_valid else None
    ctx.check(_lib.load().zim_decode(ctx.h, C.byref(cfg), _p(frames), _sample_type(frames), H, W, _p(order), _p(res),
                                     _p(mod), _p(valid), _stream()))
    return dict(order=order, residual=res, mod=mod, valid=valid)


def decode_phase_f64(ctx: Context, order, residual, post_smooth=True, hdr=False):
    """startCalculate's CV_64F phase: 2 pi order + residual, optionally
    post-smoothed (the HDR form for an HDR decode, whose invalid orders are -1)."""
    H, W = order.shape
    out = torch.empty((H, W), dtype=torch.float64, device=order.device)
    mode = (2 if post_smooth else 3) if hdr else (1 if post_smooth else 0)
    ctx.check(_lib.load().zim_decode_phase_f64(ctx.h, _p(order), _p(residual), H, W, mode, _p(out), _stream()))
    return out


def rectify(ctx: Context, cam, order, residual, post_smooth=True):
    H, W = order.shape
    shp = (ctx.rect_h, ctx.rect_w)
    base = torch.empty(shp, dtype=torch.int32, device=order.device)
    res = torch.empty(shp, dtype=torch.float32, device=order.device)
    rord = torch.empty(shp, dtype=torch.int32, device=order.device)
    ctx.check(_lib.load().zim_rectify(ctx.h, int(cam), _p(order), _p(residual), H, W, int(bool(post_smooth)),
                                      _p(base), _p(res), _p(rord), _stream()))
    return base, res, rord


def match(ctx: Context, left, right, pha_f, grad_threshold=1.0, want_best=True):
    """left/right: (base, res, order) rectified triples."""
    lb, lr, lo = left
    rb, rr, ro = right
    H, W = lo.shape
    disp = torch.empty((H, W), dtype=torch.float32, device=lo.device)
    best = torch.empty((H, W), dtype=torch.int32, device=lo.device) if want_best else None
    ctx.check(_lib.load().zim_match(ctx.h, _p(lb), _p(lr), _p(lo), _p(rb), _p(rr), _p(ro), H, W, int(pha_f),
                                    float(grad_threshold), _p(disp), _p(best), _stream()))
    return disp, best


def rectify_match(ctx: Context, left, right, pha_f, post_smooth=True, grad_threshold=1.0, hdr=False):
    """setData + stereoMatch fused (zim_rectify_match): left/right are the
    decoded (order, residual) of each camera; returns the raw disparity."""
    lo, lr = left
    ro, rr = right
    H, W = lo.shape
    disp = torch.empty((ctx.rect_h, ctx.rect_w), dtype=torch.float32, device=lo.device)
    mode = (2 if post_smooth else 3) if hdr else (1 if post_smooth else 0)
    ctx.check(_lib.load().zim_rectify_match(ctx.h, _p(lo), _p(lr), _p(ro), _p(rr), H, W, mode, int(pha_f),
                                            float(grad_threshold), _p(disp), _stream()))
    return disp


def median_reproject(ctx: Context, rcfg, disp):
    H, W = disp.shape
    dout = torch.empty_like(disp)
    xyz = torch.empty((H, W, 3), dtype=torch.float32, device=disp.device)
    mask = torch.empty((H, W), dtype=torch.uint8, device=disp.device)
    ctx.check(_lib.load().zim_median_reproject(ctx.h, C.byref(rcfg), _p(disp), H, W, _p(dout), _p(xyz), _p(mask),
                                               _stream()))
    return dout, xyz, mask


def filter_px_gaussian(ctx, xyz, mask, update_mask=False):
    H, W = mask.shape
    out = torch.empty_like(xyz)
    mo = torch.empty_like(mask) if update_mask else None
    ctx.check(_lib.load().zim_filter_px_gaussian(ctx.h, _p(xyz), _p(mask), H, W, _p(out), _p(mo), _stream()))
    return out, (mo if update_mask else mask)


def filter_ror(ctx, xyz, mask, radius, min_neighbors, window_size):
    H, W = mask.shape
    out = torch.empty_like(xyz)
    mo = torch.empty_like(mask)
    ctx.check(_lib.load().zim_filter_ror(ctx.h, _p(xyz), _p(mask), H, W, float(radius), int(min_neighbors),
                                         int(window_size), _p(out), _p(mo), _stream()))
    return out, mo


def filter_mls(ctx, xyz, mask, window, sigma, order, max_radius=0.0, iterations=1):
    H, W = mask.shape
    out = torch.empty_like(xyz)
    ctx.check(_lib.load().zim_filter_mls(ctx.h, _p(xyz), _p(mask), H, W, int(window), float(sigma), int(order),
                                         float(max_radius), int(iterations), _p(out), _stream()))
    return out


def filter_sor(ctx, xyz, mask, mean_k, std_mul=1.0, want_mean_dist=False):
    H, W = mask.shape
    mo = torch.empty_like(mask)
    md = torch.empty((H, W), dtype=torch.float32, device=mask.device) if want_mean_dist else None
    ctx.check(_lib.load().zim_filter_sor(ctx.h, _p(xyz), _p(mask), H, W, int(mean_k), float(std_mul), _p(mo), _p(md),
                                         _stream()))
    return mo, md


def sor_stats(ctx) -> dict:
    """Statistics of the last SOR run on this context (synchronises)."""
    st = _lib.SorStats()
    ctx.check(_lib.load().zim_filter_sor_stats(ctx.h, C.byref(st)))
    return dict(n_valid=st.n_valid, mean=st.mean, stddev=st.stddev, threshold=st.threshold,
                n_far_search=st.n_far_search)


def filter_metric_gaussian(ctx, xyz, mask, sigma):
    H, W = mask.shape
    out = torch.empty_like(xyz)
    ctx.check(_lib.load().zim_filter_metric_gaussian(ctx.h, _p(xyz), _p(mask), H, W, float(sigma), _p(out),
                                                     _stream()))
    return out


def compact_points(ctx, xyz, mask):
    """Valid points in PCL PointXYZ layout (N, 4) float32, row-major order."""
    H, W = mask.shape
    pts = torch.empty((H * W, 4), dtype=torch.float32, device=mask.device)
    cnt = torch.zeros(1, dtype=torch.int64, device=mask.device)
    ctx.check(_lib.load().zim_compact_points(ctx.h, _p(xyz), _p(mask), H, W, _p(pts), _p(cnt), _stream()))
    return pts[: int(cnt.item())]


def pack_ply(ctx, xyz, mask, gray=None, with_gray=False):
    """PLY vertex body of the valid points (row order) as a uint8 device tensor:
    12 bytes (float x, y, z) per point, or 15 with with_gray (+ grey as r, g, b;
    255 when gray is None)."""
    H, W = mask.shape
    rec = 15 if with_gray else 12
    body = torch.empty(H * W * rec, dtype=torch.uint8, device=mask.device)
    cnt = torch.zeros(1, dtype=torch.int64, device=mask.device)
    ctx.check(_lib.load().zim_pack_ply(ctx.h, _p(xyz), _p(mask), _p(gray) if gray is not None else None,
                                       int(bool(with_gray)), H, W, _p(body), _p(cnt), _stream()))
    return body[: int(cnt.item()) * rec]


def rectify_image(ctx, cam, image):
    """rectifyLeftImage (cam 0) or the right camera's: 8-bit image remapped
    INTER_LINEAR into the rectified frame."""
    image = image.contiguous()
    H, W = image.shape
    out = torch.empty((ctx.rect_h, ctx.rect_w), dtype=torch.uint8, device=image.device)
    ctx.check(_lib.load().zim_rectify_image(ctx.h, int(cam), _p(image), H, W, _p(out), _stream()))
    return out


def rotated_rect(roi) -> _lib.RotatedRect:
    """cv::RotatedRect from ((cx, cy), (w, h), angle) -- OpenCV's Python form -- or as is."""
    if isinstance(roi, _lib.RotatedRect):
        return roi
    (cx, cy), (w, h), a = roi
    return _lib.RotatedRect(float(cx), float(cy), float(w), float(h), float(a))


def roi_source_spans(roi, rows, cols):
    """The filled rotated rectangle in the source image: (lo, hi) column per row."""
    lo = np.empty(rows, np.int32); hi = np.empty(rows, np.int32)
    check(_lib.load().zim_roi_source_spans(C.byref(rotated_rect(roi)), int(rows), int(cols), _p(lo), _p(hi)))
    return lo, hi


@dataclass
class RectifiedROI:
    """RectifiedROI (JSLAB_PhaseEpipolarReconstructor_V2.h:97-102): rectangles as
    (x, y, width, height); mask is the full rectified-frame ROI mask (device)."""
    left_rect: tuple
    right_rect: tuple
    mask: Optional[torch.Tensor]


def prepare_roi(ctx: Context, roi, l_order, r_order, pha_f) -> Optional[RectifiedROI]:
    """prepareRectifiedROI on rectified order maps; None for an empty ROI."""
    mask = torch.empty((ctx.rect_h, ctx.rect_w), dtype=torch.uint8, device=l_order.device)
    out = _lib.RectifiedROI()
    valid = C.c_int(0)
    ctx.check(_lib.load().zim_prepare_roi(ctx.h, C.byref(rotated_rect(roi)), _p(l_order), _p(r_order), int(pha_f),
                                          C.byref(out), _p(mask), C.byref(valid), _stream()))
    if not valid.value:
        return None
    return RectifiedROI(out.left_rect.as_tuple(), out.right_rect.as_tuple(), mask)


def reconstruct_roi(ctx: Context, rcfg, roi: RectifiedROI, left, right, pha_f, want_disp=False):
    """startCalculate_v2_roi on rectified (base, res, order) triples; outputs are
    left_rect-sized (xyz, mask, disp)."""
    lb, lr, lo = left
    rb, rr, ro = right
    x, y, w, h = roi.left_rect
    xyz = torch.empty((h, w, 3), dtype=torch.float32, device=lo.device)
    mask = torch.empty((h, w), dtype=torch.uint8, device=lo.device)
    disp = torch.empty((h, w), dtype=torch.float32, device=lo.device) if want_disp else None
    rr_ = _lib.RectifiedROI(_lib.Rect(*roi.left_rect), _lib.Rect(*roi.right_rect))
    ctx.check(_lib.load().zim_reconstruct_roi(ctx.h, C.byref(rcfg), C.byref(rr_), _p(roi.mask), _p(lb), _p(lr),
                                              _p(lo), _p(rb), _p(rr), _p(ro), int(pha_f), _p(xyz), _p(mask),
                                              _p(disp), _stream()))
    return xyz, mask, disp


def fit_poly_calib(ctx: Context, Q, disps, masks):
    """computePixelwiseDepthCalibration on device disparity maps (float32) and
    masks (uint8) of the reference planes: returns (cx, cy, cz) as
    (rows, cols, 4) float32 device tensors and the plane equations (n, 4)."""
    disps = [d.contiguous() for d in disps]
    masks = [m.contiguous() for m in masks]
    n = len(disps)
    H, W = disps[0].shape
    for d, m in zip(disps, masks):
        if d.shape != (H, W) or m.shape != (H, W) or d.dtype != torch.float32 or m.dtype != torch.uint8:
            raise ZimError(_lib.ERR_INVALID_ARG, "disparities float32 and masks uint8 of one size")
    out = [torch.empty((H, W, 4), dtype=torch.float32, device=disps[0].device) for _ in range(3)]
    dp = (C.c_void_p * n)(*[d.data_ptr() for d in disps])
    mp = (C.c_void_p * n)(*[m.data_ptr() for m in masks])
    eqs = np.zeros((n, 4))
    Qa = np.ascontiguousarray(np.asarray(Q, np.float64).reshape(16))
    ctx.check(_lib.load().zim_fit_poly_calib(ctx.h, _p(Qa), dp, mp, n, H, W, *(_p(o) for o in out), _p(eqs),
                                             _stream()))
    return out[0], out[1], out[2], eqs


class JSLAB_StereoCalib_V2:
    """The V2 depth-calibration part of JSLAB_StereoCalib_V2 (JSLAB_StereoCalib_V2.h):
    loadBaseCalibration, addPlaneReferenceData, clearPlaneReferenceData,
    computePixelwiseDepthCalibration, getParams, saveCalibResult.  The base
    stereo calibration (calibrateCamera / stereoCalibrate on target images) is
    taken as given: a JSLAB_StereoCalibParams_V1 or a V1 file."""

    def __init__(self, img_size, base: Optional[JSLAB_StereoCalibParams_V1] = None, ctx: Optional[Context] = None):
        self.m_img_size = tuple(img_size)
        self._base = base
        self._ctx = ctx or Context(torch.cuda.current_device())
        self._disps, self._masks = [], []
        self._coeffs = None

    def loadBaseCalibration(self, filename: str) -> bool:
        from . import calib_io
        p = JSLAB_StereoCalibParams_V1()
        if not calib_io.loadStereoCalibParams_V1(filename, p):
            return False
        self._base = p
        self.m_img_size = tuple(p.image_size)
        return True

    def addPlaneReferenceData(self, disp_map, mask):
        self._disps.append(torch.as_tensor(disp_map).to("cuda", torch.float32).contiguous())
        self._masks.append(torch.as_tensor(mask).to("cuda", torch.uint8).contiguous())

    def clearPlaneReferenceData(self):
        self._disps, self._masks = [], []

    def computePixelwiseDepthCalibration(self):
        """stereoRectify(flags 0, alpha -1, new size = the image size), then the fit."""
        if self._base is None:
            raise ZimError(_lib.ERR_NOT_CALIBRATED, "no base calibration")
        b = self._base
        self._ctx.set_calibration(calib_struct(b.camera_matrix, b.dist_coeffs, b.R, b.t, *self.m_img_size), False)
        cx, cy, cz, eqs = fit_poly_calib(self._ctx, self._ctx.Q, self._disps, self._masks)
        self._coeffs = [t.cpu().numpy() for t in (cx, cy, cz)]
        self.plane_eqs = eqs

    def getParams(self) -> "JSLAB_StereoCalibParams_V2":
        b = self._base
        p = JSLAB_StereoCalibParams_V2([np.array(k, float) for k in b.camera_matrix],
                                       [np.array(d, float) for d in b.dist_coeffs], np.array(b.R, float),
                                       np.array(b.t, float), tuple(self.m_img_size))
        if self._coeffs is not None:
            p.xyz_calib_coeffs = [c.copy() for c in self._coeffs]
        return p

    def saveCalibResult(self, filename: str) -> bool:
        from . import calib_io
        return calib_io.saveStereoCalibParams(filename, self.getParams())


def reconstruct_pair(ctx, dcfg, rcfg, left, right, pha_f=0, out=None, want_disp=False):
    """Whole plain per-pair path on device frames.  Returns (xyz, mask, disp)."""
    F, H, W = left.shape
    if out is None:
        xyz = torch.empty((ctx.rect_h, ctx.rect_w, 3), dtype=torch.float32, device=left.device)
        mask = torch.empty((ctx.rect_h, ctx.rect_w), dtype=torch.uint8, device=left.device)
        disp = torch.empty((ctx.rect_h, ctx.rect_w), dtype=torch.float32, device=left.device) if want_disp else None
    else:
        xyz, mask, disp = out
    ctx.check(_lib.load().zim_reconstruct_pair(ctx.h, C.byref(dcfg), C.byref(rcfg), _p(left), _p(right),
                                               _sample_type(left), H, W, int(pha_f), _p(xyz), _p(mask), _p(disp),
                                               _stream()))
    return xyz, mask, disp


def reconstruct_pair_host(ctx, dcfg, rcfg, left: np.ndarray, right: np.ndarray, pha_f=0, xyz=None, mask=None,
                          disp=None, stream=None, asynchronous=False):
    """The same from host arrays (numpy or pinned CPU tensors); synchronous.
    asynchronous=True queues the copies and the pair on `stream` (a
    torch.cuda.Stream; default the current stream) and returns at once
    (zim_reconstruct_pair_host_async): the outputs are ready, and the inputs
    free, once that stream has drained.  Pass page-locked buffers."""
    F, H, W = left.shape
    st = SAMPLE_U8 if left.dtype in (np.uint8, torch.uint8) else SAMPLE_U16
    if xyz is None:
        xyz = np.empty((ctx.rect_h, ctx.rect_w, 3), np.float32)
    if mask is None:
        mask = np.empty((ctx.rect_h, ctx.rect_w), np.uint8)

    def hp(a):
        if a is None:
            return None
        if isinstance(a, torch.Tensor):
            return C.c_void_p(a.data_ptr())
        return a.ctypes.data_as(C.c_void_p)

    fn = _lib.load().zim_reconstruct_pair_host_async if asynchronous else _lib.load().zim_reconstruct_pair_host
    sp = C.c_void_p(stream.cuda_stream) if stream is not None else _stream()
    ctx.check(fn(ctx.h, C.byref(dcfg), C.byref(rcfg), hp(left), hp(right), st, H, W, int(pha_f), hp(xyz), hp(mask),
                 hp(disp), sp))
    return xyz, mask, disp


# ---------------------------------------------------------------------------
# Reference-shaped classes
# ---------------------------------------------------------------------------
@dataclass
class DecodedPhase:
    """A decoded camera: phase = 2*pi*order + residual (unsmoothed)."""
    order: torch.Tensor
    residual: torch.Tensor
    mod: Optional[torch.Tensor]
    valid: Optional[torch.Tensor]
    post_smooth: bool


class JSLAB_PhaseShiftDecoder:
    """Mirror of the reference's abstract decoder + factory (JSLAB_PhaseShiftDecoder.h:10-92)."""

    class Version(enum.Enum):
        V1 = 0
        V2 = 1

    @dataclass
    class Config:
        freq: Sequence[float] = (121.0, 110.0, 120.0)
        shift_num: Sequence[int] = (8, 8, 8)
        modulation_threshold: float = 1.0
        preblur_sigma: float = 3.0
        avg_three_phase: bool = True
        post_smooth: bool = True
        enable_hdr: bool = False
        hdr_saturation_gray: float = 255.0
        hdr_min_amplitude: float = 2.0
        encoding: int = ENC_HETERODYNE3
        gray_bits: int = 0

    @staticmethod
    def create(config: "JSLAB_PhaseShiftDecoder.Config", version: "JSLAB_PhaseShiftDecoder.Version" = None,
               ctx: Optional[Context] = None):
        """Returns a GPU decoder, or None for an invalid config (JSLAB_PhaseShiftDecoder.cpp:9-29).

        The reference's default version is V1 (the legacy decoder without order
        maps); this path implements V2 only and raises ZimError(UNSUPPORTED) for V1.
        """
        version = JSLAB_PhaseShiftDecoder.Version.V1 if version is None else version
        cfg = _config_struct(config)
        st = _lib.load().zim_decode_validate(C.byref(cfg))
        if st == _lib.ERR_INVALID_ARG:
            return None
        if st != _lib.OK:
            raise ZimError(st, "unsupported decoder configuration")
        if version != JSLAB_PhaseShiftDecoder.Version.V2:
            raise ZimError(_lib.ERR_UNSUPPORTED, "only Version.V2 is implemented on the GPU path")
        return JSLAB_PhaseShiftDecoderV2_GPU(config, ctx)


def _config_struct(config: JSLAB_PhaseShiftDecoder.Config):
    return decode_config(encoding=config.encoding, freq=config.freq, shift_num=config.shift_num,
                         gray_bits=config.gray_bits, modulation_threshold=config.modulation_threshold,
                         preblur_sigma=config.preblur_sigma, avg_three_phase=config.avg_three_phase,
                         post_smooth=config.post_smooth, enable_hdr=config.enable_hdr,
                         hdr_saturation_gray=config.hdr_saturation_gray, hdr_min_amplitude=config.hdr_min_amplitude)


class JSLAB_PhaseShiftDecoderV2_GPU(JSLAB_PhaseShiftDecoder):
    """JSLAB_PhaseShiftDecoderV2_GPU (JSLAB_PhaseShiftDecoder_V2_GPU.h:13-33) on zim_decode."""

    def __init__(self, config: JSLAB_PhaseShiftDecoder.Config, ctx: Optional[Context] = None):
        self.m_config = config
        self._cfg = _config_struct(config)
        self._ctx = ctx or Context(torch.cuda.current_device())
        self._frames = None
        self._dec: Optional[DecodedPhase] = None

    def setImages(self, images):
        """images: a (F, H, W) tensor/array or a list of F (H, W) frames, frequency-major order."""
        n = frame_count(self._cfg)
        if isinstance(images, (list, tuple)):
            if len(images) != n:
                raise ZimError(_lib.ERR_INVALID_ARG, f"expected {n} images, got {len(images)}")
            images = torch.stack([torch.as_tensor(np.asarray(i)) if not isinstance(i, torch.Tensor) else i
                                  for i in images])
        elif not isinstance(images, torch.Tensor):
            images = torch.as_tensor(np.asarray(images))
        if images.dim() != 3 or images.shape[0] != n:
            raise ZimError(_lib.ERR_INVALID_ARG, "image stack shape mismatch")
        self._frames = images.to("cuda", non_blocking=True).contiguous()

    def startCalculate(self) -> torch.Tensor:
        """Decodes and returns the absolute phase (float64, post-smoothed if configured)."""
        if self._frames is None:
            raise ZimError(_lib.ERR_INVALID_ARG, "setImages first")
        d = decode(self._ctx, self._cfg, self._frames)
        self._dec = DecodedPhase(d["order"], d["residual"], d["mod"], d["valid"], bool(self.m_config.post_smooth))
        return decode_phase_f64(self._ctx, d["order"], d["residual"], self.m_config.post_smooth,
                                self.m_config.enable_hdr)

    def getOrderMap(self) -> torch.Tensor:
        return self._dec.order.clone()

    def getModulationMap(self) -> torch.Tensor:
        return self._dec.mod.to(torch.float64)

    def getDecoded(self) -> DecodedPhase:
        return self._dec


@dataclass
class JSLAB_StereoCalibParams_V1:
    """Mirror of JSLAB_StereoCalibParams_V1 (JSLAB_StereoCalibParams_V1.h:9-20)."""
    camera_matrix: list = field(default_factory=lambda: [np.eye(3), np.eye(3)])
    dist_coeffs: list = field(default_factory=lambda: [np.zeros(5), np.zeros(5)])
    R: np.ndarray = field(default_factory=lambda: np.eye(3))
    t: np.ndarray = field(default_factory=lambda: np.zeros(3))
    image_size: tuple = (0, 0)  # (width, height) like cv::Size

    def as_struct(self):
        return calib_struct(self.camera_matrix, self.dist_coeffs, self.R, self.t, self.image_size[0],
                            self.image_size[1])


@dataclass
class JSLAB_StereoCalibParams_V2(JSLAB_StereoCalibParams_V1):
    """Mirror of JSLAB_StereoCalibParams_V2 (JSLAB_StereoCalibParams_V2.h:8-30): the V1
    fields plus xyz_calib_coeffs[0..2], per-pixel (c0, c1, c2, c3) maps for X, Y
    and Z as (rows, cols, 4) float32 (CV_32FC4)."""
    xyz_calib_coeffs: list = field(default_factory=lambda: [np.zeros((0, 0, 4), np.float32) for _ in range(3)])


class JSLAB_PhaseEpipolarReconstructor_V2:
    """Mirror of JSLAB_PhaseEpipolarReconstructor_V2 (JSLAB_PhaseEpipolarReconstructor_V2.h:11-171)."""

    @dataclass
    class Config:
        min_depth: float = 0.0
        max_depth: float = 1000.0
        min_phase_diff: float = 0.03
        max_phase_diff: float = 0.4
        grad_threshold: float = 1.0
        use_rectified_coords: bool = True
        use_disp_median_filter: bool = True
        use_full_left_rectification: bool = True
        radius_search: float = 0.7
        radius_min_neighbors: int = 10
        radius_window_size: int = 10
        use_mls: bool = False
        mls_window_size: int = 30
        mls_spatial_sigma: float = 0.6
        use_gpu_mls: bool = True
        mls_polynomial_order: int = 1
        mls_max_radius: float = 0.0
        mls_iterations: int = 3
        # additions of this path
        use_px_gaussian: bool = True
        px_gaussian_updates_mask: bool = False
        use_ror: bool = True
        use_sor: bool = False
        sor_mean_k: int = 50
        sor_std_mul: float = 1.0
        use_metric_gaussian: bool = False
        metric_gaussian_sigma: float = 0.5

        def as_struct(self):
            kw = {f.name: getattr(self, f.name) for f in fields(self) if f.name != "use_gpu_mls"}
            for k, v in kw.items():
                if isinstance(v, bool):
                    kw[k] = int(v)
            return recon_config(**kw)

    def __init__(self, config: "JSLAB_PhaseEpipolarReconstructor_V2.Config" = None, ctx: Optional[Context] = None):
        self.m_config = config or JSLAB_PhaseEpipolarReconstructor_V2.Config()
        self._ctx = ctx or Context(torch.cuda.current_device())
        self._rect = None
        self._pha_f = 0
        self._disp = None
        self._use_v2 = False

    @property
    def context(self) -> Context:
        return self._ctx

    def setCalibrationParams(self, params: JSLAB_StereoCalibParams_V1):
        self._ctx.set_calibration(params.as_struct(), self.m_config.use_full_left_rectification)

    def setCalibrationParamsV2(self, params: JSLAB_StereoCalibParams_V2):
        """setCalibrationParamsV2 (V2.cpp:340-366): the V1 geometry, then the
        coefficient maps when all three are non-empty."""
        self.setCalibrationParams(params)
        maps = [np.asarray(m) for m in params.xyz_calib_coeffs]
        self._use_v2 = all(m.size for m in maps)
        if self._use_v2:
            self._ctx.set_poly_calib(*maps)
        else:
            self._ctx.set_poly_calib()

    def setData(self, left, right, left_k=None, right_k=None, left_mod=None, pha_f: int = 0):
        """left/right: DecodedPhase (exact path) or float64 absolute-phase maps with left_k/right_k.

        A float64 map is taken as already post-smoothed (the reference's decoder
        output); it is split into order + residual and rectified without a
        second smoothing.
        """
        cams = []
        for cam, (ph, k) in enumerate(((left, left_k), (right, right_k))):
            if isinstance(ph, DecodedPhase):
                cams.append(rectify(self._ctx, cam, ph.order, ph.residual, ph.post_smooth))
                ords = ph.order
            else:
                ph = torch.as_tensor(ph).to("cuda", torch.float64)
                k = torch.as_tensor(k).to("cuda", torch.int32).contiguous()
                res = (ph - 2 * math.pi * k.to(torch.float64)).to(torch.float32).contiguous()
                cams.append(rectify(self._ctx, cam, k, res, False))
        self._rect = cams
        self._pha_f = int(pha_f)

    def startCalculate(self):
        """Runs match -> median -> reproject -> filters; returns (xyz, P)."""
        return self._calculate(0)

    def startCalculate_v2(self):
        """startCalculate_v2 (V2.cpp:482-593): reprojection through the per-pixel
        coefficient maps.  Without maps the reference writes no point, so
        neither does this (the disparity map is still computed)."""
        return self._calculate(1)

    def _calculate(self, model: int):
        if self._rect is None:
            raise ZimError(_lib.ERR_INVALID_ARG, "setData first")
        c = self.m_config
        rc = c.as_struct()
        disp, _ = match(self._ctx, self._rect[0], self._rect[1], self._pha_f, c.grad_threshold, want_best=False)
        if model == 1 and not self._use_v2:
            dmed, xyz, mask = median_reproject(self._ctx, rc, disp)
            self._disp = dmed
            return torch.zeros_like(xyz), torch.zeros_like(mask)
        rc.reproject_model = model
        dmed, xyz, mask = median_reproject(self._ctx, rc, disp)
        self._disp = dmed
        if c.use_px_gaussian:
            xyz, mask = filter_px_gaussian(self._ctx, xyz, mask, c.px_gaussian_updates_mask)
        if c.use_ror:
            xyz, mask = filter_ror(self._ctx, xyz, mask, c.radius_search, c.radius_min_neighbors,
                                   c.radius_window_size)
        if c.use_sor:
            mask, _ = filter_sor(self._ctx, xyz, mask, c.sor_mean_k, c.sor_std_mul)
            xyz = xyz * mask.unsqueeze(-1).to(xyz.dtype)
        if c.use_mls:
            xyz = filter_mls(self._ctx, xyz, mask, c.mls_window_size, c.mls_spatial_sigma, c.mls_polynomial_order,
                             c.mls_max_radius, c.mls_iterations)
        if c.use_metric_gaussian:
            xyz = filter_metric_gaussian(self._ctx, xyz, mask, c.metric_gaussian_sigma)
        return xyz, mask

    def getDisparityMap(self) -> torch.Tensor:
        return self._disp.clone()

    def prepareRectifiedROI(self, roi_original) -> Optional[RectifiedROI]:
        """prepareRectifiedROI (V2.cpp:595-675); None where the reference returns false."""
        if self._rect is None:
            return None
        return prepare_roi(self._ctx, roi_original, self._rect[0][2], self._rect[1][2], self._pha_f)

    def startCalculate_v2_roi(self, roi):
        """startCalculate_v2_roi (V2.cpp:677-913) for a rotated rectangle or a
        prepared RectifiedROI: a left_rect-sized (xyz, P), or (None, None) where
        the reference releases its outputs.  Without coefficient maps it runs
        startCalculate_v2 on the whole frame, like the reference."""
        if self._rect is None:
            raise ZimError(_lib.ERR_INVALID_ARG, "setData first")
        if not self._use_v2:
            return self.startCalculate_v2()
        if not isinstance(roi, RectifiedROI):
            roi = self.prepareRectifiedROI(roi)
            if roi is None:
                return None, None
        rc = self.m_config.as_struct()
        rc.reproject_model = 1
        xyz, mask, disp = reconstruct_roi(self._ctx, rc, roi, self._rect[0], self._rect[1], self._pha_f,
                                          want_disp=True)
        self._disp = disp
        return xyz, mask

    def rectifyLeftImage(self, image) -> torch.Tensor:
        """rectifyLeftImage (V2.cpp:920-924): the left 8-bit image in the rectified frame."""
        return rectify_image(self._ctx, 0, torch.as_tensor(image).to("cuda", torch.uint8))
