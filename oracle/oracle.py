"""ctypes wrapper of the FP64 oracle (oracle/zim_oracle.c) -- test infrastructure.

Every function takes and returns numpy arrays.  ``build()`` compiles the C
restatement with gcc (-O2 -fopenmp -ffp-contract=off, no fast-math) into
``oracle/libzim_oracle.so``.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libzim_oracle.so"
SOURCES = [HERE / "zim_oracle.c", HERE / "zim_oracle_diff.c", HERE / "zim_oracle.h"]
FLAGS = ["-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11"]

ENC_HETERODYNE3, ENC_HIERARCHICAL, ENC_GRAYCODE, ENC_GRAYCODE_COMPLEMENTARY = 0, 1, 2, 3
NEAR_WRAP, NEAR_ROUND, NEAR_MOD, NEAR_GRAY = 1, 2, 4, 8


def build() -> Path:
    h = hashlib.sha256()
    for s in SOURCES:
        h.update(s.read_bytes())
    h.update(" ".join(FLAGS).encode())
    dig = h.hexdigest()
    stamp = HERE / ".oracle.sha"
    if LIB_PATH.exists() and stamp.exists() and stamp.read_text() == dig:
        return LIB_PATH
    tmp = LIB_PATH.with_suffix(".so.tmp")
    srcs = [str(s) for s in SOURCES if s.suffix == ".c"]
    r = subprocess.run(["gcc", *FLAGS, *srcs, "-o", str(tmp), "-lm"], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("oracle build failed:\n" + r.stderr)
    os.replace(tmp, LIB_PATH)
    stamp.write_text(dig)
    return LIB_PATH


class DecodeCfg(C.Structure):
    _fields_ = [("encoding", C.c_int), ("n_freq", C.c_int), ("freq", C.c_double * 4), ("shift_num", C.c_int * 4),
                ("gray_bits", C.c_int), ("modulation_threshold", C.c_double), ("preblur_sigma", C.c_double),
                ("avg_three_phase", C.c_int), ("post_smooth", C.c_int), ("enable_hdr", C.c_int),
                ("hdr_saturation_gray", C.c_double), ("hdr_min_amplitude", C.c_double)]


class Calib(C.Structure):
    _fields_ = [("K", (C.c_double * 9) * 2), ("D", (C.c_double * 5) * 2), ("R", C.c_double * 9),
                ("t", C.c_double * 3), ("width", C.c_int), ("height", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB_PATH))
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def make_decode_cfg(encoding=ENC_HETERODYNE3, freq=(121, 110, 120), shift_num=(8, 8, 8), gray_bits=0,
                    modulation_threshold=1.0, preblur_sigma=3.0, avg_three_phase=True, post_smooth=True, n_freq=None,
                    enable_hdr=False, hdr_saturation_gray=255.0, hdr_min_amplitude=2.0):
    c = DecodeCfg()
    c.encoding = encoding
    c.n_freq = n_freq if n_freq is not None else (3 if encoding == ENC_HETERODYNE3 else
                                                 (len(freq) if encoding == ENC_HIERARCHICAL else 1))
    for i, f in enumerate(list(freq)[:4]):
        c.freq[i] = f
    for i, s in enumerate(list(shift_num)[:4]):
        c.shift_num[i] = s
    c.gray_bits = gray_bits
    c.modulation_threshold = modulation_threshold
    c.preblur_sigma = preblur_sigma
    c.avg_three_phase = int(bool(avg_three_phase))
    c.post_smooth = int(bool(post_smooth))
    c.enable_hdr = int(bool(enable_hdr))
    c.hdr_saturation_gray = float(hdr_saturation_gray)
    c.hdr_min_amplitude = float(hdr_min_amplitude)
    return c


def make_calib(K, D, R, t, width, height):
    c = Calib()
    for k in range(2):
        for i in range(9):
            c.K[k][i] = float(np.asarray(K[k], dtype=np.float64).reshape(-1)[i])
        for i in range(5):
            c.D[k][i] = float(np.asarray(D[k], dtype=np.float64).reshape(-1)[i])
    for i in range(9):
        c.R[i] = float(np.asarray(R, dtype=np.float64).reshape(-1)[i])
    for i in range(3):
        c.t[i] = float(np.asarray(t, dtype=np.float64).reshape(-1)[i])
    c.width, c.height = int(width), int(height)
    return c


def gaussian_kernel3(sigma):
    k = np.zeros(3)
    lib().zo_gaussian_kernel3(C.c_double(sigma), _p(k))
    return k


def blur3(src, k):
    src = _c(src, np.float64)
    dst = np.empty_like(src)
    k = _c(k, np.float64)
    lib().zo_blur3(_p(src), _p(dst), C.c_int(src.shape[0]), C.c_int(src.shape[1]), _p(k))
    return dst


def frame_count(cfg):
    return lib().zo_frame_count(C.byref(cfg))


def decode(cfg, frames, eps=1e-5):
    """frames: (F, H, W) sample values.  Returns phase, order, mod, valid, near."""
    fr = _c(frames, np.float64)
    F, H, W = fr.shape
    assert F == frame_count(cfg), (F, frame_count(cfg))
    phase = np.empty((H, W)); order = np.empty((H, W), np.int32); mod = np.empty((H, W))
    valid = np.empty((H, W), np.uint8); near = np.empty((H, W), np.uint8)
    rc = lib().zo_decode(C.byref(cfg), _p(fr), C.c_int(H), C.c_int(W), _p(phase), _p(order), _p(mod), _p(valid),
                         _p(near), C.c_double(eps))
    if rc:
        raise ValueError("oracle rejected the decode config")
    return phase, order, mod, valid, near


def post_smooth(phase):
    phase = _c(phase, np.float64)
    out = np.empty_like(phase)
    lib().zo_post_smooth(_p(phase), _p(out), C.c_int(phase.shape[0]), C.c_int(phase.shape[1]))
    return out


def post_smooth_hdr(phase, valid):
    phase = _c(phase, np.float64)
    valid = _c(valid, np.uint8)
    out = np.empty_like(phase)
    lib().zo_post_smooth_hdr(_p(phase), _p(valid), _p(out), C.c_int(phase.shape[0]), C.c_int(phase.shape[1]))
    return out


def stereo_rectify(calib):
    R1 = np.zeros(9); R2 = np.zeros(9); P1 = np.zeros(12); P2 = np.zeros(12); Q = np.zeros(16)
    lib().zo_stereo_rectify(C.byref(calib), _p(R1), _p(R2), _p(P1), _p(P2), _p(Q))
    return R1.reshape(3, 3), R2.reshape(3, 3), P1.reshape(3, 4), P2.reshape(3, 4), Q.reshape(4, 4)


def full_left(calib, R1, P1, P2, Q):
    R1 = _c(R1, np.float64).reshape(9).copy(); P1 = _c(P1, np.float64).reshape(12).copy()
    P2 = _c(P2, np.float64).reshape(12).copy(); Q = _c(Q, np.float64).reshape(16).copy()
    w = C.c_int(); h = C.c_int()
    lib().zo_full_left(C.byref(calib), _p(R1), _p(P1), _p(P2), _p(Q), C.byref(w), C.byref(h))
    return P1.reshape(3, 4), P2.reshape(3, 4), Q.reshape(4, 4), w.value, h.value


def rectification(calib, full_left_canvas=True):
    """setCalibrationParams: R1, R2, P1, P2, Q, rect_w, rect_h."""
    R1, R2, P1, P2, Q = stereo_rectify(calib)
    w, h = calib.width, calib.height
    if full_left_canvas:
        P1, P2, Q, w, h = full_left(calib, R1, P1, P2, Q)
    return R1, R2, P1, P2, Q, w, h


def undistort_points(K, D, pts, R=None, P=None):
    pts = _c(pts, np.float32).reshape(-1, 2)
    out = np.empty_like(pts)
    K = _c(K, np.float64).reshape(9); D = _c(D, np.float64).reshape(5)
    Rp = _p(_c(R, np.float64).reshape(9)) if R is not None else None
    Pa = _c(P, np.float64) if P is not None else None
    lib().zo_undistort_points(_p(K), _p(D), Rp, _p(Pa) if Pa is not None else None,
                              C.c_int(Pa.shape[1] if Pa is not None else 3), _p(pts), _p(out), C.c_int(len(pts)))
    return out


def init_rectify_map(K, D, R, P, w, h):
    mx = np.empty((h, w), np.float32); my = np.empty((h, w), np.float32)
    lib().zo_init_rectify_map(_p(_c(K, np.float64).reshape(9)), _p(_c(D, np.float64).reshape(5)),
                              _p(_c(R, np.float64).reshape(9)), _p(_c(P, np.float64).reshape(12)), C.c_int(w),
                              C.c_int(h), _p(mx), _p(my))
    return mx, my


def remap_linear(src, mapx, mapy):
    src = _c(src, np.float64); mapx = _c(mapx, np.float32); mapy = _c(mapy, np.float32)
    dst = np.empty(mapx.shape, np.float64)
    lib().zo_remap_linear(_p(src), C.c_int(src.shape[0]), C.c_int(src.shape[1]), _p(mapx), _p(mapy),
                          C.c_int(mapx.shape[0]), C.c_int(mapx.shape[1]), _p(dst))
    return dst


def remap_u8(src, mapx, mapy):
    src = _c(src, np.uint8); mapx = _c(mapx, np.float32); mapy = _c(mapy, np.float32)
    dst = np.empty(mapx.shape, np.uint8)
    lib().zo_remap_u8(_p(src), C.c_int(src.shape[0]), C.c_int(src.shape[1]), _p(mapx), _p(mapy),
                      C.c_int(mapx.shape[0]), C.c_int(mapx.shape[1]), _p(dst))
    return dst


def remap_nearest(src, mapx, mapy):
    src = _c(src, np.int32); mapx = _c(mapx, np.float32); mapy = _c(mapy, np.float32)
    dst = np.empty(mapx.shape, np.int32)
    lib().zo_remap_nearest(_p(src), C.c_int(src.shape[0]), C.c_int(src.shape[1]), _p(mapx), _p(mapy),
                           C.c_int(mapx.shape[0]), C.c_int(mapx.shape[1]), _p(dst))
    return dst


def stereo_match(lph, rph, lk, rk, pha_f, grad_threshold=1.0, eps=1e-5):
    lph = _c(lph, np.float64); rph = _c(rph, np.float64); lk = _c(lk, np.int32); rk = _c(rk, np.int32)
    H, W = lph.shape
    disp = np.empty((H, W)); best = np.empty((H, W), np.int32); near = np.empty((H, W), np.uint8)
    lib().zo_stereo_match(_p(lph), _p(rph), _p(lk), _p(rk), C.c_int(H), C.c_int(W), C.c_int(pha_f),
                          C.c_double(grad_threshold), _p(disp), _p(best), _p(near), C.c_double(eps))
    return disp, best, near


def stereo_match_roi(lph, lk, lmask, rph, rk, dx_off, pha_f, grad_threshold=1.0, eps=1e-5):
    """startCalculate_v2_roi's matching on cropped windows (same rows)."""
    lph = _c(lph, np.float64); lk = _c(lk, np.int32); lmask = _c(lmask, np.uint8)
    rph = _c(rph, np.float64); rk = _c(rk, np.int32)
    H, LW = lph.shape
    RW = rph.shape[1]
    disp = np.empty((H, LW)); best = np.empty((H, LW), np.int32); near = np.empty((H, LW), np.uint8)
    lib().zo_stereo_match_roi(_p(lph), _p(lk), _p(lmask), C.c_int(LW), _p(rph), _p(rk), C.c_int(RW), C.c_int(H),
                              C.c_int(dx_off), C.c_int(pha_f), C.c_double(grad_threshold), _p(disp), _p(best),
                              _p(near), C.c_double(eps))
    return disp, best, near


def median5(src):
    src = _c(src, np.float32)
    dst = np.empty_like(src)
    lib().zo_median5(_p(src), _p(dst), C.c_int(src.shape[0]), C.c_int(src.shape[1]))
    return dst


def reproject(disp, Q, R1, min_depth=0.0, max_depth=1000.0, use_rectified=True, eps=1e-5):
    disp = _c(disp, np.float32)
    H, W = disp.shape
    xyz = np.empty((H, W, 3), np.float32); mask = np.empty((H, W), np.uint8); near = np.empty((H, W), np.uint8)
    lib().zo_reproject(_p(disp), C.c_int(H), C.c_int(W), _p(_c(Q, np.float64).reshape(16)),
                       _p(_c(R1, np.float64).reshape(9)), C.c_double(min_depth), C.c_double(max_depth),
                       C.c_int(int(use_rectified)), _p(xyz), _p(mask), _p(near), C.c_double(eps))
    return xyz, mask, near


def poly_reproject(disp, maps, R1, min_depth=0.0, max_depth=1000.0, use_rectified=True):
    """startCalculate_v2's reprojection; maps = (cx, cy, cz), each (H, W, 4) float32."""
    disp = _c(disp, np.float32)
    H, W = disp.shape
    m = [_c(a, np.float32) for a in maps]
    for a in m:
        assert a.shape == (H, W, 4)
    xyz = np.empty((H, W, 3), np.float32); mask = np.empty((H, W), np.uint8)
    lib().zo_poly_reproject(_p(disp), C.c_int(H), C.c_int(W), _p(m[0]), _p(m[1]), _p(m[2]),
                            _p(_c(R1, np.float64).reshape(9)), C.c_double(min_depth), C.c_double(max_depth),
                            C.c_int(int(use_rectified)), _p(xyz), _p(mask))
    return xyz, mask


def px_gaussian(xyz, mask, update_mask=False, eps=1e-5):
    xyz = _c(xyz, np.float32); mask = _c(mask, np.uint8)
    H, W = mask.shape
    out = np.empty_like(xyz); mo = np.empty_like(mask); near = np.empty_like(mask)
    lib().zo_px_gaussian(_p(xyz), _p(mask), C.c_int(H), C.c_int(W), _p(out), _p(mo) if update_mask else None,
                         _p(near), C.c_double(eps))
    return out, (mo if update_mask else mask.copy()), near


def ror(xyz, mask, radius, min_neighbors, window_size, eps=1e-5):
    xyz = _c(xyz, np.float32); mask = _c(mask, np.uint8)
    H, W = mask.shape
    out = np.empty_like(xyz); mo = np.empty_like(mask); near = np.empty_like(mask)
    lib().zo_ror(_p(xyz), _p(mask), C.c_int(H), C.c_int(W), C.c_float(radius), C.c_int(min_neighbors),
                 C.c_int(window_size), _p(out), _p(mo), _p(near), C.c_double(eps))
    return out, mo, near


def mls(xyz, mask, window, sigma, order, max_radius=0.0, iterations=1, eps=1e-5, jitter=0.0, seed=0):
    xyz = _c(xyz, np.float32); mask = _c(mask, np.uint8)
    H, W = mask.shape
    out = np.empty(xyz.shape, np.float64); near = np.zeros_like(mask)
    lib().zo_mls(_p(xyz), _p(mask), C.c_int(H), C.c_int(W), C.c_int(window), C.c_float(sigma), C.c_int(order),
                 C.c_float(max_radius), C.c_int(iterations), _p(out), _p(near), C.c_double(eps),
                 C.c_double(jitter), C.c_ulonglong(seed))
    return out, near


def mls_sensitivity(xyz, mask, window, sigma, order, max_radius=0.0, iterations=1, jitter=1e-6, runs=2):
    """Largest output change (mm) when every neighbour offset is perturbed by a
    relative `jitter` -- the size of FP32 rounding in the offsets.  Points where
    it is large are ill-conditioned (e.g. three nearly collinear neighbours)."""
    base, _ = mls(xyz, mask, window, sigma, order, max_radius, iterations)
    sens = np.zeros(mask.shape)
    for s in range(1, runs + 1):
        o, _ = mls(xyz, mask, window, sigma, order, max_radius, iterations, jitter=jitter, seed=s)
        sens = np.maximum(sens, np.abs(o - base).max(axis=-1))
    return sens


def sor(xyz, mask, k, std_mul=1.0, eps=1e-5):
    xyz = _c(xyz, np.float32); mask = _c(mask, np.uint8)
    n = mask.size
    mo = np.empty_like(mask); md = np.empty(mask.shape); near = np.empty_like(mask); thr = C.c_double()
    rc = lib().zo_sor(_p(xyz), _p(mask), C.c_int(n), C.c_int(k), C.c_double(std_mul), _p(mo), _p(md),
                      C.byref(thr), _p(near), C.c_double(eps))
    if rc:
        return mask.copy(), md, 0.0, near
    return mo, md, thr.value, near


def metric_gaussian(xyz, mask, sigma, eps=1e-5):
    xyz = _c(xyz, np.float32); mask = _c(mask, np.uint8)
    out = np.empty_like(xyz); near = np.empty_like(mask)
    lib().zo_metric_gaussian(_p(xyz), _p(mask), C.c_int(mask.size), C.c_double(sigma), _p(out), _p(near),
                             C.c_double(eps))
    return out, near


class DiffGeom(C.Structure):
    _fields_ = [("ir", (C.c_double * 9) * 2), ("dist", (C.c_double * 3) * 2), ("Q", C.c_double * 16),
                ("baseline0", C.c_double), ("rect_w", C.c_int), ("rect_h", C.c_int), ("src_w", C.c_int),
                ("src_h", C.c_int)]


def diff_geom(ir, dist, Q, baseline0, rect_w, rect_h, src_w, src_h):
    """Fixed geometry of the differentiable forward: ir[c] = (P_c[:, :3] R_c)^-1,
    dist[c] = (p1, p2, k3), the nominal Q and baseline."""
    g = DiffGeom()
    for c in range(2):
        for a in range(9):
            g.ir[c][a] = float(np.asarray(ir[c]).ravel()[a])
        for a in range(3):
            g.dist[c][a] = float(dist[c][a])
    for a in range(16):
        g.Q[a] = float(np.asarray(Q).ravel()[a])
    g.baseline0 = float(baseline0)
    g.rect_w, g.rect_h, g.src_w, g.src_h = rect_w, rect_h, src_w, src_h
    return g


def diff_eval(geom, theta, order_l, res_l, order_r, res_r, best, plane, zmin=0.0, zmax=1e4, loss_weight=1.0,
              want_grad=True, want_points=False, want_phase_grad=False, cells=None, cells_mode=0,
              want_grad_abs=False):
    """FP64 loss of one view and (optionally) its analytic gradient, J^T J,
    points and phase gradients.  cells: int32 array of rect_h*rect_w*8 for
    cells_mode 1 (record) / 2 (reuse the recorded bilinear cells).  Returns a dict."""
    th = _c(theta, np.float64)
    ol, orr = _c(order_l, np.int32), _c(order_r, np.int32)
    rl, rr = _c(res_l, np.float64), _c(res_r, np.float64)
    bc = _c(best, np.int32)
    pl = _c(plane, np.float64)
    loss, npts = C.c_double(), C.c_double()
    grad = np.zeros(16) if want_grad else None
    jtj = np.zeros(256) if want_grad else None
    xyz = np.zeros((geom.rect_h, geom.rect_w, 3)) if want_points else None
    mask = np.zeros((geom.rect_h, geom.rect_w), np.uint8) if want_points else None
    gl = np.zeros(ol.shape) if want_phase_grad else None
    gr = np.zeros(ol.shape) if want_phase_grad else None
    ga = np.zeros(16) if want_grad_abs else None
    nul = C.c_void_p()
    lib().zo_diff_eval(C.byref(geom), _p(th), _p(ol), _p(rl), _p(orr), _p(rr), _p(bc), _p(pl), C.c_double(zmin),
                       C.c_double(zmax), C.c_double(loss_weight), C.byref(loss), C.byref(npts),
                       _p(grad) if want_grad else nul, _p(jtj) if want_grad else nul,
                       _p(xyz) if want_points else nul, _p(mask) if want_points else nul,
                       _p(gl) if want_phase_grad else nul, _p(gr) if want_phase_grad else nul,
                       _p(cells) if cells is not None else nul, C.c_int(cells_mode), _p(ga) if want_grad_abs else nul)
    out = {"loss": loss.value, "n_points": npts.value}
    if want_grad:
        out["grad"], out["jtj"] = grad, jtj.reshape(16, 16)
    if want_points:
        out["xyz"], out["mask"] = xyz, mask
    if want_phase_grad:
        out["grad_phase"] = (gl, gr)
    if want_grad_abs:
        out["grad_abs"] = ga
    return out


def diff_round_positions(on: bool):
    """zo_diff_round_positions: round diff_eval's sample positions to FP32."""
    lib().zo_diff_round_positions(C.c_int(int(bool(on))))


def _setup_prototypes():
    L = lib()
    L.zo_decode.restype = C.c_int
    L.zo_sor.restype = C.c_int
    L.zo_frame_count.restype = C.c_int


def rectify_decoded(phase_unsmoothed, order, mapx, mapy, post, hdr_valid=None):
    """setData for one camera: optional post-smooth (HDR form when the decode
    validity is given), remap linear / nearest."""
    if post:
        ph = post_smooth_hdr(phase_unsmoothed, hdr_valid) if hdr_valid is not None else post_smooth(phase_unsmoothed)
    else:
        ph = phase_unsmoothed
    return remap_linear(ph, mapx, mapy), remap_nearest(order, mapx, mapy)
