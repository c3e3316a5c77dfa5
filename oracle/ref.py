"""ctypes wrapper of oracle/_ref/libzim_ref.so: the reference's own decoder,
reconstructor and MLS, compiled from its sources by oracle/ref_build.py.

TEST INFRASTRUCTURE ONLY.  It is the checker that pins the oracle (and,
through the fixtures it writes, the CUDA path) to the reference.  The library
exists only where the reference sources were available to build it;
``available()`` says whether it can be used here.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import ref_build

_lib = None


class DecodeCfg(C.Structure):
    _fields_ = [("freq", C.c_double * 3), ("shift_num", C.c_int * 3), ("modulation_threshold", C.c_double),
                ("preblur_sigma", C.c_double), ("avg_three_phase", C.c_int), ("post_smooth", C.c_int),
                ("enable_hdr", C.c_int), ("hdr_saturation_gray", C.c_double), ("hdr_min_amplitude", C.c_double)]


class Calib(C.Structure):
    _fields_ = [("K", (C.c_double * 9) * 2), ("D", (C.c_double * 5) * 2), ("R", C.c_double * 9),
                ("t", C.c_double * 3), ("width", C.c_int), ("height", C.c_int)]


class ReconCfg(C.Structure):
    _fields_ = [("min_depth", C.c_double), ("max_depth", C.c_double), ("grad_threshold", C.c_double),
                ("use_rectified_coords", C.c_int), ("use_disp_median_filter", C.c_int),
                ("use_full_left_rectification", C.c_int), ("radius_search", C.c_float),
                ("radius_min_neighbors", C.c_int), ("radius_window_size", C.c_int), ("use_mls", C.c_int),
                ("mls_window_size", C.c_int), ("mls_spatial_sigma", C.c_float), ("mls_polynomial_order", C.c_int),
                ("mls_max_radius", C.c_float), ("mls_iterations", C.c_int)]


def available() -> bool:
    try:
        lib()
        return True
    except (FileNotFoundError, RuntimeError, OSError):
        return False


def lib():
    global _lib
    if _lib is None:
        path = ref_build.build()
        L = C.CDLL(str(path))
        L.zr_last_error.restype = C.c_char_p
        L.zr_recon_create.restype = C.c_void_p
        for f in ("zr_decode", "zr_recon_run", "zr_stereo_match", "zr_px_gaussian", "zr_ror", "zr_mls", "zr_mls_f64",
                  "zr_recon_rectification", "zr_poly_point"):
            getattr(L, f).restype = C.c_int
        L.zr_recon_run.argtypes = [C.c_void_p] + [C.c_void_p] * 5 + [C.c_int] * 4 + [C.c_void_p] * 9
        L.zr_recon_rectification.argtypes = [C.c_void_p] * 7
        L.zr_recon_destroy.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def _check(rc):
    if rc == -1:
        raise ValueError("the reference factory rejected the config (nullptr)")
    if rc:
        raise RuntimeError(lib().zr_last_error().decode())


def decode_cfg(freq=(121, 110, 120), shift_num=(8, 8, 8), modulation_threshold=1.0, preblur_sigma=3.0,
               avg_three_phase=True, post_smooth=True, enable_hdr=False, hdr_saturation_gray=255.0,
               hdr_min_amplitude=2.0, **_ignored):
    """JSLAB_PhaseShiftDecoder::Config (three frequencies).  Keys the
    reference has no field for (encoding, n_freq, gray_bits) are ignored."""
    c = DecodeCfg()
    for i in range(3):
        c.freq[i] = float(freq[i])
        c.shift_num[i] = int(shift_num[i])
    c.modulation_threshold = modulation_threshold
    c.preblur_sigma = preblur_sigma
    c.avg_three_phase = int(bool(avg_three_phase))
    c.post_smooth = int(bool(post_smooth))
    c.enable_hdr = int(bool(enable_hdr))
    c.hdr_saturation_gray = hdr_saturation_gray
    c.hdr_min_amplitude = hdr_min_amplitude
    return c


def decode(cfg: DecodeCfg, frames):
    """frames (F, H, W), u8 or float (passed as CV_64F).  Returns phase
    (startCalculate's), phase_raw (before the post-smooth), order, mod, valid."""
    if frames.dtype == np.uint8:
        fr, depth = _c(frames, np.uint8), 0
    else:
        fr, depth = _c(frames, np.float64), 6
    F, H, W = fr.shape
    assert F == sum(cfg.shift_num), (F, list(cfg.shift_num))
    ph, raw, mod = np.empty((H, W)), np.empty((H, W)), np.empty((H, W))
    k = np.empty((H, W), np.int32)
    v = np.empty((H, W), np.uint8)
    _check(lib().zr_decode(C.byref(cfg), _p(fr), C.c_int(depth), C.c_int(H), C.c_int(W), _p(ph), _p(raw), _p(k),
                           _p(mod), _p(v)))
    return ph, raw, k, mod, v


def calib(rig: dict) -> Calib:
    c = Calib()
    for cam in range(2):
        for i in range(9):
            c.K[cam][i] = float(np.asarray(rig["K"][cam], np.float64).ravel()[i])
        for i in range(5):
            c.D[cam][i] = float(np.asarray(rig["D"][cam], np.float64).ravel()[i])
    for i in range(9):
        c.R[i] = float(np.asarray(rig["R"], np.float64).ravel()[i])
    for i in range(3):
        c.t[i] = float(np.asarray(rig["t"], np.float64).ravel()[i])
    c.width, c.height = int(rig["width"]), int(rig["height"])
    return c


def recon_cfg(min_depth=0.0, max_depth=1000.0, grad_threshold=1.0, use_rectified_coords=True,
              use_disp_median_filter=True, use_full_left_rectification=True, radius_search=0.7,
              radius_min_neighbors=10, radius_window_size=10, use_mls=False, mls_window_size=30,
              mls_spatial_sigma=0.6, mls_polynomial_order=1, mls_max_radius=0.0, mls_iterations=3):
    """JSLAB_PhaseEpipolarReconstructor_V2::Config (defaults as in the reference header)."""
    c = ReconCfg()
    for k, v in locals().items():
        if k != "c":
            setattr(c, k, v if not isinstance(v, bool) else int(v))
    return c


class Reconstructor:
    """JSLAB_PhaseEpipolarReconstructor_V2 with its calibration set."""

    def __init__(self, cfg: ReconCfg, rig: dict, poly=None):
        L = lib()
        w, h = C.c_int(), C.c_int()
        cal = calib(rig)
        if poly is not None:
            m = [_c(a, np.float32) for a in poly]
            ph, pw = m[0].shape[:2]
            self._poly = m
            self.h_ = L.zr_recon_create(C.byref(cfg), C.byref(cal), _p(m[0]), _p(m[1]), _p(m[2]), C.c_int(ph),
                                        C.c_int(pw), C.byref(w), C.byref(h))
        else:
            self.h_ = L.zr_recon_create(C.byref(cfg), C.byref(cal), None, None, None, 0, 0, C.byref(w), C.byref(h))
        if not self.h_:
            raise RuntimeError(L.zr_last_error().decode())
        self.w, self.h = w.value, h.value

    def __del__(self):
        if getattr(self, "h_", None):
            lib().zr_recon_destroy(self.h_)
            self.h_ = None

    def rectification(self):
        R1, Q = np.empty(9), np.empty(16)
        maps = [np.empty((self.h, self.w), np.float32) for _ in range(4)]
        lib().zr_recon_rectification(self.h_, _p(R1), _p(Q), *[_p(m) for m in maps])
        return R1.reshape(3, 3), Q.reshape(4, 4), (maps[0], maps[1]), (maps[2], maps[3])

    def run(self, lph, rph, lk, rk, lmod, pha_f, v2=False):
        """setData + startCalculate[_v2]: xyz, P, disparity, the rectified
        (left phase, right phase, left order, right order) setData produced,
        and the reprojected (xyz, P) before the filters."""
        lph, rph, lmod = _c(lph, np.float64), _c(rph, np.float64), _c(lmod, np.float64)
        lk, rk = _c(lk, np.int32), _c(rk, np.int32)
        H, W = lph.shape
        xyz = np.empty((self.h, self.w, 3), np.float32)
        P = np.empty((self.h, self.w), np.uint8)
        disp = np.empty((self.h, self.w))
        rect = [np.empty((self.h, self.w)), np.empty((self.h, self.w)), np.empty((self.h, self.w), np.int32),
                np.empty((self.h, self.w), np.int32)]
        raw_xyz = np.empty_like(xyz)
        raw_P = np.empty_like(P)
        _check(lib().zr_recon_run(self.h_, _p(lph), _p(rph), _p(lk), _p(rk), _p(lmod), H, W, int(pha_f), int(v2),
                                  _p(xyz), _p(P), _p(disp), _p(raw_xyz), _p(raw_P), *[_p(r) for r in rect]))
        return xyz, P, disp, tuple(rect), (raw_xyz, raw_P)


def stereo_match(lph, rph, lk, rk, pha_f, grad_threshold=1.0):
    lph, rph = _c(lph, np.float64), _c(rph, np.float64)
    lk, rk = _c(lk, np.int32), _c(rk, np.int32)
    H, W = lph.shape
    disp = np.empty((H, W))
    _check(lib().zr_stereo_match(_p(lph), _p(rph), _p(lk), _p(rk), C.c_int(H), C.c_int(W), C.c_int(pha_f),
                                 C.c_double(grad_threshold), _p(disp)))
    return disp


def px_gaussian(xyz, P):
    xyz, P = _c(xyz, np.float32), _c(P, np.uint8)
    out = np.empty_like(xyz)
    _check(lib().zr_px_gaussian(_p(xyz), _p(P), C.c_int(P.shape[0]), C.c_int(P.shape[1]), _p(out)))
    return out


def ror(xyz, P, radius, min_neighbors, window):
    xyz, P = _c(xyz, np.float32), _c(P, np.uint8)
    out, op = np.empty_like(xyz), np.empty_like(P)
    _check(lib().zr_ror(_p(xyz), _p(P), C.c_int(P.shape[0]), C.c_int(P.shape[1]), C.c_float(radius),
                        C.c_int(min_neighbors), C.c_int(window), _p(out), _p(op)))
    return out, op


def poly_point(cx, cy, cz, d):
    """evaluateV2CalibPoint (JSLAB_PhaseEpipolarReconstructor_V2.cpp:13-76) for
    one pixel's coefficient vectors: (ok, (x, y, z)) in FP64."""
    f = [np.ascontiguousarray(v, np.float32) for v in (cx, cy, cz)]
    out = np.zeros(3)
    ok = lib().zr_poly_point(_p(f[0]), _p(f[1]), _p(f[2]), C.c_double(d), _p(out))
    return bool(ok), out


def mls_f64(xyz, P, window, sigma, order, max_radius=0.0, iterations=1):
    """The reference MLS source evaluated in double (oracle/ref_mls_f64.cpp); output rounded to float."""
    xyz, P = _c(xyz, np.float32), _c(P, np.uint8)
    out = np.empty_like(xyz)
    _check(lib().zr_mls_f64(_p(xyz), _p(P), C.c_int(P.shape[0]), C.c_int(P.shape[1]), C.c_int(window),
                            C.c_double(sigma), C.c_int(order), C.c_double(max_radius), C.c_int(iterations), _p(out)))
    return out


def mls(xyz, P, window, sigma, order, max_radius=0.0, iterations=1):
    xyz, P = _c(xyz, np.float32), _c(P, np.uint8)
    out = np.empty_like(xyz)
    _check(lib().zr_mls(_p(xyz), _p(P), C.c_int(P.shape[0]), C.c_int(P.shape[1]), C.c_int(window),
                        C.c_float(sigma), C.c_int(order), C.c_float(max_radius), C.c_int(iterations), _p(out)))
    return out
