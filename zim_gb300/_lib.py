"""ctypes binding of libzim_gb300.so (include/zim.h).

The library is built in-tree by ``zim_gb300._build``.  Loading fails loudly if
it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import _build

OK, ERR_INVALID_ARG, ERR_UNSUPPORTED, ERR_NOT_CALIBRATED, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_TIMEOUT, ERR_DEVICE_CHECK = range(8)
STATUS_NAMES = ["OK", "INVALID_ARG", "UNSUPPORTED", "NOT_CALIBRATED", "CUDA", "OUT_OF_MEMORY", "TIMEOUT",
                "DEVICE_CHECK"]
ENC_HETERODYNE3, ENC_HIERARCHICAL, ENC_GRAYCODE, ENC_GRAYCODE_COMPLEMENTARY = range(4)
SAMPLE_U8, SAMPLE_U16 = 0, 1


class DecodeConfig(C.Structure):
    _fields_ = [("freq", C.c_double * 4), ("shift_num", C.c_int * 4), ("modulation_threshold", C.c_double),
                ("preblur_sigma", C.c_double), ("avg_three_phase", C.c_int), ("post_smooth", C.c_int),
                ("enable_hdr", C.c_int), ("hdr_saturation_gray", C.c_double), ("hdr_min_amplitude", C.c_double),
                ("encoding", C.c_int), ("n_freq", C.c_int), ("gray_bits", C.c_int)]


class StereoCalib(C.Structure):
    _fields_ = [("camera_matrix", (C.c_double * 9) * 2), ("dist_coeffs", (C.c_double * 5) * 2),
                ("R", C.c_double * 9), ("t", C.c_double * 3), ("width", C.c_int), ("height", C.c_int)]


class ReconConfig(C.Structure):
    _fields_ = [("min_depth", C.c_double), ("max_depth", C.c_double), ("min_phase_diff", C.c_double),
                ("max_phase_diff", C.c_double), ("grad_threshold", C.c_double), ("use_rectified_coords", C.c_int),
                ("use_disp_median_filter", C.c_int), ("use_full_left_rectification", C.c_int),
                ("use_px_gaussian", C.c_int), ("px_gaussian_updates_mask", C.c_int), ("use_ror", C.c_int),
                ("radius_search", C.c_float), ("radius_min_neighbors", C.c_int), ("radius_window_size", C.c_int),
                ("use_mls", C.c_int), ("mls_window_size", C.c_int), ("mls_spatial_sigma", C.c_float),
                ("mls_polynomial_order", C.c_int), ("mls_max_radius", C.c_float), ("mls_iterations", C.c_int),
                ("use_sor", C.c_int), ("sor_mean_k", C.c_int), ("sor_std_mul", C.c_double),
                ("use_metric_gaussian", C.c_int), ("metric_gaussian_sigma", C.c_double),
                ("reproject_model", C.c_int)]


class SorStats(C.Structure):
    _fields_ = [("n_valid", C.c_double), ("mean", C.c_double), ("stddev", C.c_double), ("threshold", C.c_double),
                ("n_far_search", C.c_uint32)]


class RotatedRect(C.Structure):
    _fields_ = [("center_x", C.c_float), ("center_y", C.c_float), ("width", C.c_float), ("height", C.c_float),
                ("angle", C.c_float)]


class Rect(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("width", C.c_int), ("height", C.c_int)]

    def as_tuple(self):
        return (self.x, self.y, self.width, self.height)


class RectifiedROI(C.Structure):
    _fields_ = [("left_rect", Rect), ("right_rect", Rect)]


class PointXYZ(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float), ("pad", C.c_float)]


class BatchPair(C.Structure):
    _fields_ = [("decode", DecodeConfig), ("sample_type", C.c_int), ("rows", C.c_int), ("cols", C.c_int),
                ("calib", C.c_int), ("pha_f", C.c_int), ("frames", C.c_void_p * 2), ("xyz", C.c_void_p),
                ("mask", C.c_void_p), ("disp", C.c_void_p), ("filters", C.c_void_p)]


class BatchTuning(C.Structure):
    _fields_ = [("decode_rows", C.c_int), ("match_rows", C.c_int), ("filter_rows", C.c_int),
                ("ctas_per_sm", C.c_int)]


DIFF_NPARAMS = 16


class DiffParams(C.Structure):
    _fields_ = [("cam", (C.c_double * 6) * 2), ("baseline", C.c_double), ("rot", C.c_double * 3)]


class DiffView(C.Structure):
    _fields_ = [("order", C.c_void_p * 2), ("residual", C.c_void_p * 2), ("best_col", C.c_void_p),
                ("plane", C.c_double * 4), ("xyz", C.c_void_p), ("mask", C.c_void_p), ("grad_xyz", C.c_void_p),
                ("grad_phase", C.c_void_p * 2)]


class DiffResult(C.Structure):
    _fields_ = [("loss", C.c_double), ("n_points", C.c_double), ("grad", C.c_double * DIFF_NPARAMS),
                ("jtj", C.c_double * (DIFF_NPARAMS * DIFF_NPARAMS))]


V = C.c_void_p
I = C.c_int
D = C.c_double
Fl = C.c_float
# name -> (restype, argtypes); mirrors include/zim.h
PROTOTYPES = {
    "zim_version": (C.c_char_p, []),
    "zim_decode_config_default": (None, [V]),
    "zim_recon_config_default": (None, [V]),
    "zim_decode_frame_count": (I, [V]),
    "zim_decode_validate": (I, [V]),
    "zim_decode_max_order": (I, [V]),
    "zim_create": (I, [I, V]),
    "zim_destroy": (None, [V]),
    "zim_last_error": (C.c_char_p, [V]),
    "zim_release_scratch": (I, [V]),
    "zim_scratch_bytes": (C.c_size_t, [V]),
    "zim_launch_count": (C.c_ulonglong, [V]),
    "zim_check_device": (I, [V, V]),
    "zim_decode": (I, [V, V, V, I, I, I, V, V, V, V, V]),
    "zim_decode_phase_f64": (I, [V, V, V, I, I, I, V, V]),
    "zim_set_calibration": (I, [V, V, I]),
    "zim_get_rectification": (I, [V, V, V, V, V, V, V, V]),
    "zim_get_rectify_maps": (I, [V, I, V, V, V]),
    "zim_set_poly_calib": (I, [V, V, V, V, I, I]),
    "zim_rectify_image": (I, [V, I, V, I, I, V, V]),
    "zim_roi_source_spans": (I, [V, I, I, V, V]),
    "zim_fit_poly_calib": (I, [V, V, V, V, I, I, I, V, V, V, V, V]),
    "zim_prepare_roi": (I, [V, V, V, V, I, V, V, V, V]),
    "zim_reconstruct_roi": (I, [V, V, V, V, V, V, V, V, V, V, I, V, V, V, V]),
    "zim_pack_ply": (I, [V, V, V, V, I, I, I, V, V, V]),
    "zim_rectify": (I, [V, I, V, V, I, I, I, V, V, V, V]),
    "zim_match": (I, [V, V, V, V, V, V, V, I, I, I, D, V, V, V]),
    "zim_rectify_match": (I, [V, V, V, V, V, I, I, I, I, D, V, V]),
    "zim_median_reproject": (I, [V, V, V, I, I, V, V, V, V]),
    "zim_filter_px_gaussian": (I, [V, V, V, I, I, V, V, V]),
    "zim_filter_ror": (I, [V, V, V, I, I, Fl, I, I, V, V, V]),
    "zim_filter_mls": (I, [V, V, V, I, I, I, Fl, I, Fl, I, V, V]),
    "zim_filter_sor": (I, [V, V, V, I, I, I, D, V, V, V]),
    "zim_filter_sor_stats": (I, [V, V]),
    "zim_filter_metric_gaussian": (I, [V, V, V, I, I, D, V, V]),
    "zim_compact_points": (I, [V, V, V, I, I, V, V, V]),
    "zim_compact_points_noalloc": (I, [V, V, I, I, V, V, V]),
    "zim_reconstruct_pair": (I, [V, V, V, V, V, I, I, I, I, V, V, V, V]),
    "zim_reconstruct_pair_host": (I, [V, V, V, V, V, I, I, I, I, V, V, V, V]),
    "zim_reconstruct_pair_host_async": (I, [V, V, V, V, V, I, I, I, I, V, V, V, V]),
    "zim_batch_create": (I, [V, V, I, I, V]),
    "zim_batch_destroy": (None, [V]),
    "zim_batch_rect_size": (I, [V, I, V, V]),
    "zim_batch_submit": (I, [V, V, I, V, V]),
    "zim_batch_run": (I, [V, V]),
    "zim_batch_autotune": (I, [V, V, V, V]),
    "zim_batch_get_tuning": (I, [V, V]),
    "zim_diff_params_nominal": (I, [V, V]),
    "zim_diff_rectify": (I, [V, V, I, V, V, I, I, V, V, V, V]),
    "zim_diff_forward": (I, [V, V, V, I, I, I, D, D, V, V]),
    "zim_diff_backward": (I, [V, V, V, I, I, I, D, D, D, V, V]),
}

_lib = None


def lib_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads libzim_gb300.so (building it first if asked and absent)."""
    global _lib
    if _lib is not None:
        return _lib
    p = lib_path()
    if not p.exists():
        if not build_if_missing:
            raise RuntimeError(f"zim_gb300 CUDA library missing: {p} (run __graft_entry__.build())")
        _build.build_cuda()
    lib = C.CDLL(str(p))
    for name, (res, args) in PROTOTYPES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class ZimError(RuntimeError):
    def __init__(self, status: int, msg: str):
        self.status = status
        super().__init__(f"zim status {STATUS_NAMES[status] if 0 <= status < 8 else status}: {msg}")


def check(status: int, ctx=None) -> None:
    if status != OK:
        msg = load().zim_last_error(ctx).decode() if ctx else ""
        raise ZimError(status, msg)
