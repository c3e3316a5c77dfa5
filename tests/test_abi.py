"""C-ABI boundary checks that need no GPU: the library loads, exports every
symbol include/zim.h declares, and the pure host entry points (config defaults,
validation, frame counts) behave like the reference's factory."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    txt = (ROOT / "include" / "zim.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"ZIM_API\s+[\w\s\*]+?\b(zim_\w+)\s*\(", txt)))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "zim_decode" in names and "zim_reconstruct_pair" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(native):
    for name in declared_symbols():
        assert hasattr(native, name), name


def test_prototype_table_matches_header():
    from zim_gb300 import _lib
    assert set(declared_symbols()) == set(_lib.PROTOTYPES)


def test_struct_sizes_match_c_layout():
    from zim_gb300 import _lib
    # zim_decode_config: 4 doubles + 4 ints + 2 doubles + 3 ints(+pad) + 2 doubles + 3 ints
    assert C.sizeof(_lib.DecodeConfig) == 32 + 16 + 16 + 8 + 8 + 16 + 16
    assert C.sizeof(_lib.StereoCalib) == 2 * 9 * 8 + 2 * 5 * 8 + 9 * 8 + 3 * 8 + 8
    assert C.sizeof(_lib.PointXYZ) == 16


def test_config_defaults_mirror_reference(native):
    from zim_gb300 import api
    d = api.decode_config()
    assert d.modulation_threshold == 1.0 and d.preblur_sigma == 3.0
    assert d.avg_three_phase == 1 and d.post_smooth == 1 and d.enable_hdr == 0
    r = api.recon_config()
    # JSLAB_PhaseEpipolarReconstructor_V2::Config defaults
    assert (r.min_depth, r.max_depth, r.grad_threshold) == (0.0, 1000.0, 1.0)
    assert r.use_rectified_coords == 1 and r.use_disp_median_filter == 1 and r.use_full_left_rectification == 1
    assert abs(r.radius_search - 0.7) < 1e-6 and r.radius_min_neighbors == 10 and r.radius_window_size == 10
    assert r.use_mls == 0 and r.mls_window_size == 30 and r.mls_iterations == 3


def test_validate_like_reference_factory(native):
    from zim_gb300 import _lib, api
    L = native
    ok = api.decode_config(freq=(107, 100, 94))
    assert L.zim_decode_validate(C.byref(ok)) == _lib.OK
    for bad in ((0, 100, 94), (107, 0, 94), (107, 100, 0)):
        c = api.decode_config(freq=bad)
        assert L.zim_decode_validate(C.byref(c)) == _lib.ERR_INVALID_ARG
    c = api.decode_config(enable_hdr=True)  # HDR least squares: heterodyne and hierarchical
    assert L.zim_decode_validate(C.byref(c)) == _lib.OK
    c = api.decode_config(enable_hdr=True, shift_num=(13, 8, 8))  # the reference fit takes 3..12 steps
    assert L.zim_decode_validate(C.byref(c)) == _lib.ERR_INVALID_ARG
    c = api.decode_config(encoding=api.ENC_GRAYCODE, freq=(32,), shift_num=(4,), gray_bits=5, enable_hdr=True)
    assert L.zim_decode_validate(C.byref(c)) == _lib.ERR_UNSUPPORTED
    c = api.decode_config(shift_num=(2, 8, 8))
    assert L.zim_decode_validate(C.byref(c)) == _lib.ERR_INVALID_ARG
    c = api.decode_config(freq=(107.5, 100, 94))
    assert L.zim_decode_validate(C.byref(c)) == _lib.ERR_INVALID_ARG
    h = api.decode_config(encoding=api.ENC_HIERARCHICAL, freq=(1, 8, 64), shift_num=(4, 4, 4))
    assert L.zim_decode_validate(C.byref(h)) == _lib.OK
    assert L.zim_decode_frame_count(C.byref(h)) == 12 and L.zim_decode_max_order(C.byref(h)) == 63
    h = api.decode_config(encoding=api.ENC_HIERARCHICAL, freq=(1, 8, 60), shift_num=(4, 4, 4))
    assert L.zim_decode_validate(C.byref(h)) == _lib.ERR_INVALID_ARG
    g = api.decode_config(encoding=api.ENC_GRAYCODE_COMPLEMENTARY, freq=(32,), shift_num=(4,), gray_bits=5)
    assert L.zim_decode_validate(C.byref(g)) == _lib.OK
    assert L.zim_decode_frame_count(C.byref(g)) == 10 and L.zim_decode_max_order(C.byref(g)) == 31
    assert L.zim_decode_max_order(C.byref(ok)) == 107


def test_python_factory_returns_none_on_invalid_config(native):
    from zim_gb300 import api
    cfg = api.JSLAB_PhaseShiftDecoder.Config(freq=(0, 100, 94))
    assert api.JSLAB_PhaseShiftDecoder.create(cfg, api.JSLAB_PhaseShiftDecoder.Version.V2) is None


def test_null_arguments_are_rejected_without_a_device(native):
    from zim_gb300 import _lib
    assert native.zim_decode(None, None, None, 0, 1, 1, None, None, None, None, None) == _lib.ERR_INVALID_ARG
    assert native.zim_set_calibration(None, None, 1) == _lib.ERR_INVALID_ARG
    assert native.zim_create(0, None) == _lib.ERR_INVALID_ARG
    assert native.zim_version().decode().startswith("zim_gb300")


def test_create_without_gpu_reports_cuda_error(native):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from zim_gb300 import _lib
    h = C.c_void_p()
    assert native.zim_create(0, C.byref(h)) == _lib.ERR_CUDA
