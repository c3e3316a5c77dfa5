"""Calibration files of the reference: OpenCV FileStorage XML/YAML for the
stereo parameters and the raw ``.bin`` matrices of the V2 per-pixel
coefficient maps.

- ``loadStereoCalibParams_V1`` follows JSLAB_StereoCalibParams_V1.cpp:3-20 (keys
  LeftCameraMatrix, LeftDistortionCoefficients, RightCameraMatrix,
  RightDistortionCoefficients, RotationMatrix, TranslationVector, ImageSize).
- ``loadStereoCalibParams_V2`` follows JSLAB_StereoCalibParams_V2.cpp:20-43: the
  same file plus ``<base>_rx.bin``, ``<base>_ry.bin``, ``<base>_rz.bin`` next to
  it, where ``<base>`` is the file name up to its last dot.
- ``load_mat_binary`` / ``save_mat_binary`` follow loadMatBinary
  (JSLAB_StereoCalibParams_V2.cpp:4-17) and saveMatBinary
  (JSLAB_StereoCalib_V2.cpp:22-30): three native int32 (OpenCV type, rows,
  cols) followed by the rows of the matrix, densely packed.
- ``saveStereoCalibParams`` writes what JSLAB_StereoCalib_V1/V2::saveCalibResult
  write (JSLAB_StereoCalib_V1.cpp:59-76, JSLAB_StereoCalib_V2.cpp:90-111).

The FileStorage reader handles the node kinds these files use: ``opencv-matrix``
(rows, cols, dt, data) and a plain integer sequence (cv::Size, written as
"width height").
"""
from __future__ import annotations

import re
import xml.etree.ElementTree as ET
from typing import Dict, Optional

import numpy as np

from .api import JSLAB_StereoCalibParams_V1, JSLAB_StereoCalibParams_V2

# OpenCV depth codes (CV_8U .. CV_64F, CV_16F) and FileStorage dt letters.
_DEPTH_DTYPE = {0: np.uint8, 1: np.int8, 2: np.uint16, 3: np.int16, 4: np.int32, 5: np.float32, 6: np.float64,
                7: np.float16}
_DTYPE_DEPTH = {np.dtype(v): k for k, v in _DEPTH_DTYPE.items()}
_DT_LETTER = {"u": np.uint8, "c": np.int8, "w": np.uint16, "s": np.int16, "i": np.int32, "f": np.float32,
              "d": np.float64, "h": np.float16}
_LETTER_DT = {np.dtype(v): k for k, v in _DT_LETTER.items()}

V1_KEYS = ("LeftCameraMatrix", "LeftDistortionCoefficients", "RightCameraMatrix", "RightDistortionCoefficients",
           "RotationMatrix", "TranslationVector")


def cv_type(dtype, channels: int) -> int:
    """CV_MAKETYPE(depth, channels)."""
    return _DTYPE_DEPTH[np.dtype(dtype)] + ((int(channels) - 1) << 3)


def load_mat_binary(filename: str) -> Optional[np.ndarray]:
    """loadMatBinary: returns (rows, cols) or (rows, cols, channels), or None if
    the file cannot be opened or is shorter than its header says."""
    try:
        with open(filename, "rb") as f:
            head = f.read(12)
            if len(head) < 12:
                return None
            typ, rows, cols = np.frombuffer(head, dtype="<i4")
            depth, cn = int(typ) & 7, (int(typ) >> 3) + 1
            if depth not in _DEPTH_DTYPE or rows < 0 or cols < 0:
                return None
            dt = np.dtype(_DEPTH_DTYPE[depth])
            n = int(rows) * int(cols) * cn
            raw = f.read(n * dt.itemsize)
    except OSError:
        return None
    if len(raw) != n * dt.itemsize:
        return None
    a = np.frombuffer(raw, dtype=dt).copy()
    return a.reshape(int(rows), int(cols), cn) if cn > 1 else a.reshape(int(rows), int(cols))


def save_mat_binary(filename: str, mat: np.ndarray) -> None:
    """saveMatBinary: header (type, rows, cols) + the matrix rows."""
    a = np.ascontiguousarray(mat)
    cn = a.shape[2] if a.ndim == 3 else 1
    if a.ndim not in (2, 3):
        raise ValueError("a matrix is rows x cols [x channels]")
    with open(filename, "wb") as f:
        f.write(np.array([cv_type(a.dtype, cn), a.shape[0], a.shape[1]], dtype="<i4").tobytes())
        f.write(a.tobytes())


# ---------------------------------------------------------- FileStorage ----

def _matrix(rows: int, cols: int, dt: str, values) -> np.ndarray:
    m = re.fullmatch(r"(\d*)([ucwsifdh])", dt.strip())
    if not m:
        raise ValueError(f"unsupported FileStorage dt {dt!r}")
    cn = int(m.group(1) or 1)
    a = np.asarray([float(v) for v in values], dtype=np.float64).astype(_DT_LETTER[m.group(2)])
    if a.size != rows * cols * cn:
        raise ValueError("FileStorage matrix data length differs from rows*cols*channels")
    return a.reshape(rows, cols, cn) if cn > 1 else a.reshape(rows, cols)


def _read_xml(text: str) -> Dict[str, object]:
    root = ET.fromstring(text)
    out = {}
    for node in root:
        if node.get("type_id") == "opencv-matrix":
            out[node.tag] = _matrix(int(node.findtext("rows")), int(node.findtext("cols")), node.findtext("dt"),
                                    (node.findtext("data") or "").split())
        else:
            out[node.tag] = [float(v) for v in (node.text or "").split()]
    return out


def _read_yaml(text: str) -> Dict[str, object]:
    out = {}
    mat = re.compile(r"^(\w+):\s*!!opencv-matrix\s*\n\s+rows:\s*(\d+)\s*\n\s+cols:\s*(\d+)\s*\n\s+dt:\s*(\w+)\s*\n"
                     r"\s+data:\s*\[([^\]]*)\]", re.M)
    for m in mat.finditer(text):
        out[m.group(1)] = _matrix(int(m.group(2)), int(m.group(3)), m.group(4),
                                  [v for v in re.split(r"[\s,]+", m.group(5)) if v])
    for m in re.finditer(r"^(\w+):\s*\[([^\]]*)\]", text, re.M):
        out.setdefault(m.group(1), [float(v) for v in re.split(r"[\s,]+", m.group(2)) if v])
    return out


def read_file_storage(filename: str) -> Optional[Dict[str, object]]:
    """Top-level nodes of an OpenCV FileStorage XML or YAML file (None if it
    cannot be opened)."""
    try:
        with open(filename, "r", encoding="utf-8") as f:
            text = f.read()
    except OSError:
        return None
    return _read_yaml(text) if text.lstrip().startswith("%YAML") else _read_xml(text)


def _fmt(v) -> str:
    return repr(int(v)) if float(v).is_integer() and abs(v) < 2 ** 53 else repr(float(v))


def _xml_matrix(name: str, a: np.ndarray) -> str:
    a = np.asarray(a)
    if a.ndim == 1:
        a = a.reshape(-1, 1)
    cn = a.shape[2] if a.ndim == 3 else 1
    dt = ("" if cn == 1 else str(cn)) + _LETTER_DT[a.dtype]
    flat = [_fmt(v) if a.dtype.kind in "iu" else repr(float(v)) for v in a.reshape(-1)]
    return (f'<{name} type_id="opencv-matrix">\n  <rows>{a.shape[0]}</rows>\n  <cols>{a.shape[1]}</cols>\n'
            f"  <dt>{dt}</dt>\n  <data>\n    {' '.join(flat)}</data></{name}>\n")


def write_file_storage(filename: str, nodes: Dict[str, object]) -> None:
    """FileStorage XML with opencv-matrix nodes (numpy arrays) and integer
    sequences (tuples)."""
    parts = ['<?xml version="1.0"?>\n<opencv_storage>\n']
    for k, v in nodes.items():
        if isinstance(v, np.ndarray):
            parts.append(_xml_matrix(k, v))
        else:
            parts.append(f"<{k}>\n  {' '.join(_fmt(x) for x in v)}</{k}>\n")
    parts.append("</opencv_storage>\n")
    with open(filename, "w", encoding="utf-8") as f:
        f.write("".join(parts))


# ------------------------------------------------------ calibration files ----

def _fill_v1(nodes: Dict[str, object], params: JSLAB_StereoCalibParams_V1) -> None:
    get = lambda k: np.asarray(nodes[k], dtype=np.float64) if k in nodes else None
    K0, D0, K1, D1 = (get(k) for k in V1_KEYS[:4])
    if K0 is not None:
        params.camera_matrix[0] = K0.reshape(3, 3)
    if K1 is not None:
        params.camera_matrix[1] = K1.reshape(3, 3)
    if D0 is not None:
        params.dist_coeffs[0] = D0.reshape(-1)
    if D1 is not None:
        params.dist_coeffs[1] = D1.reshape(-1)
    if "RotationMatrix" in nodes:
        params.R = get("RotationMatrix").reshape(3, 3)
    if "TranslationVector" in nodes:
        params.t = get("TranslationVector").reshape(3)
    if "ImageSize" in nodes:
        w, h = (int(v) for v in np.asarray(nodes["ImageSize"]).reshape(-1)[:2])
        params.image_size = (w, h)


def loadStereoCalibParams_V1(filename: str, params: JSLAB_StereoCalibParams_V1) -> bool:
    """Fills params from the file; False if it cannot be opened (like the reference,
    absent keys leave the fields as they were)."""
    nodes = read_file_storage(filename)
    if nodes is None:
        return False
    _fill_v1(nodes, params)
    return True


def coeff_paths(filename: str):
    base = filename[:filename.rfind(".")] if "." in filename else filename
    return [base + s for s in ("_rx.bin", "_ry.bin", "_rz.bin")]


def loadStereoCalibParams_V2(filename: str, params: JSLAB_StereoCalibParams_V2) -> bool:
    """The V1 fields plus the three coefficient maps; True only if all three
    maps were read (the reference's return value)."""
    nodes = read_file_storage(filename)
    if nodes is None:
        return False
    _fill_v1(nodes, params)
    maps = [load_mat_binary(p) for p in coeff_paths(filename)]
    params.xyz_calib_coeffs = [m if m is not None else np.zeros((0, 0, 4), np.float32) for m in maps]
    return all(m is not None for m in maps)


def saveStereoCalibParams(filename: str, params: JSLAB_StereoCalibParams_V1) -> bool:
    """saveCalibResult: the XML file and, for V2 parameters, the three maps."""
    nodes = {
        "LeftCameraMatrix": np.asarray(params.camera_matrix[0], np.float64).reshape(3, 3),
        "LeftDistortionCoefficients": np.asarray(params.dist_coeffs[0], np.float64).reshape(1, -1),
        "RightCameraMatrix": np.asarray(params.camera_matrix[1], np.float64).reshape(3, 3),
        "RightDistortionCoefficients": np.asarray(params.dist_coeffs[1], np.float64).reshape(1, -1),
        "RotationMatrix": np.asarray(params.R, np.float64).reshape(3, 3),
        "TranslationVector": np.asarray(params.t, np.float64).reshape(3, 1),
        "ImageSize": tuple(int(v) for v in params.image_size),
    }
    try:
        write_file_storage(filename, nodes)
        if isinstance(params, JSLAB_StereoCalibParams_V2):
            for p, m in zip(coeff_paths(filename), params.xyz_calib_coeffs):
                save_mat_binary(p, np.asarray(m, np.float32))
    except OSError:
        return False
    return True


__all__ = ["load_mat_binary", "save_mat_binary", "read_file_storage", "write_file_storage", "cv_type",
           "loadStereoCalibParams_V1", "loadStereoCalibParams_V2", "saveStereoCalibParams", "coeff_paths"]
