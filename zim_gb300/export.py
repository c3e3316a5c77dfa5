"""On-disk outputs of the reference's drivers, written from device clouds.

- ``savePointCloudToPlyBinary`` / ``savePointCloudToPlyBinaryWithGray``
  (main.cpp:85-160): binary little-endian PLY, float x y z (+ uchar red green
  blue = the grey value).  The vertex body is packed on the GPU
  (zim_pack_ply) and copied out once; the host writes the header and the body.
- ``saveToTxt`` (main.cpp:162-184): "x y z" lines of the points with
  -10000 < z < 10000 and |z| > 0.0001, six significant digits like a default
  std::ostream.
- ``saveRaw64F`` (JSLAB_PhaseDisparityExporter.cpp:115-141): row-major doubles
  plus the same info text.
"""
from __future__ import annotations

import numpy as np
import torch

from . import api


def _ply_header(count: int, gray: bool) -> bytes:
    h = f"ply\nformat binary_little_endian 1.0\nelement vertex {count}\n"
    h += "property float x\nproperty float y\nproperty float z\n"
    if gray:
        h += "property uchar red\nproperty uchar green\nproperty uchar blue\n"
    return (h + "end_header\n").encode()


def _cloud(xyz, P):
    xyz = torch.as_tensor(xyz)
    P = torch.as_tensor(P)
    if xyz.dim() != 3 or xyz.shape[2] != 3 or P.shape != xyz.shape[:2] or xyz.dtype != torch.float32 \
            or P.dtype != torch.uint8:
        return None, None
    return xyz.to("cuda").contiguous(), P.to("cuda").contiguous()


def _write(ctx, xyz, P, gray, with_gray, file_name) -> bool:
    body = api.pack_ply(ctx, xyz, P, gray, with_gray).cpu().numpy()
    n = body.size // (15 if with_gray else 12)
    try:
        with open(file_name, "wb") as f:
            f.write(_ply_header(n, with_gray))
            f.write(body.tobytes())
    except OSError:
        return False
    return True


def savePointCloudToPlyBinary(xyz, P, file_name: str, ctx: api.Context) -> bool:
    xyz, P = _cloud(xyz, P)
    if xyz is None:
        return False
    return _write(ctx, xyz, P, None, False, file_name)


def savePointCloudToPlyBinaryWithGray(xyz, P, gray_image, file_name: str, ctx: api.Context,
                                      enable_gray_color: bool = True) -> bool:
    """gray_image: the rectified left image (8-bit, same size), or None for
    white points; False on a size or type mismatch, like the reference."""
    xyz, P = _cloud(xyz, P)
    if xyz is None:
        return False
    gray = None
    if enable_gray_color and gray_image is not None:
        g = torch.as_tensor(gray_image)
        if g.dtype != torch.uint8 or tuple(g.shape) != tuple(P.shape):
            return False
        gray = g.to("cuda").contiguous()
    return _write(ctx, xyz, P, gray, True, file_name)


def saveToTxt(xyz, filename: str) -> bool:
    a = torch.as_tensor(xyz).cpu().numpy().reshape(-1, 3)
    z = a[:, 2]
    keep = a[(z > -10000) & (z < 10000) & (np.abs(z) > 0.0001)]
    try:
        with open(filename, "w") as f:
            f.writelines(f"{p[0]:g} {p[1]:g} {p[2]:g}\n" for p in keep.tolist())
    except OSError:
        return False
    return True


def saveRaw64F(data, raw_path: str, info_path: str) -> bool:
    a = np.ascontiguousarray(torch.as_tensor(data).cpu().numpy())
    if a.ndim != 2 or a.size == 0 or a.dtype != np.float64:
        return False
    try:
        with open(raw_path, "wb") as f:
            f.write(a.astype("<f8").tobytes())
    except OSError:
        return False
    try:
        with open(info_path, "w") as f:
            f.write(f"rows {a.shape[0]}\ncols {a.shape[1]}\ntype CV_64FC1 (double)\n"
                    "layout row-major, one double per pixel\n"
                    "rows/cols written on the FIRST line as 'rows cols' for convenience\n")
    except OSError:
        pass
    return True


def loadRaw64F(raw_path: str, rows: int, cols: int) -> np.ndarray:
    return np.fromfile(raw_path, dtype="<f8", count=rows * cols).reshape(rows, cols)


__all__ = ["savePointCloudToPlyBinary", "savePointCloudToPlyBinaryWithGray", "saveToTxt", "saveRaw64F",
           "loadRaw64F"]
