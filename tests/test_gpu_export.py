"""Device-side parts of the on-disk outputs: the packed PLY vertex body
(zim_pack_ply) against numpy's packing of the same cloud, whole PLY files, and
rectifyLeftImage (zim_rectify_image) against the oracle's fixed-point remap,
bit-exact."""
import numpy as np
import pytest
import torch

from conftest import scene_data

PLY_GRAY = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("r", "u1"), ("g", "u1"), ("b", "u1")])


def cloud(h=61, w=97, seed=0):
    rng = np.random.default_rng(seed)
    xyz = rng.normal(0, 100, (h, w, 3)).astype(np.float32)
    mask = (rng.random((h, w)) < 0.6).astype(np.uint8)
    gray = rng.integers(0, 256, (h, w), dtype=np.uint8)
    return xyz, mask, gray


def numpy_body(xyz, mask, gray=None, with_gray=False):
    m = mask > 0
    if not with_gray:
        return xyz[m].astype("<f4").tobytes()
    rec = np.zeros(int(m.sum()), PLY_GRAY)
    p = xyz[m]
    rec["x"], rec["y"], rec["z"] = p[:, 0], p[:, 1], p[:, 2]
    g = gray[m] if gray is not None else np.full(int(m.sum()), 255, np.uint8)
    rec["r"] = rec["g"] = rec["b"] = g
    return rec.tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["xyz", "gray", "white"])
def test_pack_ply_body(ctx, variant):
    from zim_gb300 import api
    xyz, mask, gray = cloud()
    g = torch.from_numpy(gray).cuda() if variant == "gray" else None
    body = api.pack_ply(ctx, torch.from_numpy(xyz).cuda(), torch.from_numpy(mask).cuda(), g,
                        with_gray=variant != "xyz")
    want = numpy_body(xyz, mask, gray if variant == "gray" else None, variant != "xyz")
    assert body.cpu().numpy().tobytes() == want


@pytest.mark.gpu
def test_ply_files(ctx, tmp_path):
    from zim_gb300 import export
    xyz, mask, gray = cloud(seed=3)
    fn = tmp_path / "c.ply"
    assert export.savePointCloudToPlyBinaryWithGray(xyz, mask, gray, str(fn), ctx)
    data = fn.read_bytes()
    head = export._ply_header(int(mask.sum()), True)
    assert data.startswith(head) and data[len(head):] == numpy_body(xyz, mask, gray, True)
    assert export.savePointCloudToPlyBinary(xyz, mask, str(fn), ctx)
    data = fn.read_bytes()
    head = export._ply_header(int(mask.sum()), False)
    assert data.startswith(head) and data[len(head):] == numpy_body(xyz, mask)
    assert not export.savePointCloudToPlyBinaryWithGray(xyz, mask, gray[:-1], str(fn), ctx)


@pytest.mark.gpu
@pytest.mark.parametrize("cam", [0, 1])
def test_rectify_image_bit_exact(ctx, oracle_lib, cam):
    from zim_gb300 import api
    spec, L, R, _ = scene_data("config1", width=612, height=512)
    ctx.set_calibration(spec.rig.as_dict(), True)
    img = (L if cam == 0 else R)[0]
    img8 = (img >> 4).astype(np.uint8) if img.dtype == np.uint16 else img
    out = api.rectify_image(ctx, cam, torch.from_numpy(np.ascontiguousarray(img8)).cuda())
    mx, my = (t.cpu().numpy() for t in ctx.rectify_maps(cam))
    want = oracle_lib.remap_u8(img8, mx, my)
    assert np.array_equal(out.cpu().numpy(), want)
