"""zim_compact_points_noalloc: the compaction entry point that allocates no
device memory, for callers that may not call cudaMalloc (a host application
that owns all device memory through its own pool, or a capture loop that
cannot take the synchronisation cudaMalloc/cudaFree may imply).

It is called through the C ABI and compared with zim_compact_points (the
allocating entry point) on two calls in a row: compaction is integer work, so
the outputs must be identical.  This file sorts last so that a run stopping at
the first failure has already run every other test; it also passes alone.
"""
import ctypes as C

import numpy as np
import pytest
import torch


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def noalloc(native, xyz, mask):
    H, W = mask.shape
    pts = torch.full((H * W, 4), -7.0, dtype=torch.float32, device="cuda")
    cnt = torch.full((1,), 12345, dtype=torch.int64, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = native.zim_compact_points_noalloc(_ptr(xyz), _ptr(mask), H, W, _ptr(pts), _ptr(cnt), st)
    torch.cuda.synchronize()
    return rc, pts[: int(cnt.item())]


def cloud(h, w, seed, p):
    g = torch.Generator(device="cuda").manual_seed(seed)
    xyz = torch.rand((h, w, 3), device="cuda", generator=g) * 900.0
    mask = (torch.rand((h, w), device="cuda", generator=g) < p).to(torch.uint8)
    return xyz, mask


@pytest.mark.gpu
def test_noalloc_compaction_equals_allocating_entry(native, ctx):
    from zim_gb300 import _lib, api
    cases = [cloud(2092, 2501, 1, 0.75), cloud(480, 640, 2, 0.30)]
    for call in range(2):  # two calls in a row over the shared array
        for xyz, mask in cases:
            ref = api.compact_points(ctx, xyz, mask)
            rc, got = noalloc(native, xyz, mask)
            assert rc == _lib.OK
            assert got.shape == ref.shape == (int(mask.sum().item()), 4)
            assert torch.equal(got, ref), f"call {call}"


@pytest.mark.gpu
def test_noalloc_rejects_sizes_beyond_its_array(native):
    from zim_gb300 import _lib
    xyz, mask = cloud(8, 8, 3, 0.5)
    pts = torch.empty((64, 4), device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    # 8193 x 8193 > 64 Mi pixels: rejected before any work is launched
    rc = native.zim_compact_points_noalloc(_ptr(xyz), _ptr(mask), 8193, 8193, _ptr(pts), _ptr(cnt), st)
    assert rc == _lib.ERR_INVALID_ARG
    assert native.zim_compact_points_noalloc(None, _ptr(mask), 8, 8, _ptr(pts), _ptr(cnt), st) == _lib.ERR_INVALID_ARG
