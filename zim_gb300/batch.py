"""The batched path (``zim_batch_*`` in include/zim.h) on torch CUDA tensors.

    b = Batch(ctx, [rig_a, rig_b])              # one rectification per calibration
    b.submit([BatchPair(cfg, left, right, calib=0), ...], recon_config())
    b.autotune()                                 # optional: picks band heights / CTAs per SM
    b.run()                                      # replays the captured CUDA graph

Each pair gets ``xyz`` (rect_h, rect_w, 3) and ``mask`` outputs (allocated by
``submit`` unless given), equal bit for bit to what ``reconstruct_pair``
returns for it with the same config.  A pair's ``filters`` (a recon_config)
chooses its grid filters (SOR, MLS, metric Gaussian); without it the
submission's config does.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import torch

from . import _lib
from .api import Context, _p, _sample_type, _stream, calib_struct


@dataclass
class BatchPair:
    decode: _lib.DecodeConfig
    left: torch.Tensor            # (F, H, W) u8 / u16 frame stack on the device
    right: torch.Tensor
    calib: int = 0
    pha_f: int = 0
    xyz: Optional[torch.Tensor] = None
    mask: Optional[torch.Tensor] = None
    disp: Optional[torch.Tensor] = None
    filters: Optional[object] = None  # a recon_config whose grid filters apply to this pair


class Batch:
    def __init__(self, ctx: Context, calibs: Sequence, full_left: bool = True):
        self.ctx = ctx
        self._L = ctx._L
        arr = (_lib.StereoCalib * len(calibs))()
        for i, c in enumerate(calibs):
            arr[i] = c if isinstance(c, _lib.StereoCalib) else calib_struct(**c)
        h = C.c_void_p()
        ctx.check(self._L.zim_batch_create(ctx.h, arr, len(calibs), int(bool(full_left)), C.byref(h)))
        self.h = h
        self.pairs = []

    def close(self):
        if getattr(self, "h", None):
            self._L.zim_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def rect_size(self, calib: int):
        w, h = C.c_int(), C.c_int()
        self.ctx.check(self._L.zim_batch_rect_size(self.h, calib, C.byref(w), C.byref(h)))
        return w.value, h.value

    def submit(self, pairs: Sequence[BatchPair], rcfg, tuning: Optional[dict] = None):
        arr = (_lib.BatchPair * len(pairs))()
        for i, p in enumerate(pairs):
            w, h = self.rect_size(p.calib)
            dev = p.left.device
            if p.xyz is None:
                p.xyz = torch.empty((h, w, 3), dtype=torch.float32, device=dev)
            if p.mask is None:
                p.mask = torch.empty((h, w), dtype=torch.uint8, device=dev)
            s = arr[i]
            s.decode = p.decode
            s.sample_type = _sample_type(p.left)
            s.rows, s.cols = p.left.shape[1], p.left.shape[2]
            s.calib, s.pha_f = p.calib, p.pha_f
            s.frames[0] = _p(p.left).value
            s.frames[1] = _p(p.right).value
            s.xyz = _p(p.xyz).value
            s.mask = _p(p.mask).value
            s.disp = _p(p.disp).value if p.disp is not None else None
            s.filters = C.cast(C.pointer(p.filters), C.c_void_p).value if p.filters is not None else None
        t = None
        if tuning is not None:
            t = _lib.BatchTuning(**tuning)
        self.ctx.check(self._L.zim_batch_submit(self.h, arr, len(pairs), C.byref(rcfg),
                                                C.byref(t) if t is not None else None))
        self.pairs = list(pairs)
        return self

    def run(self):
        self.ctx.check(self._L.zim_batch_run(self.h, _stream()))

    def autotune(self):
        t = _lib.BatchTuning()
        ms = C.c_double()
        self.ctx.check(self._L.zim_batch_autotune(self.h, _stream(), C.byref(t), C.byref(ms)))
        return self._tuning_dict(t), ms.value

    def tuning(self) -> dict:
        t = _lib.BatchTuning()
        self.ctx.check(self._L.zim_batch_get_tuning(self.h, C.byref(t)))
        return self._tuning_dict(t)

    @staticmethod
    def _tuning_dict(t) -> dict:
        return {"decode_rows": t.decode_rows, "match_rows": t.match_rows, "filter_rows": t.filter_rows,
                "ctas_per_sm": t.ctas_per_sm}
