"""Seeded synthetic stereo fringe scenes (the benchmark's and the tests' inputs).

The scenes follow the workload descriptions this library is measured on:

* ``config0``: 640x480, f = 800 px, c = (320, 240), baseline 120 mm, no
  distortion; 4-step phase shift + 5 Gray bits + 1 complementary Gray bit, u8,
  I = A + B cos(.) + N(0, 2^2), A ~ U(80, 120), B ~ U(60, 100); a plane at
  Z = 800 mm carrying a sphere of radius 120 mm centred at Z = 700 mm.  The
  projector is 1280 px wide; 5 Gray bits code 32 periods, so the fringe period
  is 40 px (1280 / 32) rather than 32 px (which would need 40 codewords).
* ``config1``: 2448x2048 (5 MP), f = 2400 px, baseline 200 mm, k1 = -0.05,
  k2 = 0.01; 1/8/64 fringes across a 1280 px projector, 4 steps each, 12-bit
  values in u16 with sigma = 8 and the 8-bit A/B ranges scaled by 16; 20 seeded
  Gaussian bumps (5-40 mm, sigma 20-150 mm) over a plane at 900 mm plus two box
  occluders.
* ``ref_heterodyne``: the reference's own 3-frequency heterodyne (121/110/120,
  8 steps, u8) on the config-1 geometry.
* ``pose_plane``: a planar target at a seeded pose (tilt +-30 deg, depth
  600-1200 mm) on the config-1 rig.

The projector is a pinhole midway between the cameras, looking along +Z.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _build

ENC_HETERODYNE3, ENC_HIERARCHICAL, ENC_GRAYCODE, ENC_GRAYCODE_COMPLEMENTARY = range(4)


class _Scene(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("K", (C.c_double * 9) * 2), ("D", (C.c_double * 5) * 2),
                ("R", C.c_double * 9), ("t", C.c_double * 3), ("proj_K", C.c_double * 9), ("proj_width", C.c_int),
                ("proj_height", C.c_int), ("proj_R", C.c_double * 9), ("proj_t", C.c_double * 3),
                ("scene_kind", C.c_int), ("plane_z", C.c_double), ("max_relief", C.c_double),
                ("plane_n", C.c_double * 3), ("plane_d", C.c_double), ("sphere", C.c_double * 4),
                ("n_bumps", C.c_int), ("bumps", (C.c_double * 4) * 32), ("n_boxes", C.c_int),
                ("boxes", (C.c_double * 5) * 4), ("encoding", C.c_int), ("n_freq", C.c_int), ("gray_bits", C.c_int),
                ("freq", C.c_double * 4), ("shift_num", C.c_int * 4), ("bit_depth", C.c_int), ("A_lo", C.c_double),
                ("A_hi", C.c_double), ("B_lo", C.c_double), ("B_hi", C.c_double), ("noise_sigma", C.c_double),
                ("seed", C.c_uint64)]


_lib = None


def _load():
    global _lib
    if _lib is None:
        if not _build.SYNTH_LIB.exists():
            _build.build_synth()
        _lib = C.CDLL(str(_build.SYNTH_LIB))
        _lib.zs_render.restype = C.c_int
        _lib.zs_frame_count.restype = C.c_int
    return _lib


@dataclass
class Rig:
    width: int
    height: int
    K: list            # two 3x3
    D: list            # two length-5
    R: np.ndarray      # left -> right
    t: np.ndarray

    def as_dict(self):
        return dict(K=[np.asarray(k, float) for k in self.K], D=[np.asarray(d, float) for d in self.D],
                    R=np.asarray(self.R, float), t=np.asarray(self.t, float), width=self.width, height=self.height)


@dataclass
class SceneSpec:
    name: str
    rig: Rig
    encoding: int
    freq: tuple
    shift_num: tuple
    gray_bits: int = 0
    bit_depth: int = 8
    A: tuple = (80.0, 120.0)
    B: tuple = (60.0, 100.0)
    noise: float = 2.0
    seed: int = 0
    scene_kind: int = 0
    plane_z: float = 800.0
    plane_n: tuple = (0.0, 0.0, 1.0)
    plane_d: float = 800.0
    sphere: tuple = (0.0, 0.0, 0.0, 0.0)
    bumps: list = field(default_factory=list)
    boxes: list = field(default_factory=list)
    proj_width: int = 1280
    proj_height: int = 1024
    proj_f: float = 1000.0
    proj_center: tuple = (0.0, 0.0, 0.0)
    modulation_threshold: float = 0.3
    preblur_sigma: float = 3.0

    @property
    def n_freq(self):
        if self.encoding == ENC_HETERODYNE3:
            return 3
        return len(self.freq) if self.encoding == ENC_HIERARCHICAL else 1

    @property
    def sample_dtype(self):
        return np.uint8 if self.bit_depth == 8 else np.uint16

    @property
    def pha_f(self):
        if self.encoding == ENC_HETERODYNE3:
            return int(self.freq[0])
        if self.encoding == ENC_HIERARCHICAL:
            return int(self.freq[-1]) - 1
        return (1 << self.gray_bits) - 1

    def decode_kwargs(self):
        """Arguments for the decoder config of this scene."""
        return dict(encoding=self.encoding, freq=tuple(self.freq), shift_num=tuple(self.shift_num),
                    gray_bits=self.gray_bits, modulation_threshold=self.modulation_threshold,
                    preblur_sigma=self.preblur_sigma)

    def _struct(self) -> _Scene:
        s = _Scene()
        r = self.rig
        s.width, s.height = r.width, r.height
        for k in range(2):
            for i, v in enumerate(np.asarray(r.K[k], float).reshape(9)):
                s.K[k][i] = v
            for i, v in enumerate(np.asarray(r.D[k], float).reshape(5)):
                s.D[k][i] = v
        for i, v in enumerate(np.asarray(r.R, float).reshape(9)):
            s.R[i] = v
        for i, v in enumerate(np.asarray(r.t, float).reshape(3)):
            s.t[i] = v
        pk = [self.proj_f, 0, (self.proj_width - 1) / 2, 0, self.proj_f, (self.proj_height - 1) / 2, 0, 0, 1]
        for i, v in enumerate(pk):
            s.proj_K[i] = v
        s.proj_width, s.proj_height = self.proj_width, self.proj_height
        for i in range(9):
            s.proj_R[i] = 1.0 if i % 4 == 0 else 0.0
        for i in range(3):
            s.proj_t[i] = -self.proj_center[i]
        s.scene_kind = self.scene_kind
        s.plane_z = self.plane_z
        s.max_relief = sum(b[2] for b in self.bumps) + 1.0
        for i in range(3):
            s.plane_n[i] = self.plane_n[i]
        s.plane_d = self.plane_d
        for i in range(4):
            s.sphere[i] = self.sphere[i]
        s.n_bumps = len(self.bumps)
        for j, b in enumerate(self.bumps):
            for i in range(4):
                s.bumps[j][i] = b[i]
        s.n_boxes = len(self.boxes)
        for j, b in enumerate(self.boxes):
            for i in range(5):
                s.boxes[j][i] = b[i]
        s.encoding = self.encoding
        s.n_freq = self.n_freq
        s.gray_bits = self.gray_bits
        for i, f in enumerate(self.freq):
            s.freq[i] = f
        for i, n in enumerate(self.shift_num):
            s.shift_num[i] = n
        s.bit_depth = self.bit_depth
        s.A_lo, s.A_hi = self.A
        s.B_lo, s.B_hi = self.B
        s.noise_sigma = self.noise
        s.seed = self.seed & 0xFFFFFFFFFFFFFFFF
        return s

    def frame_count(self) -> int:
        return _load().zs_frame_count(C.byref(self._struct()))

    def render(self, cam: int, with_xyz: bool = False):
        """Frames (F, H, W) of camera `cam` (0 left, 1 right) [+ ground-truth xyz]."""
        s = self._struct()
        F = self.frame_count()
        frames = np.empty((F, self.rig.height, self.rig.width), self.sample_dtype)
        xyz = np.empty((self.rig.height, self.rig.width, 3), np.float32) if with_xyz else None
        _load().zs_render(C.byref(s), C.c_int(cam), frames.ctypes.data_as(C.c_void_p),
                          xyz.ctypes.data_as(C.c_void_p) if with_xyz else None)
        return (frames, xyz) if with_xyz else frames


def make_rig(width, height, f, baseline, dist=(0, 0, 0, 0, 0), cx=None, cy=None, R=None) -> Rig:
    cx = (width - 1) / 2.0 if cx is None else cx
    cy = (height - 1) / 2.0 if cy is None else cy
    K = np.array([[f, 0, cx], [0, f, cy], [0, 0, 1]], float)
    R = np.eye(3) if R is None else np.asarray(R, float)
    # right camera centre at (baseline, 0, 0) in left coordinates: X_r = R (X_l - C)
    t = -R @ np.array([baseline, 0.0, 0.0])
    return Rig(width, height, [K, K.copy()], [np.array(dist, float), np.array(dist, float)], R, t)


def config0(seed: int = 0, width: int = 640, height: int = 480) -> SceneSpec:
    s = width / 640.0
    rig = make_rig(width, height, 800.0 * s, 120.0, cx=320.0 * s, cy=240.0 * s)
    return SceneSpec(name="config0", rig=rig, encoding=ENC_GRAYCODE_COMPLEMENTARY, freq=(32,), shift_num=(4,),
                     gray_bits=5, bit_depth=8, A=(80, 120), B=(60, 100), noise=2.0, seed=seed, scene_kind=0,
                     plane_d=800.0, sphere=(60.0, 0.0, 700.0, 120.0), proj_width=1280, proj_height=1024,
                     proj_f=1280 * 800 / 760.0, proj_center=(60.0, 0.0, 0.0))


def _bumps_boxes(rng):
    bumps = [(rng.uniform(-400, 600), rng.uniform(-350, 350), rng.uniform(5, 40), rng.uniform(20, 150))
             for _ in range(20)]
    boxes = []
    for i in range(2):
        w, h = rng.uniform(120, 250), rng.uniform(120, 250)
        x0 = rng.uniform(-300, 450 - w) if i == 0 else rng.uniform(0, 500 - w)
        y0 = rng.uniform(-250, 250 - h)
        boxes.append((x0, x0 + w, y0, y0 + h, 900.0 - rng.uniform(60, 120)))
    return bumps, boxes


def config1(seed: int = 1, width: int = 2448, height: int = 2048) -> SceneSpec:
    rng = np.random.default_rng(seed)
    rig = make_rig(width, height, 2400.0 * width / 2448.0, 200.0, dist=(-0.05, 0.01, 0, 0, 0))
    bumps, boxes = _bumps_boxes(rng)
    return SceneSpec(name="config1", rig=rig, encoding=ENC_HIERARCHICAL, freq=(1, 8, 64), shift_num=(4, 4, 4),
                     bit_depth=12, A=(1280, 1920), B=(960, 1600), noise=8.0, seed=seed, scene_kind=1, plane_z=900.0,
                     bumps=bumps, boxes=boxes, proj_width=1280, proj_height=1024, proj_f=1280 * 900 / 1200.0,
                     proj_center=(100.0, 0.0, 0.0))


def ref_heterodyne(seed: int = 2, width: int = 2448, height: int = 2048, freq=(121, 110, 120), steps=8) -> SceneSpec:
    s = config1(seed, width, height)
    s.name = "ref_heterodyne"
    s.encoding = ENC_HETERODYNE3
    s.freq = tuple(freq)
    s.shift_num = (steps, steps, steps)
    s.bit_depth = 8
    s.A, s.B, s.noise = (80, 120), (60, 100), 2.0
    return s


CONFIG2_SIZES = ((640, 480), (1280, 1024), (2448, 2048), (4096, 3000))


def config2(seed: int = 7, n_pairs: int = 64, sizes=CONFIG2_SIZES):
    """The mixed batch: n_pairs stereo pairs, each with a size drawn from
    `sizes` and an encoding drawn from {4-step + 5-bit Gray + complementary bit
    (the config-0 scene and rig, scaled to the size, 8-bit), three-frequency
    1/8/64 x 4 steps in 12-bit u16 (the config-1 encoding, scene and rig,
    scaled, with a pair-specific seed)}.  Pairs of the same size and encoding
    share a calibration.  Returns (specs, calib_keys)."""
    rng = np.random.default_rng(seed)
    specs, keys = [], []
    for i in range(n_pairs):
        w, h = sizes[int(rng.integers(len(sizes)))]
        gray = bool(rng.integers(2))
        sd = int(seed * 1000 + i)
        s = config0(sd, w, h) if gray else config1(sd, w, h)
        s.name = f"config2_{i}"
        specs.append(s)
        keys.append(("gray" if gray else "freq3", w, h))
    return specs, keys


def pose_plane(seed: int = 3, width: int = 2448, height: int = 2048, pose: int = 0) -> SceneSpec:
    rng = np.random.default_rng(seed * 1000 + pose)
    s = config1(seed, width, height)
    s.name = f"pose_plane{pose}"
    tx, ty = np.deg2rad(rng.uniform(-30, 30)), np.deg2rad(rng.uniform(-30, 30))
    depth = rng.uniform(600, 1200)
    n = np.array([np.sin(tx), np.sin(ty), 1.0])
    n /= np.linalg.norm(n)
    centre = np.array([100.0, 0.0, depth])
    s.scene_kind = 2
    s.plane_n = tuple(n)
    s.plane_d = float(n @ centre)
    s.bumps, s.boxes = [], []
    return s
