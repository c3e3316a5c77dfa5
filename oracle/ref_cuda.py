"""The reference's own CUDA kernels on the GPU: a second witness for parity.

TEST INFRASTRUCTURE ONLY (the checker, never the thing measured or shipped).
oracle/ref_build.py compiles the reference's three CUDA files, device code
only, into oracle/_ref/*.cubin; this module loads those cubins through the CUDA
driver API (ctypes on libcuda) into the context torch uses and launches their
kernels on torch tensors, exactly as the reference's host launchers do
(grid of 16 x 16 blocks, the same arguments and constant tables):

  * decodeKernel            JSLAB_PhaseShiftDecoder_V2_GPU.cu:44-146, launched as at :270-278
  * buildOrderRangeKernel,  JSLAB_PhaseEpipolarReconstructor_V2_GPU.cu:18-37 and :45-113,
    stereoMatchKernel       launched as at :460-463
  * medianFilter5x5Kernel   same file :119-150
  * reprojectTo3DKernel     :157-213
  * gaussianFilterKernel    :220-274 (its weights: getGaussianKernel(3, 0.7) outer product, :395-400)
  * radiusOutlierKernel     :281-347
  * mlsKernel               JSLAB_MLS_Filter.cu:165-391, launched as at :434-439

Only the kernels run here; the launchers' host code (cv::Mat conversions,
allocation) is what this module restates.
"""
from __future__ import annotations

import ctypes as C
import json
import math
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
INDEX = REF_DIR / "ref_cubins.json"


def available() -> bool:
    if not INDEX.exists():
        return False
    idx = json.loads(INDEX.read_text())
    return all((REF_DIR / f).exists() for f in idx)


class _Driver:
    def __init__(self):
        self.lib = C.CDLL("libcuda.so.1")
        self._ok(self.lib.cuInit(0), "cuInit")

    def _ok(self, r, what):
        if r != 0:
            raise RuntimeError(f"{what} failed: CUresult {r}")


def _launch_args(args):
    """ctypes storage for each argument and the void* array cuLaunchKernel wants."""
    store = []
    for a in args:
        if isinstance(a, C._SimpleCData):
            store.append(a)
        else:
            raise TypeError(f"kernel argument {a!r} is not a ctypes value")
    arr = (C.c_void_p * len(store))(*[C.cast(C.pointer(v), C.c_void_p) for v in store])
    return store, arr


class RefCuda:
    """The loaded cubins (in the current CUDA context, which torch creates)."""

    def __init__(self):
        import torch
        if not available():
            raise FileNotFoundError("oracle/_ref cubins not built (oracle/ref_build.py builds them where the "
                                    "reference's sources are)")
        torch.cuda.init()
        torch.empty(1, device="cuda")  # the primary context is current on this thread
        self.drv = _Driver()
        lib = self.drv.lib
        lib.cuModuleLoadData.argtypes = [C.POINTER(C.c_void_p), C.c_void_p]
        lib.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
        lib.cuModuleGetGlobal_v2.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_size_t), C.c_void_p, C.c_char_p]
        lib.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                       C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.c_void_p]
        lib.cuMemcpyHtoD_v2.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
        self.modules, self.funcs = {}, {}
        self._images = []
        for cubin, names in json.loads(INDEX.read_text()).items():
            img = C.create_string_buffer((REF_DIR / cubin).read_bytes())
            self._images.append(img)
            mod = C.c_void_p()
            self.drv._ok(lib.cuModuleLoadData(C.byref(mod), C.cast(img, C.c_void_p)), f"cuModuleLoadData({cubin})")
            self.modules[cubin] = mod
            for mangled in names:
                fn = C.c_void_p()
                self.drv._ok(lib.cuModuleGetFunction(C.byref(fn), mod, mangled.encode()), f"get {mangled}")
                # the plain name: the identifier after the _Z<len> prefix
                i = 2
                while mangled[i].isdigit():
                    i += 1
                n = int(mangled[2:i])
                self.funcs[mangled[i:i + n]] = fn

    def set_constant(self, cubin, name, data: bytes):
        ptr, size = C.c_uint64(), C.c_size_t()
        lib = self.drv.lib
        self.drv._ok(lib.cuModuleGetGlobal_v2(C.byref(ptr), C.byref(size), self.modules[cubin], name.encode()),
                     f"cuModuleGetGlobal({name})")
        assert size.value == len(data), (name, size.value, len(data))
        buf = C.create_string_buffer(data, len(data))
        self.drv._ok(lib.cuMemcpyHtoD_v2(ptr.value, buf, len(data)), "cuMemcpyHtoD")

    def launch2d(self, name, rows, cols, *args):
        """The reference launchers' shape: 16 x 16 blocks over the image."""
        import torch
        store, arr = _launch_args(args)
        st = torch.cuda.current_stream().cuda_stream
        self.drv._ok(self.drv.lib.cuLaunchKernel(self.funcs[name], (cols + 15) // 16, (rows + 15) // 16, 1, 16, 16,
                                                 1, 0, C.c_void_p(st), arr, None), f"launch {name}")
        del store


def ptr(t):
    return C.c_void_p(t.data_ptr())


def gaussian_kernel3(sigma: float):
    """getGaussianKernel(3, sigma) as OpenCV defines it for sigma > 0:
    exp(-(i - 1)^2 / (2 sigma^2)) normalised to sum 1, in double."""
    g = [math.exp(-((i - 1) ** 2) / (2.0 * sigma * sigma)) for i in range(3)]
    s = sum(g)
    return [v / s for v in g]


def decode(rc: RefCuda, frames_u8, shift_num, freq, modulation_threshold, preblur_sigma, avg_three=False):
    """decodeKernel on a u8 frame stack (sum(shift_num) x rows x cols, frame
    order of the reference).  Returns (phase f64, k i32, mod f64) tensors."""
    import struct

    import torch
    F, rows, cols = frames_u8.shape
    g = gaussian_kernel3(preblur_sigma)
    blur = [g[i] * g[j] for i in range(3) for j in range(3)]
    rc.set_constant("JSLAB_PhaseShiftDecoder_V2_GPU.cubin", "c_blur", struct.pack("9d", *blur))
    sins, coss = [], []
    for n in shift_num:
        for k in range(n):
            sins.append(math.sin(2.0 * math.pi * k / n))
            coss.append(math.cos(2.0 * math.pi * k / n))
    dev = frames_u8.device
    d_sin = torch.tensor(sins, dtype=torch.float64, device=dev)
    d_cos = torch.tensor(coss, dtype=torch.float64, device=dev)
    phase = torch.zeros((rows, cols), dtype=torch.float64, device=dev)
    mod = torch.zeros((rows, cols), dtype=torch.float64, device=dev)
    kmap = torch.zeros((rows, cols), dtype=torch.int32, device=dev)
    s0, s1, s2 = shift_num
    I = C.c_int
    rc.launch2d("decodeKernel", rows, cols, ptr(frames_u8), I(rows), I(cols), ptr(d_sin), ptr(d_cos), I(s0), I(s1),
                I(s2), I(0), I(s0), I(s0 + s1), I(0), I(s0), I(s0 + s1), C.c_double(freq[0]), C.c_double(freq[1]),
                C.c_double(freq[2]), C.c_double(modulation_threshold), I(1 if avg_three else 0), ptr(phase), ptr(kmap),
                ptr(mod))
    torch.cuda.synchronize()
    return phase, kmap, mod


def stereo_match(rc: RefCuda, l_phase, r_phase, l_k, r_k, pha_f, grad_threshold):
    """buildOrderRangeKernel + stereoMatchKernel on rectified maps (f64 phase,
    i32 order); the span tables initialised as the launcher does."""
    import torch
    rows, cols = l_phase.shape
    knum = pha_f if pha_f > 0 else 0
    dev = l_phase.device
    col_min = torch.full((rows * (knum + 1),), 0x7F7F7F7F, dtype=torch.int32, device=dev)
    col_max = torch.full((rows * (knum + 1),), -1, dtype=torch.int32, device=dev)
    disp = torch.zeros((rows, cols), dtype=torch.float32, device=dev)
    I = C.c_int
    rc.launch2d("buildOrderRangeKernel", rows, cols, ptr(r_k), I(rows), I(cols), I(knum), ptr(col_min), ptr(col_max))
    rc.launch2d("stereoMatchKernel", rows, cols, ptr(l_phase), ptr(r_phase), ptr(l_k), ptr(r_k), ptr(col_min),
                ptr(col_max), I(rows), I(cols), I(pha_f), C.c_double(grad_threshold), ptr(disp))
    torch.cuda.synchronize()
    return disp


def median5(rc: RefCuda, disp):
    import torch
    rows, cols = disp.shape
    out = torch.zeros_like(disp)
    rc.launch2d("medianFilter5x5Kernel", rows, cols, ptr(disp), ptr(out), C.c_int(rows), C.c_int(cols))
    torch.cuda.synchronize()
    return out


def reproject(rc: RefCuda, disp, Q, R1, min_depth, max_depth, use_rectified):
    import torch
    rows, cols = disp.shape
    dev = disp.device
    dQ = torch.tensor(list(Q), dtype=torch.float64, device=dev)
    dR = torch.tensor(list(R1), dtype=torch.float64, device=dev)
    xyz = torch.zeros((rows, cols, 3), dtype=torch.float32, device=dev)
    P = torch.zeros((rows, cols), dtype=torch.uint8, device=dev)
    rc.launch2d("reprojectTo3DKernel", rows, cols, ptr(disp), C.c_int(rows), C.c_int(cols), ptr(dQ), ptr(dR),
                C.c_double(min_depth), C.c_double(max_depth), C.c_int(1 if use_rectified else 0), ptr(xyz), ptr(P))
    torch.cuda.synchronize()
    return xyz, P


def px_gaussian(rc: RefCuda, xyz, P):
    """gaussianFilterKernel; its weights are the float outer product of
    getGaussianKernel(3, 0.7, CV_32F) (each 1-D weight rounded to float, the
    product rounded to float)."""
    import struct

    import numpy as np
    import torch
    g = np.array(gaussian_kernel3(0.7), dtype=np.float32)
    w = [float(np.float32(g[i]) * np.float32(g[j])) for i in range(3) for j in range(3)]
    rc.set_constant("JSLAB_PhaseEpipolarReconstructor_V2_GPU.cubin", "c_pc_gauss", struct.pack("9f", *w))
    rows, cols = P.shape
    out = torch.zeros_like(xyz)
    Pout = torch.zeros_like(P)
    rc.launch2d("gaussianFilterKernel", rows, cols, ptr(xyz), ptr(P), ptr(out), ptr(Pout), C.c_int(rows),
                C.c_int(cols))
    torch.cuda.synchronize()
    return out, Pout


def ror(rc: RefCuda, xyz, P, radius, min_neighbors, window_size):
    import torch
    rows, cols = P.shape
    out = torch.zeros_like(xyz)
    Pout = torch.zeros_like(P)
    rc.launch2d("radiusOutlierKernel", rows, cols, ptr(xyz), ptr(P), ptr(out), ptr(Pout), C.c_int(rows),
                C.c_int(cols), C.c_float(radius * radius), C.c_int(min_neighbors), C.c_int(window_size // 2))
    torch.cuda.synchronize()
    return out, Pout


def mls(rc: RefCuda, xyz, P, window, sigma, order, max_radius):
    """One mlsKernel pass with the launcher's derived arguments."""
    import numpy as np
    import torch
    rows, cols = P.shape
    s = np.float32(sigma)
    inv_2s2 = np.float32(1.0) / (np.float32(2.0) * s * s)
    r2c = np.float32(max_radius) * np.float32(max_radius) if max_radius > 0 else np.float32(9.0) * s * s
    out = torch.zeros_like(xyz)
    rc.launch2d("mlsKernel", rows, cols, ptr(xyz), ptr(P), ptr(out), C.c_int(rows), C.c_int(cols), C.c_int(window),
                C.c_float(float(inv_2s2)), C.c_int(3), C.c_int(order), C.c_float(float(r2c)))
    torch.cuda.synchronize()
    return out
