"""Builds oracle/_ref/libzim_ref.so from the reference's own C++ sources.

TEST INFRASTRUCTURE ONLY.  The library is the checker the oracle is pinned
against: the reference's decoder V2 (with its factory and V1, which the factory
names), its reconstructor V2 and its CPU MLS, compiled with g++ straight from
the reference tree (nothing is copied into this repository), against the small
OpenCV stand-in in oracle/cvshim/ whose image primitives are the oracle's own
restatements (oracle/zim_oracle.c), plus oracle/ref_bridge.cpp (a C interface
for ctypes).

    python oracle/ref_build.py [--ref PATH]

Compiled, from PhaseShiftGrayCode3D/src/ of the reference:
  * JSLAB_PhaseShiftDecoder.cpp, JSLAB_PhaseShiftDecoder_V1.cpp,
    JSLAB_PhaseShiftDecoder_V2.cpp (whole files);
  * JSLAB_PhaseEpipolarReconstructor_V2.cpp lines 1-593 and 915-1006: the
    filters, calibration, setData, startCalculate, startCalculate_v2,
    getDisparityMap, rectifyLeftImage and stereoMatch.  Lines 595-914 (the ROI
    path) and 1008-1423 (the interactive ROI picker: HighGUI windows, mouse
    callbacks, contour and flood-fill tools) need OpenCV modules the stand-in
    does not provide; they reach g++ as nothing, and `#line` markers keep every
    diagnostic and debug line on the reference file's own numbering.
    oracle/ref_recon_tail.inc is appended to that unit: it exposes the
    file-local evaluateV2CalibPoint (lines 13-76) to the tests;
  * JSLAB_MLS_Filter.cpp (whole file), and a second time through
    oracle/ref_mls_f64.cpp, which includes it with its `float` arithmetic
    widened to double (the oracle's FP64 MLS is pinned to that build; the
    FP32 one bounds the reference's own rounding).
Also built, as a second witness on the GPU (build_cubins): the reference's
three CUDA files JSLAB_PhaseShiftDecoder_V2_GPU.cu, JSLAB_PhaseEpipolarReconstructor_V2_GPU.cu
and JSLAB_MLS_Filter.cu, device code only (nvcc -cubin for sm_103a), into
oracle/_ref/*.cubin, with the entry names ptxas reports written to
oracle/_ref/ref_cubins.json.  A cubin holds GPU code only, so it runs on any
host of the GPU; oracle/ref_cuda.py loads it through the CUDA driver API.
Needs g++ with OpenMP and nvcc; the reference tree exists only where it was
mounted, so this build runs there (never on a machine without it).
"""
from __future__ import annotations

import argparse
import hashlib
import os
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT_DIR = HERE / "_ref"
LIB_PATH = OUT_DIR / "libzim_ref.so"
DEFAULT_REF = Path("/root/reference")
SRC_SUBDIR = Path("PhaseShiftGrayCode3D") / "src"

WHOLE = ["JSLAB_PhaseShiftDecoder.cpp", "JSLAB_PhaseShiftDecoder_V1.cpp", "JSLAB_PhaseShiftDecoder_V2.cpp",
         "JSLAB_MLS_Filter.cpp"]
PARTIAL = {"JSLAB_PhaseEpipolarReconstructor_V2.cpp": [(1, 593), (915, 1006)]}

CXXFLAGS = ["-O2", "-fopenmp", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-w",
            "-D__declspec(x)=", "-Dprivate=public"]
CFLAGS = ["-O2", "-fopenmp", "-std=c11", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]


def ref_src(ref: Path | None = None) -> Path:
    return Path(ref or os.environ.get("ZIM_REFERENCE", DEFAULT_REF)) / SRC_SUBDIR


def sources_present(ref: Path | None = None) -> bool:
    s = ref_src(ref)
    return all((s / f).exists() for f in WHOLE + list(PARTIAL))


def _digest(src: Path) -> str:
    h = hashlib.sha256()
    for f in sorted(WHOLE + list(PARTIAL)):
        h.update((src / f).read_bytes())
    for p in sorted((HERE / "cvshim").rglob("*")) + [HERE / "ref_bridge.cpp", HERE / "ref_mls_f64.cpp",
                                                      HERE / "ref_recon_tail.inc",
                                                      HERE / "zim_oracle.c",
                                                      HERE / "zim_oracle.h", Path(__file__)]:
        if p.is_file():
            h.update(p.read_bytes())
    h.update(" ".join(CXXFLAGS + CFLAGS).encode())
    return h.hexdigest()


def _run(cmd, stdin=None):
    r = subprocess.run(cmd, input=stdin, capture_output=True)
    if r.returncode:
        raise RuntimeError("oracle/_ref build failed: " + " ".join(map(str, cmd[:6])) + " ...\n" +
                           r.stderr.decode(errors="replace")[-4000:])


def build(ref: Path | None = None, force: bool = False) -> Path:
    """Compiles (if the sources changed) and returns the path of libzim_ref.so."""
    src = ref_src(ref)
    if not all((src / f).exists() for f in WHOLE + list(PARTIAL)):
        if LIB_PATH.exists():
            return LIB_PATH
        raise FileNotFoundError(f"reference sources not found under {src}")
    OUT_DIR.mkdir(exist_ok=True)
    stamp = OUT_DIR / "build.sha"
    dig = _digest(src)
    if not force and LIB_PATH.exists() and stamp.exists() and stamp.read_text() == dig:
        return LIB_PATH
    inc = ["-I", str(HERE / "cvshim"), "-I", str(HERE / "cvshim" / "opencv2"), "-I", str(src)]
    with tempfile.TemporaryDirectory() as tmp:
        objs = []
        jobs = []
        for f in WHOLE:
            o = Path(tmp) / (Path(f).stem + ".o")
            jobs.append((["g++", *CXXFLAGS, *inc, "-c", str(src / f), "-o", str(o)], None))
            objs.append(o)
        for f, ranges in PARTIAL.items():
            lines = (src / f).read_bytes().split(b"\n")
            text = bytearray()
            for a, b in ranges:
                text += f'#line {a} "{src / f}"\n'.encode()
                text += b"\n".join(lines[a - 1:b]) + b"\n"
            text += f'#line 1 "{HERE / "ref_recon_tail.inc"}"\n'.encode() + (HERE / "ref_recon_tail.inc").read_bytes()
            o = Path(tmp) / (Path(f).stem + ".o")
            # The selected lines go to g++ on its standard input: no copy is
            # written.  This file's filter loops put statements between the two
            # loops of `omp parallel for collapse(2)`, which MSVC (OpenMP 2.0,
            # the reference's compiler) ignores with a warning and g++ rejects,
            # so its OpenMP pragmas are left off: the loops run serially, with
            # the same per-pixel results.
            flags = [x for x in CXXFLAGS if x != "-fopenmp"]
            jobs.append((["g++", *flags, *inc, "-x", "c++", "-c", "-", "-o", str(o)], bytes(text)))
            objs.append(o)
        for f in ["cvshim/zim_cv.cpp", "ref_bridge.cpp", "ref_mls_f64.cpp"]:
            o = Path(tmp) / (Path(f).stem + ".o")
            jobs.append((["g++", *CXXFLAGS, *inc, "-c", str(HERE / f), "-o", str(o)], None))
            objs.append(o)
        o = Path(tmp) / "zim_oracle.o"
        jobs.append((["gcc", *CFLAGS, "-c", str(HERE / "zim_oracle.c"), "-o", str(o)], None))
        objs.append(o)
        procs = [(subprocess.Popen(cmd, stdin=subprocess.PIPE if data else None, stdout=subprocess.PIPE,
                                   stderr=subprocess.PIPE), cmd, data) for cmd, data in jobs]
        for p, cmd, data in procs:
            _, err = p.communicate(data)
            if p.returncode:
                raise RuntimeError("oracle/_ref build failed: " + " ".join(map(str, cmd[-4:])) + "\n" +
                                   err.decode(errors="replace")[-4000:])
        tmp_lib = LIB_PATH.with_suffix(".so.tmp")
        _run(["g++", "-shared", "-fopenmp", *map(str, objs), "-o", str(tmp_lib), "-lm"])
        os.replace(tmp_lib, LIB_PATH)
    stamp.write_text(dig)
    return LIB_PATH


CUDA_FILES = ["JSLAB_PhaseShiftDecoder_V2_GPU.cu", "JSLAB_PhaseEpipolarReconstructor_V2_GPU.cu",
              "JSLAB_MLS_Filter.cu"]
CUBIN_JSON = OUT_DIR / "ref_cubins.json"
NVCC_FLAGS = ["-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-w",
              "-D__declspec(x)=", "-Xptxas", "-v"]


def build_cubins(ref: Path | None = None, force: bool = False) -> Path:
    """Compiles the reference's CUDA files into cubins (device code only) and
    returns the index file mapping each cubin to its kernels' entry names."""
    import json
    src = ref_src(ref)
    if not all((src / f).exists() for f in CUDA_FILES):
        if CUBIN_JSON.exists():
            return CUBIN_JSON
        raise FileNotFoundError(f"reference CUDA sources not found under {src}")
    OUT_DIR.mkdir(exist_ok=True)
    h = hashlib.sha256()
    for f in CUDA_FILES:
        h.update((src / f).read_bytes())
    for p in sorted((HERE / "cvshim").rglob("*")) + [Path(__file__)]:
        if p.is_file():
            h.update(p.read_bytes())
    stamp = OUT_DIR / "cubins.sha"
    dig = h.hexdigest()
    if not force and CUBIN_JSON.exists() and stamp.exists() and stamp.read_text() == dig:
        return CUBIN_JSON
    nvcc = os.environ.get("NVCC") or "nvcc"
    inc = ["-I", str(HERE / "cvshim"), "-I", str(HERE / "cvshim" / "opencv2"), "-I", str(src)]
    index = {}
    procs = []
    for f in CUDA_FILES:
        out = OUT_DIR / (Path(f).stem + ".cubin")
        cmd = [nvcc, *NVCC_FLAGS, *inc, str(src / f), "-o", str(out)]
        procs.append((f, out, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE)))
    for f, out, p in procs:
        o, e = p.communicate()
        if p.returncode:
            raise RuntimeError(f"cubin build of {f} failed:\n" + e.decode(errors="replace")[-4000:])
        # ptxas -v names every entry it compiles: "Compiling entry function '<mangled>'"
        names = []
        for line in (o + e).decode(errors="replace").splitlines():
            if "Compiling entry function '" in line:
                names.append(line.split("'")[1])
        index[out.name] = sorted(set(names))
    CUBIN_JSON.write_text(json.dumps(index, indent=1))
    stamp.write_text(dig)
    return CUBIN_JSON


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", type=Path, default=None)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build(a.ref, a.force))
    print(build_cubins(a.ref, a.force))


if __name__ == "__main__":
    sys.exit(main())
