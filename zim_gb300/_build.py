"""Builds the native parts of zim_gb300 in-tree.

* ``libzim_gb300.so`` -- the CUDA library behind ``include/zim.h``, compiled
  for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``).
* ``libzim_synth.so`` -- the synthetic scene renderer (C, OpenMP).

Translation units compile in parallel; a unit is rebuilt when its source, a
header it may include or the flags change.  No cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libzim_gb300.so"
SYNTH_LIB = PKG / "libzim_synth.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-fvisibility=hidden", "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
# per-file extra flags: the FP64 map arithmetic must not be contracted into FMAs
FILE_FLAGS = {"calib.cu": ["--fmad=false"]}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _digest(paths, flags) -> str:
    h = hashlib.sha256()
    for p in paths:
        h.update(Path(p).read_bytes())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build_cuda(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "zim.h"]
    sources = sorted(CSRC.glob("*.cu"))
    nv = nvcc()
    objs, jobs = [], []
    for src in sources:
        flags = NVCC_FLAGS + ARCH + FILE_FLAGS.get(src.name, [])
        obj = BUILD / (src.stem + ".o")
        stamp = BUILD / (src.stem + ".sha")
        dig = _digest([src] + headers, flags)
        objs.append(obj)
        if obj.exists() and stamp.exists() and stamp.read_text() == dig:
            continue
        jobs.append(([nv, *flags, "-c", str(src), "-o", str(obj)], stamp, dig))
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_run, cmd) for cmd, _, _ in jobs]
        for f, (cmd, stamp, dig) in zip(futs, jobs):
            out = f.result()
            if verbose and out.strip():
                print(out)
            stamp.write_text(dig)
    link_dig = _digest(objs, ARCH)
    link_stamp = BUILD / "link.sha"
    if not (LIB.exists() and link_stamp.exists() and link_stamp.read_text() == link_dig):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nv, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"])
        os.replace(tmp, LIB)
        link_stamp.write_text(link_dig)
    return LIB


def build_synth() -> Path:
    src = PKG / "synth" / "zim_synth.c"
    flags = ["-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11"]
    stamp = BUILD / "synth.sha"
    BUILD.mkdir(exist_ok=True)
    dig = _digest([src, PKG / "synth" / "zim_synth.h"], flags)
    if SYNTH_LIB.exists() and stamp.exists() and stamp.read_text() == dig:
        return SYNTH_LIB
    tmp = SYNTH_LIB.with_suffix(".so.tmp")
    _run(["gcc", *flags, str(src), "-o", str(tmp), "-lm"])
    os.replace(tmp, SYNTH_LIB)
    stamp.write_text(dig)
    return SYNTH_LIB


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_cuda, verbose)
        b = ex.submit(build_synth)
        a.result()
        b.result()


if __name__ == "__main__":
    build_all(verbose=True)
