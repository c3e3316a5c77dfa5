"""The header-only C++ adapter (include/zim_jslab.hpp): compiles with g++
against the C ABI (CPU), and reconstructs an analytic plane (GPU)."""
import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "jslab_adapter_test.cpp"
OUT = ROOT / "zim_gb300" / "_build" / "jslab_adapter_test"
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def build():
    OUT.parent.mkdir(exist_ok=True)
    pkg = ROOT / "zim_gb300"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", str(ROOT / "include"), "-I", str(CUDA / "include"), str(SRC),
           "-o", str(OUT), "-L", str(pkg), "-lzim_gb300", "-L", str(CUDA / "lib64"), "-lcudart",
           f"-Wl,-rpath,{pkg}", f"-Wl,-rpath,{CUDA / 'lib64'}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return OUT


def test_adapter_compiles_and_links(native):
    assert build().exists()


@pytest.mark.gpu
def test_adapter_reconstructs_plane(native, tmp_path):
    exe = build()
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=300)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
