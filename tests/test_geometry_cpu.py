"""Tile geometry of the FP32 tile passes, checked on the CPU.

Builds tests/geometry_check.cpp against the library's own headers
(fwi_gb300/csrc/prop.h, common.cuh) with g++ and runs it: the tile-grid
origin rule, the tile role of every tile against its points, and what the
interior passes assume of an interior tile (for groups of several windows
too) over about 1800 grid shapes.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


def test_tile_geometry(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("needs g++ and the CUDA headers")
    exe = tmp_path / "geometry_check"
    subprocess.run([gxx, "-std=c++17", "-O2", f"-I{CUDA_INC}", f"-I{os.path.join(ROOT, 'fwi_gb300', 'csrc')}",
                    os.path.join(ROOT, "tests", "geometry_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.startswith("OK"), out.stdout
