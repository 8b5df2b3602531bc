"""The small-shot cluster path's plan, checked on the CPU.

Builds tests/cluster_plan_check.cpp against fwi_gb300/csrc/cluster_plan.h with g++ and runs it:
over a sweep of window widths, grid heights, layer widths and image types, the row partition
covers the interior with CTAs of at least 8 rows, fits the shared memory, keeps the kernels'
alignments and has the least largest-CTA cost (brute force on small grids); refused plans are
ones that cannot fit.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


def test_cluster_plan(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("needs g++ and the CUDA headers")
    exe = tmp_path / "cluster_plan_check"
    subprocess.run([gxx, "-std=c++17", "-O2", "-include", "cuda_runtime.h", f"-I{CUDA_INC}",
                    f"-I{os.path.join(ROOT, 'fwi_gb300', 'csrc')}",
                    os.path.join(ROOT, "tests", "cluster_plan_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.startswith("OK"), out.stdout
