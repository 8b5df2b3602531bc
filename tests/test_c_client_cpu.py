"""Both C-ABIs from a C99 client (tests/c_client.c): the headers compile as
C99 with warnings as errors, every compatibility entry point resolves at link
time, and the host-side entry points run without a GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


def test_c99_client_builds_links_and_runs(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("needs gcc and the CUDA headers")
    from fwi_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    exe = tmp_path / "c_client"
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    "-I", CUDA_INC, os.path.join(ROOT, "tests", "c_client.c"), "-L", libdir, "-lfwi_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "compat 17" in out.stdout and "invalid argument" in out.stdout
