"""The drop-in claim at link level: the reference's own src/main.c, compiled
unchanged as C99 against its own headers (with a one-rank MPI stand-in,
tests/mpi_stub/mpi.h, for the MPI it uses), links against libfwi_gb300.so
and the CUDA runtime with no symbol left unresolved; the library replaces
the reference's two CUDA objects.  Needs the reference checkout, named by
the environment variable FWI_REFERENCE_ROOT; skipped where it is not given."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("FWI_REFERENCE_ROOT", "")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def test_reference_main_links_against_the_library(tmp_path):
    main_c = os.path.join(REF, "src", "main.c") if REF else ""
    cudart = os.path.join(CUDA, "lib64")
    gcc = shutil.which("gcc")
    if not main_c or not os.path.exists(main_c) or gcc is None or not os.path.exists(os.path.join(CUDA, "include", "cuda_runtime.h")):
        pytest.skip("needs the reference checkout, gcc and the CUDA toolkit")
    from fwi_gb300 import build
    libdir = os.path.dirname(build.build())
    obj, exe = tmp_path / "main.o", tmp_path / "fwi_main"
    subprocess.run([gcc, "-std=c99", "-w", "-I", os.path.join(ROOT, "tests", "mpi_stub"), "-I",
                    os.path.join(REF, "include"), "-I", os.path.join(CUDA, "include"), "-c", main_c, "-o", str(obj)],
                   check=True)
    link = subprocess.run([gcc, str(obj), "-L", libdir, "-lfwi_gb300", "-L", cudart, "-lcudart", "-lm",
                           f"-Wl,-rpath,{libdir}", "-o", str(exe)], capture_output=True, text=True)
    assert link.returncode == 0, link.stderr
    assert "undefined reference" not in link.stderr
