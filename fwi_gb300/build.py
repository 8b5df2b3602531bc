"""Builds libfwi_gb300.so (sm_103a) in-tree: fwi_gb300/lib/libfwi_gb300.so.

Translation units compile in parallel with one -gencode (compute_103a ->
sm_103a); objects go to fwi_gb300/_build/.  No cmake, no torch extension
machinery: plain nvcc, so the same recipe runs on x86 and aarch64 hosts.

    python -m fwi_gb300.build [--force] [-j N]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libfwi_gb300.so")

UNITS = ["compat.cu", "native.cu", "prop_f32.cu", "prop_f64.cu", "noalloc.cu"]
# compat.cu reproduces the reference's arithmetic operation for operation: no multiply-add contraction
UNIT_FLAGS = {"compat.cu": ["--fmad=false"]}
C_UNITS = ["driver.c"]  # host C over the C-ABI
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(not os.path.exists(d) or os.path.getmtime(d) > t for d in deps)


def _depfile_deps(dep: str):
    """Prerequisites listed in a make-style dependency file (nvcc / gcc -MD), or None."""
    try:
        text = open(dep).read()
    except OSError:
        return None
    text = text.replace("\\\n", " ")
    _, _, rhs = text.partition(":")
    return [d for d in rhs.split() if d != "\\"]


def _deps(src: str, obj: str, local_headers):
    """Every header the last compile of `src` read (from its -MD file), else all local headers."""
    listed = _depfile_deps(obj[:-2] + ".d")
    return [src] + (listed if listed is not None else local_headers)


def build(force: bool = False, jobs: int = 4, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    inc = os.path.join(os.path.dirname(PKG), "include")
    # without a dependency file (first build), any local header counts
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))] + [
        os.path.join(inc, h) for h in os.listdir(inc) if h.endswith(".h")]
    objs, todo = [], []
    for u in UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, _deps(src, obj, headers)):
            todo.append([nvcc(), *ARCH, *NVCC_FLAGS, *UNIT_FLAGS.get(u, []), "-I", inc, "-MD", "-MF",
                         obj[:-2] + ".d", "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
        return p

    cc = os.environ.get("CC", "gcc")
    for u in C_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u.replace(".c", ".o"))
        objs.append(obj)
        if force or _stale(obj, _deps(src, obj, headers)):
            todo.append([cc, "-O2", "-fPIC", "-std=c11", "-Wall", "-I", inc, "-MD", "-MF", obj[:-2] + ".d",
                         "-c", src, "-o", obj])

    with ThreadPoolExecutor(max_workers=max(1, jobs)) as ex:
        list(ex.map(run, todo))
    if force or todo or _stale(LIB, objs):
        run([nvcc(), *ARCH, "-shared", "--cudart", "static", "-o", LIB, *objs])
    return LIB


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-j", type=int, default=4)
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args(argv)
    print(build(force=a.force, jobs=a.j, verbose=a.v))


if __name__ == "__main__":
    sys.exit(main())
