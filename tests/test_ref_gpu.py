"""The reference's own CUDA kernels, compiled unchanged for sm_103a into
oracle/_ref (where the reference checkout was available at build time), run on
the GPU: shot 0 of the fixtures sequenced as src/main.c:318-495 does it,
against the fixtures made from the same kernels run as C on the CPU.  nvcc
contracts multiply-adds by default (as the reference's Makefile builds the
kernels) and the CPU build does not, so the two agree to FP32 rounding carried
over 300 steps, not bit for bit (the library's reference-compatible ABI is bit
for bit, tests/test_compat_gpu.py).  Skipped where the cubin was not built."""
import os

import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_small.npz"))


def rel(a, b):
    return float(np.linalg.norm((np.asarray(a, np.float64) - b).ravel()) / np.linalg.norm(np.asarray(b).ravel()))


def test_reference_gpu_kernels_reproduce_the_fixtures():
    if not po.ref_gpu_available():
        pytest.skip("the reference's kernels were not compiled for the GPU (no reference checkout at build time)")
    nx, nz, nt, cpml, sz = (int(G[k]) for k in ("nx", "nz", "nt", "cpml", "sz"))
    secs, fi, g, res = po.ref_gpu_shot(G["vel_i"], G["eps_i"], G["del_i"], G["obs"][0], nx, nz, nt, cpml,
                                       float(G["dh"]), float(G["dt"]), float(G["f"]), int(G["shots_sx"][0]), sz,
                                       runs=2)
    e_res = rel(res, G["res"][0])
    e_g = [rel(a, G[k]) for a, k in zip(g, ("gcx_shot0", "gcz_shot0", "gdx_shot0"))]
    print(f"[parity] reference kernels on the GPU vs the same kernels on the CPU: residual {e_res:.3e}, "
          f"gradients {e_g[0]:.3e} {e_g[1]:.3e} {e_g[2]:.3e}, misfit {fi:.9g} vs {float(G['fi'][0]):.9g}, "
          f"{secs[-1] * 1e3:.2f} ms per shot")
    assert len(secs) == 2 and all(s > 0 for s in secs)
    assert e_res <= 1e-5
    assert max(e_g) <= 1e-4
    assert abs(fi - float(G["fi"][0])) <= 1e-5 * float(G["fi"][0])
