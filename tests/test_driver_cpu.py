"""The C driver's inversion policy (fwi_gb300/csrc/driver.c) on the CPU.

driver.c is built with tests/driver_mock.c, a stand-in for the library's
entry points over a quadratic misfit (see that file), and driven through
ctypes: the reference's line search (halving on a NaN or larger misfit,
alpha and the halving count kept over the band unless reset_alpha, restore
and stop after max_halvings), the optional FP64 Armijo test, and the band
loop (frequencies, observed data per band, restart from the initial model).
The same driver on the real library is tested on the GPU in
tests/test_driver_gpu.py.
"""
import ctypes as C
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from fwi_gb300.native import BandObsFn, InvertOpts, make_shots

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("needs gcc")
    so = tmp_path_factory.mktemp("driver") / "libdrivermock.so"
    subprocess.run([gcc, "-shared", "-fPIC", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "fwi_gb300", "csrc", "driver.c"), os.path.join(ROOT, "tests", "driver_mock.c"),
                    "-lm", "-o", str(so)], check=True)
    L = C.CDLL(str(so))
    L.mock_create.restype = C.c_void_p
    L.mock_create.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float]
    L.mock_set.argtypes = [C.c_void_p, C.c_float, C.c_float]
    L.mock_trials.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    L.mock_freqs.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    L.mock_counts.argtypes = [C.c_void_p, C.c_void_p]
    L.mock_model.restype = C.c_float
    L.mock_model.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.mock_free.argtypes = [C.c_void_p]
    L.fwi_invert_defaults.argtypes = [C.POINTER(InvertOpts)]
    L.fwi_invert.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(InvertOpts),
                             C.c_void_p, C.POINTER(C.c_int)]
    L.fwi_invert_bands.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_float, C.c_float, C.c_int,
                                   C.c_int, BandObsFn, C.c_void_p, C.POINTER(InvertOpts), C.c_int, C.c_void_p,
                                   C.c_void_p]
    return L


SHOTS = make_shots([dict(sx=10, sz=5, rz=5, rx0=4, rx1=20, nt=10)])
OBS = np.zeros(16 * 10, np.float32)


def opts(lib, **kw):
    o = InvertOpts()
    lib.fwi_invert_defaults(C.byref(o))
    o.first_alpha[0] = o.first_alpha[1] = o.first_alpha[2] = 0.5
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def invert(lib, rscale=1.0, nan_above=math.inf, **kw):
    ctx = lib.mock_create(4, 2, 0.0, 1.0)
    lib.mock_set(ctx, rscale, nan_above)
    o = opts(lib, **kw)
    hist = np.zeros(o.iterations, np.float64)
    done = C.c_int(0)
    rc = lib.fwi_invert(ctx, SHOTS, 1, OBS.ctypes.data, None, C.byref(o), hist.ctypes.data, C.byref(done))
    tr = np.zeros(256, np.float32)
    n = lib.mock_trials(ctx, tr.ctypes.data, 256)
    counts = np.zeros(5, np.int32)
    lib.mock_counts(ctx, counts.ctypes.data)
    model = lib.mock_model(ctx, 0, 0)
    lib.mock_free(ctx)
    return rc, done.value, hist, tr[:n].tolist(), counts.tolist(), model


def test_converges_on_a_quadratic(lib):
    rc, done, hist, trials, counts, model = invert(lib, iterations=4)
    assert rc == 0 and done == 4
    assert hist.tolist() == [12.0, 3.0, 0.0, 0.0]  # 1/2 |m - t|^2 over 3 x 8 points
    assert trials == [1.0, 1.0, 1.0] and counts[3] == 1 and model == 1.0


def test_halving_keeps_alpha_over_the_band_as_the_reference(lib):
    _, _, _, trials, counts, _ = invert(lib, nan_above=0.3, iterations=4)
    assert trials == [1.0, 0.5, 0.25, 0.25, 0.25] and counts[2] == 0
    _, _, _, trials, _, _ = invert(lib, nan_above=0.3, iterations=4, reset_alpha=1)
    assert trials == [1.0, 0.5, 0.25] * 3


def test_too_many_halvings_restore_the_model_and_end_the_band(lib):
    rc, done, _, trials, counts, model = invert(lib, nan_above=0.0, iterations=4)
    assert rc == 0 and done == 2
    assert trials == [1.0 / 2 ** k for k in range(6)]  # max_halvings = 5
    assert counts[2] == 1 and model == 0.5  # m_back after the first step


def test_armijo_asks_for_a_sufficient_decrease(lib):
    # direction 4 g: alpha 1 overshoots, alpha 1/2 only matches the misfit, 1/4 reaches the minimum
    _, _, _, trials, _, _ = invert(lib, rscale=4.0, iterations=2)
    assert trials == [1.0, 0.5]
    _, _, _, trials, _, model = invert(lib, rscale=4.0, iterations=2, armijo_c1=1e-4)
    assert trials == [1.0, 0.5, 0.25] and model == 1.0


@pytest.mark.parametrize("restart", [1, 0])
def test_band_loop(lib, restart):
    ctx = lib.mock_create(4, 2, 0.0, 1.0)
    seen = []
    buf = np.zeros(16 * 10, np.float32)

    @BandObsFn
    def band_obs(user, band, f, obs):
        seen.append((band, round(f, 3)))
        obs[0] = buf.ctypes.data
        return 0

    o = opts(lib, iterations=2)
    hist = np.zeros(3 * o.iterations, np.float64)
    done = np.zeros(3, np.int32)
    rc = lib.fwi_invert_bands(ctx, SHOTS, 1, None, 3.0, 3.0, 3, 10, band_obs, None, C.byref(o), restart,
                              hist.ctypes.data, done.ctypes.data)
    fr = np.zeros(8, np.float32)
    nf = lib.mock_freqs(ctx, fr.ctypes.data, 8)
    counts = np.zeros(5, np.int32)
    lib.mock_counts(ctx, counts.ctypes.data)
    lib.mock_free(ctx)
    assert rc == 0 and done.tolist() == [2, 2, 2]
    assert fr[:nf].tolist() == [3.0, 6.0, 9.0] and seen == [(0, 3.0), (1, 6.0), (2, 9.0)]
    assert counts[0] == 6 and counts[4] == (2 if restart else 0)
    if restart:  # every band starts from the initial model: the same misfit history
        assert hist[0] == hist[2] == hist[4] == 12.0
