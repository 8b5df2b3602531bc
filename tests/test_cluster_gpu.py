"""Small shots resident on chip (one thread-block cluster per shot, every step
in one launch; prop_cluster.cuh), which FP32 exact-adjoint contexts with full
image storage use where the window fits a cluster's shared memory.  Checked
against the FP64 oracle, against the tile passes (environment FWI_CLUSTER=0),
with two shots of different windows and lengths in one batch, every image
type, and the misfit-only call.  Tolerances (relative L2): gradients 1e-4 of
the FP64 oracle, 1e-5 of the tile passes (the same arithmetic in another
order: FP32 rounding over 260 steps); misfit 1e-5 and 1e-6."""
import numpy as np
import pytest

from test_native_gpu import oracle_exact, wavelet, exact_problem

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm((np.asarray(a, np.float64) - b).ravel()) / np.linalg.norm(np.asarray(b).ravel()))


@pytest.fixture(scope="module")
def case():
    p = exact_problem(seed=21, nx=160, nz=120, nt=260)
    nx, nz = p["nx"], p["nz"]
    shots = [dict(sx=40, sz=6, rz=6, rx0=4, rx1=nx - 4, nt=p["nt"], x0=0, nxw=0),
             dict(sx=70, sz=nz - 10, rz=5, rx0=30, rx1=nx - 10, nt=p["nt"] - 60, x0=20, nxw=nx - 24)]
    from fwi_gb300 import Context, MODE_EXACT, PREC_FP64, make_shots
    ctx = Context(nx=nx, nz=nz, dh=p["dh"], dt=p["dt"], cpml=p["cpml"], f_cpml=p["f"], nt_max=p["nt"], max_shots=2,
                  mode=MODE_EXACT, precision=PREC_FP64)
    ctx.set_wavelet(wavelet(p))
    ctx.set_model(p["vh"] * 1.03, p["vp"] * 0.98, p["vn"] * 1.02)
    obs = ctx.forward(make_shots(shots))
    mask = np.ones(sum(s["rx1"] - s["rx0"] for s in shots), np.uint8)
    mask[::9] = 0
    J, g = oracle_exact(p, shots, obs, mask)
    return p, shots, obs, mask, J, g


def run(p, shots, obs, mask, sprec=0, cluster=True, monkeypatch=None):
    from fwi_gb300 import Context, MODE_EXACT, make_shots
    if not cluster:
        monkeypatch.setenv("FWI_CLUSTER", "0")
    ctx = Context(nx=p["nx"], nz=p["nz"], dh=p["dh"], dt=p["dt"], cpml=p["cpml"], f_cpml=p["f"], nt_max=p["nt"],
                  max_shots=2, mode=MODE_EXACT, store_prec=sprec)
    ctx.set_wavelet(wavelet(p).astype(np.float32))
    ctx.set_model(*(np.ascontiguousarray(p[k], np.float32) for k in ("vh", "vp", "vn")))
    sh = make_shots(shots)
    r = ctx.gradient(sh, obs.astype(np.float32), mask)
    launches = ctx.last_launches()
    J = ctx.misfit(sh, obs.astype(np.float32), mask)
    if not cluster:
        monkeypatch.delenv("FWI_CLUSTER")
    return r, launches, J


def test_cluster_path_matches_fp64_oracle_and_tile_passes(case, monkeypatch):
    p, shots, obs, mask, J, g = case
    (Jc, *gc), lc, Jm = run(p, shots, obs, mask)
    (Jt, *gt), lt, _ = run(p, shots, obs, mask, cluster=False, monkeypatch=monkeypatch)
    e_or = [rel(a, b) for a, b in zip(gc, g)]
    e_tile = [rel(a, b) for a, b in zip(gc, gt)]
    print(f"[parity] cluster path: vs FP64 oracle {e_or[0]:.3e} {e_or[1]:.3e} {e_or[2]:.3e}, vs tile passes "
          f"{e_tile[0]:.3e} {e_tile[1]:.3e} {e_tile[2]:.3e}, misfit {abs(Jc - J) / J:.3e}; launches {lc} vs {lt}")
    assert lc < 10 < lt  # one launch per pass and batch, not per step
    assert abs(Jc - J) <= 1e-5 * J and abs(Jc - Jt) <= 1e-6 * Jt
    assert Jm == Jc  # the misfit-only call runs the same forward
    assert max(e_or) <= 1e-4 and max(e_tile) <= 1e-5


@pytest.mark.parametrize("sprec,tol", [(1, 2e-3), (2, 2e-2)])
def test_cluster_path_reduced_precision_images(case, sprec, tol, monkeypatch):
    p, shots, obs, mask, _, _ = case
    (Jc, *gc), _, _ = run(p, shots, obs, mask, sprec=sprec)
    (Jt, *gt), _, _ = run(p, shots, obs, mask, sprec=sprec, cluster=False, monkeypatch=monkeypatch)
    (J32, *g32), _, _ = run(p, shots, obs, mask)
    assert Jc == J32  # the images do not enter the misfit
    for a, b, c in zip(gc, gt, g32):
        assert rel(a, c) <= tol and rel(a, b) <= tol


@pytest.fixture(scope="module")
def c1_case():
    """A C1-sized grid (209 x 209, 20-point layer): 16 CTAs of unequal rows (fewer at the
    bottom layer), one image buffer for FP32 images and two for FP16 in the adjoint."""
    p = exact_problem(seed=5, nx=209, nz=209, nt=240)
    p["cpml"] = 20
    nx, nz = p["nx"], p["nz"]
    shots = [dict(sx=104, sz=6, rz=6, rx0=4, rx1=nx - 4, nt=p["nt"], x0=0, nxw=0)]
    from fwi_gb300 import Context, MODE_EXACT, PREC_FP64, make_shots
    ctx = Context(nx=nx, nz=nz, dh=p["dh"], dt=p["dt"], cpml=p["cpml"], f_cpml=p["f"], nt_max=p["nt"], max_shots=1,
                  mode=MODE_EXACT, precision=PREC_FP64)
    ctx.set_wavelet(wavelet(p))
    ctx.set_model(p["vh"] * 1.03, p["vp"] * 0.98, p["vn"] * 1.02)
    obs = ctx.forward(make_shots(shots))
    mask = np.ones(nx - 8, np.uint8)
    J, g = oracle_exact(p, shots, obs, mask)
    return p, shots, obs, mask, J, g


@pytest.mark.parametrize("sprec,tol_tile", [(0, 1e-5), (1, 2e-3)])
def test_cluster_path_c1_grid_unequal_rows(c1_case, sprec, tol_tile, monkeypatch):
    p, shots, obs, mask, J, g = c1_case
    (Jc, *gc), lc, _ = run(p, shots, obs, mask, sprec=sprec)
    (Jt, *gt), lt, _ = run(p, shots, obs, mask, sprec=sprec, cluster=False, monkeypatch=monkeypatch)
    e_or = [rel(a, b) for a, b in zip(gc, g)]
    e_tile = [rel(a, b) for a, b in zip(gc, gt)]
    print(f"[parity] cluster path, 209 x 209, images {sprec}: vs FP64 oracle {max(e_or):.3e}, vs tile passes "
          f"{max(e_tile):.3e}; launches {lc} vs {lt}")
    assert lc < 10 < lt
    assert abs(Jc - J) <= 1e-5 * J and abs(Jc - Jt) <= 1e-6 * Jt
    assert max(e_tile) <= tol_tile and max(e_or) <= (1e-4 if sprec == 0 else tol_tile)


@pytest.mark.parametrize("shape", [
    dict(nx=40, nz=44, cpml=4, nt=90),     # no CPML point inside the interior (layer width = frame)
    dict(nx=96, nz=200, cpml=30, nt=80),   # 16 CTAs over 192 rows, wide layers (side band 52 of 88 columns)
    dict(nx=72, nz=36, cpml=10, nt=3),     # 3 CTAs, three steps
])
def test_cluster_path_edge_shapes(shape, monkeypatch):
    """Shapes at the edges of the cluster path's plan (no layer work, wide layers, a handful of
    CTAs, a few steps), against the FP64 oracle and the tile passes, with random observed data;
    source and receivers in the bottom layer, so that the two wavefields meet within the steps."""
    p = exact_problem(seed=3, nx=shape["nx"], nz=shape["nz"], nt=shape["nt"])
    p["cpml"] = shape["cpml"]
    nx, nz, nt = p["nx"], p["nz"], p["nt"]
    shots = [dict(sx=nx // 2, sz=nz - 6, rz=nz - 8, rx0=4, rx1=nx - 4, nt=nt, x0=0, nxw=0)]
    rng = np.random.default_rng(2)
    obs = 1e-3 * rng.standard_normal(nt * (nx - 8))
    mask = np.ones(nx - 8, np.uint8)
    J, g = oracle_exact(p, shots, obs, mask)
    (Jc, *gc), lc, _ = run(p, shots, obs, mask)
    (Jt, *gt), lt, _ = run(p, shots, obs, mask, cluster=False, monkeypatch=monkeypatch)
    assert lc < 10 < lt
    assert abs(Jc - J) <= 1e-5 * J and abs(Jc - Jt) <= 1e-6 * Jt
    for a, b, c in zip(gc, g, gt):
        assert np.linalg.norm(b) > 0
        assert rel(a, b) <= 1e-4 and rel(a, c) <= 1e-5


def test_cluster_path_single_step(monkeypatch):
    """One step: the misfit of the first samples, a gradient of zeros (no image before the first
    update), as the tile passes give."""
    p = exact_problem(seed=3, nx=72, nz=36, nt=1)
    nx, nz = p["nx"], p["nz"]
    shots = [dict(sx=nx // 2, sz=nz - 6, rz=nz - 8, rx0=4, rx1=nx - 4, nt=1, x0=0, nxw=0)]
    obs = 1e-3 * np.random.default_rng(4).standard_normal(nx - 8)
    mask = np.ones(nx - 8, np.uint8)
    (Jc, *gc), lc, _ = run(p, shots, obs, mask)
    (Jt, *gt), _, _ = run(p, shots, obs, mask, cluster=False, monkeypatch=monkeypatch)
    assert lc < 10 and abs(Jc - Jt) <= 1e-6 * Jt
    for a, c in zip(gc, gt):
        assert np.all(np.isfinite(a)) and np.allclose(a, c, rtol=1e-5, atol=1e-30)
