"""The native-semantics oracle: forward equals the reference restatement, and
its EXACT adjoint passes the dot-product and finite-difference tests in FP64."""
import numpy as np
import pytest

from oracle import pyoracle as po


def small_problem(dtype=np.float64, nx=48, nz=40, nt=200, cpml=10, seed=3, f=20.0):
    rng = np.random.default_rng(seed)
    vel = 2000 + 600 * rng.random((nz, nx))
    eps = 0.2 * rng.random((nz, nx))
    dl = np.minimum(0.1 * rng.random((nz, nx)), eps)
    vp = vel ** 2
    dh, dt = 10.0, 1e-3
    ax, bx, az, bz = po.cpml_profiles(nx, nz, cpml, dh, dt, f, dtype=dtype)
    return dict(nx=nx, nz=nz, nt=nt, cpml=cpml, dh=dh, dt=dt, ax=ax, bx=bx, az=az, bz=bz,
                source=po.ricker(nt, dt, f, dtype=dtype), vh=(vp * (1 + 2 * eps)).astype(dtype),
                vp=vp.astype(dtype), vn=(vp * (1 + 2 * dl)).astype(dtype))


@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-13), (np.float32, 2e-5)])
def test_forward_equals_reference_restatement(dtype, tol):
    p = small_problem(dtype)
    nx, cpml = p["nx"], p["cpml"]
    shot, _ = po.forward_shot(p, 21, 7)  # reference geometry is 1-based
    rec = po.exact_forward(p, 20, 6, 6, cpml, nx - cpml)
    err = np.abs(rec - shot[:, cpml:nx - cpml]).max() / np.abs(shot).max()
    assert err < tol


def test_dot_product_fp64():
    p = small_problem()
    nx = p["nx"]
    rng = np.random.default_rng(11)
    w = rng.standard_normal(p["nt"])
    r = rng.standard_normal((p["nt"], nx - 8))
    d = po.exact_forward(p, 17, 6, 9, 4, nx - 4, wavelet=w)
    _, _, _, _, tr = po.exact_gradient(p, 17, 6, 9, 4, nx - 4, wavelet=w, adjoint_source=r,
                                       want_adj_trace=True)
    lhs, rhs = float((d * r).sum()), float((w * tr).sum())
    assert abs(lhs - rhs) / max(abs(lhs), abs(rhs)) < 1e-11


def test_dot_product_source_in_cpml_fp64():
    """Source and receivers inside the absorbing layers exercise every CPML term."""
    p = small_problem(seed=5)
    nx, nz = p["nx"], p["nz"]
    rng = np.random.default_rng(12)
    w = rng.standard_normal(p["nt"])
    r = rng.standard_normal((p["nt"], nx - 8))
    d = po.exact_forward(p, 6, nz - 7, nz - 6, 4, nx - 4, wavelet=w)
    _, _, _, _, tr = po.exact_gradient(p, 6, nz - 7, nz - 6, 4, nx - 4, wavelet=w,
                                       adjoint_source=r, want_adj_trace=True)
    lhs, rhs = float((d * r).sum()), float((w * tr).sum())
    assert abs(lhs - rhs) / max(abs(lhs), abs(rhs)) < 1e-11


def test_finite_difference_gradient_fp64():
    p = small_problem(nt=160, seed=4)
    nx, nz = p["nx"], p["nz"]
    geo = (22, 6, 6, 4, nx - 4)
    true = dict(p, vh=p["vh"] * 1.02, vp=p["vp"] * 0.99, vn=p["vn"] * 1.01)
    obs = po.exact_forward(true, *geo)
    mask = np.ones(nx - 8, np.uint8)
    mask[::7] = 0
    J0, gh, gp, gn = po.exact_gradient(p, *geo, obs=obs, mask=mask)
    rng = np.random.default_rng(21)
    scale = float(p["vp"].mean()) * 1e-3
    for _ in range(3):
        dm = [rng.standard_normal((nz, nx)) * scale for _ in range(3)]
        pred = sum(float((g * d).sum()) for g, d in zip((gh, gp, gn), dm))
        e = 1e-2

        def J(s):
            q = dict(p, vh=p["vh"] + s * dm[0], vp=p["vp"] + s * dm[1], vn=p["vn"] + s * dm[2])
            return po.exact_gradient(q, *geo, obs=obs, mask=mask)[0]
        fd = (J(e) - J(-e)) / (2 * e)
        assert abs(fd / pred - 1) < 1e-4


def test_misfit_is_half_sum_of_masked_squares():
    p = small_problem(nt=80)
    nx = p["nx"]
    geo = (20, 6, 6, 4, nx - 4)
    rec = po.exact_forward(p, *geo)
    obs = rec * 0.5
    mask = np.ones(nx - 8, np.uint8)
    mask[3] = 0
    J = po.exact_gradient(p, *geo, obs=obs, mask=mask)[0]
    res = (rec - obs) * mask[None, :]
    assert abs(J - 0.5 * float((res ** 2).sum())) <= 1e-12 * J
