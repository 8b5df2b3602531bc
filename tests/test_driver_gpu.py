"""The C host driver (fwi_invert): one band of src/main.c:396-801's loop over
the native ABI.  Checked against the same policy written out in Python over
the same entry points (identical misfit history, bit for bit), and the
misfit must not increase from one iteration to the next."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_small.npz"))
NX, NZ, NT, CPML, SZ = (int(G[k]) for k in ("nx", "nz", "nt", "cpml", "sz"))


def make_ctx():
    import fwi_gb300
    ctx = fwi_gb300.Context(nx=NX, nz=NZ, dh=float(G["dh"]), dt=float(G["dt"]), cpml=CPML,
                            f_cpml=float(G["f"]), nt_max=NT, max_shots=2, mode=fwi_gb300.MODE_EXACT)
    ctx.set_wavelet(G["source"])
    ctx.set_model(G["vh_i"], G["vp_i"], G["vn_i"])
    shots = fwi_gb300.make_shots([(int(sx) - 1, SZ - 1, SZ - 1, CPML, NX - CPML, NT) for sx in G["shots_sx"]])
    obs = np.concatenate([G["obs"][k][:, CPML:NX - CPML].ravel() for k in range(2)]).astype(np.float32)
    return ctx, shots, obs


def python_policy(ctx, shots, obs, iterations, m=5, first=(3e5, 2e5, 2.5e5), alpha0=1.0, max_halvings=5):
    """src/main.c:396-801 (one band) over the Python bindings."""
    hist = []
    alpha, count = alpha0, 0
    for n in range(iterations):
        phi = ctx.gradient(shots, obs)[0]
        hist.append(phi)
        if n == 0:
            ctx.first_step(*first)
            continue
        ctx.lbfgs_direction(m)
        trial, stop = 1e10, False
        while trial > phi:
            ctx.lbfgs_update(alpha, alpha, alpha)
            trial = ctx.misfit(shots, obs)
            if np.isnan(trial):
                trial, count, alpha = 1e30, count + 1, np.float32(alpha * 0.5)
            elif trial > phi:
                count, alpha = count + 1, np.float32(alpha * 0.5)
            if count > max_halvings:
                ctx.restore_model()
                stop = True
                break
        if stop:
            break
    return np.array(hist)


def test_c_driver_equals_policy_and_decreases():
    ctx, shots, obs = make_ctx()
    hist_c = ctx.invert(shots, obs, iterations=5)
    ctx2, shots2, obs2 = make_ctx()
    hist_py = python_policy(ctx2, shots2, obs2, 5)
    assert len(hist_c) == len(hist_py) >= 3
    assert np.array_equal(hist_c, hist_py)
    assert np.all(np.diff(hist_c) <= 0), hist_c
    assert hist_c[-1] < hist_c[0]


def test_frequency_switch_changes_wavelet_and_layers():
    ctx, shots, obs = make_ctx()
    a = ctx.forward(shots)
    ctx.set_frequency(float(G["f"]) * 2, NT)
    b = ctx.forward(shots)
    ctx.set_frequency(float(G["f"]), NT)
    c = ctx.forward(shots)
    assert not np.allclose(a, b)
    # back at the first band: the same Ricker (main.c's formula) and CPML profiles
    ctx.set_wavelet(G["source"])
    d = ctx.forward(shots)
    assert float(np.abs(c - d).max()) <= 1e-6 * float(np.abs(d).max())
    assert np.array_equal(a, d)
