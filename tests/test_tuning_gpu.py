"""Autotuner (fwi_autotune / fwi_set_tuning) on the GPU.

A tuned launch choice is applied to later calls, is reproducible bit for bit
when given again with fwi_set_tuning, and stays within FP32 rounding of the
built-in choice (relative L2 1e-5 on the gradients, 1e-6 on the misfit);
batches of several windows keep one shot per block.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = float(np.float32(1e-3))


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def problem(seed=21, nx=136, nz=88, nt=220):
    rng = np.random.default_rng(seed)
    vel = 1900 + 700 * rng.random((nz, nx))
    for _ in range(4):
        vel = (vel + np.roll(vel, 1, 0) + np.roll(vel, 1, 1)) / 3
    vp = vel ** 2
    return dict(nx=nx, nz=nz, nt=nt, cpml=12, dh=10.0, f=18.0,
                vh=(vp * 1.3).astype(np.float32), vp=vp.astype(np.float32), vn=(vp * 1.15).astype(np.float32))


def context(p, batch, **kw):
    from fwi_gb300 import Context, MODE_EXACT, PREC_FP32
    ctx = Context(nx=p["nx"], nz=p["nz"], dh=p["dh"], dt=DT, cpml=p["cpml"], f_cpml=p["f"], nt_max=p["nt"],
                  max_shots=batch, mode=MODE_EXACT, precision=PREC_FP32, store_prec=1, **kw)
    ctx.set_ricker(p["f"], p["nt"])
    return ctx


def observed(p, shots, batch):
    ctx = context(p, batch)
    ctx.set_model(p["vh"] * 1.02, p["vp"] * 0.98, p["vn"] * 1.01)
    return ctx.forward(shots)


@pytest.fixture(scope="module")
def one_window():
    """Six shots on the whole model: one window, so every choice is open."""
    from fwi_gb300 import make_shots
    p = problem()
    shots = make_shots([dict(sx=14 + 20 * k, sz=6, rz=5, rx0=4, rx1=p["nx"] - 4, nt=p["nt"] - 10 * (k % 2), x0=0,
                             nxw=0) for k in range(6)])
    return p, shots, observed(p, shots, 6)


def test_autotune_choice_is_applied_and_reproducible(one_window):
    p, shots, obs = one_window
    res, tunings = [], []
    for how in ("tuned", "given", "built-in"):
        ctx = context(p, 6)
        ctx.set_model(p["vh"], p["vp"], p["vn"])
        if how == "tuned":
            t = ctx.autotune(shots, steps=24)
            tunings.append(t)
        elif how == "given":
            ctx.set_tuning(shots, tunings[0])
        res.append(ctx.gradient(shots, obs))
        del ctx
    t = tunings[0]
    for ph in ("forward", "adjoint"):
        c = t[ph]
        assert 1 <= c["shots_per_group"] <= 6 and 1 <= c["layer_shots_per_group"] <= 6
        assert c["inline_strip"] in (0, 1)
        assert 0 < t[f"{ph}_us"] <= t[f"default_{ph}_us"]
    assert t["trials"] > 2
    tuned, given, builtin = res
    assert tuned[0] == given[0]
    for a, b in zip(tuned[1:], given[1:]):
        assert np.array_equal(a, b)
    assert abs(tuned[0] - builtin[0]) <= 1e-6 * abs(builtin[0])
    for a, b in zip(tuned[1:], builtin[1:]):
        assert rel_l2(a, b) <= 1e-5, rel_l2(a, b)


def phase(sg, sl, inl):
    return dict(shots_per_group=sg, layer_shots_per_group=sl, inline_strip=inl)


@pytest.mark.parametrize("fwd,adj", [((1, 1, 0), (1, 1, 0)), ((2, 6, 1), (3, 2, 1)), ((6, 1, 0), (6, 1, 0)),
                                     ((3, 2, 1), (2, 6, 0))])
def test_every_choice_gives_the_same_gradient(one_window, fwd, adj):
    p, shots, obs = one_window
    out = []
    for choice in (None, dict(forward=phase(*fwd), adjoint=phase(*adj))):
        ctx = context(p, 6)
        ctx.set_model(p["vh"], p["vp"], p["vn"])
        if choice:
            ctx.set_tuning(shots, choice)
        out.append(ctx.gradient(shots, obs))
        del ctx
    assert abs(out[0][0] - out[1][0]) <= 1e-6 * abs(out[0][0])
    for a, b in zip(out[1][1:], out[0][1:]):
        assert rel_l2(a, b) <= 1e-5, rel_l2(a, b)


def test_several_windows_keep_one_shot_per_layer_block():
    from fwi_gb300 import FwiError, make_shots
    p = problem(seed=22, nx=120, nz=72, nt=160)
    shots = make_shots([dict(sx=30, sz=6, rz=5, rx0=4, rx1=p["nx"] - 4, nt=p["nt"], x0=0, nxw=0),
                        dict(sx=60, sz=8, rz=5, rx0=24, rx1=p["nx"] - 8, nt=p["nt"] - 30, x0=20, nxw=p["nx"] - 24)])
    obs = observed(p, shots, 2)
    ctx = context(p, 2, max_window=p["nx"])
    ctx.set_model(p["vh"], p["vp"], p["vn"])
    t = ctx.autotune(shots, steps=16)
    for ph in ("forward", "adjoint"):  # interior groups may hold both windows; layer groups one shot
        assert t[ph]["layer_shots_per_group"] == 1 and t[ph]["inline_strip"] == 0
        assert t[ph]["shots_per_group"] in (1, 2)
    with pytest.raises(FwiError) as e:
        ctx.set_tuning(shots, dict(forward=phase(1, 1, 0), adjoint=phase(2, 2, 0)))
    assert e.value.status == -1  # FWI_ERR_ARG
    J, *g = ctx.gradient(shots, obs)
    assert np.isfinite(J) and all(np.all(np.isfinite(a)) for a in g)
