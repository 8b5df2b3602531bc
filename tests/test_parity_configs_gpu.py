"""Parity at the benchmark configurations' own geometry, on the GPU.

C1 (201 x 201 physical grid, 209 x 209 with the 4-point frame, nt = 2000,
dt = 1 ms, dh = 10 m, 10 Hz Ricker at physical (100, 2), seeded five-layer
model with a Gaussian anomaly; fwi_gb300.synth.c1):

  * REF_COMPAT (the reference's gradient) against the oracle's restatement of
    the reference's arithmetic (FP32 storage, FP64-promoted stencils,
    src/parallelcalls.cu, sequenced as src/main.c:318-495), through the
    native C-ABI and through the reference-compatible C-ABI
    (launchPropagation / res_h / launchBackPropagation).  Receivers as the
    reference places them: row sz - 1, columns [CPML, nx - CPML)
    (src/parallelcalls.cu:107-116).
  * EXACT (the discrete adjoint) in FP64 against the FP64 oracle, and in FP32
    against the FP64 oracle, with C1's own receiver spread (all 201 physical
    columns).

A C2 window (the C2 model's first 208 columns and 128 rows, nt = 3000, 8 Hz)
pins the FP64 GPU path to the FP64 oracle over C2's full trace length.

Gradients are compared over the whole grid and over the rows the model update
changes (iz > 15, the reference's near-surface `layer`,
include/parallelcalls.h:6; src/parallelcalls.cu:343-404): most of the
gradient's norm, and of the FP32 error, sits in the rows around the sources
and receivers, which no update reads.

A dot-product test of the exact adjoint through the public entry points:
<DF dm, r> (DF dm: the derivative of fwi_forward's traces along a model
perturbation, central differences with Richardson extrapolation, FP64)
against <dm, fwi_gradient with residual r>.

Tolerances are written beside each assertion; the achieved values print with
pytest -s.
"""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

LAYER = 15
F32_DT, F32_R = float(np.float32(1e-3)), float(np.float32(1e-6))


def rel(a, b, rows=0):
    a, b = np.asarray(a, np.float64)[rows:], np.asarray(b, np.float64)[rows:]
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def report(name, **vals):
    print(f"[parity] {name}: " + ", ".join(f"{k} {v:.3e}" for k, v in vals.items()))


# ------------------------------------------------------------------ C1, reference arithmetic

@pytest.fixture(scope="module")
def c1_ref():
    """C1 in the reference's geometry and arithmetic: traces of the true model and the
    gradient of the initial model, from the oracle's restatement (FP32 and FP64)."""
    from fwi_gb300 import synth
    w = synth.c1()
    s = w.shots[0]
    po.set_threads(16)
    out = {"w": w, "sx": s["sx"] + 1, "sz": s["sz"] + 1}  # the reference's 1-based source
    dt32 = float(np.float32(w.dt))  # as the context's configuration holds dt and R
    for dt_ in (np.float32, np.float64):
        ax, bx, az, bz = po.cpml_profiles(w.nx, w.nz, w.cpml, w.dh, dt32, w.f, R=F32_R, dtype=dt_)
        base = dict(nx=w.nx, nz=w.nz, nt=w.nt, cpml=w.cpml, dh=w.dh, dt=dt32, ax=ax, bx=bx, az=az, bz=bz,
                    source=po.ricker(w.nt, dt32, w.f, dtype=dt_))
        true = dict(base, **dict(zip(("vh", "vp", "vn"), (a.astype(dt_) for a in w.squared()))))
        ini = dict(base, **dict(zip(("vh", "vp", "vn"), (a.astype(dt_) for a in w.squared(initial=True)))))
        obs, _ = po.forward_shot(true, out["sx"], out["sz"])
        if dt_ == np.float32:
            obs32 = obs
        fi, gx, gz, gd, res = po.gradient_shot(ini, out["sx"], out["sz"], obs32.astype(dt_))
        out[dt_] = dict(prob=ini, obs=obs, fi=float(fi), g=(gx, gz, gd), res=res)
    return out


def c1_ref_ctx(w, precision, wavelet):
    from fwi_gb300 import Context, MODE_REF_COMPAT
    ctx = Context(nx=w.nx, nz=w.nz, dh=w.dh, dt=w.dt, cpml=w.cpml, f_cpml=w.f, nt_max=w.nt, max_shots=1,
                  mode=MODE_REF_COMPAT, precision=precision)
    ctx.set_wavelet(np.ascontiguousarray(wavelet, ctx.dtype))
    return ctx


def test_c1_ref_compat_native_matches_reference_arithmetic(c1_ref):
    """The native FP32 path in REF_COMPAT mode against the reference's arithmetic.
    Over 2000 steps two FP32 evaluations of the same scheme part by about the
    reference's own FP32 error (its plain-form leapfrog rounds each small update
    against the field: traces 1.1e-4 from its own FP64 evaluation, gradients
    3.3e-3 / 1.1e-4 / 1.3e-3), so the native path is held to the FP64 evaluation
    of the reference's arithmetic, and must be closer to it than the reference's
    own FP32 result is."""
    from fwi_gb300 import PREC_FP32, make_shots
    w, sx, sz = c1_ref["w"], c1_ref["sx"], c1_ref["sz"]
    r32, r64 = c1_ref[np.float32], c1_ref[np.float64]
    cp = w.cpml
    shots = make_shots([(sx - 1, sz - 1, sz - 1, cp, w.nx - cp, w.nt)])
    ctx = c1_ref_ctx(w, PREC_FP32, r32["prob"]["source"])
    ctx.set_model(*w.squared())
    tr = ctx.forward(shots).reshape(w.nt, w.nx - 2 * cp)
    t32, t64 = r32["obs"][:, cp:w.nx - cp], r64["obs"][:, cp:w.nx - cp]
    ctx.set_model(*w.squared(initial=True))
    J, gh, gp, gn = ctx.gradient(shots, np.ascontiguousarray(t32))
    g = (gh, gp, gn)
    e = dict(traces_vs_ref32=rel(tr, t32), traces_vs_ref64=rel(tr, t64), ref32_traces_vs_ref64=rel(t32, t64),
             misfit_vs_ref64=abs(J - r64["fi"]) / r64["fi"], ref32_misfit_vs_ref64=abs(r32["fi"] - r64["fi"]) / r64["fi"])
    g64 = [rel(a, b) for a, b in zip(g, r64["g"])]
    g64u = [rel(a, b, LAYER + 1) for a, b in zip(g, r64["g"])]
    ref = [rel(a, b) for a, b in zip(r32["g"], r64["g"])]
    g32 = [rel(a, b) for a, b in zip(g, r32["g"])]
    report("C1 REF_COMPAT native FP32 vs the reference's arithmetic", **e,
           **{f"g_vs_ref64_{k}": v for k, v in zip(("hor", "po", "nmo"), g64)},
           **{f"upd_vs_ref64_{k}": v for k, v in zip(("hor", "po", "nmo"), g64u)},
           **{f"ref32_g_vs_ref64_{k}": v for k, v in zip(("hor", "po", "nmo"), ref)},
           **{f"g_vs_ref32_{k}": v for k, v in zip(("hor", "po", "nmo"), g32)})
    assert e["traces_vs_ref64"] <= 2e-5                      # measured 5e-6 class
    assert e["traces_vs_ref32"] <= 2e-4                      # the reference's own FP32 error, 1.1e-4
    assert e["misfit_vs_ref64"] <= 1e-5
    assert max(g64u) <= 1e-4                                 # the rows the update changes
    assert all(a <= b for a, b in zip(g64, ref))             # no farther from FP64 than the reference's FP32
    assert max(g32) <= 5e-3


def test_c1_ref_compat_fp64_matches_reference_arithmetic_in_fp64(c1_ref):
    from fwi_gb300 import PREC_FP64, make_shots
    w, sx, sz = c1_ref["w"], c1_ref["sx"], c1_ref["sz"]
    r64 = c1_ref[np.float64]
    cp = w.cpml
    shots = make_shots([(sx - 1, sz - 1, sz - 1, cp, w.nx - cp, w.nt)])
    ctx = c1_ref_ctx(w, PREC_FP64, r64["prob"]["source"])
    ctx.set_model(*(a.astype(np.float64) for a in w.squared(initial=True)))
    obs = np.ascontiguousarray(c1_ref[np.float32]["obs"][:, cp:w.nx - cp], np.float64)
    J, gh, gp, gn = ctx.gradient(shots, obs)
    e = [rel(a, b) for a, b in zip((gh, gp, gn), r64["g"])]
    report("C1 REF_COMPAT native FP64 vs reference arithmetic in FP64", misfit=abs(J - r64["fi"]) / r64["fi"],
           g_hor=e[0], g_po=e[1], g_nmo=e[2])
    # the FP64 oracle's profiles and wavelet come from FP32 inputs promoted, as the context's
    assert abs(J - r64["fi"]) <= 1e-9 * r64["fi"]
    assert max(e) <= 1e-8


def test_c1_ref_compat_through_launch_functions_matches_reference_arithmetic(c1_ref):
    """The drop-in ABI at C1 size: src/main.c's sequence for one shot through
    launchPropagation / res_h / launchBackPropagation, 2000 steps, reproduces the
    reference's arithmetic bit for bit (traces, residual, the three gradients)."""
    from compat_shot import compat_gradient_shot
    from fwi_gb300 import native
    L = native.lib()
    w, sx, sz = c1_ref["w"], c1_ref["sx"], c1_ref["sz"]
    r32 = c1_ref[np.float32]
    p = r32["prob"]
    res, syn, g = compat_gradient_shot(L, w.nx, w.nz, w.nt, w.cpml, w.dh, w.dt, p["ax"], p["bx"], p["az"], p["bz"],
                                       p["vh"], p["vp"], p["vn"], p["source"], sx, sz, r32["obs"])
    assert L.fwi_compat_last_error() == 0
    e_res = rel(res, r32["res"])
    e_all = [rel(a, b) for a, b in zip(g, r32["g"])]
    report("C1 compat ABI FP32 vs reference arithmetic", residual=e_res, g_hor=e_all[0], g_po=e_all[1],
           g_nmo=e_all[2])
    assert np.array_equal(res, r32["res"])
    for a, b in zip(g, r32["g"]):
        assert np.array_equal(a, b)


# ------------------------------------------------------------------ exact adjoint vs the FP64 oracle

def wavelet(w, nt):
    """The Ricker wavelet of src/main.c:328-332 in FP64, from dt as the context holds it."""
    return po.ricker(nt, float(np.float32(w.dt)), w.f, dtype=np.float64)


def exact_oracle(w, model, shot, obs=None):
    """FP64 oracle of the native semantics: (traces, J, gradients) of one shot."""
    dt32 = float(np.float32(w.dt))
    ax, bx, az, bz = po.cpml_profiles(w.nx, w.nz, w.cpml, w.dh, dt32, w.f, R=F32_R, dtype=np.float64)
    p = dict(nx=w.nx, nz=w.nz, nt=shot["nt"], cpml=w.cpml, dh=w.dh, dt=dt32, ax=ax, bx=bx, az=az, bz=bz,
             source=wavelet(w, shot["nt"]),
             **dict(zip(("vh", "vp", "vn"), (np.ascontiguousarray(a, np.float64) for a in model))))
    geo = (shot["sx"], shot["sz"], shot["rz"], shot["rx0"], shot["rx1"])
    tr = po.exact_forward(p, *geo)
    if obs is None:
        return tr, None, None
    J, gh, gp, gn = po.exact_gradient(p, *geo, obs=obs)
    return tr, J, (gh, gp, gn)


def exact_ctx(w, precision, nt):
    from fwi_gb300 import Context, MODE_EXACT
    ctx = Context(nx=w.nx, nz=w.nz, dh=w.dh, dt=w.dt, cpml=w.cpml, f_cpml=w.f, nt_max=nt, max_shots=1,
                  mode=MODE_EXACT, precision=precision)
    ctx.set_wavelet(np.ascontiguousarray(wavelet(w, nt), ctx.dtype))
    return ctx


@pytest.fixture(scope="module")
def c1_exact():
    from fwi_gb300 import synth
    w = synth.c1()
    po.set_threads(16)
    shot = w.shots[0]
    obs, _, _ = exact_oracle(w, w.squared(), shot)
    _, J, g = exact_oracle(w, w.squared(initial=True), shot, obs=obs)
    return w, shot, obs, J, g


def test_c1_exact_fp64_matches_fp64_oracle(c1_exact):
    from fwi_gb300 import PREC_FP64, make_shots
    w, shot, obs, J, g = c1_exact
    ctx = exact_ctx(w, PREC_FP64, shot["nt"])
    ctx.set_model(*(a.astype(np.float64) for a in w.squared(initial=True)))
    Jg, *gg = ctx.gradient(make_shots([shot]), np.ascontiguousarray(obs))
    e = [rel(a, b) for a, b in zip(gg, g)]
    report("C1 EXACT FP64 vs FP64 oracle", misfit=abs(Jg - J) / J, g_hor=e[0], g_po=e[1], g_nmo=e[2])
    assert abs(Jg - J) <= 1e-10 * J
    assert max(e) <= 1e-10


def test_c1_exact_fp32_matches_fp64_oracle(c1_exact):
    from fwi_gb300 import PREC_FP32, make_shots
    w, shot, obs, J, g = c1_exact
    ctx = exact_ctx(w, PREC_FP32, shot["nt"])
    ctx.set_model(*w.squared(initial=True))
    Jg, *gg = ctx.gradient(make_shots([shot]), np.ascontiguousarray(obs, np.float32))
    e_all = [rel(a, b) for a, b in zip(gg, g)]
    e_upd = [rel(a, b, LAYER + 1) for a, b in zip(gg, g)]
    report("C1 EXACT FP32 vs FP64 oracle", misfit=abs(Jg - J) / J, g_hor=e_all[0], g_po=e_all[1], g_nmo=e_all[2],
           upd_hor=e_upd[0], upd_po=e_upd[1], upd_nmo=e_upd[2])
    assert abs(Jg - J) <= 1e-5 * J
    assert max(e_upd) <= 1e-4    # the target, on the rows the update changes
    assert max(e_all) <= 2e-3


def test_c2_window_fp64_matches_fp64_oracle_over_3000_steps():
    """The C2 model's first 208 columns and 128 rows (with the frame), C2's
    trace length (nt = 3000) and wavelet, C2's first shot position."""
    from fwi_gb300 import PREC_FP32, PREC_FP64, make_shots, synth
    c2 = synth.c2(shots=32)
    po.set_threads(16)
    nx, nz = 208, 128

    w = SimpleNamespace(nx=nx, nz=nz, dh=c2.dh, dt=c2.dt, f=c2.f, cpml=c2.cpml, nt=c2.nt)
    cut = lambda ms: [np.ascontiguousarray(a[:nz, :nx]) for a in ms]
    true, ini = cut(c2.squared()), cut(c2.squared(initial=True))
    shot = dict(sx=c2.shots[0]["sx"], sz=6, rz=6, rx0=4, rx1=nx - 4, nt=c2.nt, x0=0, nxw=0)
    obs, _, _ = exact_oracle(w, true, shot)
    _, J, g = exact_oracle(w, ini, shot, obs=obs)
    res = {}
    for prec, dt_ in ((PREC_FP64, np.float64), (PREC_FP32, np.float32)):
        ctx = exact_ctx(w, prec, shot["nt"])
        ctx.set_model(*(a.astype(dt_) for a in ini))
        Jg, *gg = ctx.gradient(make_shots([shot]), np.ascontiguousarray(obs, dt_))
        res[prec] = (abs(Jg - J) / J, [rel(a, b) for a, b in zip(gg, g)], [rel(a, b, LAYER + 1) for a, b in zip(gg, g)])
        del ctx
    (m64, e64, _), (m32, e32, u32) = res[PREC_FP64], res[PREC_FP32]
    report("C2 window nt 3000 EXACT FP64 vs FP64 oracle", misfit=m64, g_hor=e64[0], g_po=e64[1], g_nmo=e64[2])
    report("C2 window nt 3000 EXACT FP32 vs FP64 oracle", misfit=m32, g_hor=e32[0], g_po=e32[1], g_nmo=e32[2],
           upd_hor=u32[0], upd_po=u32[1], upd_nmo=u32[2])
    assert m64 <= 1e-10 and max(e64) <= 1e-10
    # FP32, stated: on this narrow window (CPML on three sides within 108 points) measured
    # 4.2e-4 / 6.2e-5 / 7.9e-5 on the update rows; the full-width C2 figure is the benchmark's
    assert m32 <= 1e-5 and max(u32) <= 1e-3 and max(e32) <= 5e-3


# ------------------------------------------------------------------ dot-product test of the exact adjoint

def dot_problem():
    rng = np.random.default_rng(9)
    nx, nz, nt = 72, 56, 260
    vel = 1900 + 700 * rng.random((nz, nx))
    for _ in range(4):
        vel = (vel + np.roll(vel, 1, 0) + np.roll(vel, 1, 1)) / 3
    eps = 0.15 + 0.05 * rng.random((nz, nx))
    dl = 0.05 + 0.05 * rng.random((nz, nx))
    vp = vel ** 2
    model = (vp * (1 + 2 * eps), vp, vp * (1 + 2 * dl))

    def smooth(a):
        for _ in range(3):
            a = (a + np.roll(a, 1, 0) + np.roll(a, -1, 0) + np.roll(a, 1, 1) + np.roll(a, -1, 1)) / 5
        return a
    dm = [smooth(rng.standard_normal((nz, nx))) * m.mean() for m in model]
    # two shots: one at the surface, one with source and receivers inside the CPML layers
    shots = [dict(sx=20, sz=6, rz=6, rx0=4, rx1=nx - 4, nt=nt, x0=0, nxw=0),
             dict(sx=6, sz=nz - 7, rz=nz - 6, rx0=4, rx1=nx - 4, nt=nt, x0=0, nxw=0)]
    r = rng.standard_normal(sum(s["nt"] * (s["rx1"] - s["rx0"]) for s in shots))
    return nx, nz, nt, model, dm, shots, r


def dot_ctx(nx, nz, nt, precision):
    from fwi_gb300 import Context, MODE_EXACT
    ctx = Context(nx=nx, nz=nz, dh=10.0, dt=F32_DT, cpml=12, f_cpml=20.0, nt_max=nt, max_shots=2,
                  mode=MODE_EXACT, precision=precision)
    ctx.set_wavelet(po.ricker(nt, F32_DT, 20.0, dtype=ctx.dtype))
    return ctx


def test_dot_product_of_the_exact_adjoint_through_the_entry_points():
    """<DF dm, r> = <dm, DF^T r>: DF^T r is fwi_gradient with observed data
    F(m) - r (its residual is then r), DF dm the derivative of fwi_forward's
    traces along dm (FP64, central differences at e and e/2 combined by
    Richardson extrapolation, truncation O(e^4)).  FP64: agreement to 1e-9
    (6.5e-10 measured here, 5e-11 on the CPU oracle with the same
    construction).  FP32: the FP32 adjoint against the FP64 derivative, within
    2e-5 (1.1e-5 measured)."""
    from fwi_gb300 import PREC_FP32, PREC_FP64, make_shots
    nx, nz, nt, model, dm, shots, r = dot_problem()
    sh = make_shots(shots)
    c64 = dot_ctx(nx, nz, nt, PREC_FP64)
    c64.set_model(*model)
    F0 = c64.forward(sh)
    _, *g64 = c64.gradient(sh, F0 - r)
    rhs64 = sum(float((a * b).sum()) for a, b in zip(g64, dm))

    def F(s):
        c64.set_model(*(m + s * d for m, d in zip(model, dm)))
        return c64.forward(sh)
    e = 1e-3
    D1 = (F(e) - F(-e)) / (2 * e)
    D2 = (F(e / 2) - F(-e / 2)) / e
    lhs = float((((4 * D2 - D1) / 3) * r).sum())
    err64 = abs(lhs - rhs64) / abs(lhs)

    c32 = dot_ctx(nx, nz, nt, PREC_FP32)
    c32.set_model(*(m.astype(np.float32) for m in model))
    F32 = c32.forward(sh)
    _, *g32 = c32.gradient(sh, (F32 - r.astype(np.float32)).astype(np.float32))
    rhs32 = sum(float((a.astype(np.float64) * b).sum()) for a, b in zip(g32, dm))
    err32 = abs(lhs - rhs32) / abs(lhs)
    report("dot-product test, exact adjoint", fp64=err64, fp32=err32)
    assert err64 <= 1e-9
    assert err32 <= 2e-5
