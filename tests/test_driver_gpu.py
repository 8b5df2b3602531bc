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


def test_direction_slope_is_the_misfit_derivative():
    """fwi_direction_slope against the misfit along the trial line m_back - alpha r
    (FP64 context: Richardson extrapolation of two one-sided differences)."""
    import fwi_gb300
    ctx = fwi_gb300.Context(nx=NX, nz=NZ, dh=float(G["dh"]), dt=float(G["dt"]), cpml=CPML,
                            f_cpml=float(G["f"]), nt_max=NT, max_shots=2, mode=fwi_gb300.MODE_EXACT,
                            precision=fwi_gb300.PREC_FP64)
    ctx.set_wavelet(G["source"].astype(np.float64))
    ctx.set_model(*(G[k].astype(np.float64) for k in ("vh_i", "vp_i", "vn_i")))
    shots = fwi_gb300.make_shots([(int(sx) - 1, SZ - 1, SZ - 1, CPML, NX - CPML, NT) for sx in G["shots_sx"]])
    obs = np.concatenate([G["obs"][k][:, CPML:NX - CPML].ravel() for k in range(2)]).astype(np.float64)
    ctx.gradient(shots, obs)
    ctx.first_step(3e5, 2e5, 2.5e5)
    J0 = ctx.gradient(shots, obs)[0]
    ctx.lbfgs_direction(5)
    slope = float(ctx.direction_slope().sum())
    assert slope > 0  # a descent direction

    def drop(a):
        ctx.lbfgs_update(a, a, a)
        return (J0 - ctx.misfit(shots, obs)) / a

    a = 1e-3
    est = 2 * drop(a / 2) - drop(a)
    assert abs(est - slope) <= 1e-3 * abs(slope), (est, slope)


def test_armijo_option_keeps_descent():
    ctx, shots, obs = make_ctx()
    hist = ctx.invert(shots, obs, iterations=5, armijo_c1=1e-4)
    assert len(hist) >= 3
    assert np.all(np.diff(hist) <= 0), hist


def test_bands_equal_band_by_band_calls():
    """fwi_invert_bands with observed data from a callback = set_frequency + fwi_invert
    per band, bit for bit; each band's misfit decreases."""
    import fwi_gb300
    f0 = float(G["f"])
    true, shots, _ = make_ctx()
    true.set_model(G["vh_t"], G["vp_t"], G["vn_t"])

    def band_obs(band, f):
        true.set_frequency(f, NT)
        return true.forward(shots)

    ctx, _, _ = make_ctx()
    hists = ctx.invert_bands(shots, band_obs, f0, 3.0, 2, NT, iterations=3)
    ref, _, _ = make_ctx()
    manual = []
    for b in range(2):
        ref.set_frequency(f0 + 3.0 * b, NT)
        manual.append(ref.invert(shots, band_obs(b, f0 + 3.0 * b), iterations=3))
    assert len(hists) == 2
    for h, m in zip(hists, manual):
        assert np.array_equal(h, m)
        assert h[-1] < h[0]
    assert np.array_equal(ctx.get_model()[1], ref.get_model()[1])


def test_model_files_round_trip(tmp_path):
    """Raw float32 Vp / eps / delta in (the reference's *_ori.bin), squared
    velocities out (its *_ini.bin)."""
    import fwi_gb300
    ctx, _, _ = make_ctx()
    rng = np.random.default_rng(4)
    vp = (2000 + 500 * rng.random((NZ, NX))).astype(np.float32)
    eps = (0.1 + 0.1 * rng.random((NZ, NX))).astype(np.float32)
    dl = (0.05 * rng.random((NZ, NX))).astype(np.float32)
    paths = [str(tmp_path / n) for n in ("vp_ori.bin", "vh_ori.bin", "vn_ori.bin")]
    for a, p in zip((vp, eps, dl), paths):
        a.tofile(p)
    ctx.load_model_files(*paths)
    got = ctx.get_model()
    ctx2, _, _ = make_ctx()
    ctx2.set_model_vti(vp, eps, dl)
    for a, b in zip(got, ctx2.get_model()):
        assert np.array_equal(a, b)
    outs = [str(tmp_path / n) for n in ("vh_ini.bin", "vp_ini.bin", "vn_ini.bin")]
    ctx.save_model_files(*outs)
    for a, p in zip(got, outs):
        assert np.array_equal(np.fromfile(p, np.float32).reshape(NZ, NX), a)
    with pytest.raises(fwi_gb300.FwiError):
        ctx.load_model_files(paths[0], paths[1], str(tmp_path / "missing.bin"))


def test_curvature_guard_keeps_the_direction_downhill():
    """A history pair with y.s < 0 for one parameter: the reference's two-loop
    (no guard) scales that parameter's direction by a negative gamma, uphill;
    fwi_set_lbfgs_guard skips the pair, and every parameter's direction is a
    descent direction (g . r > 0 on the rows the update changes)."""
    rng = np.random.default_rng(3)
    m0 = [G["vh_i"], G["vp_i"], G["vn_i"]]
    g0 = [rng.standard_normal((NZ, NX)).astype(np.float32) for _ in range(3)]
    stats = {}
    for guard in (False, True):
        ctx, _, _ = make_ctx()
        ctx.set_model(*m0)
        ctx.set_gradient(*g0)
        ctx.first_step(3e5, 2e5, 2.5e5)
        m1 = ctx.get_model()
        s = [a.astype(np.float64) - b for a, b in zip(m1, m0)]
        # v_hor: the gradient falls along the step (y.s < 0); v_po, v_nmo: it grows (y.s > 0)
        k = [-1e-6, 1e-6, 1e-6]
        g1 = [(g + kk * sv).astype(np.float32) for g, kk, sv in zip(g0, k, s)]
        ctx.set_gradient(*g1)
        ctx.set_lbfgs_guard(guard)
        st = ctx.lbfgs_direction(5)
        slope = ctx.direction_slope()
        stats[guard] = (st, slope)
    (st0, sl0), (st1, sl1) = stats[False], stats[True]
    assert st0[6] < 0 < st0[7] and st0[8] > 0      # y.s of the newest pair, v_hor negative
    assert st0[0] < 0                               # unguarded gamma for v_hor: negative
    assert sl0[0] < 0                               # ... so its direction points uphill
    assert np.all(st1[0:3] > 0) and np.all(np.asarray(sl1) > 0)
    np.testing.assert_allclose(st1[1:3], st0[1:3], rtol=1e-12)  # the other parameters unchanged
