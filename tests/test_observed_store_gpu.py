"""Observed data kept on the device (fwi_store_observed, fwi_model_observed):
gradients and misfits read from the store equal those computed from the same
records passed in, bit for bit (FP32 store), or within the stated FP16 error;
records modelled on the device from a model equal fwi_forward's; the
multiscale loop re-models each band's records there (the reference's
per-band regeneration, src/main.c:321-366) and gives the history the
caller-supplied records give."""
import numpy as np
import pytest

from test_native_gpu import exact_problem, exact_shots, wavelet

pytestmark = pytest.mark.gpu


def ctx_for(p, batch=2):
    from fwi_gb300 import Context, MODE_EXACT
    ctx = Context(nx=p["nx"], nz=p["nz"], dh=p["dh"], dt=p["dt"], cpml=p["cpml"], f_cpml=p["f"], nt_max=p["nt"],
                  max_shots=batch, mode=MODE_EXACT)
    ctx.set_wavelet(wavelet(p).astype(np.float32))
    return ctx


def models(p, scale=(1.0, 1.0, 1.0)):
    return [np.ascontiguousarray(p[k] * s, np.float32) for k, s in zip(("vh", "vp", "vn"), scale)]


def test_store_and_model_observed_equal_passed_records():
    from fwi_gb300 import FwiError, SPREC_FP16, make_shots
    p = exact_problem(dtype=np.float32)
    shots = make_shots(exact_shots(p))
    true, ini = models(p, (1.03, 0.98, 1.02)), models(p)
    ctx = ctx_for(p)
    ctx.set_model(*true)
    obs = ctx.forward(shots)
    ctx.set_model(*ini)
    mask = np.ones(sum(s.nrec for s in shots), np.uint8)
    mask[::7] = 0
    want = ctx.gradient(shots, obs, mask)
    # FP32 store from host records
    ctx.store_observed(shots, obs)
    got = ctx.gradient(shots, None, mask)
    assert got[0] == want[0] and all(np.array_equal(a, b) for a, b in zip(got[1:], want[1:]))
    assert ctx.misfit(shots, None, mask) == want[0]
    # records modelled on the device from the true model; the context keeps its own model
    ctx.model_observed(shots, *true)
    assert all(np.array_equal(a, b) for a, b in zip(ctx.get_model(), ini))
    got = ctx.gradient(shots, None, mask)
    assert got[0] == want[0] and all(np.array_equal(a, b) for a, b in zip(got[1:], want[1:]))
    # FP16 store: 2 B per sample, one scale per trace
    ctx.store_observed(shots, obs, SPREC_FP16)
    g16 = ctx.gradient(shots, None, mask)
    rel = [float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(g16[1:], want[1:])]
    print(f"[parity] FP16 observed store vs FP32 records: misfit {abs(g16[0] - want[0]) / want[0]:.3e}, "
          f"gradients {rel[0]:.3e} {rel[1]:.3e} {rel[2]:.3e}")
    assert abs(g16[0] - want[0]) <= 1e-3 * want[0] and max(rel) <= 1e-2
    ctx.model_observed(shots, *true, store_prec=SPREC_FP16)
    g16m = ctx.gradient(shots, None, mask)
    assert g16m[0] == g16[0] and all(np.array_equal(a, b) for a, b in zip(g16m[1:], g16[1:]))
    # other shots than the stored ones, or no store at all, are refused
    with pytest.raises(FwiError):
        ctx.gradient(make_shots(exact_shots(p)[:1]), None)
    ctx.free_observed()
    with pytest.raises(FwiError):
        ctx.misfit(shots, None)


def test_bands_remodelled_on_the_device_equal_caller_records():
    from fwi_gb300 import make_shots
    p = exact_problem(dtype=np.float32)
    shots = make_shots(exact_shots(p))
    true, ini = models(p, (1.03, 0.98, 1.02)), models(p)
    nt, f0 = p["nt"], 15.0
    twin = ctx_for(p)  # the caller's own modelling of each band's records
    twin.set_model(*true)

    def host_obs(band, f):
        twin.set_frequency(f, nt)
        return twin.forward(shots)

    ctx = ctx_for(p)
    ctx.set_model(*ini)
    want = ctx.invert_bands(shots, host_obs, f0, 5.0, 2, nt, iterations=2)
    ctx2 = ctx_for(p)
    ctx2.set_model(*ini)

    def device_obs(band, f):
        ctx2.model_observed(shots, *true)  # at the band's frequency, set by the loop before the call
        return None

    got = ctx2.invert_bands(shots, device_obs, f0, 5.0, 2, nt, iterations=2)
    assert len(got) == len(want) == 2
    for a, b in zip(got, want):
        assert len(a) == len(b) and np.array_equal(a, b)
