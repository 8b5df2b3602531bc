"""The seeded synthetic workloads C1-C5 (fwi_gb300/synth.py): stable time
steps, and shot geometry the library accepts (windows inside the model,
sources and receivers on interior points of their windows, masks sized to
the receivers)."""
import numpy as np
import pytest

from fwi_gb300 import synth


def interior(ix, iz, nx, nz):
    return 3 < ix < nx - 4 and 3 < iz < nz - 4


@pytest.mark.parametrize("name,kw", [("C1", {}), ("C2", {}), ("C3", dict(shots=8, nt=600)), ("C4", dict(shots=16)),
                                     ("C5", dict(shots=16, nt=800))])
def test_workload_is_stable_and_its_shots_fit(name, kw):
    w = synth.WORKLOADS[name](**kw)
    assert 0 < w.cfl() <= synth.CFL_LIMIT
    for a in (w.vel, w.eps, w.delta, w.vel0, w.eps0, w.delta0):
        assert a.shape == (w.nz, w.nx) and np.all(np.isfinite(a))
    assert np.all(w.delta <= w.eps + 1e-6)  # VTI: delta <= epsilon
    for s in w.shots:
        x0, nxw = s["x0"], s["nxw"] or w.nx
        assert 0 <= x0 and x0 + nxw <= w.nx and nxw >= 2 * w.cpml + 9
        assert interior(s["sx"] - x0, s["sz"], nxw, w.nz)
        assert s["rx1"] > s["rx0"]
        assert interior(s["rx0"] - x0, s["rz"], nxw, w.nz) and interior(s["rx1"] - 1 - x0, s["rz"], nxw, w.nz)
        assert 0 < s["nt"] <= w.nt
    if w.mask is not None:
        assert w.mask.size == sum(s["rx1"] - s["rx0"] for s in w.shots)


def test_unstable_time_step_is_refused():
    w = synth.c1()
    with pytest.raises(ValueError):
        synth.Workload("too coarse", w.nx, w.nz, w.dh, 10 * w.dt, w.nt, w.f, w.cpml, w.shots, w.vel, w.eps, w.delta)
