"""Seeded synthetic workloads for the five benchmark configurations.

No field data or model files ship with the reference (src/main.c:101-123
reads files that are absent), so every workload is a seeded synthetic model
with the sizes and value ranges of its configuration:

  C1  201 x 201, dh 10 m, nt 2000, dt 1 ms, 5 flat layers + Gaussian anomaly,
      one shot at (100, 2), 201 receivers at z = 2, 10 Hz, seed 1
  C2  601 x 301, dh 10 m, nt 3000, dt 1 ms, 3 dipping interfaces + 2 anomalies,
      32 shots evenly spaced at z = 2, 601 receivers each, 8 Hz, seed 2
  C3  2001 x 801, dh 12.5 m, nt 6000, dt 1 ms, 8 layers, 2 normal faults
      (50-150 m throw), eps 0-0.25, delta 0-0.12, 64 shots, seed 3
  C4  4001 x 1201, dh 10 m, 256 shots with apertures U(400, 1600) columns and
      nt U(2000, 8000), dt 0.8 ms, 12 Hz, 10 % trace dropout, seed 4
  C5  4001 x 1201, dh 10 m, 512 shots, nt 8000, dt 0.8 ms, bands 3/6/9/12 Hz,
      faulted model with a high-velocity wedge (Vp up to 4500 m/s), seed 5

Grid convention: the physical grid is padded by the reference's 4-point zero
frame on every side (the frame is never updated, src/parallelcalls.cu:96),
so physical (x, z) is computational (x + 4, z + 4) and "z = 2" is an
updated row.  The CPML layers (20 points) lie inside the padded grid.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

FRAME = 4
CFL_LIMIT = 0.5546  # 2-D 8th-order leapfrog: vmax dt / dh <= 2 / sqrt(2 sum |c2|)


@dataclass
class Workload:
    name: str
    nx: int            # computational grid (physical + 2 * FRAME)
    nz: int
    dh: float
    dt: float
    nt: int
    f: float
    cpml: int
    shots: list        # dicts: sx, sz, rz, rx0, rx1, nt, x0, nxw (computational coordinates)
    vel: np.ndarray    # true Vp, epsilon, delta [nz][nx] (float32)
    eps: np.ndarray
    delta: np.ndarray
    vel0: np.ndarray = None  # initial model
    eps0: np.ndarray = None
    delta0: np.ndarray = None
    mask: np.ndarray = None  # per-shot receiver masks, concatenated (uint8) or None
    bands: list = field(default_factory=list)
    note: str = ""

    @property
    def points(self):
        return self.nx * self.nz

    def squared(self, initial=False):
        """(v_hor, v_po, v_nmo) as the reference's pre_variables forms them."""
        v, e, d = (self.vel0, self.eps0, self.delta0) if initial else (self.vel, self.eps, self.delta)
        vp = (v * v).astype(np.float32)
        return ((vp * (1 + 2 * e)).astype(np.float32), vp, (vp * (1 + 2 * d)).astype(np.float32))

    def point_updates(self, shots=None):
        """Forward + adjoint point updates of a gradient over `shots` (windows and nt per shot),
        counting every grid point of each shot's window, the 4-point frame included."""
        sh = self.shots if shots is None else shots
        return sum(2 * (s["nxw"] or self.nx) * self.nz * s["nt"] for s in sh)

    def physical_point_updates(self, shots=None):
        """The same over the points a step updates: each window without its 4-point frame
        (601 x 301 per shot and step for C2, not 609 x 309)."""
        sh = self.shots if shots is None else shots
        return sum(2 * ((s["nxw"] or self.nx) - 2 * FRAME) * (self.nz - 2 * FRAME) * s["nt"] for s in sh)

    def cfl(self):
        vmax = float((self.vel * np.sqrt(1 + 2 * np.maximum(self.eps, self.delta))).max())
        return vmax * self.dt / self.dh

    def __post_init__(self):
        # the true model's fastest speed bounds the smoothed initial model's
        if self.cfl() > CFL_LIMIT:
            raise ValueError(f"{self.name}: vmax dt / dh = {self.cfl():.4f} above the stability limit {CFL_LIMIT}")


def _gauss_smooth(a, sigma):
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(a.astype(np.float64), sigma, mode="nearest").astype(np.float32)


def _pad(a):
    return np.pad(a, FRAME, mode="edge").astype(np.float32)


def _layers(nzp, nxp, depths, values, dips=None):
    """Piecewise-constant model: value k below interface k (depth in points at x=0, dip in points/point)."""
    z = np.arange(nzp, dtype=np.float64)[:, None]
    x = np.arange(nxp, dtype=np.float64)[None, :]
    out = np.full((nzp, nxp), values[0], np.float64)
    for k, d in enumerate(depths):
        dip = 0.0 if dips is None else dips[k]
        out = np.where(z >= d + dip * x, values[k + 1], out)
    return out


def _anomaly(nzp, nxp, cx, cz, sigma, amp):
    z = np.arange(nzp)[:, None]
    x = np.arange(nxp)[None, :]
    return amp * np.exp(-((x - cx) ** 2 + (z - cz) ** 2) / (2.0 * sigma ** 2))


def _surface_shots(nxp, count, nt, z_phys=2, rec=(None, None)):
    """Evenly spaced sources at physical depth z_phys; receivers on all physical columns."""
    nx = nxp + 2 * FRAME
    xs = np.linspace(0, nxp - 1, count + 2)[1:-1] if count > 1 else [nxp // 2]
    r0 = FRAME if rec[0] is None else rec[0]
    r1 = nx - FRAME if rec[1] is None else rec[1]
    return [dict(sx=int(round(x)) + FRAME, sz=z_phys + FRAME, rz=z_phys + FRAME, rx0=r0, rx1=r1, nt=nt,
                 x0=0, nxw=0) for x in xs]


def _vti(nzp, nxp, rng, n_layers, emax, dmax, depths, dips=None):
    eps_l = rng.uniform(0.0, emax, n_layers)
    del_l = np.array([rng.uniform(0.0, min(dmax, e)) for e in eps_l])
    eps = _layers(nzp, nxp, depths, eps_l, dips)
    dl = _layers(nzp, nxp, depths, del_l, dips)
    return eps, dl


def c1(seed=1):
    rng = np.random.default_rng(seed)
    nxp = nzp = 201
    depths = np.sort(rng.uniform(0.1, 0.9, 4)) * nzp
    vel = _layers(nzp, nxp, depths, np.linspace(1500, 3500, 5))
    vel += _anomaly(nzp, nxp, nxp * 0.5, nzp * 0.55, 8, 200.0)
    eps, dl = _vti(nzp, nxp, rng, 5, 0.2, 0.1, depths)
    w = Workload("C1 plain single-shot gradient 201x201 nt=2000", nxp + 8, nzp + 8, 10.0, 1e-3, 2000, 10.0, 20,
                 [dict(sx=100 + FRAME, sz=2 + FRAME, rz=2 + FRAME, rx0=FRAME, rx1=nxp + FRAME, nt=2000, x0=0,
                       nxw=0)],
                 _pad(vel), _pad(eps), _pad(dl))
    w.vel0, w.eps0, w.delta0 = (_gauss_smooth(a, 10) for a in (w.vel, w.eps, w.delta))
    return w


def c2(seed=2, shots=32, nt=3000):
    rng = np.random.default_rng(seed)
    nxp, nzp = 601, 301
    depths = np.sort(rng.uniform(0.2, 0.8, 3)) * nzp
    dips = rng.uniform(-0.08, 0.08, 3)
    vel = _layers(nzp, nxp, depths, [1600, 2100, 2600, 3200], dips)
    vel += _anomaly(nzp, nxp, nxp * 0.3, nzp * 0.45, 12, 250.0)
    vel += _anomaly(nzp, nxp, nxp * 0.7, nzp * 0.6, 15, -200.0)
    eps, dl = _vti(nzp, nxp, rng, 4, 0.2, 0.1, depths, dips)
    w = Workload("C2 batched FWI 601x301 nt=3000 32 shots", nxp + 8, nzp + 8, 10.0, 1e-3, nt, 8.0, 20,
                 _surface_shots(nxp, shots, nt), _pad(vel), _pad(eps), _pad(dl))
    w.vel0, w.eps0, w.delta0 = (_gauss_smooth(a, 10) for a in (w.vel, w.eps, w.delta))
    return w


def _faulted(nzp, nxp, rng, n_layers, vmin, vmax_, dh, faults=2):
    depths = np.sort(rng.uniform(0.1, 0.92, n_layers - 1)) * nzp
    vals = np.linspace(vmin, vmax_, n_layers)
    z = np.arange(nzp, dtype=np.float64)[:, None]
    x = np.arange(nxp, dtype=np.float64)[None, :]
    shift = np.zeros((1, nxp))
    for _ in range(faults):
        xf = rng.uniform(0.25, 0.75) * nxp
        throw = rng.uniform(50.0, 150.0) / dh
        shift = shift + np.where(x > xf, throw, 0.0)
    out = np.full((nzp, nxp), vals[0])
    for k, d in enumerate(depths):
        out = np.where(z >= d + shift, vals[k + 1], out)
    return out, depths, shift


def c3(seed=3, shots=64, nt=6000):
    rng = np.random.default_rng(seed)
    nxp, nzp = 2001, 801
    vel, depths, shift = _faulted(nzp, nxp, rng, 8, 1600.0, 4200.0, 12.5)
    e_l = rng.uniform(0, 0.25, 8)
    d_l = np.array([rng.uniform(0, min(0.12, e)) for e in e_l])
    z = np.arange(nzp, dtype=np.float64)[:, None]
    eps = np.full((nzp, nxp), e_l[0])
    dl = np.full((nzp, nxp), d_l[0])
    for k, d in enumerate(depths):
        eps = np.where(z >= d + shift, e_l[k + 1], eps)
        dl = np.where(z >= d + shift, d_l[k + 1], dl)
    w = Workload("C3 checkpointed gradient 2001x801 nt=6000 64 shots", nxp + 8, nzp + 8, 12.5, 1e-3, nt, 10.0, 20,
                 _surface_shots(nxp, shots, nt), _pad(vel), _pad(eps), _pad(dl))
    w.vel0, w.eps0, w.delta0 = (_gauss_smooth(a, 10) for a in (w.vel, w.eps, w.delta))
    return w


def c4(seed=4, shots=256):
    rng = np.random.default_rng(seed)
    nxp, nzp = 4001, 1201
    vel, depths, shift = _faulted(nzp, nxp, rng, 8, 1600.0, 4200.0, 10.0)
    eps = np.full((nzp, nxp), 0.1)
    dl = np.full((nzp, nxp), 0.05)
    nx = nxp + 8
    sh = []
    for k in range(shots):
        ap = int(rng.integers(400, 1601))
        x0 = int(rng.integers(0, nx - ap + 1))
        nt = int(rng.integers(2000, 8001))
        sx = x0 + ap // 2
        sh.append(dict(sx=sx, sz=2 + FRAME, rz=2 + FRAME, rx0=x0 + FRAME, rx1=x0 + ap - FRAME, nt=nt, x0=x0, nxw=ap))
    mask = np.concatenate([(rng.random(s["rx1"] - s["rx0"]) >= 0.10).astype(np.uint8) for s in sh])
    w = Workload(f"C4 uneven batch 4001x1201 {shots} shots", nx, nzp + 8, 10.0, 8e-4, max(s["nt"] for s in sh), 12.0,
                 20, sh, _pad(vel), _pad(eps), _pad(dl), mask=mask)
    w.vel0, w.eps0, w.delta0 = (_gauss_smooth(a, 10) for a in (w.vel, w.eps, w.delta))
    return w


def c5(seed=5, shots=512, nt=8000):
    rng = np.random.default_rng(seed)
    nxp, nzp = 4001, 1201
    vel, depths, shift = _faulted(nzp, nxp, rng, 8, 1600.0, 3800.0, 10.0)
    z = np.arange(nzp)[:, None]
    x = np.arange(nxp)[None, :]
    wedge = (z > 0.35 * nzp) & (z < 0.35 * nzp + 0.4 * (x - 0.3 * nxp)) & (x > 0.3 * nxp)
    vel = np.where(wedge, 4500.0, vel)
    eps = np.full((nzp, nxp), 0.12)
    dl = np.full((nzp, nxp), 0.06)
    w = Workload(f"C5 multiscale 4001x1201 nt={nt} {shots} shots", nxp + 8, nzp + 8, 10.0, 8e-4, nt, 3.0, 20,
                 _surface_shots(nxp, shots, nt), _pad(vel), _pad(eps), _pad(dl), bands=[3.0, 6.0, 9.0, 12.0])
    w.vel0, w.eps0, w.delta0 = (_gauss_smooth(a, 10) for a in (w.vel, w.eps, w.delta))
    return w


WORKLOADS = {"C1": c1, "C2": c2, "C3": c3, "C4": c4, "C5": c5}
