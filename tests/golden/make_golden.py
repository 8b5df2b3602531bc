"""Generate the golden fixtures of tests/golden/ from the reference's own kernels.

The reference (danielvn/Fwi) ships no tests, fixtures or input models.  These
fixtures pin the path by RUNNING the reference's kernels: `make -C oracle ref`
compiles src/parallelcalls.cu from the reference checkout for the CPU
(oracle/ref_shim), and oracle/_ref/libref.so then sequences them the way
src/main.c does (launch grids of src/serialcalls.cu).  The inputs are small
seeded synthetic models.

Usage (needs the reference checkout, given by --ref-root or FWI_REFERENCE_ROOT):
    python tests/golden/make_golden.py [--ref-root PATH]

Writes tests/golden/ref_small.npz.  Host-side inputs that src/main.c computes
on the CPU (the Ricker wavelet, d0 and L of the CPML profiles, the norms and
dot products of the L-BFGS two-loop) come from plain transcriptions of
src/main.c in the fixture script and the reference driver.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as po  # noqa: E402


def seq_sum_sq_f32(a):
    """float accumulation of powf(x, 2) in index order (src/main.c:551-555)."""
    s = np.float32(0)
    for v in a.ravel():
        s = np.float32(s + np.float32(v * v))
    return s


def layered_model(nx, nz, rng, vmin=1800.0, vmax=3200.0):
    """Smooth layered Vp with an anomaly, plus epsilon/delta (delta <= epsilon)."""
    z = np.arange(nz)[:, None] * np.ones((1, nx))
    x = np.ones((nz, 1)) * np.arange(nx)[None, :]
    depths = np.sort(rng.uniform(0.2, 0.9, 3)) * nz
    vel = np.full((nz, nx), vmin)
    eps = np.zeros((nz, nx))
    dl = np.zeros((nz, nx))
    for k, d in enumerate(depths):
        below = z >= d + 2.0 * np.sin(x / 9.0 + k)
        vel[below] = vmin + (k + 1) * (vmax - vmin) / len(depths)
        e = rng.uniform(0.0, 0.2)
        eps[below] = e
        dl[below] = rng.uniform(0.0, min(0.1, e))
    vel += 150.0 * np.exp(-(((x - nx * 0.55) / 6.0) ** 2 + ((z - nz * 0.6) / 5.0) ** 2))
    return vel.astype(np.float32), eps.astype(np.float32), dl.astype(np.float32)


def smooth(a, passes=6):
    out = a.astype(np.float64)
    for _ in range(passes):
        p = np.pad(out, 1, mode="edge")
        out = (p[:-2, 1:-1] + p[2:, 1:-1] + p[1:-1, :-2] + p[1:-1, 2:] + 4 * p[1:-1, 1:-1]) / 8.0
    return out.astype(np.float32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=os.environ.get("FWI_REFERENCE_ROOT"),
                    help="the reference checkout (default: $FWI_REFERENCE_ROOT)")
    args = ap.parse_args()
    if not args.ref_root:
        ap.error("give --ref-root or set FWI_REFERENCE_ROOT to the reference checkout")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref",
                    f"REF_ROOT={args.ref_root}"], check=True)
    ref = po.ref_lib()
    assert ref is not None, "oracle/_ref/libref.so was not built"
    P = po._ptr

    nx, nz, nt, cpml, sz = 64, 48, 300, 10, 5
    dh, dt, f, vmax, Rc = 10.0, 1e-3, 25.0, 6000.0, 1e-6
    shots_sx = [21, 43]
    rng = np.random.default_rng(20261203)
    vel_t, eps_t, del_t = layered_model(nx, nz, rng)
    vel_i, eps_i, del_i = smooth(vel_t), smooth(eps_t), smooth(del_t)

    # src/main.c:48-51: L and d0 in float
    L = np.float32(cpml * np.float32(dh))
    d0 = np.float32(-3 * np.log(np.float64(np.float32(Rc))) / np.float64(np.float32(2 * L)))
    ax, bx, az, bz = (np.zeros(n, np.float32) for n in (nx, nx, nz, nz))
    ref.ref_cpml_x(P(ax), P(bx), cpml, vmax, nx, dt, dh, f, d0, L)
    ref.ref_cpml_z(P(az), P(bz), cpml, vmax, nz, dt, dh, f, d0, L)
    source = po.ricker(nt, dt, f)

    def prevar(vel, eps, dl):
        out = [np.zeros((nz, nx), np.float32) for _ in range(3)]
        ref.ref_pre_variables(P(vel), P(eps), P(dl), *[P(o) for o in out], nx, nz)
        return out

    vh_t, vp_t, vn_t = prevar(vel_t, eps_t, del_t)
    vh_i, vp_i, vn_i = prevar(vel_i, eps_i, del_i)
    base = dict(nx=nx, nz=nz, nt=nt, cpml=cpml, dh=dh, dt=dt, ax=ax, bx=bx, az=az, bz=bz,
                source=source)
    ptrue = dict(base, vh=vh_t, vp=vp_t, vn=vn_t)
    pinit = dict(base, vh=vh_i, vp=vp_i, vn=vn_i)

    out = dict(nx=nx, nz=nz, nt=nt, cpml=cpml, sz=sz, dh=dh, dt=dt, f=f, vmax=vmax, R=Rc,
               L=L, d0=d0, shots_sx=np.array(shots_sx, np.int32),
               vel_t=vel_t, eps_t=eps_t, del_t=del_t, vel_i=vel_i, eps_i=eps_i, del_i=del_i,
               ax=ax, bx=bx, az=az, bz=bz, source=source,
               vh_t=vh_t, vp_t=vp_t, vn_t=vn_t, vh_i=vh_i, vp_i=vp_i, vn_i=vn_i)

    # observed data (true model) with snapshots of shot 0, src/main.c:334-366
    obs = []
    for k, sx in enumerate(shots_sx):
        shot, snap = po.forward_shot(ptrue, sx, sz, snap=(k == 0), library=ref)
        obs.append(shot)
        if k == 0:
            out["snap0_steps"] = np.array([0, 1, 2, 150, 299], np.int32)
            out["snap0"] = snap[out["snap0_steps"]]
    out["obs"] = np.stack(obs)

    # gradient of the initial model, summed over shots as src/main.c:408-496
    g = [np.zeros((nz, nx), np.float32) for _ in range(3)]
    fis, res = [], []
    for k, sx in enumerate(shots_sx):
        fi, gx, gz, gd, r = po.gradient_shot(pinit, sx, sz, obs[k], library=ref)
        fis.append(fi)
        res.append(r)
        out[f"gcx_shot{k}"], out[f"gcz_shot{k}"], out[f"gdx_shot{k}"] = gx, gz, gd
    # the reference accumulates all shots into one gradient: redo it that way
    for k, sx in enumerate(shots_sx):
        ref.ref_gradient_shot(nx, nz, nt, cpml, sx, sz, dh, dt,
                              *[P(pinit[q]) for q in ("ax", "bx", "az", "bz", "vh", "vp", "vn",
                                                       "source")],
                              P(obs[k]), P(g[0]), P(g[1]), P(g[2]), None, nt)
    fiTotal = np.float32(0)
    for fi in fis:
        fiTotal = np.float32(fiTotal + np.float32(fi))
    out["fi"] = np.array(fis, np.float32)
    out["fi_total"] = fiTotal
    out["res"] = np.stack(res)
    out["gcx"], out["gcz"], out["gdx"] = g

    # iteration 0: norms, NORMAL, UpdateModel (src/main.c:539-568)
    norms = [np.float32(np.sqrt(seq_sum_sq_f32(a))) for a in g]
    gn = [a.copy() for a in g]
    ref.ref_normal(P(gn[0]), P(gn[1]), P(gn[2]), nx, nz, *norms)
    vh1, vp1, vn1 = vh_i.copy(), vp_i.copy(), vn_i.copy()
    ref.ref_update_model(P(gn[0]), P(gn[1]), P(gn[2]), P(vh1), P(vp1), P(vn1),
                         3e5, 2e5, 2.5e5, nx, nz)
    out["norms"] = np.array(norms, np.float32)
    out["gcx_n"], out["gcz_n"], out["gdx_n"] = gn
    out["vh_1"], out["vp_1"], out["vn_1"] = vh1, vp1, vn1

    # iteration 1: gradient at the updated model, then the L-BFGS direction in
    # slot 0 and update_LBFGS with alpha = 1 (src/main.c:569-693)
    p1 = dict(base, vh=vh1, vp=vp1, vn=vn1)
    g1 = [np.zeros((nz, nx), np.float32) for _ in range(3)]
    for k, sx in enumerate(shots_sx):
        ref.ref_gradient_shot(nx, nz, nt, cpml, sx, sz, dh, dt,
                              *[P(p1[q]) for q in ("ax", "bx", "az", "bz", "vh", "vp", "vn",
                                                    "source")],
                              P(obs[k]), P(g1[0]), P(g1[1]), P(g1[2]), None, nt)
    out["gcx_1"], out["gcz_1"], out["gdx_1"] = g1

    def lbfgs_state(seed_hist=None):
        st = {n: np.zeros((5, nz, nx), np.float32) for n in
              "s_vp s_vn s_vh y_gcz y_gdx y_gcx".split()}
        st.update(v_po=vp1.copy(), v_nmo=vn1.copy(), v_hor=vh1.copy(),
                  back_vpo=vp_i.copy(), back_vnmo=vn_i.copy(), back_vhor=vh_i.copy(),
                  gcz=g1[1].copy(), gdx=g1[2].copy(), gcx=g1[0].copy(),
                  back_gcz=g[1].copy(), back_gdx=g[2].copy(), back_gcx=g[0].copy())
        for n in "q_gcz q_gdx q_gcx r_b1 r_b2 r_b3".split():
            st[n] = np.zeros((nz, nx), np.float32)
        return st

    st = lbfgs_state()
    sig, eps, gam = po.lbfgs_direction(st, 0, library=ref)
    for n in "s_vp s_vn s_vh y_gcz y_gdx y_gcx".split():
        out[f"lb0_{n}"] = st[n][:1]
    for n in "q_gcz q_gdx q_gcx r_b1 r_b2 r_b3".split():
        out[f"lb0_{n}"] = st[n]
    out["lb0_sigma"], out["lb0_epsilon"], out["lb0_gamma"] = sig, eps, gam
    # the model is backed up before the trial update (src/main.c:683-688), so the
    # trial model is v_1 - alpha r
    vp2, vn2, vh2 = vp1.copy(), vn1.copy(), vh1.copy()
    ref.ref_update_lbfgs(P(st["r_b1"]), P(st["r_b2"]), P(st["r_b3"]), P(vp2), P(vn2), P(vh2),
                         P(vp1), P(vn1), P(vh1), nx, nz, 1.0, 1.0, 1.0, 1, 1, 1, 0, 0)
    out["vp_2"], out["vn_2"], out["vh_2"] = vp2, vn2, vh2
    # the same update with the optional clamps on (flags of src/parallelcalls.cu:343-404)
    vp3, vn3, vh3 = vp1.copy(), vn1.copy(), vh1.copy()
    ref.ref_update_lbfgs(P(st["r_b1"]), P(st["r_b2"]), P(st["r_b3"]), P(vp3), P(vn3), P(vh3),
                         P(vp1), P(vn1), P(vh1), nx, nz, 40.0, 40.0, 40.0, 1, 1, 1, 1, 1)
    out["vp_3"], out["vn_3"], out["vh_3"] = vp3, vn3, vh3

    # a deeper history: slots 0..1 filled with seeded curvature pairs, direction in slot 2
    st = lbfgs_state()
    hr = np.random.default_rng(7)
    for n_s, n_y in (("s_vp", "y_gcz"), ("s_vn", "y_gdx"), ("s_vh", "y_gcx")):
        for slot in range(2):
            s = hr.standard_normal((nz, nx)).astype(np.float32) * 1e3
            st[n_s][slot] = s
            st[n_y][slot] = (s * 1e-4 + hr.standard_normal((nz, nx)) * 1e-2).astype(np.float32)
    for n in "s_vp s_vn s_vh y_gcz y_gdx y_gcx".split():
        out[f"lb2_in_{n}"] = st[n][:2].copy()
    sig, eps, gam = po.lbfgs_direction(st, 2, library=ref)
    for n in "s_vp s_vn s_vh y_gcz y_gdx y_gcx".split():
        out[f"lb2_{n}"] = st[n][:3]
    for n in "q_gcz q_gdx q_gcx r_b1 r_b2 r_b3".split():
        out[f"lb2_{n}"] = st[n]
    out["lb2_sigma"], out["lb2_epsilon"], out["lb2_gamma"] = sig, eps, gam

    path = os.path.join(HERE, "ref_small.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KiB)")


if __name__ == "__main__":
    main()
