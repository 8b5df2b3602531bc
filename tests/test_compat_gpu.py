"""Parity of the reference-compatible C-ABI (include/fwi_compat.h) on the GPU.

Every entry point is called through the C-ABI with device buffers and
compared with the oracle / the golden fixtures made from the reference's own
kernels.  Tolerances:
  - element-wise kernels (pre_variables, NORMAL, UpdateModel, the L-BFGS
    axpys, res): bit-exact (explicitly rounded FP32, as the reference's
    formulas);
  - CPML profiles: within 2 ulp (FP64 exp on the device vs the host's);
  - stencil kernels, one step: bit-exact (the reference's mixed FP32 / FP64
    stencil arithmetic, operation for operation, no multiply-add contraction);
  - one full shot sequenced as src/main.c (forward with host snapshots,
    residual, adjoint + imaging): bit-exact residual traces and gradients.
"""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
G = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_small.npz"))
NX, NZ, NT, CPML, SZ = (int(G[k]) for k in ("nx", "nz", "nt", "cpml", "sz"))
DH, DT = float(G["dh"]), float(G["dt"])


@pytest.fixture(scope="module")
def L():
    from fwi_gb300 import native
    return native.lib()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def zeros(*shape):
    return torch.zeros(*shape, dtype=torch.float32, device="cuda")


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def P(t):
    return t.data_ptr()


_KEEP = []


def D(a):
    """Device copy that stays alive for the whole test (a bare temporary would be
    freed, and its memory handed to the next allocation, before the kernel runs)."""
    t = dev(a)
    _KEEP.append(t)
    return t


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def test_pre_variables_bitexact(L):
    for p in ("t", "i"):
        vel, eps, dl = dev(G[f"vel_{p}"]), dev(G[f"eps_{p}"]), dev(G[f"del_{p}"])
        vh, vp, vn = zeros(NZ, NX), zeros(NZ, NX), zeros(NZ, NX)
        L.pre_variables_h(P(vel), P(eps), P(dl), P(vh), P(vp), P(vn), NX, NZ)
        assert np.array_equal(host(vh), G[f"vh_{p}"])
        assert np.array_equal(host(vp), G[f"vp_{p}"])
        assert np.array_equal(host(vn), G[f"vn_{p}"])
    assert L.fwi_compat_last_error() == 0


def test_cpml_profiles(L):
    ax, bx, az, bz = zeros(NX), zeros(NX), zeros(NZ), zeros(NZ)
    args = (CPML, float(G["vmax"]))
    L.CPML_x_h(P(ax), P(bx), *args, NX, DT, DH, float(G["f"]), float(G["d0"]), float(G["L"]))
    L.CPML_z_h(P(az), P(bz), *args, NZ, DT, DH, float(G["f"]), float(G["d0"]), float(G["L"]))
    for t, k in ((ax, "ax"), (bx, "bx"), (az, "az"), (bz, "bz")):
        got, want = host(t), G[k]
        assert np.array_equal(got == 0, want == 0), k
        np.testing.assert_allclose(got, want, rtol=2.5e-7, atol=0, err_msg=k)


def test_normal_and_update_model_bitexact(L):
    g = [dev(G[k]) for k in ("gcx", "gcz", "gdx")]
    L.NORMAL_h(P(g[0]), P(g[1]), P(g[2]), NX, NZ, *[float(x) for x in G["norms"]])
    for t, k in zip(g, ("gcx_n", "gcz_n", "gdx_n")):
        assert np.array_equal(host(t), G[k]), k
    vh, vp, vn = dev(G["vh_i"]), dev(G["vp_i"]), dev(G["vn_i"])
    L.UpdateModel_h(P(g[0]), P(g[1]), P(g[2]), P(vh), P(vp), P(vn), 3e5, 2e5, 2.5e5, NX, NZ)
    assert np.array_equal(host(vh), G["vh_1"]) and np.array_equal(host(vp), G["vp_1"])
    assert np.array_equal(host(vn), G["vn_1"])


def _lbfgs_direction_compat(L, k, hist=None):
    """src/main.c:570-682 driven through the compat ABI; host dots as the oracle's."""
    O = po.lib()
    n = NX * NZ
    H = {nm: zeros(5, NZ, NX) for nm in "s_vp s_vn s_vh y_gcz y_gdx y_gcx".split()}
    if hist:
        for nm, a in hist.items():
            H[nm][: a.shape[0]] = dev(a)
    vpo, vnmo, vhor = dev(G["vp_1"]), dev(G["vn_1"]), dev(G["vh_1"])
    bvpo, bvnmo, bvhor = dev(G["vp_i"]), dev(G["vn_i"]), dev(G["vh_i"])
    gcz, gdx, gcx = dev(G["gcz_1"]), dev(G["gdx_1"]), dev(G["gcx_1"])
    bgcz, bgdx, bgcx = dev(G["gcz"]), dev(G["gdx"]), dev(G["gcx"])
    q = [gcz.clone(), gdx.clone(), gcx.clone()]
    r = [zeros(NZ, NX) for _ in range(3)]
    L.compute_sy_h(P(H["s_vp"]), P(H["s_vn"]), P(H["s_vh"]), P(H["y_gcz"]), P(H["y_gdx"]),
                   P(H["y_gcx"]), P(vpo), P(vnmo), P(vhor), P(bvpo), P(bvnmo), P(bvhor), P(gcz),
                   P(gdx), P(gcx), P(bgcz), P(bgdx), P(bgcx), NX, NZ, k)
    sv = [[0.0] * 5 for _ in range(3)]
    ev = [[0.0] * 5 for _ in range(3)]
    pairs = (("y_gcz", "s_vp"), ("y_gdx", "s_vn"), ("y_gcx", "s_vh"))

    def hd(a, b):
        a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
        return O.orc_host_halfdot_f32(a.ctypes.data, b.ctypes.data, n)

    for l in range(k, -1, -1):
        for c, (yn, sn) in enumerate(pairs):
            y, s = host(H[yn][l]), host(H[sn][l])
            sv[c][l] = np.float32(1.0 / hd(y, s))
            ev[c][l] = np.float32(sv[c][l] * np.float32(hd(host(q[c]), s)))
        L.compute_qi_h(P(q[0]), P(q[1]), P(q[2]), P(H["y_gcz"]), P(H["y_gdx"]), P(H["y_gcx"]),
                       ev[0][l], ev[1][l], ev[2][l], NX, NZ, l)
    gam = []
    for yn, sn in pairs:
        s, y = np.ascontiguousarray(host(H[sn][k])), np.ascontiguousarray(host(H[yn][k]))
        sy, yy = C.c_float(), C.c_float()
        O.orc_host_sy_yy_f32(s.ctypes.data, y.ctypes.data, n, C.byref(sy), C.byref(yy))
        gam.append(np.float32(np.float32(sy.value) / np.float32(yy.value)))
    L.compute_ri_h(P(r[0]), P(r[1]), P(r[2]), P(q[0]), P(q[1]), P(q[2]), *[float(x) for x in gam],
                   NX, NZ)
    for l in range(0, k + 1):
        beta = [np.float32(sv[c][l] * np.float32(hd(host(H[yn][l]), host(r[c]))))
                for c, (yn, _) in enumerate(pairs)]
        L.update_r_h(P(r[0]), P(r[1]), P(r[2]), P(H["s_vp"]), P(H["s_vn"]), P(H["s_vh"]),
                     ev[0][l], ev[1][l], ev[2][l], *[float(b) for b in beta], NX, NZ, l)
    return [host(t) for t in r], np.array(gam, np.float32)


@pytest.mark.parametrize("k", [0, 2])
def test_lbfgs_axpys_bitexact(L, k):
    hist = None
    if k == 2:
        hist = {nm: G[f"lb2_in_{nm}"] for nm in "s_vp s_vn s_vh y_gcz y_gdx y_gcx".split()}
    r, gam = _lbfgs_direction_compat(L, k, hist)
    assert np.array_equal(gam, G[f"lb{k}_gamma"])
    for t, nm in zip(r, ("r_b1", "r_b2", "r_b3")):
        assert np.array_equal(t, G[f"lb{k}_{nm}"]), nm


def test_update_lbfgs_bitexact(L):
    r = [dev(G[k]) for k in ("lb0_r_b1", "lb0_r_b2", "lb0_r_b3")]
    for alpha, fmin, fmax, tag in ((1.0, 0, 0, "2"), (40.0, 1, 1, "3")):
        vp, vn, vh = dev(G["vp_1"]), dev(G["vn_1"]), dev(G["vh_1"])
        bp, bn, bh = dev(G["vp_1"]), dev(G["vn_1"]), dev(G["vh_1"])
        L.update_LBFGS_h(P(r[0]), P(r[1]), P(r[2]), P(vp), P(vn), P(vh), P(bp), P(bn), P(bh), NX,
                         NZ, alpha, alpha, alpha, 1, 1, 1, fmin, fmax)
        assert np.array_equal(host(vp), G[f"vp_{tag}"]) and np.array_equal(host(vn), G[f"vn_{tag}"])
        assert np.array_equal(host(vh), G[f"vh_{tag}"])


def _random_state(seed):
    """White-noise fields (zero frame)."""
    rng = np.random.default_rng(seed)

    def field():
        a = rng.standard_normal((NZ, NX))
        a[:4] = a[-4:] = 0
        a[:, :4] = a[:, -4:] = 0
        return a.astype(np.float32)
    return field


def test_single_step_kernels_against_oracle(L):
    O = po.lib()
    sm = _random_state(5)
    Pp, Fp, Pq, Fq = sm(), sm(), sm(), sm()
    psx, psz, zx, zz = (sm() * 0.1 for _ in range(4))
    ax, bx, az, bz = (G[k] for k in ("ax", "bx", "az", "bz"))
    vh, vp, vn, src = G["vh_i"], G["vp_i"], G["vn_i"], G["source"]
    dh2 = np.float32(DH * DH)
    C_ = np.float32(np.float32(DT * DT) / dh2)
    ptr = po._ptr

    def tol(got, want):
        return np.array_equal(got, want)

    # SecondDerivate_P
    p2o, r2o = np.zeros_like(Pp), np.zeros_like(Pp)
    O.orc_second_derivate_p_f32(ptr(Pp), ptr(Fp), ptr(p2o), ptr(r2o), dh2, NX, NZ)
    p2g, r2g = zeros(NZ, NX), zeros(NZ, NX)
    L.SecondDerivate_P_h(P(D(Pp)), P(D(Fp)), P(p2g), P(r2g), float(dh2), NX, NZ)
    assert tol(host(p2g), p2o) and tol(host(r2g), r2o)
    # PSI_F
    a_o, b_o = psx.copy(), psz.copy()
    O.orc_psi_f_f32(ptr(Pp), ptr(Fp), ptr(ax), ptr(bx), ptr(az), ptr(bz), ptr(a_o), ptr(b_o), NX, NZ, DH, CPML)
    a_g, b_g = dev(psx), dev(psz)
    L.PSI_F_h(P(D(Pp)), P(D(Fp)), P(D(ax)), P(D(bx)), P(D(az)), P(D(bz)), P(a_g), P(b_g), NX, NZ,
              DH, CPML)
    assert tol(host(a_g), a_o) and tol(host(b_g), b_o)
    # ZETA_F (on the oracle's p2/r2/psi)
    zx_o, zz_o, ap_o, af_o = zx.copy(), zz.copy(), np.zeros_like(zx), np.zeros_like(zx)
    O.orc_zeta_f_f32(ptr(p2o), ptr(r2o), ptr(ax), ptr(bx), ptr(az), ptr(bz), ptr(a_o), ptr(b_o), ptr(zx_o),
                     ptr(zz_o), ptr(ap_o), ptr(af_o), NX, NZ, DH, CPML)
    zx_g, zz_g, ap_g, af_g = dev(zx), dev(zz), zeros(NZ, NX), zeros(NZ, NX)
    L.ZETA_F_h(P(D(p2o)), P(D(r2o)), 0, 0, P(D(ax)), P(D(bx)), P(D(az)), P(D(bz)), P(D(a_o)),
               P(D(b_o)), P(zx_g), P(zz_g), P(ap_g), P(af_g), NX, NZ, DH, float(dh2), CPML)
    for g_, o_ in ((zx_g, zx_o), (zz_g, zz_o), (ap_g, ap_o), (af_g, af_o)):
        assert tol(host(g_), o_)
    # propagator_F (source and receivers on row sz-1)
    Pn_o, Fn_o, PF_o, shot_o = Pq.copy(), Fq.copy(), np.zeros_like(Pq), np.zeros((NT, NX), np.float32)
    O.orc_propagator_f_f32(ptr(p2o), ptr(r2o), ptr(PF_o), ptr(Pp), ptr(Fp), ptr(Pn_o), ptr(Fn_o), ptr(vh),
                           ptr(vp), ptr(vn), ptr(ap_o), ptr(af_o), ptr(src), ptr(shot_o), C_, dh2, NX, NZ,
                           21, SZ, 40, CPML)
    Pn_g, Fn_g, PF_g, shot_g = dev(Pq), dev(Fq), zeros(NZ, NX), zeros(NT, NX)
    L.propagator_F_h(P(D(p2o)), P(D(r2o)), P(PF_g), P(D(Pp)), P(D(Fp)), P(Pn_g), P(Fn_g), P(D(vh)),
                     P(D(vp)), P(D(vn)), P(D(ap_o)), P(D(af_o)), P(D(src)), P(shot_g), float(C_),
                     float(dh2), NX, NZ, 21, SZ, 40, CPML)
    for g_, o_ in ((Pn_g, Pn_o), (Fn_g, Fn_o), (PF_g, PF_o), (shot_g, shot_o)):
        assert tol(host(g_), o_)
    # res
    s1, s2 = sm()[:NZ], sm()[:NZ]
    ro = np.zeros_like(s1)
    O.orc_res_f32(ptr(ro), ptr(s1), ptr(s2), NX, NZ)
    rg = zeros(NZ, NX)
    L.res_h(P(rg), P(D(s1)), P(D(s2)), NX, NZ)
    assert np.array_equal(host(rg), ro)
    assert L.fwi_compat_last_error() == 0


def test_one_shot_through_launch_functions_matches_reference(L):
    """src/main.c:408-495 for shot 0 of the fixtures, through launchPropagation /
    res_h / launchBackPropagation with the reference's buffer layout and aliasing."""
    from compat_shot import compat_gradient_shot
    res, _, g = compat_gradient_shot(L, NX, NZ, NT, CPML, DH, DT, G["ax"], G["bx"], G["az"], G["bz"], G["vh_i"],
                                     G["vp_i"], G["vn_i"], G["source"], int(G["shots_sx"][0]), SZ, G["obs"][0])
    assert np.array_equal(res, G["res"][0]), rel_l2(res, G["res"][0])
    assert L.fwi_compat_last_error() == 0
    for t, k in zip(g, ("gcx_shot0", "gcz_shot0", "gdx_shot0")):
        assert np.array_equal(t, G[k]), (k, rel_l2(t, G[k]))
