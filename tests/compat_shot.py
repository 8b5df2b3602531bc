"""One shot sequenced as src/main.c:408-495 does it, through the
reference-compatible C-ABI (launchPropagation, res_h, launchBackPropagation)
with the reference's buffer layout: one 2 nx nz allocation per time level
(F = P + nx nz), the time levels swapped by the caller, the adjoint's CPML
arrays aliasing the forward's (src/main.c:162-193), the forward snapshots in
pinned host memory.  Shared by the GPU parity tests."""
import ctypes as C

import numpy as np


def _blocking_stream():
    for name in ("libcudart.so", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            rt = C.CDLL(name)
            s = C.c_void_p()
            if rt.cudaStreamCreate(C.byref(s)) == 0:
                return rt, s.value
        except OSError:
            continue
    return None, 0


def compat_gradient_shot(L, nx, nz, nt, cpml, dh, dt, ax, bx, az, bz, vh, vp, vn, source, sx, sz, obs):
    """Returns (res [nt, nx], synthetic traces [nt, nx], (gcx, gcz, gdx) [nz, nx]); sx, sz are
    the reference's 1-based source coordinates, obs the observed shot record [nt, nx]."""
    import torch

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()

    def zeros(k):
        return torch.zeros(k, dtype=torch.float32, device="cuda")

    def P(t):
        return t.data_ptr()

    rt, s1 = _blocking_stream()
    _, s2 = _blocking_stream()
    n = nx * nz
    # C = (dt * dt) / dh2 in FP32 operations, as src/main.c:55 forms it from float dt and dh
    f32 = np.float32
    dh2 = f32(f32(dh) * f32(dh))
    C_ = float(f32(f32(dt) * f32(dt)) / dh2)
    a_x, b_x, a_z, b_z = (dev(a) for a in (ax, bx, az, bz))
    v_hor, v_po, v_nmo = dev(vh), dev(vp), dev(vn)
    src = dev(source)
    lvlA, lvlB, pre2 = zeros(2 * n), zeros(2 * n), zeros(2 * n)
    PF, p2, r2 = zeros(n), zeros(n), zeros(n)
    psi_px, psi_fz, z_px, z_fz, aten_p, aten_f = (zeros(n) for _ in range(6))
    shot1 = dev(obs)
    shot2, Res = zeros(nt * nx), zeros(nt * nx)
    PF_h = torch.zeros(nt * 2 * n, dtype=torch.float32).pin_memory()
    f4 = 4
    P_pre, P_past = lvlA, lvlB
    for it in range(nt):
        L.launchPropagation(s1, s2, PF_h.data_ptr() + 2 * it * n * f4, P(PF), P(P_past), P(P_pre),
                            P(P_past) + n * f4, P(P_pre) + n * f4, P(p2), P(r2), float(dh2), nx, nz,
                            P(a_x), P(b_x), P(a_z), P(b_z), P(psi_px), P(psi_fz), dh, cpml, P(z_px),
                            P(z_fz), P(aten_p), P(aten_f), P(v_hor), P(v_po), P(v_nmo), P(src),
                            P(shot2), C_, sx, sz, it)
        P_pre, P_past = P_past, P_pre
    L.res_h(P(Res), P(shot1), P(shot2), nx, nt)
    torch.cuda.synchronize()
    res = Res.cpu().numpy().reshape(nt, nx)
    syn = shot2.cpu().numpy().reshape(nt, nx)

    for t in (lvlA, lvlB, psi_px, psi_fz, z_px, z_fz, aten_p, aten_f):
        t.zero_()
    psixcx, psixcz, atenxcx, atenxcz, atenzdx, atenzcz = (zeros(n) for _ in range(6))
    aux = [zeros(n) for _ in range(4)]
    p2c = [zeros(n) for _ in range(4)]
    g = [zeros(n) for _ in range(3)]
    P_pre, P_past = lvlA, lvlB
    for it in range(nt):
        L.launchBackPropagation(s1, s2, nx, nz, nt, PF_h.data_ptr() + (nt - it - 1) * n * 2 * f4, P(P_pre),
                                P(P_past), P(P_pre) + n * f4, P(P_past) + n * f4, *[P(a) for a in aux],
                                P(v_hor), P(v_po), P(v_nmo), *[P(a) for a in p2c], float(dh2), P(pre2),
                                P(pre2) + n * f4, P(a_x), P(b_x), P(a_z), P(b_z), P(psixcx), P(psixcz),
                                P(psi_px), P(psi_fz), dh, cpml, P(z_px), P(z_fz), P(aten_f), P(aten_p),
                                P(atenxcx), P(atenxcz), P(atenzdx), P(atenzcz), P(Res), C_, P(PF), it, sx,
                                sz, dt, P(g[0]), P(g[1]), P(g[2]))
        P_pre, P_past = P_past, P_pre
    torch.cuda.synchronize()
    grads = tuple(t.cpu().numpy().reshape(nz, nx) for t in g)
    if rt is not None:
        rt.cudaStreamDestroy(C.c_void_p(s1))
        rt.cudaStreamDestroy(C.c_void_p(s2))
    return res, syn, grads
