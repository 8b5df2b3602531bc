"""ctypes bindings of the CPU oracle (test infrastructure only).

Only tests/, the smoke check in __graft_entry__.py and bench.py's CPU
baseline / reference arm import this module, to check results against it or
to time it as the CPU baseline.  The product library never does.

`lib()` loads oracle/liboracle.so (the C restatement, vti_oracle.h), building
it with `make -C oracle` when it is missing.  `ref_lib()` loads
oracle/_ref/libref.so, the reference's own kernels compiled for the CPU, which
exists only where the reference sources were available at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

_i, _f, _d, _p = C.c_int, C.c_float, C.c_double, C.c_void_p


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and, with ref=True, _ref/libref.so)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_p)


def _sig(lib, name, args, res=None):
    fn = getattr(lib, name)
    fn.argtypes = args
    fn.restype = res
    return fn


def _declare(lib, prefix, suffix, real):
    r = real
    s = suffix
    _sig(lib, f"{prefix}pre_variables{s}", [_p] * 6 + [_i, _i])
    _sig(lib, f"{prefix}cpml_x{s}", [_p, _p, _i, r, _i, r, r, r, r, r])
    _sig(lib, f"{prefix}cpml_z{s}", [_p, _p, _i, r, _i, r, r, r, r, r])
    _sig(lib, f"{prefix}psi_f{s}", [_p] * 8 + [_i, _i, r, _i])
    _sig(lib, f"{prefix}zeta_f{s}", [_p] * 12 + [_i, _i, r, _i])
    _sig(lib, f"{prefix}second_derivate_p{s}", [_p] * 4 + [r, _i, _i])
    _sig(lib, f"{prefix}propagator_f{s}", [_p] * 14 + [r, r] + [_i] * 6)
    _sig(lib, f"{prefix}res{s}", [_p] * 3 + [_i, _i])
    _sig(lib, f"{prefix}entry_point{s}", [_p] * 9 + [_i, _i])
    _sig(lib, f"{prefix}psi_r{s}", [_p] * 12 + [_i, _i, r, _i])
    _sig(lib, f"{prefix}second_derivate{s}", [_p] * 8 + [r, _i, _i])
    _sig(lib, f"{prefix}zeta_r{s}", [_p] * 20 + [_i, _i, r, _i])
    _sig(lib, f"{prefix}retro_propagation{s}", [_p] * 6 + [r, r] + [_i] * 6 + [_p] * 8)
    _sig(lib, f"{prefix}gradient{s}", [_p] * 7 + [r, r, _i, _i])
    _sig(lib, f"{prefix}normal{s}", [_p] * 3 + [_i, _i, r, r, r])
    _sig(lib, f"{prefix}update_model{s}", [_p] * 6 + [r, r, r, _i, _i])
    _sig(lib, f"{prefix}compute_sy{s}", [_p] * 18 + [_i, _i, _i])
    _sig(lib, f"{prefix}compute_qi{s}", [_p] * 6 + [r, r, r, _i, _i, _i])
    _sig(lib, f"{prefix}compute_ri{s}", [_p] * 6 + [r, r, r, _i, _i])
    _sig(lib, f"{prefix}update_r{s}", [_p] * 6 + [r] * 6 + [_i, _i, _i])
    _sig(lib, f"{prefix}update_lbfgs{s}", [_p] * 9 + [_i, _i, r, r, r] + [_i] * 5)
    _sig(lib, f"{prefix}forward_shot{s}", [_i] * 6 + [r, r] + [_p] * 10)
    _sig(lib, f"{prefix}gradient_shot{s}", [_i] * 6 + [r, r] + [_p] * 13 + [_i], r)
    _sig(lib, f"{prefix}lbfgs_direction{s}", [_i, _i, _i] + [_p] * 27)


def lib():
    """The restatement (liboracle.so), with argument types declared."""
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        for s, r in (("_f32", _f), ("_f64", _d)):
            _declare(L, "orc_", s, r)
            _sig(L, f"orc_host_misfit{s}", [_p, C.c_long], r)
            _sig(L, f"orc_host_norm{s}", [_p, C.c_long], r)
            _sig(L, f"orc_host_halfdot{s}", [_p, _p, C.c_long], r)
            _sig(L, f"orc_host_sy_yy{s}", [_p, _p, C.c_long, _p, _p])
            _sig(L, f"orc_ricker{s}", [_p, _i, r, r])
            _sig(L, f"orc_setup_cpml{s}", [_p] * 4 + [_i] * 3 + [r] * 5)
            _sig(L, f"orx_forward{s}", [_i] * 4 + [r, r] + [_p] * 7 + [_i, _i, _p, _i, _i, _i] + [_p] * 3 + [_i])
            _sig(L, f"orx_gradient_shot{s}",
                 [_i] * 4 + [r, r] + [_p] * 7 + [_i, _i, _p, _i, _i, _i, _p, _p, _i] + [_p] * 5, _d)
        _sig(L, "orc_set_threads", [_i])
        _sig(L, "orc_get_threads", [], _i)
        _LIB = L
    return _LIB


def ref_lib():
    """The reference's kernels compiled for the CPU (oracle/_ref/libref.so) or None."""
    global _REF
    if _REF is None:
        path = os.path.join(HERE, "_ref", "libref.so")
        if not os.path.exists(path):
            return None
        L = C.CDLL(path)
        _declare(L, "ref_", "", _f)
        _REF = L
    return _REF


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


# ----------------------------------------------------------------- helpers

def _sfx(dtype):
    return "_f32" if np.dtype(dtype) == np.float32 else "_f64"


def cpml_profiles(nx, nz, cpml, dh, dt, f, vmax=6000.0, R=1e-6, dtype=np.float32):
    """(a_x, b_x, a_z, b_z) as src/main.c:48-51, 276-279, 318-319 build them."""
    ax, bx = np.zeros(nx, dtype), np.zeros(nx, dtype)
    az, bz = np.zeros(nz, dtype), np.zeros(nz, dtype)
    getattr(lib(), "orc_setup_cpml" + _sfx(dtype))(
        _ptr(ax), _ptr(bx), _ptr(az), _ptr(bz), nx, nz, cpml, dh, dt, f, vmax, R)
    return ax, bx, az, bz


def ricker(nt, dt, f, dtype=np.float32):
    """Ricker wavelet of src/main.c:328-332."""
    s = np.zeros(nt, dtype)
    getattr(lib(), "orc_ricker" + _sfx(dtype))(_ptr(s), nt, dt, f)
    return s


def pre_variables(vel, eps, delta):
    """(v_hor, v_po, v_nmo) from (Vp, epsilon, delta), src/parallelcalls.cu:3-16."""
    dt = vel.dtype
    nz, nx = vel.shape
    vh, vp, vn = (np.zeros_like(vel) for _ in range(3))
    getattr(lib(), "orc_pre_variables" + _sfx(dt))(
        _ptr(vel), _ptr(eps), _ptr(delta), _ptr(vh), _ptr(vp), _ptr(vn), nx, nz)
    return vh, vp, vn


def forward_shot(prob, sx, sz, snap=False, library=None):
    """One shot as src/main.c models it.  prob: dict with nx, nz, nt, cpml, dh, dt,
    ax, bx, az, bz, vh, vp, vn, source (numpy arrays of one dtype).
    Returns (shot[nt, nx], snap[nt, 2, nz, nx] or None)."""
    dt_ = prob["vh"].dtype
    nx, nz, nt = prob["nx"], prob["nz"], prob["nt"]
    shot = np.zeros((nt, nx), dt_)
    sn = np.zeros((nt, 2, nz, nx), dt_) if snap else None
    fn = (getattr(library, "ref_forward_shot") if library is not None
          else getattr(lib(), "orc_forward_shot" + _sfx(dt_)))
    fn(nx, nz, nt, prob["cpml"], sx, sz, prob["dh"], prob["dt"],
       *[_ptr(prob[k]) for k in ("ax", "bx", "az", "bz", "vh", "vp", "vn", "source")],
       _ptr(shot), _ptr(sn))
    return shot, sn


def gradient_shot(prob, sx, sz, obs, nt_adj=None, library=None):
    """Misfit and reference gradient of one shot (src/main.c:408-495).
    Returns (fi, gcx, gcz, gdx, res)."""
    dt_ = prob["vh"].dtype
    nx, nz, nt = prob["nx"], prob["nz"], prob["nt"]
    g = [np.zeros((nz, nx), dt_) for _ in range(3)]
    res = np.zeros((nt, nx), dt_)
    fn = (getattr(library, "ref_gradient_shot") if library is not None
          else getattr(lib(), "orc_gradient_shot" + _sfx(dt_)))
    fi = fn(nx, nz, nt, prob["cpml"], sx, sz, prob["dh"], prob["dt"],
            *[_ptr(prob[k]) for k in ("ax", "bx", "az", "bz", "vh", "vp", "vn", "source")],
            _ptr(np.ascontiguousarray(obs, dt_)), *[_ptr(a) for a in g], _ptr(res),
            nt if nt_adj is None else nt_adj)
    return fi, g[0], g[1], g[2], res


def exact_forward(prob, sx, sz, rz, rx0, rx1, wavelet=None, images=False, exact=True):
    """Native-semantics forward: rec[nt, rx1-rx0] (+ G, H images [nt, nz, nx])."""
    dt_ = prob["vh"].dtype
    nx, nz, nt = prob["nx"], prob["nz"], prob["nt"]
    w = prob["source"] if wavelet is None else np.ascontiguousarray(wavelet, dt_)
    rec = np.zeros((nt, rx1 - rx0), dt_)
    G = np.zeros((nt, nz, nx), dt_) if images else None
    H = np.zeros((nt, nz, nx), dt_) if images else None
    getattr(lib(), "orx_forward" + _sfx(dt_))(
        nx, nz, nt, prob["cpml"], prob["dh"], prob["dt"],
        *[_ptr(prob[k]) for k in ("ax", "bx", "az", "bz", "vh", "vp", "vn")],
        sx, sz, _ptr(w), rz, rx0, rx1, _ptr(rec), _ptr(G), _ptr(H), 1 if exact else 0)
    return (rec, G, H) if images else rec


def exact_gradient(prob, sx, sz, rz, rx0, rx1, obs=None, mask=None, wavelet=None,
                   adjoint_source=None, want_adj_trace=False):
    """Misfit (FP64) and EXACT gradient (dJ/dv_hor, dJ/dv_po, dJ/dv_nmo) of one shot.
    With adjoint_source, back-propagates that [nt, nrec] field instead of the
    residual; with want_adj_trace, also returns the adjoint trace at the source."""
    dt_ = prob["vh"].dtype
    nx, nz, nt = prob["nx"], prob["nz"], prob["nt"]
    w = prob["source"] if wavelet is None else np.ascontiguousarray(wavelet, dt_)
    g = [np.zeros((nz, nx), dt_) for _ in range(3)]
    tr = np.zeros(nt, dt_) if want_adj_trace else None
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    J = getattr(lib(), "orx_gradient_shot" + _sfx(dt_))(
        nx, nz, nt, prob["cpml"], prob["dh"], prob["dt"],
        *[_ptr(prob[k]) for k in ("ax", "bx", "az", "bz", "vh", "vp", "vn")],
        sx, sz, _ptr(w), rz, rx0, rx1,
        _ptr(None if obs is None else np.ascontiguousarray(obs, dt_)), _ptr(m), 1,
        _ptr(g[0]), _ptr(g[1]), _ptr(g[2]), _ptr(tr),
        _ptr(None if adjoint_source is None else np.ascontiguousarray(adjoint_source, dt_)))
    out = (J, g[0], g[1], g[2])
    return out + (tr,) if want_adj_trace else out


def lbfgs_direction(state, k, library=None):
    """One two-loop direction as src/main.c:570-682 (m = 5).  `state` is a dict of
    float32 arrays (modified in place, as the reference's device buffers are):
    s_vp s_vn s_vh y_gcz y_gdx y_gcx [5, nz, nx]; v_po v_nmo v_hor back_vpo
    back_vnmo back_vhor gcz gdx gcx back_gcz back_gdx back_gcx q_gcz q_gdx q_gcx
    r_b1 r_b2 r_b3 [nz, nx].  Returns (sigma[3,5], epsilon[3,5], gamma[3])."""
    nz, nx = state["v_po"].shape
    sig = np.zeros((3, 5), np.float32)
    eps = np.zeros((3, 5), np.float32)
    gam = np.zeros(3, np.float32)
    names = ("s_vp s_vn s_vh y_gcz y_gdx y_gcx v_po v_nmo v_hor back_vpo back_vnmo back_vhor "
             "gcz gdx gcx back_gcz back_gdx back_gcx q_gcz q_gdx q_gcx r_b1 r_b2 r_b3").split()
    fn = (library.ref_lbfgs_direction if library is not None
          else lib().orc_lbfgs_direction_f32)
    fn(nx, nz, k, *[_ptr(state[n]) for n in names], _ptr(sig), _ptr(eps), _ptr(gam))
    return sig, eps, gam


# ----------------------------------------------------------------- the reference's kernels on the GPU

def ref_gpu_available() -> bool:
    """The reference's kernels compiled for sm_103a and their shot driver exist (oracle/_ref)."""
    return all(os.path.exists(os.path.join(HERE, "_ref", f)) for f in ("parallelcalls.cubin", "ref_gpu_shot"))


def ref_gpu_shot(vel, eps, delta, obs, nx, nz, nt, cpml, dh, dt, f, sx, sz, runs=1):
    """One shot of the reference's own CUDA kernels, sequenced as src/main.c:318-495
    (oracle/ref_gpu/ref_gpu_shot.cpp): model (Vp, epsilon, delta) [nz][nx] and the
    observed record [nt][nx] in, 1-based source (sx, sz).  Runs the shot `runs` times;
    returns (seconds per run, misfit, (gcx, gcz, gdx), res)."""
    import json
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        for name, a in (("vel", vel), ("eps", eps), ("delta", delta), ("obs", obs)):
            np.ascontiguousarray(a, np.float32).tofile(os.path.join(d, f"{name}.f32"))
        out = subprocess.run([os.path.join(HERE, "_ref", "ref_gpu_shot"), os.path.join(HERE, "_ref", "parallelcalls.cubin"),
                              d, str(nx), str(nz), str(nt), str(cpml), repr(float(dh)), repr(float(dt)),
                              repr(float(f)), str(sx), str(sz), str(runs)],
                             capture_output=True, text=True, check=True).stdout
        r = json.loads(out.strip().splitlines()[-1])
        g = tuple(np.fromfile(os.path.join(d, f"{k}.f32"), np.float32).reshape(nz, nx) for k in ("gcx", "gcz", "gdx"))
        res = np.fromfile(os.path.join(d, "res.f32"), np.float32).reshape(nt, nx)
    return r["seconds_per_shot"], r["misfit"], g, res
