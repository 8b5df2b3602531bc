"""ctypes bindings of libfwi_gb300.so: the native ABI (include/fwi.h) and the
reference-compatible ABI (include/fwi_compat.h).

Array arguments are anything exposing a data pointer: numpy arrays (host) or
torch tensors (host or CUDA; `data_ptr()`).  The library detects host versus
device memory per call.  There is no fallback: if the shared library is not
built, `lib()` raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libfwi_gb300.so")

FWI_OK = 0
FWI_ERR_ARG = -1
FWI_ERR_CUDA = -2
FWI_ERR_NOMEM = -3
FWI_ERR_STATE = -4
FWI_ERR_NUMERIC = -5
FWI_ERR_UNSUPPORTED = -6
FWI_ERR_NODEVICE = -7

MODE_REF_COMPAT, MODE_EXACT = 0, 1
PREC_FP32, PREC_FP64 = 0, 1
STORE_FULL, STORE_CHECKPOINT, STORE_BOUNDARY = 0, 1, 2
SPREC_NATIVE, SPREC_FP16, SPREC_BF16 = 0, 1, 2

COMPAT_SYMBOLS = [
    "pre_variables_h", "CPML_x_h", "CPML_z_h", "PSI_F_h", "ZETA_F_h", "propagator_F_h", "res_h",
    "SecondDerivate_P_h", "launchPropagation", "launchBackPropagation", "NORMAL_h", "UpdateModel_h",
    "compute_sy_h", "compute_qi_h", "compute_ri_h", "update_r_h", "update_LBFGS_h",
]


class FwiError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        msg = lib().fwi_strerror(status).decode() if _LIB is not None else str(status)
        super().__init__(f"{what}: {msg} ({status})")


class Config(C.Structure):
    _fields_ = [("nx", C.c_int), ("nz", C.c_int), ("dh", C.c_float), ("dt", C.c_float),
                ("cpml", C.c_int), ("f_cpml", C.c_float), ("vmax", C.c_float), ("r_coef", C.c_float),
                ("nt_max", C.c_int), ("max_shots", C.c_int), ("max_window", C.c_int),
                ("max_receivers", C.c_int), ("mode", C.c_int), ("precision", C.c_int),
                ("store", C.c_int), ("store_prec", C.c_int), ("ckpt_every", C.c_int),
                ("device", C.c_int)]


class InvertOpts(C.Structure):
    _fields_ = [("iterations", C.c_int), ("lbfgs_m", C.c_int), ("first_alpha", C.c_float * 3),
                ("alpha0", C.c_float), ("max_halvings", C.c_int), ("reset_alpha", C.c_int),
                ("flag_min", C.c_int), ("flag_max", C.c_int), ("armijo_c1", C.c_double),
                ("curvature_guard", C.c_int)]


class PhaseChoice(C.Structure):
    _fields_ = [("shots_per_group", C.c_int), ("layer_shots_per_group", C.c_int), ("inline_strip", C.c_int)]


class Tuning(C.Structure):
    _fields_ = [("forward", PhaseChoice), ("adjoint", PhaseChoice), ("trials", C.c_int),
                ("forward_us", C.c_double), ("adjoint_us", C.c_double),
                ("default_forward_us", C.c_double), ("default_adjoint_us", C.c_double)]


# int (*)(void *user, int band, float f, const void **obs)
BandObsFn = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_float, C.POINTER(C.c_void_p))


class Shot(C.Structure):
    _fields_ = [("sx", C.c_int), ("sz", C.c_int), ("rz", C.c_int), ("rx0", C.c_int),
                ("rx1", C.c_int), ("nt", C.c_int), ("x0", C.c_int), ("nxw", C.c_int)]

    @property
    def nrec(self):
        return self.rx1 - self.rx0


_LIB = None
_p, _i, _f, _d, _l = C.c_void_p, C.c_int, C.c_float, C.c_double, C.c_long


def _sig(L, name, args, res=_i):
    fn = getattr(L, name)
    fn.argtypes = args
    fn.restype = res


def lib() -> C.CDLL:
    """Load the library (built by fwi_gb300.build / __graft_entry__.build)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is not built; run `python -m fwi_gb300.build`")
        L = C.CDLL(LIB_PATH)
        cfgp, shotp = C.POINTER(Config), C.POINTER(Shot)
        _sig(L, "fwi_config_default", [cfgp], None)
        _sig(L, "fwi_config_bytes", [cfgp], C.c_size_t)
        _sig(L, "fwi_create", [cfgp, C.POINTER(_p)])
        _sig(L, "fwi_destroy", [_p], None)
        _sig(L, "fwi_strerror", [_i], C.c_char_p)
        _sig(L, "fwi_last_cuda_error", [_p])
        _sig(L, "fwi_set_model", [_p, _p, _p, _p])
        _sig(L, "fwi_set_model_vti", [_p, _p, _p, _p])
        _sig(L, "fwi_get_model", [_p, _p, _p, _p])
        _sig(L, "fwi_set_wavelet", [_p, _p, _i])
        _sig(L, "fwi_set_ricker", [_p, _f, _i])
        _sig(L, "fwi_forward", [_p, shotp, _i, _p])
        _sig(L, "fwi_gradient", [_p, shotp, _i, _p, _p, _p, _p, _p, C.POINTER(_d)])
        _sig(L, "fwi_misfit", [_p, shotp, _i, _p, _p, C.POINTER(_d)])
        _sig(L, "fwi_set_gradient", [_p, _p, _p, _p])
        _sig(L, "fwi_first_step", [_p, _f, _f, _f])
        _sig(L, "fwi_lbfgs_direction", [_p, _i, _p])
        _sig(L, "fwi_lbfgs_update", [_p, _f, _f, _f, _i, _i])
        _sig(L, "fwi_restore_model", [_p])
        _sig(L, "fwi_gradient_vti", [_p, _p, _p, _p])
        _sig(L, "fwi_last_timing", [_p, _p])
        _sig(L, "fwi_set_tile_timing", [_p, _i])
        _sig(L, "fwi_last_tile_timing", [_p, _p])
        _sig(L, "fwi_last_recompute_timing", [_p, _p])
        _sig(L, "fwi_last_launches", [_p], _l)
        _sig(L, "fwi_autotune", [_p, shotp, _i, _i, C.POINTER(Tuning)])
        _sig(L, "fwi_set_tuning", [_p, shotp, _i, C.POINTER(Tuning)])
        _sig(L, "fwi_check_bounded_wait", [_p, _l])
        _sig(L, "fwi_set_graphs", [_p, _i])
        _sig(L, "fwi_graph_stats", [_p, _p])
        _sig(L, "fwi_strip_points", [_i, _i, _i, _p, _p, _l], _l)
        _sig(L, "fwi_residual_misfit_noalloc", [_p, _p, _p, _p, _l, _i, _p, _p])
        _sig(L, "fwi_invert_defaults", [C.POINTER(InvertOpts)], None)
        _sig(L, "fwi_invert", [_p, shotp, _i, _p, _p, C.POINTER(InvertOpts), _p, C.POINTER(_i)])
        _sig(L, "fwi_invert_bands", [_p, shotp, _i, _p, _f, _f, _i, _i, BandObsFn, _p, C.POINTER(InvertOpts), _i,
                                     _p, _p])
        _sig(L, "fwi_direction_slope", [_p, _p])
        _sig(L, "fwi_set_lbfgs_guard", [_p, _i])
        _sig(L, "fwi_store_observed", [_p, shotp, _i, _p, _i])
        _sig(L, "fwi_model_observed", [_p, shotp, _i, _p, _p, _p, _i])
        _sig(L, "fwi_free_observed", [_p])
        _sig(L, "fwi_load_model_files", [_p, C.c_char_p, C.c_char_p, C.c_char_p])
        _sig(L, "fwi_save_model_files", [_p, C.c_char_p, C.c_char_p, C.c_char_p])
        _sig(L, "fwi_set_frequency", [_p, _f, _i])
        # reference-compatible ABI: float* device pointers, ints, floats
        _sig(L, "pre_variables_h", [_p] * 6 + [_i, _i], None)
        _sig(L, "CPML_x_h", [_p, _p, _i, _f, _i, _f, _f, _f, _f, _f], None)
        _sig(L, "CPML_z_h", [_p, _p, _i, _f, _i, _f, _f, _f, _f, _f], None)
        _sig(L, "PSI_F_h", [_p] * 8 + [_i, _i, _f, _i], None)
        _sig(L, "ZETA_F_h", [_p] * 14 + [_i, _i, _f, _f, _i], None)
        _sig(L, "propagator_F_h", [_p] * 14 + [_f, _f] + [_i] * 6, None)
        _sig(L, "res_h", [_p] * 3 + [_i, _i], None)
        _sig(L, "SecondDerivate_P_h", [_p] * 4 + [_f, _i, _i], None)
        _sig(L, "launchPropagation", [_p] * 10 + [_f, _i, _i] + [_p] * 6 + [_f, _i] + [_p] * 9 +
             [_f, _i, _i, _i], None)
        _sig(L, "launchBackPropagation", [_p, _p, _i, _i, _i] + [_p] * 16 + [_f] + [_p] * 10 +
             [_f, _i] + [_p] * 9 + [_f, _p, _i, _i, _i, _f, _p, _p, _p], None)
        _sig(L, "NORMAL_h", [_p] * 3 + [_i, _i, _f, _f, _f], None)
        _sig(L, "UpdateModel_h", [_p] * 6 + [_f, _f, _f, _i, _i], None)
        _sig(L, "compute_sy_h", [_p] * 18 + [_i, _i, _i], None)
        _sig(L, "compute_qi_h", [_p] * 6 + [_f, _f, _f, _i, _i, _i], None)
        _sig(L, "compute_ri_h", [_p] * 6 + [_f, _f, _f, _i, _i], None)
        _sig(L, "update_r_h", [_p] * 6 + [_f] * 6 + [_i, _i, _i], None)
        _sig(L, "update_LBFGS_h", [_p] * 9 + [_i, _i, _f, _f, _f] + [_i] * 5, None)
        _sig(L, "fwi_compat_last_error", [])
        _LIB = L
    return _LIB


def ptr(x):
    """Raw address of an array-like (numpy, torch) or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        if not x.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous")
        return x.ctypes.data
    raise TypeError(f"cannot take the address of {type(x)}")


def _check(status, what):
    if status != FWI_OK:
        raise FwiError(status, what)


def make_shots(specs):
    """Shot array from dicts / tuples (sx, sz, rz, rx0, rx1, nt[, x0, nxw])."""
    arr = (Shot * len(specs))()
    for k, s in enumerate(specs):
        if isinstance(s, dict):
            vals = [s.get(n, 0) for n, _ in Shot._fields_]
        else:
            vals = list(s) + [0] * (8 - len(s))
        for (n, _), v in zip(Shot._fields_, vals):
            setattr(arr[k], n, int(v))
    return arr


def strip_points(nx, nz, cpml):
    """(ix, iz) of the CPML strip points, in the strip kernels' order (host only)."""
    L = lib()
    n = L.fwi_strip_points(nx, nz, cpml, None, None, 0)
    ix = np.zeros(max(n, 1), np.int32)
    iz = np.zeros(max(n, 1), np.int32)
    L.fwi_strip_points(nx, nz, cpml, ix.ctypes.data, iz.ctypes.data, n)
    return ix[:n], iz[:n]


def _checked(x, dtype, size, what):
    """Host numpy arrays must have the context's element type and at least `size` elements."""
    if isinstance(x, np.ndarray):
        if x.dtype != dtype:
            raise TypeError(f"{what}: dtype {x.dtype}, the context computes in {np.dtype(dtype)}")
        if x.size < size:
            raise ValueError(f"{what}: {x.size} elements, {size} needed")
        if not x.flags.c_contiguous:
            raise ValueError(f"{what}: not C-contiguous")
    elif hasattr(x, "dtype") and hasattr(x, "numel"):
        want = "torch.float64" if np.dtype(dtype) == np.float64 else "torch.float32"
        if str(x.dtype) != want and what != "mask":
            raise TypeError(f"{what}: dtype {x.dtype}, expected {want}")
        if x.numel() < size:
            raise ValueError(f"{what}: {x.numel()} elements, {size} needed")
    return x


class Context:
    """One native context (include/fwi.h)."""

    def __init__(self, **kw):
        L = lib()
        cfg = Config()
        L.fwi_config_default(C.byref(cfg))
        for k, v in kw.items():
            if not hasattr(cfg, k):
                raise TypeError(f"unknown config field {k}")
            setattr(cfg, k, v)
        self.cfg = cfg
        self.dtype = np.float64 if cfg.precision == PREC_FP64 else np.float32
        h = _p()
        _check(L.fwi_create(C.byref(cfg), C.byref(h)), "fwi_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().fwi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def _grid(self, *arrays, what="model"):
        n = self.cfg.nx * self.cfg.nz
        return [_checked(a, self.dtype, n, what) for a in arrays]

    def set_model(self, vh, vp, vn):
        vh, vp, vn = self._grid(vh, vp, vn)
        _check(lib().fwi_set_model(self._h, ptr(vh), ptr(vp), ptr(vn)), "fwi_set_model")

    def set_model_vti(self, vel, eps, delta):
        vel, eps, delta = self._grid(vel, eps, delta)
        _check(lib().fwi_set_model_vti(self._h, ptr(vel), ptr(eps), ptr(delta)), "fwi_set_model_vti")

    def get_model(self):
        out = [np.zeros((self.cfg.nz, self.cfg.nx), self.dtype) for _ in range(3)]
        _check(lib().fwi_get_model(self._h, *[ptr(o) for o in out]), "fwi_get_model")
        return out

    def set_wavelet(self, w):
        w = np.ascontiguousarray(w, self.dtype) if isinstance(w, np.ndarray) else w
        _checked(w, self.dtype, len(w), "wavelet")
        _check(lib().fwi_set_wavelet(self._h, ptr(w), len(w)), "fwi_set_wavelet")

    def set_frequency(self, f, nt):
        _check(lib().fwi_set_frequency(self._h, float(f), int(nt)), "fwi_set_frequency")

    def invert(self, shots, obs, mask=None, **opts):
        """One band of the reference's inversion loop in the C driver; returns the misfits."""
        o = InvertOpts()
        lib().fwi_invert_defaults(C.byref(o))
        for k, v in opts.items():
            if k == "first_alpha":
                o.first_alpha[:] = list(v)
            else:
                setattr(o, k, v)
        self._inputs(shots, obs, mask)
        hist = np.zeros(o.iterations, np.float64)  # obs None: the records kept on the device
        done = C.c_int(0)
        _check(lib().fwi_invert(self._h, shots, len(shots), ptr(obs), ptr(mask), C.byref(o),
                                hist.ctypes.data, C.byref(done)), "fwi_invert")
        return hist[: done.value]

    def invert_bands(self, shots, band_obs, f0, df, nbands, nt, mask=None, restart_model=False, **opts):
        """Multiscale loop of the C driver; band_obs(band, f) returns that band's observed
        data (host or device array).  Returns the misfits of each band."""
        o = InvertOpts()
        lib().fwi_invert_defaults(C.byref(o))
        for k, v in opts.items():
            if k == "first_alpha":
                o.first_alpha[:] = list(v)
            else:
                setattr(o, k, v)
        keep = []

        def cb(user, band, f, out):
            try:
                d = band_obs(band, float(f))
                if isinstance(d, np.ndarray):
                    d = np.ascontiguousarray(d, self.dtype)
                keep.append(d)
                out[0] = C.c_void_p(ptr(d))
                return 0
            except Exception:  # noqa: BLE001 - reported to the driver as a failed band
                return 1

        fn = BandObsFn(cb)
        if mask is not None:
            mask = np.ascontiguousarray(mask, np.uint8)
        hist = np.zeros(nbands * o.iterations, np.float64)
        done = np.zeros(nbands, np.int32)
        _check(lib().fwi_invert_bands(self._h, shots, len(shots), ptr(mask), float(f0), float(df), int(nbands),
                                      int(nt), fn, None, C.byref(o), 1 if restart_model else 0,
                                      hist.ctypes.data, done.ctypes.data), "fwi_invert_bands")
        return [hist[b * o.iterations: b * o.iterations + done[b]] for b in range(nbands)]

    def set_lbfgs_guard(self, on=True):
        """Skip history pairs without positive curvature in later L-BFGS directions."""
        _check(lib().fwi_set_lbfgs_guard(self._h, 1 if on else 0), "fwi_set_lbfgs_guard")

    def direction_slope(self):
        out = np.zeros(3, np.float64)
        _check(lib().fwi_direction_slope(self._h, out.ctypes.data), "fwi_direction_slope")
        return out

    def load_model_files(self, vp_path, eps_path, delta_path):
        _check(lib().fwi_load_model_files(self._h, *(os.fsencode(p) for p in (vp_path, eps_path, delta_path))),
               "fwi_load_model_files")

    def save_model_files(self, vh_path, vp_path, vn_path):
        _check(lib().fwi_save_model_files(self._h, *(os.fsencode(p) for p in (vh_path, vp_path, vn_path))),
               "fwi_save_model_files")

    def set_ricker(self, f, nt):
        _check(lib().fwi_set_ricker(self._h, float(f), int(nt)), "fwi_set_ricker")

    def forward(self, shots, out=None):
        n = sum(s.nt * s.nrec for s in shots)
        if out is None:
            out = np.zeros(n, self.dtype)
        _checked(out, self.dtype, n, "traces")
        _check(lib().fwi_forward(self._h, shots, len(shots), ptr(out)), "fwi_forward")
        return out

    def gradient(self, shots, obs, mask=None, out=None):
        """Returns (misfit, g_vh, g_vp, g_vn); `out` may give three destination arrays."""
        if out is None:
            out = [np.zeros((self.cfg.nz, self.cfg.nx), self.dtype) for _ in range(3)]
        self._grid(*out, what="gradient")
        self._inputs(shots, obs, mask)
        J = C.c_double(0)
        _check(lib().fwi_gradient(self._h, shots, len(shots), ptr(obs), ptr(mask),
                                  *[ptr(o) for o in out], C.byref(J)), "fwi_gradient")
        return (J.value, *out)

    def _inputs(self, shots, obs, mask):
        if obs is not None:  # None: the records kept on the device (store_observed / model_observed)
            _checked(obs, self.dtype, sum(s.nt * s.nrec for s in shots), "obs")
        if mask is not None:
            _checked(mask, np.uint8, sum(s.nrec for s in shots), "mask")

    def misfit(self, shots, obs, mask=None):
        self._inputs(shots, obs, mask)
        J = C.c_double(0)
        _check(lib().fwi_misfit(self._h, shots, len(shots), ptr(obs), ptr(mask), C.byref(J)),
               "fwi_misfit")
        return J.value

    def store_observed(self, shots, obs, store_prec=0):
        """Keep these shots' records on the device (FP32, or FP16 with per-trace scales)."""
        self._inputs(shots, obs, None)
        _check(lib().fwi_store_observed(self._h, shots, len(shots), ptr(obs), int(store_prec)), "fwi_store_observed")

    def model_observed(self, shots, vh, vp, vn, store_prec=0):
        """Model these shots' records on the device from (vh, vp, vn) into the store."""
        vh, vp, vn = self._grid(vh, vp, vn)
        _check(lib().fwi_model_observed(self._h, shots, len(shots), ptr(vh), ptr(vp), ptr(vn), int(store_prec)),
               "fwi_model_observed")

    def free_observed(self):
        _check(lib().fwi_free_observed(self._h), "fwi_free_observed")

    def set_gradient(self, gh, gp, gn):
        gh, gp, gn = self._grid(gh, gp, gn, what="gradient")
        _check(lib().fwi_set_gradient(self._h, ptr(gh), ptr(gp), ptr(gn)), "fwi_set_gradient")

    def first_step(self, a_hor, a_po, a_nmo):
        _check(lib().fwi_first_step(self._h, a_hor, a_po, a_nmo), "fwi_first_step")

    def lbfgs_direction(self, m=5):
        st = np.zeros(12, np.float64)
        _check(lib().fwi_lbfgs_direction(self._h, m, st.ctypes.data), "fwi_lbfgs_direction")
        return st

    def lbfgs_update(self, av, ad, ae, flag_min=0, flag_max=0):
        _check(lib().fwi_lbfgs_update(self._h, av, ad, ae, flag_min, flag_max), "fwi_lbfgs_update")

    def restore_model(self):
        _check(lib().fwi_restore_model(self._h), "fwi_restore_model")

    def gradient_vti(self):
        out = [np.zeros((self.cfg.nz, self.cfg.nx), self.dtype) for _ in range(3)]
        _check(lib().fwi_gradient_vti(self._h, *[ptr(o) for o in out]), "fwi_gradient_vti")
        return out

    def last_timing(self):
        t = np.zeros(4, np.float32)
        _check(lib().fwi_last_timing(self._h, t.ctypes.data), "fwi_last_timing")
        return t

    def last_cuda_error(self):
        """The cudaError_t of the last CUDA call that failed in this context (0: none)."""
        return int(lib().fwi_last_cuda_error(self._h))

    def last_launches(self):
        return int(lib().fwi_last_launches(self._h))

    def autotune(self, shots, steps=48):
        """Times candidate launch choices per batch shape of `shots` and keeps the fastest
        (fwi_autotune); returns the first batch's choice and step times."""
        t = Tuning()
        _check(lib().fwi_autotune(self._h, shots, len(shots), int(steps), C.byref(t)), "fwi_autotune")
        out = {f: getattr(t, f) for f, _ in Tuning._fields_}
        for ph in ("forward", "adjoint"):
            out[ph] = {f: getattr(out[ph], f) for f, _ in PhaseChoice._fields_}
        return out

    def set_tuning(self, shots, choice):
        """Records a launch choice ({"forward": {...}, "adjoint": {...}} as autotune returns) for the
        batch shapes of `shots`."""
        t = Tuning()
        for ph in ("forward", "adjoint"):
            for f, _ in PhaseChoice._fields_:
                setattr(getattr(t, ph), f, int(choice[ph][f]))
        _check(lib().fwi_set_tuning(self._h, shots, len(shots), C.byref(t)), "fwi_set_tuning")

    def check_bounded_wait(self, polls=64):
        """Status of fwi_check_bounded_wait (FWI_ERR_CUDA: the wait gave up and said so)."""
        return int(lib().fwi_check_bounded_wait(self._h, int(polls)))

    def set_graphs(self, on=True):
        """CUDA graph replay of repeated batch sections (on by default)."""
        _check(lib().fwi_set_graphs(self._h, 1 if on else 0), "fwi_set_graphs")

    def graph_stats(self):
        """(sections replayed, sections captured) since creation."""
        t = np.zeros(2, np.int64)
        _check(lib().fwi_graph_stats(self._h, t.ctypes.data), "fwi_graph_stats")
        return tuple(int(v) for v in t)

    def graph_replays(self):
        return self.graph_stats()[0]

    def set_tile_timing(self, on=True):
        _check(lib().fwi_set_tile_timing(self._h, 1 if on else 0), "fwi_set_tile_timing")

    def last_tile_timing(self):
        """(forward ms, forward points, adjoint ms, adjoint points) per interior tile launch."""
        t = np.zeros(4, np.float64)
        _check(lib().fwi_last_tile_timing(self._h, t.ctypes.data), "fwi_last_tile_timing")
        return t

    def last_recompute_timing(self):
        """(ms, points) per interior tile launch of the checkpoint segment recompute, and the forward
        steps the last call recomputed."""
        t = np.zeros(3, np.float64)
        _check(lib().fwi_last_recompute_timing(self._h, t.ctypes.data), "fwi_last_recompute_timing")
        return t
