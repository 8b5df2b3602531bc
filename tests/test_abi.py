"""The C-ABI library: loads without a GPU, exports every symbol the headers
declare, and its host-side logic (strip enumeration, configuration checks)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import fwi_gb300
from fwi_gb300 import native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DECL = re.compile(r"^(?:void|int|long|size_t|const char\s*\*)\s*\**\s*([A-Za-z_]\w*)\s*\(", re.M)


def header_symbols():
    out = {}
    for h in ("fwi.h", "fwi_compat.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        out[h] = sorted(set(DECL.findall(text)))
    return out


@pytest.fixture(scope="module")
def built():
    from fwi_gb300 import build
    build.build()
    return native.lib()


def test_headers_declare_the_reference_surface():
    syms = header_symbols()
    assert set(native.COMPAT_SYMBOLS) <= set(syms["fwi_compat.h"])
    assert len(native.COMPAT_SYMBOLS) == 17  # include/serialcalls.h:9-31 of the reference


def test_library_exports_every_declared_symbol(built):
    out = subprocess.run(["nm", "-D", "--defined-only", native.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    for h, syms in header_symbols().items():
        missing = [s for s in syms if s not in exported]
        assert not missing, f"{h}: not exported: {missing}"
    for s in sum(header_symbols().values(), []):
        assert hasattr(built, s)


def test_build_targets_sm_103a_only():
    from fwi_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


@pytest.mark.parametrize("nx,nz,cpml", [(64, 48, 10), (201, 201, 20), (49, 29, 20), (30, 30, 4),
                                        (40, 30, 2), (609, 309, 20), (12, 12, 20)])
def test_strip_points_match_the_reference_predicate(built, nx, nz, cpml):
    ix, iz = fwi_gb300.strip_points(nx, nz, cpml)
    want = {(x, z) for z in range(nz) for x in range(nx)
            if 3 < x < nx - 4 and 3 < z < nz - 4 and (x < cpml or x > nx - cpml - 1 or z > nz - cpml - 1)}
    got = list(zip(ix.tolist(), iz.tolist()))
    assert len(got) == len(set(got)) == len(want)
    assert set(got) == want


def test_config_defaults_and_bytes(built):
    cfg = native.Config()
    built.fwi_config_default(C.byref(cfg))
    assert (cfg.nx, cfg.nz, cfg.cpml, cfg.vmax) == (201, 201, 20, 6000.0)
    b1 = built.fwi_config_bytes(C.byref(cfg))
    cfg.max_shots = 4
    b4 = built.fwi_config_bytes(C.byref(cfg))
    cfg.store_prec = native.SPREC_FP16
    b4h = built.fwi_config_bytes(C.byref(cfg))
    assert b1 < b4 and b4h < b4
    # long records: checkpoints and boundary rings need far less than every step's images
    cfg.nt_max = 6000
    full = built.fwi_config_bytes(C.byref(cfg))
    cfg.store = native.STORE_CHECKPOINT
    ckpt = built.fwi_config_bytes(C.byref(cfg))
    cfg.store = native.STORE_BOUNDARY
    ring = built.fwi_config_bytes(C.byref(cfg))
    assert ckpt < full / 4 and ring < full / 4


def test_invalid_configuration_is_rejected_before_any_device_call(built):
    for bad in (dict(nx=20), dict(cpml=-1), dict(nt_max=0), dict(max_shots=0), dict(mode=7),
                dict(max_window=10_000), dict(ckpt_every=-1), dict(device=-1)):
        with pytest.raises(native.FwiError) as e:
            native.Context(**bad)
        assert e.value.status == native.FWI_ERR_ARG


def test_strerror_covers_every_status(built):
    for s in range(0, -8, -1):
        assert built.fwi_strerror(s).decode() != "unknown status"


def test_checkpoint_interval_trades_memory_for_recompute(built):
    """The automatic interval (0) is the memory-minimal one (checkpoints + the two-segment image
    buffer, within the rounding of the segment count); a longer one costs memory in proportion.
    C2 batch: 609 x 309 grid, nt 3000, 32 shots, FP16 images."""
    def gb(k):
        cfg = native.Config()
        built.fwi_config_default(C.byref(cfg))
        cfg.nx, cfg.nz, cfg.dh, cfg.dt, cfg.cpml, cfg.f_cpml = 609, 309, 10.0, 0.001, 20, 8.0
        cfg.nt_max, cfg.max_shots, cfg.max_window, cfg.max_receivers = 3000, 32, 609, 601
        cfg.mode, cfg.store, cfg.store_prec = native.MODE_EXACT, native.STORE_CHECKPOINT, native.SPREC_FP16
        cfg.ckpt_every = k
        return built.fwi_config_bytes(C.byref(cfg)) / 1e9

    auto = gb(0)
    assert auto == gb(110)  # ceil(sqrt(8 nt / (4 * 0.5)))
    assert auto <= 1.01 * min(gb(k) for k in range(20, 400))
    assert auto < gb(375) < gb(750) < gb(3000)
    assert round(auto, 1) == 12.4 and round(gb(375), 1) == 21.8 and round(gb(750), 1) == 39.9
