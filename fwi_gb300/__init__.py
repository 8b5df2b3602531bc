"""GB300-native (sm_103a) 2-D pseudo-acoustic VTI FWI gradient path.

The product is the shared library fwi_gb300/lib/libfwi_gb300.so (CUDA
kernels behind two C-ABIs: include/fwi.h and include/fwi_compat.h).  This
package holds its build recipe (`fwi_gb300.build`), ctypes bindings
(`fwi_gb300.native`) and the seeded synthetic workloads (`fwi_gb300.synth`).
"""
from .native import (Context, FwiError, Shot, lib, make_shots, ptr, strip_points,  # noqa: F401
                     MODE_EXACT, MODE_REF_COMPAT, PREC_FP32, PREC_FP64, SPREC_BF16,
                     SPREC_FP16, SPREC_NATIVE, STORE_BOUNDARY, STORE_CHECKPOINT, STORE_FULL)
