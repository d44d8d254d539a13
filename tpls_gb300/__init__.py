"""tpls_gb300 -- GB300 (sm_103a) implementation of the TPLS per-timestep hot
path behind a C ABI (include/tpls_gpu.h) that mirrors the reference's
Fortran subroutine interfaces.

The compute path is the native library tpls_gb300/_lib/libtpls_gb300.so;
there is no CPU fallback.
"""
from .api import (F, FIELD_KIND, STATE_FIELDS, Params, TplsError, TplsGpu, base_profile, load_library,
                  shape_of)

__all__ = ["F", "FIELD_KIND", "STATE_FIELDS", "Params", "TplsError", "TplsGpu", "base_profile",
           "load_library", "shape_of"]
