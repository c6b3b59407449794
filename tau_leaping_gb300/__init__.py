"""GB300-native tau-leaping engine for StochKit reaction networks.

The engine is libtl.so (CUDA kernels for sm_103a behind the C ABI declared
in include/tl.h); this package is its Python binding plus the build recipe.
"""
from . import _ffi
from ._ffi import (FLAG_COMPAT_REFERENCE, FLAG_KEEP_SAMPLES, FLAG_SENSITIVITY, VARIANT_AUTO, VARIANT_CTA,
                   VARIANT_PLAIN, VARIANT_THREAD, VARIANT_WARP, TLError)
from .model import Model, SimResult, philox, poisson

__all__ = ["Model", "SimResult", "philox", "poisson", "TLError", "VARIANT_AUTO", "VARIANT_THREAD",
           "VARIANT_WARP", "VARIANT_CTA", "VARIANT_PLAIN", "FLAG_KEEP_SAMPLES", "FLAG_SENSITIVITY",
           "FLAG_COMPAT_REFERENCE", "_ffi"]
