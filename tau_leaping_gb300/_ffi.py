"""ctypes binding of libtl.so (include/tl.h).

This is the binding a Python caller of the C ABI writes; the tests and
bench.py drive the engine through it.  Loading fails loudly when the
library has not been built: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "libtl.so"

c_i32, c_u32, c_i64, c_u64, c_dbl, c_vp = C.c_int32, C.c_uint32, C.c_int64, C.c_uint64, C.c_double, C.c_void_p
P = C.POINTER

TL_OK = 0
STATUS = {
    0: "TL_OK", 1: "TL_ERR_INVALID_ARGUMENT", 2: "TL_ERR_INVALID_MODEL", 3: "TL_ERR_UNSUPPORTED",
    4: "TL_ERR_OVERFLOW", 5: "TL_ERR_STEP_CAP", 6: "TL_ERR_CUDA", 7: "TL_ERR_WAIT_TIMEOUT",
    8: "TL_ERR_NO_DEVICE", 9: "TL_ERR_OUT_OF_MEMORY", 10: "TL_ERR_IO", 11: "TL_ERR_PARSE",
    12: "TL_ERR_NUMERIC",
}

VARIANT_AUTO, VARIANT_THREAD, VARIANT_WARP, VARIANT_CTA, VARIANT_PLAIN = 0, 1, 2, 3, 4
VARIANT_LANES2, VARIANT_LANES4, VARIANT_LANES8, VARIANT_LANES16 = 5, 6, 7, 8
FLAG_SENSITIVITY = 1 << 0
FLAG_KEEP_SAMPLES = 1 << 1
FLAG_AUTOTUNE_MEASURE = 1 << 2
FLAG_NO_STAGE = 1 << 3
FLAG_GRAPH = 1 << 4
FLAG_GLOBAL_SLOTS = 1 << 5
FLAG_COMPAT_G = 1 << 8
FLAG_COMPAT_CRIT = 1 << 9
FLAG_COMPAT_STOICH = 1 << 10
FLAG_COMPAT_TAU2 = 1 << 11
FLAG_COMPAT_SSA = 1 << 12
FLAG_COMPAT_POISSON = 1 << 13
FLAG_COMPAT_REFERENCE = (FLAG_COMPAT_G | FLAG_COMPAT_CRIT | FLAG_COMPAT_STOICH | FLAG_COMPAT_TAU2 |
                         FLAG_COMPAT_SSA | FLAG_COMPAT_POISSON)
GEN_DIMER, GEN_TOY, GEN_CHAIN, GEN_COLLOID = 1, 2, 3, 4


class ModelDesc(C.Structure):
    _fields_ = [("n_species", c_i32), ("n_channels", c_i32), ("nnz", c_i32),
                ("x0", P(c_i64)), ("rate", P(c_dbl)), ("col_ptr", P(c_i32)), ("row_ind", P(c_i32)),
                ("stoich", P(C.c_int8)), ("pop_bits", c_i32)]


class ModelInfo(C.Structure):
    _fields_ = [("n_species", c_i32), ("n_channels", c_i32), ("nnz_raw", c_i32), ("nnz_net", c_i32),
                ("pop_bits", c_i32), ("max_order", c_i32)]


class GenParams(C.Structure):
    _fields_ = [("family", c_i32), ("n_species", c_i32), ("n_channels", c_i32), ("pop_bits", c_i32),
                ("x0_min", c_i64), ("x0_max", c_i64), ("rate_min", c_dbl), ("rate_max", c_dbl),
                ("rate_assoc", c_dbl), ("rate_dissoc", c_dbl), ("seed", c_u64)]


class RunCfg(C.Structure):
    _fields_ = [("t_final", c_dbl), ("eps", c_dbl), ("n_realizations", c_i64), ("seed", c_u64),
                ("n_intervals", c_i32), ("n_tracked", c_i32), ("tracked", P(c_i32)),
                ("n_rate_sets", c_i32), ("rate_sets", P(c_dbl)), ("t_final_sets", P(c_dbl)),
                ("variant", c_i32), ("block_threads", c_i32), ("flags", c_u32), ("n_critical", c_i32),
                ("ssa_factor", c_i32), ("ssa_block", c_i32), ("max_steps", c_i64), ("stream", c_vp),
                ("realization_offset", c_i64), ("max_halvings", c_i32), ("stage_wait_polls", c_i32)]


class Result(C.Structure):
    _fields_ = [("times", P(c_dbl)), ("mean", P(c_dbl)), ("stddev", P(c_dbl)), ("samples", P(c_i64)),
                ("leaps", c_i64), ("ssa_steps", c_i64), ("rejections", c_i64), ("truncated", c_i64),
                ("kernel_ms", c_dbl), ("total_ms", c_dbl), ("variant_used", c_i32),
                ("block_threads_used", c_i32), ("grid_used", c_i32), ("launches", c_i32)]


class GradResult(C.Structure):
    _fields_ = [("grad", P(c_dbl)), ("grad_stderr", P(c_dbl)), ("mean_final", P(c_dbl))]


class BatchItem(C.Structure):
    _fields_ = [("model", c_vp), ("cfg", P(RunCfg)), ("result", P(Result)), ("grad", P(GradResult))]


# name -> (restype, argtypes); every symbol include/tl.h declares.
SIGNATURES = {
    "tl_model_create": (c_i32, [P(ModelDesc), P(c_vp)]),
    "tl_model_from_stochkit": (c_i32, [C.c_char_p, c_i32, P(c_vp)]),
    "tl_model_destroy": (None, [c_vp]),
    "tl_model_get_info": (c_i32, [c_vp, P(ModelInfo)]),
    "tl_model_species_name": (C.c_char_p, [c_vp, c_i32]),
    "tl_model_species_index": (c_i32, [c_vp, C.c_char_p]),
    "tl_model_get_desc": (c_i32, [c_vp, P(c_i64), P(c_dbl), P(c_i32), P(c_i32), P(C.c_int8)]),
    "tl_model_write_stochkit": (c_i32, [c_vp, C.c_char_p]),
    "tl_gen_params_init": (None, [P(GenParams), c_i32]),
    "tl_model_generate": (c_i32, [P(GenParams), P(c_vp)]),
    "tl_model_get_tables": (c_i32, [c_vp, P(C.c_int8), P(c_i32), P(c_i32), P(c_i32), P(c_i32)]),
    "tl_run_cfg_init": (None, [P(RunCfg)]),
    "tl_simulate": (c_i32, [c_vp, P(RunCfg), P(Result)]),
    "tl_sensitivity": (c_i32, [c_vp, P(RunCfg), P(Result), P(GradResult)]),
    "tl_simulate_batch": (c_i32, [P(BatchItem), c_i32, c_vp]),
    "tl_simulate_static": (c_i32, [c_vp, P(RunCfg), P(Result)]),
    "tl_eval_leap": (c_i32, [c_vp, P(c_i64), c_i32, c_dbl, c_u32, c_i32, P(C.c_float), P(C.c_uint8),
                             P(C.c_float), P(C.c_float), P(C.c_float), P(c_dbl)]),
    "tl_replay": (c_i32, [c_vp, P(c_i64), P(c_i32), c_i32, c_i32, P(c_i64)]),
    "tl_philox": (c_i32, [P(c_u32), P(c_u32), c_i32, P(c_u32)]),
    "tl_poisson": (c_i32, [P(C.c_float), c_i32, c_u64, c_u32, c_i32, P(c_i32)]),
    "tl_merge_moments": (c_i32, [c_i32, c_i32, P(c_i64), P(c_dbl), P(c_dbl), P(c_i64), P(c_dbl), P(c_dbl)]),
    "tl_status_str": (C.c_char_p, [c_i32]),
    "tl_last_error": (C.c_char_p, []),
    "tl_abi_version": (c_i32, []),
    "tl_set_device": (c_i32, [c_i32]),
}

_lib = None


def lib() -> C.CDLL:
    """Load libtl.so (once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("TL_LIBTL", _LIB_PATH))
        if not path.exists():
            raise ImportError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; "
                              f"g.build()'` (the CUDA engine has no fallback)")
        L = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class TLError(RuntimeError):
    def __init__(self, status: int, where: str):
        detail = lib().tl_last_error().decode(errors="replace")
        super().__init__(f"{where}: {STATUS.get(status, status)} ({detail})")
        self.status = status


def check(status: int, where: str) -> int:
    if status != TL_OK:
        raise TLError(status, where)
    return status
