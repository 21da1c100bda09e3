"""ctypes binding of libs2kit_gb300.so (the C ABI declared in include/s2kit_gb300.h).

The library is loaded from the package directory only.  There is no fallback: if the
shared object is missing, importing the bindings raises, so nothing silently runs a CPU
path in its place.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libs2kit_gb300.so")

dp = C.POINTER(C.c_double)
fp = C.POINTER(C.c_float)
dpp = C.POINTER(dp)
vp = C.c_void_p

# every symbol include/s2kit_gb300.h declares: name -> (restype, argtypes)
SIGNATURES = {
    "FSTSemiMemo": (None, [dp, dp, dp, dp, C.c_int, dpp, dp, C.c_int, C.c_int, vp, vp, dp]),
    "InvFSTSemiMemo": (None, [dp, dp, dp, dp, C.c_int, dpp, dp, C.c_int, C.c_int, vp, vp]),
    "FZTSemiMemo": (None, [dp, dp, dp, dp, C.c_int, dp, dp, C.c_int, vp, dp]),
    "ConvOn2SphereSemiMemo": (None, [dp, dp, dp, dp, dp, dp, C.c_int, dp]),
    "FSTSemiFly": (None, [dp, dp, dp, dp, C.c_int, dp, C.c_int, C.c_int, vp, vp, dp]),
    "InvFSTSemiFly": (None, [dp, dp, dp, dp, C.c_int, dp, C.c_int, C.c_int, vp, vp]),
    "FZTSemiFly": (None, [dp, dp, dp, dp, C.c_int, dp, C.c_int, vp, dp]),
    "ConvOn2SphereSemiFly": (None, [dp, dp, dp, dp, dp, dp, C.c_int, dp]),
    "DLTSemi": (None, [dp, C.c_int, C.c_int, dp, dp, dp, dp, vp]),
    "InvDLTSemi": (None, [dp, C.c_int, C.c_int, dp, dp, dp, dp, vp]),
    "DLTNaive": (None, [dp, C.c_int, C.c_int, dp, dp, dp, dp]),
    "InvDLTNaive": (None, [dp, C.c_int, C.c_int, dp, dp]),
    "GenerateWeightsForDLT": (None, [C.c_int, dp]),
    "GenerateCosPmlTable": (None, [C.c_int, C.c_int, dp, dp]),
    "TransposeCosPmlTable": (None, [C.c_int, C.c_int, dp, dp]),
    "Spharmonic_Pml_Table": (dpp, [C.c_int, dp, dp]),
    "Transpose_Spharmonic_Pml_Table": (dpp, [dpp, C.c_int, dp]),
    "SemiNaive_Naive_Pml_Table": (dpp, [C.c_int, C.c_int, dp, dp]),
    "Transpose_SemiNaive_Naive_Pml_Table": (dpp, [dpp, C.c_int, C.c_int, dp, dp]),
    "GeneratePmlTable": (None, [C.c_int, C.c_int, dp, dp]),
    "Pmm_L2": (None, [C.c_int, dp, C.c_int, dp]),
    "TableSize": (C.c_int, [C.c_int, C.c_int]),
    "Spharmonic_TableSize": (C.c_int, [C.c_int]),
    "Reduced_SpharmonicTableSize": (C.c_int, [C.c_int, C.c_int]),
    "Reduced_Naive_TableSize": (C.c_int, [C.c_int, C.c_int]),
    "TableOffset": (C.c_int, [C.c_int, C.c_int]),
    "RowSize": (C.c_int, [C.c_int, C.c_int]),
    "Transpose_RowSize": (C.c_int, [C.c_int, C.c_int, C.c_int]),
    "IndexOfHarmonicCoeff": (C.c_int, [C.c_int, C.c_int, C.c_int]),
    "TransMult": (None, [dp, dp, dp, dp, dp, dp, C.c_int]),
    "AcosOfChebyshevNodes": (None, [C.c_int, dp]),
    "ChebyshevNodes": (None, [C.c_int, dp]),
    "s2g_last_error": (C.c_char_p, []),
    "s2g_version": (C.c_char_p, []),
    "s2g_cache_clear": (C.c_int, []),
    "s2g_plan_create": (C.c_int, [C.POINTER(vp), C.c_int, C.c_int]),
    "s2g_plan_destroy": (C.c_int, [vp]),
    "s2g_plan_create_fly": (C.c_int, [C.POINTER(vp), C.c_int]),
    "s2g_plan_workspace_size": (C.c_size_t, [vp, C.c_int, C.c_int]),
    "s2g_fst": (C.c_int, [vp, vp, vp, vp, vp, C.c_int, C.c_int, vp]),
    "s2g_inv_fst": (C.c_int, [vp, vp, vp, vp, vp, C.c_int, C.c_int, vp]),
    "s2g_fzt": (C.c_int, [vp, vp, vp, vp, vp, C.c_int, C.c_int, vp]),
    "s2g_transmult": (C.c_int, [C.c_int, vp, vp, vp, vp, vp, vp, C.c_int, vp]),
    "s2g_conv": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, C.c_int, vp]),
    "s2g_fst_real_f32": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int, vp]),
    "s2g_inv_fst_real_f32": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int, vp]),
    "s2g_fst_real_f32_host": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int]),
    "s2g_inv_fst_real_f32_host": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int]),
    "s2g_fst_real_f32_host_async": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int]),
    "s2g_inv_fst_real_f32_host_async": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int]),
    "s2g_plan_wait": (C.c_int, [vp]),
    "s2g_fst_complex_f32": (C.c_int, [vp, vp, vp, vp, vp, C.c_int, C.c_int, vp]),
    "s2g_inv_fst_complex_f32": (C.c_int, [vp, vp, vp, vp, vp, C.c_int, C.c_int, vp]),
    "s2g_plan_sync_status": (C.c_int, [vp]),
    "s2g_fst_refined": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int, vp]),
    "s2g_inv_fst_refined": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int, vp]),
    "s2g_fst_noalloc": (C.c_int, [vp, vp, vp, vp, C.c_int, vp, vp, vp, C.c_int, C.c_int, vp]),
    "s2g_group_create": (C.c_int, [C.POINTER(vp), C.c_int, C.POINTER(C.c_int), C.c_int]),
    "s2g_group_destroy": (C.c_int, [vp]),
    "s2g_group_layout": (C.c_int, [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                   C.POINTER(C.c_int64)]),
    "s2g_group_fst": (C.c_int, [vp, vp, vp, vp, vp]),
    "s2g_group_inv_fst": (C.c_int, [vp, vp, vp, vp, vp]),
    "s2g_group_fst_inv": (C.c_int, [vp, vp, vp, vp, vp, vp]),
    "s2g_group_autotune": (C.c_int, [vp, C.c_int]),
    "s2g_group_set_tiles": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int)]),
    "s2g_group_set_dct_ctas": (C.c_int, [vp, C.c_int]),
    "s2g_group_describe": (C.c_int, [vp, C.c_char_p, C.c_size_t]),
    "s2g_group_sync_status": (C.c_int, [vp]),
    "s2g_set_contraction_kernel": (C.c_int, [C.c_int]),
    "s2g_test_stall_contraction": (C.c_int, [C.c_int]),
    "s2g_tables_save": (C.c_int, [C.c_int, C.c_int, C.c_char_p]),
    "s2g_tables_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "s2g_selftest_tc": (C.c_int, [C.c_int, C.c_int, C.c_int, vp, vp, vp]),
    "s2g_prof_enable": (C.c_int, [C.c_int]),
    "s2g_prof_report": (C.c_int, [C.c_char_p, C.c_size_t]),
    "s2g_launch_count": (C.c_ulonglong, []),
}

_lib = None


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads (building first if needed and allowed) the in-tree shared library."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(f"{LIB_PATH} is missing: run python -m s2kit_gb300.build")
        from . import build as _b
        _b.build()
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class S2GError(RuntimeError):
    pass


def check(status: int, what: str = "") -> None:
    if status != 0:
        msg = load().s2g_last_error().decode(errors="replace")
        raise S2GError(f"{what} failed with status {status}: {msg}")
