"""C ABI checks that need no GPU: the library loads, exports every declared symbol, the
integer layout helpers equal the reference's, and device entry points fail loudly (with a
status and a message) instead of falling back to a CPU path."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import s2kit_gb300 as s2
from s2kit_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "s2kit_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", src)
    skip = {"if", "while", "for", "sizeof", "return"}
    return sorted({n for n in names if n not in skip})


def test_header_declares_expected_api():
    names = declared_functions()
    for n in ("FSTSemiMemo", "InvFSTSemiMemo", "FZTSemiMemo", "ConvOn2SphereSemiMemo", "FSTSemiFly", "InvFSTSemiFly",
              "FZTSemiFly", "ConvOn2SphereSemiFly", "DLTSemi", "InvDLTSemi",
              "SemiNaive_Naive_Pml_Table", "s2g_plan_create", "s2g_fst_real_f32"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = s2.load()
    raw = C.CDLL(s2.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(raw, n)]
    assert not missing, missing
    # and the Python binding covers them
    from s2kit_gb300._lib import SIGNATURES
    assert set(declared_functions()) <= set(SIGNATURES)
    assert lib.s2g_version().startswith(b"s2kit_gb300")


def test_integer_helpers_match_oracle(oracle):
    for bw in (2, 8, 17, 64, 256):
        for m in range(0, bw, max(1, bw // 16)):
            assert api.TableSize(m, bw) == oracle.table_size(m, bw)
            for l in range(m, bw, max(1, bw // 8)):
                assert api.TableOffset(m, l) == oracle.table_offset(m, l)
                assert api.RowSize(m, l) == oracle.lib.orc_row_size(m, l)
                assert api.IndexOfHarmonicCoeff(m, l, bw) == oracle.index(m, l, bw)
                assert api.IndexOfHarmonicCoeff(-m, l, bw) == oracle.index(-m, l, bw)
            for row in range(bw):
                assert api.Transpose_RowSize(row, m, bw) == oracle.lib.orc_transpose_row_size(row, m, bw)
        for cut in (1, bw // 2 or 1, bw):
            assert api.Reduced_SpharmonicTableSize(bw, cut) == oracle.lib.orc_reduced_spharmonic_table_size(bw, cut)
            assert api.Reduced_Naive_TableSize(bw, cut) == oracle.lib.orc_reduced_naive_table_size(bw, cut)


def test_spharmonic_table_size_formula():
    # cospml.c:85-92 closed form (an upper bound) up to bw 512, exact sum beyond
    for bw in (2, 8, 64, 512):
        assert api.Spharmonic_TableSize(bw) == ((4 * bw ** 3 + 6 * bw ** 2 - 8 * bw) // 24) + bw
        assert api.Spharmonic_TableSize(bw) >= api.Reduced_SpharmonicTableSize(bw, bw)
    assert api.Spharmonic_TableSize(1024) == api.Reduced_SpharmonicTableSize(1024, 1024)


def test_index_matches_vectorised_helper():
    from tests._util import harmonic_index
    bw = 32
    for m in range(-(bw - 1), bw):
        for l in range(abs(m), bw):
            assert api.IndexOfHarmonicCoeff(m, l, bw) == int(harmonic_index(m, l, bw))


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU failure path")
def test_device_entry_points_fail_loudly_without_gpu():
    lib = s2.load()
    h = C.c_void_p()
    st = lib.s2g_plan_create(C.byref(h), 64, 64)
    assert st != 0
    assert lib.s2g_last_error()  # a message, not a silent fallback
    with pytest.raises(s2.S2GError):
        api.Plan(64)


def test_argument_validation_without_gpu():
    lib = s2.load()
    h = C.c_void_p()
    assert lib.s2g_plan_create(None, 64, 64) == 1
    assert lib.s2g_plan_create(C.byref(h), 1, 1) == 1       # bw < 2
    assert lib.s2g_plan_create(C.byref(h), 64, 0) == 1      # cutoff < 1
    assert lib.s2g_plan_create(C.byref(h), 64, 65) == 1     # cutoff > bw
    assert lib.s2g_plan_create(C.byref(h), 4096, 4096) == 4  # beyond this build
    assert lib.s2g_fst(None, None, None, None, None, 1, 1, None) == 1
    assert lib.s2g_transmult(8, None, None, None, None, None, None, 1, None) == 1
