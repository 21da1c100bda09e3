"""ctypes harness for the CPU oracle (liboracle.so) and the reference build (oracle/_ref).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() (as the checker)
and bench.py's cpu_baseline / reference legs.  Never used by the product path in
s2kit_gb300/.

`Oracle` wraps the C restatement in s2oracle.c (every function there cites the S2kit
file:line it restates).  `Reference` wraps the unmodified S2kit sources compiled here by
`make -C oracle ref` against oracle/fftw_shim; it exists only where the reference checkout
is present and is used to pin the restatement and to generate tests/golden fixtures.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libs2kit_ref.so")
REF_BIN = os.path.join(HERE, "_ref", "bin")

COMPLEX, REAL = 0, 1
_lock = threading.Lock()

_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)


def build(force: bool = False) -> str:
    """Compile liboracle.so (and, if the reference checkout exists, oracle/_ref)."""
    with _lock:
        if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(
                os.path.join(HERE, "s2oracle.c")):
            subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB


def build_ref(ref: str | None = None) -> bool:
    """Builds oracle/_ref from the S2kit checkout at `ref` (or $S2_REFERENCE_DIR); False if absent."""
    ref = ref or os.environ.get("S2_REFERENCE_DIR", "")
    if not ref or not os.path.isdir(os.path.join(ref, "src")):
        return False
    with _lock:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref}"], check=True,
                       stdout=subprocess.DEVNULL)
    return os.path.exists(REF_LIB)


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


class Oracle:
    """FP64 CPU restatement of the S2kit memo path (s2oracle.c)."""

    def __init__(self):
        self.lib = C.CDLL(build())
        L = self.lib
        L.orc_index_of_harmonic_coeff.restype = C.c_int
        L.orc_index_of_harmonic_coeff.argtypes = [C.c_int] * 3
        for name in ("orc_table_size", "orc_table_offset"):
            getattr(L, name).restype = C.c_int64
            getattr(L, name).argtypes = [C.c_int, C.c_int]
        L.orc_reduced_spharmonic_table_size.restype = C.c_int64
        L.orc_reduced_spharmonic_table_size.argtypes = [C.c_int, C.c_int]
        L.orc_reduced_naive_table_size.restype = C.c_int64
        L.orc_reduced_naive_table_size.argtypes = [C.c_int, C.c_int]
        L.orc_row_size.restype = C.c_int
        L.orc_row_size.argtypes = [C.c_int, C.c_int]
        L.orc_transpose_row_size.restype = C.c_int
        L.orc_transpose_row_size.argtypes = [C.c_int] * 3
        L.orc_dft.argtypes = [C.c_int, _dp, _dp, C.c_int]
        for name in ("orc_redft10", "orc_redft01", "orc_redft10_direct", "orc_redft01_direct"):
            getattr(L, name).argtypes = [C.c_int, _dp, _dp]
        L.orc_generate_weights.argtypes = [C.c_int, _dp]
        L.orc_generate_cos_pml_table.argtypes = [C.c_int, C.c_int, _dp]
        L.orc_transpose_cos_pml_table.argtypes = [C.c_int, C.c_int, _dp, _dp]
        L.orc_generate_pml_table.argtypes = [C.c_int, C.c_int, _dp]
        L.orc_tables_new.restype = C.c_void_p
        L.orc_tables_new.argtypes = [C.c_int, C.c_int]
        L.orc_tables_new_mt.restype = C.c_void_p
        L.orc_tables_new_mt.argtypes = [C.c_int, C.c_int, C.c_int]
        L.orc_tables_free.argtypes = [C.c_void_p]
        L.orc_tables_total.restype = C.c_int64
        L.orc_tables_total.argtypes = [C.c_void_p]
        L.orc_tables_fwd.restype = _dp
        L.orc_tables_fwd.argtypes = [C.c_void_p]
        L.orc_tables_inv.restype = _dp
        L.orc_tables_inv.argtypes = [C.c_void_p]
        L.orc_tables_offsets.restype = _i64p
        L.orc_tables_offsets.argtypes = [C.c_void_p]
        L.orc_dlt_semi.argtypes = [_dp, C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_inv_dlt_semi.argtypes = [_dp, C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_dlt_naive.argtypes = [_dp, C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_inv_dlt_naive.argtypes = [_dp, C.c_int, C.c_int, _dp, _dp]
        L.orc_fst.argtypes = [_dp, _dp, _dp, _dp, C.c_int, C.c_void_p, _dp, C.c_int, C.c_int]
        L.orc_inv_fst.argtypes = [_dp, _dp, _dp, _dp, C.c_int, C.c_void_p, C.c_int, C.c_int]
        L.orc_fzt.argtypes = [_dp, _dp, _dp, _dp, C.c_int, _dp, _dp, C.c_int]
        L.orc_transmult.argtypes = [_dp] * 6 + [C.c_int]
        L.orc_conv.argtypes = [_dp] * 6 + [C.c_int]
        L.orc_conv_tables.argtypes = [_dp] * 6 + [C.c_int, C.c_void_p]
        L.orc_bench_roundtrip.restype = C.c_double
        L.orc_bench_roundtrip.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp]
        self._tables = {}

    # ---- helpers -------------------------------------------------------------------
    def index(self, m: int, l: int, bw: int) -> int:
        return self.lib.orc_index_of_harmonic_coeff(m, l, bw)

    def table_size(self, m: int, bw: int) -> int:
        return self.lib.orc_table_size(m, bw)

    def table_offset(self, m: int, l: int) -> int:
        return self.lib.orc_table_offset(m, l)

    def weights(self, bw: int) -> np.ndarray:
        w = np.empty(4 * bw)
        self.lib.orc_generate_weights(bw, _ptr(w))
        return w

    def cos_pml_table(self, bw: int, m: int) -> np.ndarray:
        t = np.empty(max(1, self.table_size(m, bw)))
        self.lib.orc_generate_cos_pml_table(bw, m, _ptr(t))
        return t[: self.table_size(m, bw)]

    def transpose_cos_pml_table(self, bw: int, m: int, table: np.ndarray) -> np.ndarray:
        table = np.ascontiguousarray(table, dtype=np.float64)
        out = np.empty(max(1, self.table_size(m, bw)))
        self.lib.orc_transpose_cos_pml_table(bw, m, _ptr(table), _ptr(out))
        return out[: self.table_size(m, bw)]

    def pml_table(self, bw: int, m: int) -> np.ndarray:
        t = np.empty(2 * bw * (bw - m))
        self.lib.orc_generate_pml_table(bw, m, _ptr(t))
        return t

    def tables(self, bw: int, cutoff: int):
        """(handle, fwd ndarray view, inv ndarray view, offsets ndarray) cached per (bw, cutoff)."""
        key = (bw, cutoff)
        if key not in self._tables:
            # orders generated on all host cores (identical values to one thread)
            h = self.lib.orc_tables_new_mt(bw, cutoff, os.cpu_count() or 1)
            n = self.lib.orc_tables_total(h)
            fwd = np.ctypeslib.as_array(self.lib.orc_tables_fwd(h), shape=(max(n, 1),))[:n]
            inv = np.ctypeslib.as_array(self.lib.orc_tables_inv(h), shape=(max(n, 1),))[:n]
            off = np.ctypeslib.as_array(self.lib.orc_tables_offsets(h), shape=(bw,)).copy()
            self._tables[key] = (h, fwd, inv, off)
        return self._tables[key]

    def drop_tables(self, bw: int, cutoff: int) -> None:
        """Frees the cached tables of (bw, cutoff) (2.9 GB of host memory at bw 1024)."""
        entry = self._tables.pop((bw, cutoff), None)
        if entry is not None:
            self.lib.orc_tables_free(C.c_void_p(entry[0]))

    # ---- transforms ----------------------------------------------------------------
    def redft10(self, x: np.ndarray, direct: bool = False) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        (self.lib.orc_redft10_direct if direct else self.lib.orc_redft10)(len(x), _ptr(x), _ptr(y))
        return y

    def redft01(self, x: np.ndarray, direct: bool = False) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        (self.lib.orc_redft01_direct if direct else self.lib.orc_redft01)(len(x), _ptr(x), _ptr(y))
        return y

    def dft(self, re: np.ndarray, im: np.ndarray, sign: int = -1):
        re = np.array(re, dtype=np.float64)
        im = np.array(im, dtype=np.float64)
        self.lib.orc_dft(len(re), _ptr(re), _ptr(im), sign)
        return re, im

    def dlt_semi(self, data, bw, m, table, weights):
        data = np.ascontiguousarray(data, dtype=np.float64)
        out = np.empty(bw - m)
        self.lib.orc_dlt_semi(_ptr(data), bw, m, _ptr(out), _ptr(np.ascontiguousarray(table)),
                              _ptr(np.ascontiguousarray(weights)))
        return out

    def inv_dlt_semi(self, coeffs, bw, m, ttable, sin_values):
        coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
        out = np.empty(2 * bw)
        self.lib.orc_inv_dlt_semi(_ptr(coeffs), bw, m, _ptr(out), _ptr(np.ascontiguousarray(ttable)),
                                  _ptr(np.ascontiguousarray(sin_values)))
        return out

    def dlt_naive(self, data, bw, m, weights, table):
        data = np.ascontiguousarray(data, dtype=np.float64)
        out = np.empty(bw - m)
        self.lib.orc_dlt_naive(_ptr(data), bw, m, _ptr(np.ascontiguousarray(weights)), _ptr(out),
                               _ptr(np.ascontiguousarray(table)))
        return out

    def inv_dlt_naive(self, coeffs, bw, m, table):
        coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
        out = np.empty(2 * bw)
        self.lib.orc_inv_dlt_naive(_ptr(coeffs), bw, m, _ptr(out), _ptr(np.ascontiguousarray(table)))
        return out

    def fst(self, rdata, idata, bw, data_format=REAL, cutoff=None):
        cutoff = bw if cutoff is None else cutoff
        h = self.tables(bw, cutoff)[0]
        rdata = np.ascontiguousarray(rdata, dtype=np.float64).reshape(-1)
        idata = np.ascontiguousarray(idata, dtype=np.float64).reshape(-1)
        rc = np.empty(bw * bw)
        ic = np.empty(bw * bw)
        w = self.weights(bw)
        self.lib.orc_fst(_ptr(rdata), _ptr(idata), _ptr(rc), _ptr(ic), bw, h, _ptr(w), data_format, cutoff)
        return rc, ic

    def inv_fst(self, rcoeffs, icoeffs, bw, data_format=REAL, cutoff=None):
        cutoff = bw if cutoff is None else cutoff
        h = self.tables(bw, cutoff)[0]
        rcoeffs = np.ascontiguousarray(rcoeffs, dtype=np.float64)
        icoeffs = np.ascontiguousarray(icoeffs, dtype=np.float64)
        rd = np.empty(4 * bw * bw)
        idd = np.empty(4 * bw * bw)
        self.lib.orc_inv_fst(_ptr(rcoeffs), _ptr(icoeffs), _ptr(rd), _ptr(idd), bw, h, data_format, cutoff)
        return rd, idd

    def fzt(self, rdata, idata, bw, data_format=REAL):
        tab = self.cos_pml_table(bw, 0)
        w = self.weights(bw)
        rdata = np.ascontiguousarray(rdata, dtype=np.float64).reshape(-1)
        idata = np.ascontiguousarray(idata, dtype=np.float64).reshape(-1)
        rr = np.empty(bw)
        ii = np.empty(2 * bw)
        self.lib.orc_fzt(_ptr(rdata), _ptr(idata), _ptr(rr), _ptr(ii), bw, _ptr(tab), _ptr(w), data_format)
        return rr, ii

    def transmult(self, rd, idd, rf, iff, bw):
        args = [np.ascontiguousarray(a, dtype=np.float64) for a in (rd, idd, rf, iff)]
        rr = np.empty(bw * bw)
        ir = np.empty(bw * bw)
        self.lib.orc_transmult(*[_ptr(a) for a in args], _ptr(rr), _ptr(ir), bw)
        return rr, ir

    def conv(self, rdata, idata, rfilter, ifilter, bw, cached_tables: bool = False):
        """ConvOn2SphereSemiMemo.  With cached_tables the (bw, bw) tables of tables() are used
        instead of tables built inside the call (same values, no second copy at large bw)."""
        args = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in (rdata, idata, rfilter, ifilter)]
        rr = np.empty(4 * bw * bw)
        ir = np.empty(4 * bw * bw)
        if cached_tables:
            self.lib.orc_conv_tables(*[_ptr(a) for a in args], _ptr(rr), _ptr(ir), bw, self.tables(bw, bw)[0])
        else:
            self.lib.orc_conv(*[_ptr(a) for a in args], _ptr(rr), _ptr(ir), bw)
        return rr, ir

    def bench_roundtrip(self, bw: int, coeffs: np.ndarray, nthreads: int):
        """coeffs: (nfunc, 2, bw*bw) float64.  Returns (seconds, output coeffs)."""
        coeffs = np.ascontiguousarray(coeffs, dtype=np.float64)
        out = np.empty_like(coeffs)
        secs = self.lib.orc_bench_roundtrip(bw, coeffs.shape[0], nthreads, _ptr(coeffs), _ptr(out))
        return secs, out


class Reference:
    """The unmodified S2kit C sources (built by `make -C oracle ref`), through their own API."""

    def __init__(self, ref: str | None = None):
        if not os.path.exists(REF_LIB) and not build_ref(ref):
            raise RuntimeError("reference build not available (oracle/_ref; set S2_REFERENCE_DIR to build it)")
        L = self.lib = C.CDLL(REF_LIB)
        L.TableSize.restype = C.c_int
        L.TableSize.argtypes = [C.c_int, C.c_int]
        L.TableOffset.restype = C.c_int
        L.TableOffset.argtypes = [C.c_int, C.c_int]
        L.Transpose_RowSize.restype = C.c_int
        L.Transpose_RowSize.argtypes = [C.c_int] * 3
        L.Reduced_Naive_TableSize.restype = C.c_int
        L.Reduced_Naive_TableSize.argtypes = [C.c_int, C.c_int]
        L.Reduced_SpharmonicTableSize.restype = C.c_int
        L.Reduced_SpharmonicTableSize.argtypes = [C.c_int, C.c_int]
        L.Spharmonic_TableSize.restype = C.c_int
        L.Spharmonic_TableSize.argtypes = [C.c_int]
        L.IndexOfHarmonicCoeff.restype = C.c_int
        L.IndexOfHarmonicCoeff.argtypes = [C.c_int] * 3
        L.SemiNaive_Naive_Pml_Table.restype = C.POINTER(_dp)
        L.SemiNaive_Naive_Pml_Table.argtypes = [C.c_int, C.c_int, _dp, _dp]
        L.Transpose_SemiNaive_Naive_Pml_Table.restype = C.POINTER(_dp)
        L.Transpose_SemiNaive_Naive_Pml_Table.argtypes = [C.POINTER(_dp), C.c_int, C.c_int, _dp, _dp]
        L.GenerateCosPmlTable.argtypes = [C.c_int, C.c_int, _dp, _dp]
        L.TransposeCosPmlTable.argtypes = [C.c_int, C.c_int, _dp, _dp]
        L.GeneratePmlTable.argtypes = [C.c_int, C.c_int, _dp, _dp]
        L.GenerateWeightsForDLT.argtypes = [C.c_int, _dp]
        L.fftw_plan_r2r_1d.restype = C.c_void_p
        L.fftw_plan_r2r_1d.argtypes = [C.c_int, _dp, _dp, C.c_int, C.c_uint]
        L.fftw_plan_guru_split_dft.restype = C.c_void_p
        L.fftw_plan_guru_split_dft.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, _dp, _dp, _dp, _dp,
                                               C.c_uint]
        L.fftw_destroy_plan.argtypes = [C.c_void_p]
        vp = C.c_void_p
        L.FSTSemiMemo.argtypes = [_dp, _dp, _dp, _dp, C.c_int, C.POINTER(_dp), _dp, C.c_int, C.c_int,
                                  C.POINTER(vp), C.POINTER(vp), _dp]
        L.InvFSTSemiMemo.argtypes = [_dp, _dp, _dp, _dp, C.c_int, C.POINTER(_dp), _dp, C.c_int, C.c_int,
                                     C.POINTER(vp), C.POINTER(vp)]
        L.FZTSemiMemo.argtypes = [_dp, _dp, _dp, _dp, C.c_int, _dp, _dp, C.c_int, C.POINTER(vp), _dp]
        L.ConvOn2SphereSemiMemo.argtypes = [_dp] * 6 + [C.c_int, _dp]
        L.TransMult.argtypes = [_dp] * 6 + [C.c_int]
        L.DLTSemi.argtypes = [_dp, C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.POINTER(vp)]
        # on-the-fly family (src/FST_semi_fly.c): tables generated per order inside each call
        L.FSTSemiFly.argtypes = [_dp, _dp, _dp, _dp, C.c_int, _dp, C.c_int, C.c_int, C.POINTER(vp), C.POINTER(vp),
                                 _dp]
        L.InvFSTSemiFly.argtypes = [_dp, _dp, _dp, _dp, C.c_int, _dp, C.c_int, C.c_int, C.POINTER(vp),
                                    C.POINTER(vp)]
        L.FZTSemiFly.argtypes = [_dp, _dp, _dp, _dp, C.c_int, _dp, C.c_int, C.POINTER(vp), _dp]
        L.ConvOn2SphereSemiFly.argtypes = [_dp] * 6 + [C.c_int, _dp]
        L.InvDLTSemi.argtypes = [_dp, C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.POINTER(vp)]
        self._keep = []

    class _Dim(C.Structure):
        _fields_ = [("n", C.c_int), ("is_", C.c_int), ("os", C.c_int)]

    def _plans(self, bw):
        L = self.lib
        n = 2 * bw
        scratch = np.zeros(2 * n * n + 4 * n)
        p = _ptr(scratch)
        dct = L.fftw_plan_r2r_1d(n, p, p, 5, 1 << 6)
        idct = L.fftw_plan_r2r_1d(n, p, p, 4, 1 << 6)
        d = (self._Dim * 1)(self._Dim(n, 1, n))
        h = (self._Dim * 1)(self._Dim(n, n, 1))
        fft = L.fftw_plan_guru_split_dft(1, C.cast(d, C.c_void_p), 1, C.cast(h, C.c_void_p), p, p, p, p, 1 << 6)
        d2 = (self._Dim * 1)(self._Dim(n, n, 1))
        h2 = (self._Dim * 1)(self._Dim(n, 1, n))
        ifft = L.fftw_plan_guru_split_dft(1, C.cast(d2, C.c_void_p), 1, C.cast(h2, C.c_void_p), p, p, p, p,
                                          1 << 6)
        self._keep.append(scratch)
        return [C.c_void_p(x) for x in (dct, idct, fft, ifft)]

    def tables(self, bw, cutoff):
        L = self.lib
        size = L.Reduced_Naive_TableSize(bw, cutoff) + L.Reduced_SpharmonicTableSize(bw, cutoff)
        ws = np.zeros(16 * bw + 8 * bw * bw)
        # SemiNaive_Naive_Pml_Table writes 2*bw samples for order m = cutoff even when
        # cutoff == bw (cospml.c:464-467), past the documented size: pad the buffers.
        fwd = np.zeros(size + 4 * bw)
        inv = np.zeros(size + 4 * bw)
        tf = L.SemiNaive_Naive_Pml_Table(bw, cutoff, _ptr(fwd), _ptr(ws))
        ti = L.Transpose_SemiNaive_Naive_Pml_Table(tf, bw, cutoff, _ptr(inv), _ptr(ws))
        self._keep += [fwd, inv, ws]
        return tf, ti, fwd[:size], inv[:size]

    def weights(self, bw):
        w = np.zeros(4 * bw)
        self.lib.GenerateWeightsForDLT(bw, _ptr(w))
        return w

    def fst(self, rdata, idata, bw, data_format=REAL, cutoff=None, tables=None):
        cutoff = bw if cutoff is None else cutoff
        tf, _, _, _ = tables or self.tables(bw, cutoff)
        dct, _, fft, _ = self._plans(bw)
        w = self.weights(bw)
        rdata = np.array(rdata, dtype=np.float64).reshape(-1)
        idata = np.array(idata, dtype=np.float64).reshape(-1)
        rc = np.zeros(bw * bw)
        ic = np.zeros(bw * bw)
        ws = np.zeros(8 * bw * bw + 16 * bw)
        self.lib.FSTSemiMemo(_ptr(rdata), _ptr(idata), _ptr(rc), _ptr(ic), bw, tf, _ptr(ws), data_format, cutoff,
                             C.byref(dct), C.byref(fft), _ptr(w))
        return rc, ic

    def inv_fst(self, rcoeffs, icoeffs, bw, data_format=REAL, cutoff=None, tables=None):
        cutoff = bw if cutoff is None else cutoff
        _, ti, _, _ = tables or self.tables(bw, cutoff)
        _, idct, _, ifft = self._plans(bw)
        rc = np.array(rcoeffs, dtype=np.float64)
        ic = np.array(icoeffs, dtype=np.float64)
        rd = np.zeros(4 * bw * bw)
        idd = np.zeros(4 * bw * bw)
        ws = np.zeros(8 * bw * bw + 16 * bw)
        self.lib.InvFSTSemiMemo(_ptr(rc), _ptr(ic), _ptr(rd), _ptr(idd), bw, ti, _ptr(ws), data_format, cutoff,
                                C.byref(idct), C.byref(ifft))
        return rd, idd

    def fzt(self, rdata, idata, bw, data_format=REAL):
        tf, _, _, _ = self.tables(bw, bw)
        dct, _, _, _ = self._plans(bw)
        w = self.weights(bw)
        rdata = np.array(rdata, dtype=np.float64).reshape(-1)
        idata = np.array(idata, dtype=np.float64).reshape(-1)
        rr = np.zeros(2 * bw)
        ii = np.zeros(2 * bw)
        ws = np.zeros(16 * bw)
        self.lib.FZTSemiMemo(_ptr(rdata), _ptr(idata), _ptr(rr), _ptr(ii), bw, tf[0], _ptr(ws), data_format,
                             C.byref(dct), _ptr(w))
        return rr[:bw], ii

    # ---- on-the-fly family: workspace sizes as documented at FST_semi_fly.c:58, 225, 447.  FZTSemiFly
    # documents 12*bw (:383) but uses 4*bw + 2*bw*bw (:394-397) plus GenerateCosPmlTable's 9*bw
    # (cospml.c:143), i.e. 2*bw*bw + 13*bw; the documented size corrupts the heap, so more is passed
    def fst_fly(self, rdata, idata, bw, data_format=REAL, cutoff=None):
        cutoff = bw if cutoff is None else cutoff
        dct, _, fft, _ = self._plans(bw)
        w = self.weights(bw)
        rdata = np.array(rdata, dtype=np.float64).reshape(-1)
        idata = np.array(idata, dtype=np.float64).reshape(-1)
        rc, ic = np.zeros(bw * bw), np.zeros(bw * bw)
        ws = np.zeros(10 * bw * bw + 24 * bw)
        self.lib.FSTSemiFly(_ptr(rdata), _ptr(idata), _ptr(rc), _ptr(ic), bw, _ptr(ws), data_format, cutoff,
                            C.byref(dct), C.byref(fft), _ptr(w))
        return rc, ic

    def inv_fst_fly(self, rcoeffs, icoeffs, bw, data_format=REAL, cutoff=None):
        cutoff = bw if cutoff is None else cutoff
        _, idct, _, ifft = self._plans(bw)
        rc = np.array(rcoeffs, dtype=np.float64)
        ic = np.array(icoeffs, dtype=np.float64)
        rd, idd = np.zeros(4 * bw * bw), np.zeros(4 * bw * bw)
        ws = np.zeros(10 * bw * bw + 24 * bw)
        self.lib.InvFSTSemiFly(_ptr(rc), _ptr(ic), _ptr(rd), _ptr(idd), bw, _ptr(ws), data_format, cutoff,
                               C.byref(idct), C.byref(ifft))
        return rd, idd

    def fzt_fly(self, rdata, idata, bw, data_format=REAL):
        dct, _, _, _ = self._plans(bw)
        w = self.weights(bw)
        rdata = np.array(rdata, dtype=np.float64).reshape(-1)
        idata = np.array(idata, dtype=np.float64).reshape(-1)
        rr, ii = np.zeros(2 * bw), np.zeros(2 * bw)
        ws = np.zeros(2 * bw * bw + 16 * bw)
        self.lib.FZTSemiFly(_ptr(rdata), _ptr(idata), _ptr(rr), _ptr(ii), bw, _ptr(ws), data_format, C.byref(dct),
                            _ptr(w))
        return rr[:bw], ii

    def conv_fly(self, rdata, idata, rfilter, ifilter, bw):
        args = [np.array(a, dtype=np.float64).reshape(-1) for a in (rdata, idata, rfilter, ifilter)]
        rr, ir = np.zeros(4 * bw * bw), np.zeros(4 * bw * bw)
        ws = np.zeros(14 * bw * bw + 26 * bw)
        self.lib.ConvOn2SphereSemiFly(*[_ptr(a) for a in args], _ptr(rr), _ptr(ir), bw, _ptr(ws))
        return rr, ir

    def conv(self, rdata, idata, rfilter, ifilter, bw):
        L = self.lib
        size = L.Reduced_Naive_TableSize(bw, bw) + L.Reduced_SpharmonicTableSize(bw, bw)
        args = [np.array(a, dtype=np.float64).reshape(-1) for a in (rdata, idata, rfilter, ifilter)]
        rr = np.zeros(4 * bw * bw)
        ir = np.zeros(4 * bw * bw)
        ws = np.zeros(2 * size + 12 * bw * bw + 12 * bw)
        L.ConvOn2SphereSemiMemo(*[_ptr(a) for a in args], _ptr(rr), _ptr(ir), bw, _ptr(ws))
        return rr, ir
