"""Python mirror of S2kit's memo-path interface over the GB300 C ABI.

The functions below keep the reference names, argument order and meaning
(include/s2kit/FST_semi_memo.h, seminaive.h, naive.h, cospml.h, weights.h, util.h), with
numpy float64 arrays standing in for the caller-owned C buffers; they call the drop-in
entry points of libs2kit_gb300.so, which run on the GPU.  `Plan` exposes the batched
device-pointer API (torch CUDA tensors or raw device addresses).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, dp, dpp, load

COMPLEX, REAL = 0, 1
PREC_FP64, PREC_BF16X3, PREC_BF16X2, PREC_FP16X2 = 0, 1, 2, 3


def _p(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.dtype == np.float64 and a.flags.c_contiguous, "float64 C-contiguous array expected"
        return a.ctypes.data_as(dp)
    return a


class PmlTable:
    """A `double**` table returned by the table builders, with the buffer it points into."""

    def __init__(self, ptr, space: np.ndarray, bw: int, cutoff: int):
        self.ptr, self.space, self.bw, self.cutoff = ptr, space, bw, cutoff

    @property
    def _as_parameter_(self):
        return self.ptr


def _table(t):
    return t.ptr if isinstance(t, PmlTable) else t


# ---- sizes and indices (cospml.c, util.c) ----------------------------------------------
def TableSize(m, bw): return load().TableSize(m, bw)
def Spharmonic_TableSize(bw): return load().Spharmonic_TableSize(bw)
def Reduced_SpharmonicTableSize(bw, m): return load().Reduced_SpharmonicTableSize(bw, m)
def Reduced_Naive_TableSize(bw, m): return load().Reduced_Naive_TableSize(bw, m)
def TableOffset(m, l): return load().TableOffset(m, l)
def RowSize(m, l): return load().RowSize(m, l)
def Transpose_RowSize(row, m, bw): return load().Transpose_RowSize(row, m, bw)
def IndexOfHarmonicCoeff(m, l, bw): return load().IndexOfHarmonicCoeff(m, l, bw)


# ---- table builders (cospml.c, pml.c, pmm.c, weights.c, chebyshev_nodes.c) -----------------
def GenerateWeightsForDLT(bw, weights):
    load().GenerateWeightsForDLT(bw, _p(weights))


def GenerateCosPmlTable(bw, m, tablespace, workspace=None):
    load().GenerateCosPmlTable(bw, m, _p(tablespace), None)


def TransposeCosPmlTable(bw, m, cos_pml_table, result):
    load().TransposeCosPmlTable(bw, m, _p(cos_pml_table), _p(result))


def GeneratePmlTable(bw, m, pml_table, workspace=None):
    load().GeneratePmlTable(bw, m, _p(pml_table), None)


def Pmm_L2(m, eval_points, n, result):
    load().Pmm_L2(m, _p(eval_points), n, _p(result))


def ChebyshevNodes(n, eval_points):
    load().ChebyshevNodes(n, _p(eval_points))


def AcosOfChebyshevNodes(n, eval_points):
    load().AcosOfChebyshevNodes(n, _p(eval_points))


def Spharmonic_Pml_Table(bw, resultspace, workspace=None):
    ptr = load().Spharmonic_Pml_Table(bw, _p(resultspace), None)
    return PmlTable(ptr, resultspace, bw, bw) if ptr else None


def Transpose_Spharmonic_Pml_Table(spharmonic_pml_table, bw, resultspace):
    ptr = load().Transpose_Spharmonic_Pml_Table(_table(spharmonic_pml_table), bw, _p(resultspace))
    return PmlTable(ptr, resultspace, bw, bw) if ptr else None


def SemiNaive_Naive_Pml_Table(bw, m, resultspace, workspace=None):
    ptr = load().SemiNaive_Naive_Pml_Table(bw, m, _p(resultspace), None)
    return PmlTable(ptr, resultspace, bw, m) if ptr else None


def Transpose_SemiNaive_Naive_Pml_Table(seminaive_naive_pml_table, bw, m, resultspace, workspace=None):
    ptr = load().Transpose_SemiNaive_Naive_Pml_Table(_table(seminaive_naive_pml_table), bw, m, _p(resultspace),
                                                     None)
    return PmlTable(ptr, resultspace, bw, m) if ptr else None


# ---- transforms (FST_semi_memo.c, seminaive.c, naive.c, util.c) ----------------------------
def FSTSemiMemo(rdata, idata, rcoeffs, icoeffs, bw, seminaive_naive_table, workspace, data_format, cutoff,
                DCT_plan=None, FFT_plan=None, weights=None):
    load().FSTSemiMemo(_p(rdata), _p(idata), _p(rcoeffs), _p(icoeffs), bw, _table(seminaive_naive_table),
                       _p(workspace), data_format, cutoff, None, None, _p(weights))


def InvFSTSemiMemo(rcoeffs, icoeffs, rdata, idata, bw, transpose_seminaive_naive_table, workspace, data_format,
                   cutoff, inv_DCT_plan=None, inv_FFT_plan=None):
    load().InvFSTSemiMemo(_p(rcoeffs), _p(icoeffs), _p(rdata), _p(idata), bw,
                          _table(transpose_seminaive_naive_table), _p(workspace), data_format, cutoff, None, None)


def FZTSemiMemo(rdata, idata, rres, ires, bw, cos_pml_table, workspace, data_format, DCT_plan=None, weights=None):
    load().FZTSemiMemo(_p(rdata), _p(idata), _p(rres), _p(ires), bw, _p(cos_pml_table), _p(workspace),
                       data_format, None, _p(weights))


def ConvOn2SphereSemiMemo(rdata, idata, rfilter, ifilter, rres, ires, bw, workspace=None):
    load().ConvOn2SphereSemiMemo(_p(rdata), _p(idata), _p(rfilter), _p(ifilter), _p(rres), _p(ires), bw,
                                 _p(workspace))


# On-the-fly family (src/FST_semi_fly.c): same arguments as the reference, no table argument.
def FSTSemiFly(rdata, idata, rcoeffs, icoeffs, bw, workspace, data_format, cutoff, DCT_plan=None, FFT_plan=None,
               weights=None):
    load().FSTSemiFly(_p(rdata), _p(idata), _p(rcoeffs), _p(icoeffs), bw, _p(workspace), data_format, cutoff, None,
                      None, _p(weights))


def InvFSTSemiFly(rcoeffs, icoeffs, rdata, idata, bw, workspace, data_format, cutoff, inv_DCT_plan=None,
                  inv_FFT_plan=None):
    load().InvFSTSemiFly(_p(rcoeffs), _p(icoeffs), _p(rdata), _p(idata), bw, _p(workspace), data_format, cutoff,
                         None, None)


def FZTSemiFly(rdata, idata, rres, ires, bw, workspace, data_format, DCT_plan=None, weights=None):
    load().FZTSemiFly(_p(rdata), _p(idata), _p(rres), _p(ires), bw, _p(workspace), data_format, None, _p(weights))


def ConvOn2SphereSemiFly(rdata, idata, rfilter, ifilter, rres, ires, bw, workspace=None):
    load().ConvOn2SphereSemiFly(_p(rdata), _p(idata), _p(rfilter), _p(ifilter), _p(rres), _p(ires), bw,
                                _p(workspace))


def DLTSemi(data, bw, m, result, workspace, cos_pml_table, weights, plan=None):
    load().DLTSemi(_p(data), bw, m, _p(result), _p(workspace), _p(cos_pml_table), _p(weights), None)


def InvDLTSemi(coeffs, bw, m, result, trans_cos_pml_table, sin_values, workspace=None, plan=None):
    load().InvDLTSemi(_p(coeffs), bw, m, _p(result), _p(trans_cos_pml_table), _p(sin_values), _p(workspace), None)


def DLTNaive(data, bw, m, weights, result, pml_table, workspace=None):
    load().DLTNaive(_p(data), bw, m, _p(weights), _p(result), _p(pml_table), _p(workspace))


def InvDLTNaive(coeffs, bw, m, result, pml_table):
    load().InvDLTNaive(_p(coeffs), bw, m, _p(result), _p(pml_table))


def TransMult(rdatacoeffs, idatacoeffs, rfiltercoeffs, ifiltercoeffs, rres, ires, bw):
    load().TransMult(_p(rdatacoeffs), _p(idatacoeffs), _p(rfiltercoeffs), _p(ifiltercoeffs), _p(rres), _p(ires),
                     bw)


# ---- batched device API -------------------------------------------------------------------
def _addr(x):
    """Device address of a torch tensor (or an int address)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def _stream(s):
    if s is None:
        return None
    if isinstance(s, int):
        return s
    return s.cuda_stream  # torch.cuda.Stream


class Plan:
    """Batched transforms of bandwidth `bw` on the current CUDA device (s2g_plan).

    fly=True makes an on-the-fly plan (s2g_plan_create_fly): no Legendre table on the device,
    the FP64 transforms (fst, inv_fst, fzt, conv) generate the Legendre functions inside their
    kernels (the FSTSemiFly family)."""

    def __init__(self, bw: int, cutoff: int | None = None, fly: bool = False):
        self.lib = load()
        self.bw = bw
        self.cutoff = bw if cutoff is None else cutoff
        self.fly = fly
        h = C.c_void_p()
        if fly:
            check(self.lib.s2g_plan_create_fly(C.byref(h), bw), "s2g_plan_create_fly")
        else:
            check(self.lib.s2g_plan_create(C.byref(h), bw, self.cutoff), "s2g_plan_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.s2g_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync_status(self):
        """Waits for the device and raises if a tensor-core kernel recorded a failure."""
        check(self.lib.s2g_plan_sync_status(self.h), "device status")

    def workspace_size(self, batch: int, precision: int = PREC_FP64) -> int:
        return self.lib.s2g_plan_workspace_size(self.h, batch, precision)

    def fst(self, rdata, idata, rcoeffs, icoeffs, batch, data_format=REAL, stream=None):
        check(self.lib.s2g_fst(self.h, _addr(rdata), _addr(idata), _addr(rcoeffs), _addr(icoeffs), batch,
                               data_format, _stream(stream)), "s2g_fst")

    def inv_fst(self, rcoeffs, icoeffs, rdata, idata, batch, data_format=REAL, stream=None):
        check(self.lib.s2g_inv_fst(self.h, _addr(rcoeffs), _addr(icoeffs), _addr(rdata), _addr(idata), batch,
                                   data_format, _stream(stream)), "s2g_inv_fst")

    def fzt(self, rdata, idata, rres, ires, batch, data_format=REAL, stream=None):
        check(self.lib.s2g_fzt(self.h, _addr(rdata), _addr(idata), _addr(rres), _addr(ires), batch, data_format,
                               _stream(stream)), "s2g_fzt")

    def conv(self, rdata, idata, rfilter, ifilter, rres, ires, batch, stream=None):
        check(self.lib.s2g_conv(self.h, _addr(rdata), _addr(idata), _addr(rfilter), _addr(ifilter), _addr(rres),
                                _addr(ires), batch, _stream(stream)), "s2g_conv")

    def fst_real_f32(self, grid, rcoeffs, icoeffs, batch, precision=PREC_BF16X3, stream=None):
        check(self.lib.s2g_fst_real_f32(self.h, _addr(grid), _addr(rcoeffs), _addr(icoeffs), batch, precision,
                                        _stream(stream)), "s2g_fst_real_f32")

    def inv_fst_real_f32(self, rcoeffs, icoeffs, grid, batch, precision=PREC_BF16X3, stream=None):
        check(self.lib.s2g_inv_fst_real_f32(self.h, _addr(rcoeffs), _addr(icoeffs), _addr(grid), batch, precision,
                                            _stream(stream)), "s2g_inv_fst_real_f32")

    def fst_complex_f32(self, rgrid, igrid, rcoeffs, icoeffs, batch, precision=PREC_BF16X3, stream=None):
        """COMPLEX data on the split path: the real and imaginary fields through the real-field
        transform, combined per coefficient (every order written)."""
        check(self.lib.s2g_fst_complex_f32(self.h, _addr(rgrid), _addr(igrid), _addr(rcoeffs), _addr(icoeffs), batch,
                                           precision, _stream(stream)), "s2g_fst_complex_f32")

    def inv_fst_complex_f32(self, rcoeffs, icoeffs, rgrid, igrid, batch, precision=PREC_BF16X3, stream=None):
        check(self.lib.s2g_inv_fst_complex_f32(self.h, _addr(rcoeffs), _addr(icoeffs), _addr(rgrid), _addr(igrid),
                                               batch, precision, _stream(stream)), "s2g_inv_fst_complex_f32")

    def fst_refined(self, grid, rcoeffs, icoeffs, batch, precision=PREC_BF16X3, stream=None):
        """FP64 in/out forward: split contraction plus one FP64-residual refinement step."""
        check(self.lib.s2g_fst_refined(self.h, _addr(grid), _addr(rcoeffs), _addr(icoeffs), batch, precision,
                                       _stream(stream)), "s2g_fst_refined")

    def inv_fst_refined(self, rcoeffs, icoeffs, grid, batch, precision=PREC_BF16X3, stream=None):
        check(self.lib.s2g_inv_fst_refined(self.h, _addr(rcoeffs), _addr(icoeffs), _addr(grid), batch, precision,
                                           _stream(stream)), "s2g_inv_fst_refined")

    def fst_real_f32_host(self, grid: np.ndarray, rcoeffs: np.ndarray, icoeffs: np.ndarray, batch, precision):
        check(self.lib.s2g_fst_real_f32_host(self.h, grid.ctypes.data, rcoeffs.ctypes.data, icoeffs.ctypes.data,
                                             batch, precision), "s2g_fst_real_f32_host")

    def inv_fst_real_f32_host(self, rcoeffs: np.ndarray, icoeffs: np.ndarray, grid: np.ndarray, batch, precision):
        check(self.lib.s2g_inv_fst_real_f32_host(self.h, rcoeffs.ctypes.data, icoeffs.ctypes.data, grid.ctypes.data,
                                                 batch, precision), "s2g_inv_fst_real_f32_host")

    def fst_real_f32_host_async(self, grid: np.ndarray, rcoeffs: np.ndarray, icoeffs: np.ndarray, batch, precision):
        """Queued host-buffer forward; the buffers stay in use until wait()."""
        check(self.lib.s2g_fst_real_f32_host_async(self.h, grid.ctypes.data, rcoeffs.ctypes.data,
                                                   icoeffs.ctypes.data, batch, precision),
              "s2g_fst_real_f32_host_async")

    def inv_fst_real_f32_host_async(self, rcoeffs: np.ndarray, icoeffs: np.ndarray, grid: np.ndarray, batch,
                                    precision):
        check(self.lib.s2g_inv_fst_real_f32_host_async(self.h, rcoeffs.ctypes.data, icoeffs.ctypes.data,
                                                       grid.ctypes.data, batch, precision),
              "s2g_inv_fst_real_f32_host_async")

    def wait(self):
        """Waits for the host-buffer calls queued on this plan."""
        check(self.lib.s2g_plan_wait(self.h), "s2g_plan_wait")


class Group:
    """Grouped transforms of many real functions of uneven bandwidth (s2g_group_*).

    ``bws``: bandwidth of each function (16 .. 256, or a power of two up to 512; at most 16
    distinct bandwidths).  Device buffers are flat
    float32 tensors: the grid holds the functions' (2 bw)^2 samples back to back, rcoeffs/icoeffs
    their bw^2 coefficients; ``grid_offsets``/``coeff_offsets`` give each function's start.
    """

    def __init__(self, bws, precision=PREC_FP16X2):
        self.lib = load()
        self.bws = [int(b) for b in bws]
        self.precision = precision
        h = C.c_void_p()
        arr = (C.c_int * len(self.bws))(*self.bws)
        check(self.lib.s2g_group_create(C.byref(h), len(self.bws), arr, precision), "s2g_group_create")
        self.h = h
        n = len(self.bws)
        go, co = (C.c_int64 * n)(), (C.c_int64 * n)()
        gt, ct = C.c_int64(), C.c_int64()
        check(self.lib.s2g_group_layout(self.h, go, co, C.byref(gt), C.byref(ct)), "s2g_group_layout")
        self.grid_offsets = np.array(go[:], dtype=np.int64)
        self.coeff_offsets = np.array(co[:], dtype=np.int64)
        self.grid_total, self.coeff_total = gt.value, ct.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.s2g_group_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fst(self, grid, rcoeffs, icoeffs, stream=None):
        check(self.lib.s2g_group_fst(self.h, _addr(grid), _addr(rcoeffs), _addr(icoeffs), _stream(stream)),
              "s2g_group_fst")

    def inv_fst(self, rcoeffs, icoeffs, grid, stream=None):
        check(self.lib.s2g_group_inv_fst(self.h, _addr(rcoeffs), _addr(icoeffs), _addr(grid), _stream(stream)),
              "s2g_group_inv_fst")

    def fst_inv(self, grid, rcoeffs, icoeffs, grid_out, stream=None):
        check(self.lib.s2g_group_fst_inv(self.h, _addr(grid), _addr(rcoeffs), _addr(icoeffs), _addr(grid_out),
                                         _stream(stream)), "s2g_group_fst_inv")

    def autotune(self, force=False):
        check(self.lib.s2g_group_autotune(self.h, 1 if force else 0), "s2g_group_autotune")

    def set_tiles(self, table_stages=0, tile_n=None, dct_ctas_per_sm=None):
        arr = None if tile_n is None else (C.c_int * len(tile_n))(*tile_n)
        check(self.lib.s2g_group_set_tiles(self.h, table_stages, arr), "s2g_group_set_tiles")
        if dct_ctas_per_sm is not None:
            check(self.lib.s2g_group_set_dct_ctas(self.h, dct_ctas_per_sm), "s2g_group_set_dct_ctas")

    def describe(self) -> dict:
        import json
        buf = C.create_string_buffer(4096)
        check(self.lib.s2g_group_describe(self.h, buf, len(buf)), "s2g_group_describe")
        return json.loads(buf.value.decode())

    def sync_status(self):
        check(self.lib.s2g_group_sync_status(self.h), "group device status")


def selftest_tc(A, B, D, nprod=6):
    """D = A @ B.T on one tcgen05 tile (torch CUDA float32 tensors, A 128 x K, B N x K)."""
    check(load().s2g_selftest_tc(B.shape[0], A.shape[1], nprod, _addr(A), _addr(B), _addr(D)), "s2g_selftest_tc")


def transmult(bw, rd, id_, rf, if_, rr, ir, batch, stream=None):
    check(load().s2g_transmult(bw, _addr(rd), _addr(id_), _addr(rf), _addr(if_), _addr(rr), _addr(ir), batch,
                               _stream(stream)), "s2g_transmult")
