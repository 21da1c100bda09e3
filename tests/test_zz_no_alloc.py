"""The forward transform entry point that allocates no device memory (s2g_fst_noalloc).

It serves callers that cannot call cudaMalloc/cudaFree (code inside a framework that has
already reserved its device memory, or code that cannot accept the synchronisation an
allocation implies): its scratch is a fixed __device__ array.  The test calls it through the
C ABI twice in a row, with different inputs, and checks each result against the existing
batched entry point s2g_fst on the same inputs, with the FP64 tolerance of the other tests.
This file is collected last so that a failure here never hides the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

import s2kit_gb300 as s2
from s2kit_gb300 import api
from tests._util import rel_err_norm

pytestmark = pytest.mark.gpu
TOL = 1e-11


def _device_tables(torch, bw, cutoff):
    size = api.Reduced_Naive_TableSize(bw, cutoff) + api.Reduced_SpharmonicTableSize(bw, cutoff)
    space = np.zeros(size)
    api.SemiNaive_Naive_Pml_Table(bw, cutoff, space, None)
    off = np.zeros(bw, dtype=np.int64)
    o = 0
    for m in range(bw):
        off[m] = o
        o += api.TableSize(m, bw) if m < cutoff else 2 * bw * (bw - m)
    w = np.zeros(4 * bw)
    api.GenerateWeightsForDLT(bw, w)
    return torch.from_numpy(space).cuda(), torch.from_numpy(off).cuda(), torch.from_numpy(w).cuda()


def _call(lib, rd, idd, rc, ic, bw, tab, off, w, fmt, cutoff):
    st = lib.s2g_fst_noalloc(rd.data_ptr(), idd.data_ptr() if idd is not None else None, rc.data_ptr(),
                             ic.data_ptr(), bw, tab.data_ptr(), off.data_ptr(), w.data_ptr(), fmt, cutoff, None)
    assert st == 0, lib.s2g_last_error()


@pytest.mark.parametrize("bw,cutoff", [(64, 64), (256, 256), (32, 8), (48, 48), (255, 40)])
def test_noalloc_matches_fst_twice(bw, cutoff):
    import torch
    lib = s2.load()
    tab, off, w = _device_tables(torch, bw, cutoff)
    plan = api.Plan(bw, cutoff)
    rng = np.random.default_rng(bw + cutoff)
    n = 2 * bw
    for call, fmt in enumerate((api.REAL, api.COMPLEX)):
        rd = torch.from_numpy(rng.standard_normal(n * n)).cuda()
        idd = torch.from_numpy(rng.standard_normal(n * n)).cuda()
        rc = torch.full((bw * bw,), float("nan"), dtype=torch.float64, device="cuda")
        ic = torch.full_like(rc, float("nan"))
        _call(lib, rd, idd, rc, ic, bw, tab, off, w, fmt, cutoff)
        ref_r = torch.zeros_like(rc)
        ref_i = torch.zeros_like(rc)
        plan.fst(rd, idd, ref_r, ref_i, 1, fmt)
        torch.cuda.synchronize()
        assert torch.isfinite(rc).all() and torch.isfinite(ic).all(), f"call {call}"
        err = rel_err_norm(rc.cpu().numpy(), ic.cpu().numpy(), ref_r.cpu().numpy(), ref_i.cpu().numpy())
        assert err <= TOL, (call, err)


def _noalloc_inputs(torch, rng, bw):
    n = 2 * bw
    rd = torch.from_numpy(rng.standard_normal(n * n)).cuda()
    idd = torch.from_numpy(rng.standard_normal(n * n)).cuda()
    rc = torch.full((bw * bw,), float("nan"), dtype=torch.float64, device="cuda")
    return rd, idd, rc, torch.full_like(rc, float("nan"))


def test_noalloc_non_power_of_two_allocates_nothing(oracle):
    """A bandwidth whose 2 bw is not a power of two: the length-2bw DFTs are Bluestein
    convolutions, whose tables the other entry points build with cudaMalloc on the first use of
    each length.  Here free device memory must not change across the first call at a length no
    other call in this process has used (bw 100, 2 bw = 200), and both calls in a row (REAL, then
    COMPLEX) must match the oracle to the FP64 parity bar."""
    import torch
    lib = s2.load()
    rng = np.random.default_rng(7)
    # a first call at another non-power-of-two length loads this library's kernels and looks up
    # the scratch array's address (module loading may reserve device memory once per process)
    tab, off, w = _device_tables(torch, 24, 24)
    rd, idd, rc, ic = _noalloc_inputs(torch, rng, 24)
    _call(lib, rd, idd, rc, ic, 24, tab, off, w, api.REAL, 24)
    bw, cutoff = 100, 100
    tab, off, w = _device_tables(torch, bw, cutoff)
    inputs = [_noalloc_inputs(torch, rng, bw) for _ in range(2)]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for (rd, idd, rc, ic), fmt in zip(inputs, (api.REAL, api.COMPLEX)):
        _call(lib, rd, idd, rc, ic, bw, tab, off, w, fmt, cutoff)
        torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, (free0, free1)
    for call, ((rd, idd, rc, ic), fmt) in enumerate(zip(inputs, (api.REAL, api.COMPLEX))):
        er, ei = oracle.fst(rd.cpu().numpy(), idd.cpu().numpy(), bw, fmt, cutoff)
        err = rel_err_norm(rc.cpu().numpy(), ic.cpu().numpy(), er, ei)
        assert err <= TOL, (call, err)


def test_noalloc_rejects_bandwidth_beyond_scratch():
    import torch
    lib = s2.load()
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    off = torch.zeros(16, dtype=torch.int64, device="cuda")
    st = lib.s2g_fst_noalloc(x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(), 512, x.data_ptr(),
                             off.data_ptr(), x.data_ptr(), api.REAL, 512, None)
    assert st == 1
    assert b"bandwidth 512" in lib.s2g_last_error()
