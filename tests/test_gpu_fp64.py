"""FP64 GPU path vs the oracle and the reference's golden data, through the C ABI.

Tolerances: the reference's own FP64 results are the target; FFT/DCT implementations and
FMA contraction differ, so results agree to rounding.  Normwise relative error
max|gpu - ref| / max|ref| <= 1e-11 is the parity bar (the plain FP64 GPU path within 1e-11
relative of the reference).
"""
import numpy as np
import pytest

from s2kit_gb300 import api
from tests._util import harmonic_index, real_field_coeffs, rel_err_norm

pytestmark = pytest.mark.gpu
TOL = 1e-11


def _tables(bw, cutoff):
    size = api.Reduced_Naive_TableSize(bw, cutoff) + api.Reduced_SpharmonicTableSize(bw, cutoff)
    fwd_space = np.zeros(size)
    inv_space = np.zeros(size)
    t = api.SemiNaive_Naive_Pml_Table(bw, cutoff, fwd_space, None)
    tt = api.Transpose_SemiNaive_Naive_Pml_Table(t, bw, cutoff, inv_space, None)
    return t, tt


def _weights(bw):
    w = np.zeros(4 * bw)
    api.GenerateWeightsForDLT(bw, w)
    return w


def _fst(rdata, idata, bw, fmt, cutoff, t=None):
    t = t or _tables(bw, cutoff)[0]
    rc, ic = np.zeros(bw * bw), np.zeros(bw * bw)
    api.FSTSemiMemo(np.ascontiguousarray(rdata, dtype=np.float64), np.ascontiguousarray(idata, dtype=np.float64),
                    rc, ic, bw, t, None, fmt, cutoff, None, None, _weights(bw))
    return rc, ic


def _inv(rc, ic, bw, fmt, cutoff, tt=None):
    tt = tt or _tables(bw, cutoff)[1]
    rd, idd = np.zeros(4 * bw * bw), np.zeros(4 * bw * bw)
    api.InvFSTSemiMemo(np.ascontiguousarray(rc), np.ascontiguousarray(ic), rd, idd, bw, tt, None, fmt, cutoff)
    return rd, idd


# ---------------------------------------------------------------------------------- tables
@pytest.mark.parametrize("bw,cut", [(16, 16), (16, 5)])
def test_tables_match_reference(golden, bw, cut):
    g = golden(f"ref_tables_bw{bw}_cut{cut}")
    t, tt = _tables(bw, cut)
    scale = np.abs(g["fwd"]).max()
    assert np.abs(t.space - g["fwd"]).max() <= 1e-13 * scale
    assert np.abs(tt.space - g["inv"]).max() <= 1e-13 * scale


@pytest.mark.parametrize("bw", [64, 256, 512])
def test_tables_match_oracle_large(oracle, bw):
    _, fwd, inv, _ = oracle.tables(bw, bw)
    t, tt = _tables(bw, bw)
    scale = np.abs(fwd).max()
    assert np.abs(t.space - fwd).max() <= 1e-12 * scale
    assert np.abs(tt.space - inv).max() <= 1e-12 * scale


def test_weights_and_nodes(golden, oracle):
    g = golden("ref_weights")
    for bw in (16, 64, 256):
        assert np.abs(_weights(bw) - g[f"w{bw}"]).max() <= 1e-14
    n = 64
    a = np.zeros(n)
    c = np.zeros(n)
    api.AcosOfChebyshevNodes(n, a)
    api.ChebyshevNodes(n, c)
    k = np.arange(n)
    assert np.abs(a - (2 * k + 1) * np.pi / (2 * n)).max() <= 1e-15
    assert np.abs(c - np.cos((2 * k + 1) * np.pi / (2 * n))).max() <= 1e-15
    r = np.zeros(n)
    api.Pmm_L2(5, a, n, r)
    ref = np.zeros(n)
    oracle.lib.orc_pmm_l2(5, a.ctypes.data_as(__import__("ctypes").POINTER(__import__("ctypes").c_double)), n,
                          ref.ctypes.data_as(__import__("ctypes").POINTER(__import__("ctypes").c_double)))
    assert np.abs(r - ref).max() <= 1e-14 * np.abs(ref).max()


def test_single_order_builders(oracle):
    bw = 32
    for m in (0, 1, 7, 30, 31):
        n = api.TableSize(m, bw)
        tab = np.zeros(n)
        api.GenerateCosPmlTable(bw, m, tab, None)
        ref = oracle.cos_pml_table(bw, m)
        assert np.abs(tab - ref).max() <= 1e-13 * np.abs(ref).max()
        tr = np.zeros(n)
        api.TransposeCosPmlTable(bw, m, tab, tr)
        assert np.abs(tr - oracle.transpose_cos_pml_table(bw, m, tab)).max() == 0.0
        p = np.zeros(2 * bw * (bw - m))
        api.GeneratePmlTable(bw, m, p, None)
        ref = oracle.pml_table(bw, m)
        assert np.abs(p - ref).max() <= 1e-13 * np.abs(ref).max()


# ------------------------------------------------------------------------- known answers
@pytest.mark.parametrize("name", ["y20_bw8", "y31_bw8", "y43_bw23", "yMix_bw17"])
def test_known_answers(golden, name):
    g = golden(f"ka_{name}")
    bw = int(g["bw"])
    rc, ic = _fst(g["rdata"], g["idata"], bw, api.COMPLEX, bw)
    exp = np.zeros(bw * bw, dtype=complex)
    for m, l, re, im in g["expected"]:
        exp[harmonic_index(int(m), int(l), bw)] = re + 1j * im
    assert np.abs(rc + 1j * ic - exp).max() <= 1e-13


# ----------------------------------------------------------------- reference fixtures
@pytest.mark.parametrize("case", ["bw8_cut8_complex", "bw16_cut4_complex", "bw32_cut32_real", "bw64_cut64_real",
                                  "bw64_cut16_complex"])
def test_reference_sht_fixtures(golden, case):
    g = golden(f"ref_sht_{case}")
    bw, cut, fmt = int(g["bw"]), int(g["cutoff"]), int(g["fmt"])
    t, tt = _tables(bw, cut)
    gr, gi = _inv(g["rcoeffs"], g["icoeffs"], bw, fmt, cut, tt)
    scale = np.abs(g["inv_r"]).max()
    assert np.abs(gr - g["inv_r"]).max() <= TOL * scale
    assert np.abs(gi - g["inv_i"]).max() <= TOL * scale
    fr, fi = _fst(g["noise_r"], g["noise_i"], bw, fmt, cut, t)
    assert rel_err_norm(fr, fi, g["fwd_noise_r"], g["fwd_noise_i"]) <= TOL
    rr, ri = _fst(g["inv_r"], g["inv_i"], bw, fmt, cut, t)
    assert rel_err_norm(rr, ri, g["rt_r"], g["rt_i"]) <= TOL


@pytest.mark.parametrize("bw", [64, 128])
def test_conv_golden(golden, bw):
    g = golden(f"conv_bw{bw}")
    z = np.zeros_like(g["signal"])
    rr, ri = np.zeros_like(z), np.zeros_like(z)
    api.ConvOn2SphereSemiMemo(g["signal"], z, g["filter"], z.copy(), rr, ri, bw, None)
    assert np.abs(rr - g["golden"]).max() <= 1e-14


def test_fzt_and_transmult(golden):
    g = golden("ref_fzt_transmult_bw16")
    bw = int(g["bw"])
    tab = np.zeros(api.TableSize(0, bw))
    api.GenerateCosPmlTable(bw, 0, tab, None)
    rr, ri = np.zeros(bw), np.full(2 * bw, 7.0)
    api.FZTSemiMemo(g["data_r"], g["data_i"], rr, ri, bw, tab, None, api.COMPLEX, None, _weights(bw))
    assert np.abs(rr - g["fzt_complex_r"]).max() <= 1e-13
    assert np.abs(ri[:bw] - g["fzt_complex_i"]).max() <= 1e-13
    assert np.all(ri[bw:] == 7.0)
    api.FZTSemiMemo(g["data_r"], g["data_i"], rr, ri, bw, tab, None, api.REAL, None, _weights(bw))
    assert np.abs(rr - g["fzt_real_r"]).max() <= 1e-13
    assert np.all(ri == 0.0)  # 2*bw zeros, FST_semi_memo.c:406
    tr, ti = np.zeros(bw * bw), np.zeros(bw * bw)
    api.TransMult(g["tm_data_r"], g["tm_data_i"], g["tm_filter_r"], g["tm_filter_i"], tr, ti, bw)
    assert np.abs(tr - g["tm_out_r"]).max() <= 1e-14
    assert np.abs(ti - g["tm_out_i"]).max() <= 1e-14


# ------------------------------------------------------------------------- 1-D DLTs
@pytest.mark.parametrize("bw,m", [(16, 0), (16, 3), (64, 10), (64, 63), (256, 1)])
def test_dlt_semi_and_naive(oracle, bw, m):
    rng = np.random.default_rng(bw + m)
    w = _weights(bw)
    tab = oracle.cos_pml_table(bw, m)
    ttab = oracle.transpose_cos_pml_table(bw, m, tab)
    data = rng.standard_normal(2 * bw)
    res = np.zeros(bw - m)
    api.DLTSemi(data, bw, m, res, None, np.ascontiguousarray(tab), w)
    ref = oracle.dlt_semi(data, bw, m, tab, w)
    assert np.abs(res - ref).max() <= 1e-12 * np.abs(ref).max()
    coeffs = rng.standard_normal(bw - m)
    sinv = np.sin((2 * np.arange(2 * bw) + 1) * np.pi / (4 * bw))
    out = np.zeros(2 * bw)
    api.InvDLTSemi(coeffs, bw, m, out, np.ascontiguousarray(ttab), sinv, None)
    ref = oracle.inv_dlt_semi(coeffs, bw, m, ttab, sinv)
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()
    ptab = oracle.pml_table(bw, m)
    res = np.zeros(bw - m)
    api.DLTNaive(data, bw, m, w, res, ptab, None)
    ref = oracle.dlt_naive(data, bw, m, w, ptab)
    assert np.abs(res - ref).max() <= 1e-12 * np.abs(ref).max()
    out = np.zeros(2 * bw)
    api.InvDLTNaive(coeffs, bw, m, out, ptab)
    ref = oracle.inv_dlt_naive(coeffs, bw, m, ptab)
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()


# ------------------------------------------------------------------ sphere transforms
@pytest.mark.parametrize("bw,cut,fmt", [(2, 2, 1), (2, 1, 0), (4, 4, 0), (8, 3, 1), (32, 32, 0), (64, 16, 1),
                                        (128, 128, 1), (12, 12, 0), (17, 17, 0), (9, 4, 1)])
def test_dropin_vs_oracle(oracle, bw, cut, fmt):
    rng = np.random.default_rng(bw * 7 + cut)
    n = 2 * bw
    rd = rng.standard_normal(n * n)
    idd = rng.standard_normal(n * n) if fmt == api.COMPLEX else np.zeros(n * n)
    fr, fi = _fst(rd, idd, bw, fmt, cut)
    orr, ori = oracle.fst(rd, idd, bw, fmt, cut)
    assert rel_err_norm(fr, fi, orr, ori) <= TOL
    if fmt == api.REAL:
        rc, ic = real_field_coeffs(rng, bw, 1.0)
    else:
        rc, ic = rng.standard_normal(bw * bw), rng.standard_normal(bw * bw)
    gr, gi = _inv(rc, ic, bw, fmt, cut)
    orr, ori = oracle.inv_fst(rc, ic, bw, fmt, cut)
    s = np.abs(orr).max()
    assert np.abs(gr - orr).max() <= TOL * s and np.abs(gi - ori).max() <= TOL * s


def test_single_function_roundtrip_bw64():
    """B=64 real field, N(0,1) coefficients with conjugate symmetry: InvFST then FST <= 1e-11."""
    rng = np.random.default_rng(2024)
    rc, ic = real_field_coeffs(rng, 64, 0.0)
    t, tt = _tables(64, 64)
    gr, gi = _inv(rc, ic, 64, api.REAL, 64, tt)
    fr, fi = _fst(gr, gi, 64, api.REAL, 64, t)
    assert rel_err_norm(fr, fi, rc, ic) <= 1e-11


# ------------------------------------------------------------------ batched device API
def _torch():
    import torch
    return torch


@pytest.mark.parametrize("bw,cut", [(64, 64), (32, 10), (256, 256)])
def test_batched_real_fast_path(oracle, bw, cut):
    torch = _torch()
    nb = 5
    rng = np.random.default_rng(bw)
    rc, ic = real_field_coeffs(rng, bw, 1.0, nfunc=nb)
    plan = api.Plan(bw, cut)
    d_rc = torch.from_numpy(rc).cuda()
    d_ic = torch.from_numpy(ic).cuda()
    grid = torch.zeros(nb, 4 * bw * bw, dtype=torch.float64, device="cuda")
    plan.inv_fst(d_rc, d_ic, grid, None, nb, api.REAL)  # real output only
    o_rc = torch.zeros_like(d_rc)
    o_ic = torch.zeros_like(d_ic)
    plan.fst(grid, None, o_rc, o_ic, nb, api.REAL)      # imaginary samples zero
    torch.cuda.synchronize()
    g = grid.cpu().numpy()
    for f in range(nb):
        er, ei = oracle.inv_fst(rc[f], ic[f], bw, api.REAL, cut)
        assert np.abs(g[f] - er).max() <= TOL * np.abs(er).max()
        orc, oic = oracle.fst(g[f], np.zeros_like(g[f]), bw, api.REAL, cut)
        assert rel_err_norm(o_rc[f].cpu().numpy(), o_ic[f].cpu().numpy(), orc, oic) <= TOL
        assert rel_err_norm(o_rc[f].cpu().numpy(), o_ic[f].cpu().numpy(), rc[f], ic[f]) <= 1e-10


def test_batched_complex_and_conv(oracle):
    torch = _torch()
    bw, nb = 32, 3
    rng = np.random.default_rng(11)
    n = 2 * bw
    rd = rng.standard_normal((nb, n * n))
    idd = rng.standard_normal((nb, n * n))
    plan = api.Plan(bw, bw)
    d = [torch.from_numpy(x).cuda() for x in (rd, idd)]
    rc = torch.zeros(nb, bw * bw, dtype=torch.float64, device="cuda")
    ic = torch.zeros_like(rc)
    plan.fst(d[0], d[1], rc, ic, nb, api.COMPLEX)
    gr = torch.zeros_like(d[0])
    gi = torch.zeros_like(d[0])
    plan.inv_fst(rc, ic, gr, gi, nb, api.COMPLEX)
    zr = torch.zeros(nb, bw, dtype=torch.float64, device="cuda")
    zi = torch.zeros_like(zr)
    plan.fzt(d[0], d[1], zr, zi, nb, api.COMPLEX)
    # convolution of each function with the next one's samples as filter
    filt = torch.roll(d[0], 1, 0).contiguous()
    cr = torch.zeros_like(d[0])
    ci = torch.zeros_like(d[0])
    plan.conv(d[0], torch.zeros_like(d[0]), filt, torch.zeros_like(filt), cr, ci, nb)
    torch.cuda.synchronize()
    for f in range(nb):
        orc, oic = oracle.fst(rd[f], idd[f], bw, api.COMPLEX, bw)
        assert rel_err_norm(rc[f].cpu().numpy(), ic[f].cpu().numpy(), orc, oic) <= TOL
        er, ei = oracle.inv_fst(orc, oic, bw, api.COMPLEX, bw)
        assert rel_err_norm(gr[f].cpu().numpy(), gi[f].cpu().numpy(), er, ei) <= TOL
        ozr, ozi = oracle.fzt(rd[f], idd[f], bw, api.COMPLEX)
        assert np.abs(zr[f].cpu().numpy() - ozr).max() <= TOL * np.abs(ozr).max()
        assert np.abs(zi[f].cpu().numpy() - ozi[:bw]).max() <= TOL * np.abs(ozi[:bw]).max()
        occ, _ = oracle.conv(rd[f], np.zeros(n * n), rd[(f - 1) % nb], np.zeros(n * n), bw)
        assert np.abs(cr[f].cpu().numpy() - occ).max() <= TOL * np.abs(occ).max()


def test_single_function_bw256_fwd_inv_conv(oracle):
    """B=256 real field, coefficients N(0,1)(1+l)^-1; forward+inverse and the zonal-filter
    convolution h_l^0 = exp(-l(l+1)/(2*40^2)) against the oracle."""
    torch = _torch()
    bw = 256
    rng = np.random.default_rng(256)
    rc, ic = real_field_coeffs(rng, bw, 1.0)
    l = np.arange(bw)
    hr, hi = np.zeros(bw * bw), np.zeros(bw * bw)
    hr[harmonic_index(0, l, bw)] = np.exp(-l * (l + 1) / (2 * 40.0 ** 2))
    fgrid, _ = oracle.inv_fst(hr, hi, bw, api.REAL, bw)
    plan = api.Plan(bw, bw)
    d_rc, d_ic = torch.from_numpy(rc).cuda(), torch.from_numpy(ic).cuda()
    grid = torch.zeros(4 * bw * bw, dtype=torch.float64, device="cuda")
    plan.inv_fst(d_rc, d_ic, grid, None, 1, api.REAL)
    o_rc, o_ic = torch.zeros_like(d_rc), torch.zeros_like(d_ic)
    plan.fst(grid, None, o_rc, o_ic, 1, api.REAL)
    out_r = torch.zeros_like(grid)
    out_i = torch.zeros_like(grid)
    z = torch.zeros_like(grid)
    plan.conv(grid, z, torch.from_numpy(fgrid).cuda(), z, out_r, out_i, 1)
    torch.cuda.synchronize()
    eg, _ = oracle.inv_fst(rc, ic, bw, api.REAL, bw)
    assert np.abs(grid.cpu().numpy() - eg).max() <= TOL * np.abs(eg).max()
    assert rel_err_norm(o_rc.cpu().numpy(), o_ic.cpu().numpy(), rc, ic) <= TOL
    oc, _ = oracle.conv(eg, np.zeros_like(eg), fgrid, np.zeros_like(fgrid), bw)
    assert np.abs(out_r.cpu().numpy() - oc).max() <= TOL * np.abs(oc).max()


def test_status_errors_on_gpu():
    import ctypes as C

    import s2kit_gb300 as s2
    lib = s2.load()
    h = C.c_void_p()
    assert lib.s2g_plan_create(C.byref(h), 64, 0) == 1
    plan = api.Plan(16, 16)
    with pytest.raises(s2.S2GError):
        plan.fst(None, None, None, None, 1)
    with pytest.raises(s2.S2GError):
        plan.fst(1, None, 1, 1, 0)  # batch 0


@pytest.mark.parametrize("bw,fmt", [(31, api.REAL), (48, api.COMPLEX), (127, api.REAL), (255, api.COMPLEX)])
def test_fp64_non_power_of_two_bandwidths_vs_oracle(oracle, bw, fmt):
    """Odd and non-power-of-two bandwidths on the batched FP64 path, whose length-2bw DFTs run as
    Bluestein convolutions (power-of-two FFTs against precomputed chirp spectra), against the
    oracle, both directions, to the FP64 parity bar."""
    torch = _torch()
    nb = 2
    rng = np.random.default_rng(bw)
    if fmt == api.REAL:
        rc, ic = real_field_coeffs(rng, bw, 1.0, nfunc=nb)
    else:
        rc, ic = rng.standard_normal((nb, bw * bw)), rng.standard_normal((nb, bw * bw))
    plan = api.Plan(bw, bw)
    d_rc, d_ic = torch.from_numpy(rc).cuda(), torch.from_numpy(ic).cuda()
    gr = torch.zeros(nb, 4 * bw * bw, dtype=torch.float64, device="cuda")
    gi = torch.zeros_like(gr)
    plan.inv_fst(d_rc, d_ic, gr, gi if fmt == api.COMPLEX else None, nb, fmt)
    o_r, o_i = torch.zeros_like(d_rc), torch.zeros_like(d_ic)
    plan.fst(gr, gi if fmt == api.COMPLEX else None, o_r, o_i, nb, fmt)
    torch.cuda.synchronize()
    for f in range(nb):
        er, ei = oracle.inv_fst(rc[f], ic[f], bw, fmt, bw)
        g_r = gr[f].cpu().numpy()
        g_i = gi[f].cpu().numpy() if fmt == api.COMPLEX else np.zeros_like(g_r)
        if fmt == api.REAL:
            ei = np.zeros_like(er)
        assert rel_err_norm(g_r, g_i, er, ei) <= TOL
        assert rel_err_norm(o_r[f].cpu().numpy(), o_i[f].cpu().numpy(), rc[f], ic[f]) <= TOL
