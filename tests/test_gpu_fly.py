"""On-the-fly drop-ins (FSTSemiFly, InvFSTSemiFly, FZTSemiFly, ConvOn2SphereSemiFly; reference
src/FST_semi_fly.c) through the C ABI, against the reference's own outputs (ref_fly.npz, made by
tests/golden/make_golden.py from the unmodified reference build) and against the memo drop-ins.
Tolerance: the FP64 parity bar, normwise 1e-11."""
import numpy as np
import pytest

from oracle.oracle import COMPLEX, REAL
from s2kit_gb300 import api
from tests._util import real_field_coeffs, rel_err_norm

pytestmark = pytest.mark.gpu
TOL = 1e-11
CASES = [(16, 16, REAL), (16, 6, COMPLEX), (32, 32, REAL), (32, 20, COMPLEX)]


def _weights(bw):
    w = np.zeros(4 * bw)
    api.GenerateWeightsForDLT(bw, w)
    return w


@pytest.mark.parametrize("bw,cut,fmt", CASES)
def test_fly_forward_inverse_vs_reference(golden, bw, cut, fmt):
    g = golden("ref_fly")
    tag = f"bw{bw}_cut{cut}_{'real' if fmt else 'complex'}"
    rc, ic = np.zeros(bw * bw), np.zeros(bw * bw)
    ws = np.zeros(10 * bw * bw + 24 * bw)
    api.FSTSemiFly(np.ascontiguousarray(g[f"{tag}_grid_r"]), np.ascontiguousarray(g[f"{tag}_grid_i"]), rc, ic, bw,
                   ws, fmt, cut, None, None, _weights(bw))
    assert rel_err_norm(rc, ic, g[f"{tag}_fst_r"], g[f"{tag}_fst_i"]) <= TOL
    rd, idd = np.zeros(4 * bw * bw), np.zeros(4 * bw * bw)
    api.InvFSTSemiFly(np.ascontiguousarray(g[f"{tag}_coef_r"]), np.ascontiguousarray(g[f"{tag}_coef_i"]), rd, idd,
                      bw, ws, fmt, cut)
    assert rel_err_norm(rd, idd, g[f"{tag}_inv_r"], g[f"{tag}_inv_i"]) <= TOL


def test_fly_fzt_and_conv_vs_reference(golden):
    g = golden("ref_fly")
    bw = 16
    for fmt, key in ((COMPLEX, "complex"), (REAL, "real")):
        rr, ri = np.zeros(2 * bw), np.full(2 * bw, np.nan)
        api.FZTSemiFly(np.ascontiguousarray(g["fzt_bw16_data_r"]), np.ascontiguousarray(g["fzt_bw16_data_i"]), rr,
                       ri, bw, np.zeros(2 * bw * bw + 16 * bw), fmt, None, _weights(bw))
        assert rel_err_norm(rr[:bw], ri[:bw], g[f"fzt_bw16_{key}_r"][:bw], g[f"fzt_bw16_{key}_i"][:bw]) <= TOL
        if fmt == REAL:  # the reference writes 2*bw imaginary zeros (FST_semi_fly.c:424)
            assert (ri == 0).all()
    z = np.zeros(4 * bw * bw)
    cr, ci = np.zeros(4 * bw * bw), np.zeros(4 * bw * bw)
    api.ConvOn2SphereSemiFly(np.ascontiguousarray(g["conv_bw16_signal"]), z, np.ascontiguousarray(g["conv_bw16_filter"]),
                             z.copy(), cr, ci, bw, np.zeros(14 * bw * bw + 26 * bw))
    assert rel_err_norm(cr, ci, g["conv_bw16_out_r"], g["conv_bw16_out_i"]) <= TOL


@pytest.mark.parametrize("bw,cut,fmt", [(64, 64, REAL), (64, 24, COMPLEX), (128, 128, REAL)])
def test_fly_matches_memo(bw, cut, fmt):
    """Fly and memo drop-ins give the same transforms (the memo one on the caller's table).  The
    fly kernels use the naive form at every order and the memo path the seminaive one below the
    cutoff: equal in exact arithmetic, apart by their FP64 rounding (2.3e-13 measured at bw 128
    on noise), held to 1e-12."""
    rng = np.random.default_rng(bw + cut)
    n = 2 * bw
    rd = rng.standard_normal(n * n)
    idd = rng.standard_normal(n * n) if fmt == COMPLEX else np.zeros(n * n)
    size = api.Reduced_Naive_TableSize(bw, cut) + api.Reduced_SpharmonicTableSize(bw, cut)
    fwd_space, inv_space = np.zeros(size), np.zeros(size)
    t = api.SemiNaive_Naive_Pml_Table(bw, cut, fwd_space, None)
    tt = api.Transpose_SemiNaive_Naive_Pml_Table(t, bw, cut, inv_space, None)
    a_r, a_i = np.zeros(bw * bw), np.zeros(bw * bw)
    api.FSTSemiMemo(rd, idd, a_r, a_i, bw, t, None, fmt, cut, None, None, _weights(bw))
    b_r, b_i = np.zeros(bw * bw), np.zeros(bw * bw)
    api.FSTSemiFly(rd, idd, b_r, b_i, bw, None, fmt, cut, None, None, _weights(bw))
    assert rel_err_norm(b_r, b_i, a_r, a_i) <= 1e-12
    g1r, g1i = np.zeros(n * n), np.zeros(n * n)
    api.InvFSTSemiMemo(a_r, a_i, g1r, g1i, bw, tt, None, fmt, cut)
    g2r, g2i = np.zeros(n * n), np.zeros(n * n)
    api.InvFSTSemiFly(a_r, a_i, g2r, g2i, bw, None, fmt, cut)
    assert rel_err_norm(g2r, g2i, g1r, g1i) <= 1e-12


@pytest.mark.parametrize("bw,fmt,nb", [(100, COMPLEX, 2), (255, REAL, 2), (256, COMPLEX, 8), (64, REAL, 9)])
def test_fly_plan_vs_oracle(oracle, bw, fmt, nb):
    """The batched on-the-fly plan (s2g_plan_create_fly) against the oracle, both directions and
    FZT, at odd / non-power-of-two and power-of-two bandwidths and batches that are not a
    multiple of the kernels' function groups."""
    import torch
    rng = np.random.default_rng(bw * 7 + nb)
    n = 2 * bw
    rd = rng.standard_normal((nb, n * n))
    idd = rng.standard_normal((nb, n * n)) if fmt == COMPLEX else np.zeros((nb, n * n))
    if fmt == REAL:
        rc, ic = real_field_coeffs(rng, bw, 1.0, nfunc=nb)
    else:
        rc, ic = rng.standard_normal((nb, bw * bw)), rng.standard_normal((nb, bw * bw))
    plan = api.Plan(bw, fly=True)
    d_rd, d_id = torch.from_numpy(rd).cuda(), torch.from_numpy(idd).cuda()
    o_r = torch.full((nb, bw * bw), float("nan"), dtype=torch.float64, device="cuda")
    o_i = torch.full_like(o_r, float("nan"))
    plan.fst(d_rd, d_id if fmt == COMPLEX else None, o_r, o_i, nb, fmt)
    g_r = torch.full((nb, n * n), float("nan"), dtype=torch.float64, device="cuda")
    g_i = torch.full_like(g_r, float("nan"))
    plan.inv_fst(torch.from_numpy(rc).cuda(), torch.from_numpy(ic).cuda(), g_r, g_i if fmt == COMPLEX else None, nb,
                 fmt)
    z_r = torch.full((nb, bw), float("nan"), dtype=torch.float64, device="cuda")
    z_i = torch.full_like(z_r, float("nan"))
    plan.fzt(d_rd, d_id, z_r, z_i, nb, fmt)
    torch.cuda.synchronize()
    for f in range(nb):
        er, ei = oracle.fst(rd[f], idd[f], bw, fmt, bw)
        assert rel_err_norm(o_r[f].cpu().numpy(), o_i[f].cpu().numpy(), er, ei) <= TOL
        gr, gi = oracle.inv_fst(rc[f], ic[f], bw, fmt, bw)
        got_i = g_i[f].cpu().numpy() if fmt == COMPLEX else np.zeros(n * n)
        if fmt == REAL:
            gi = np.zeros(n * n)
        assert rel_err_norm(g_r[f].cpu().numpy(), got_i, gr, gi) <= TOL
        zr, zi = oracle.fzt(rd[f], idd[f], bw, fmt)
        got_zi = z_i[f].cpu().numpy()
        assert rel_err_norm(z_r[f].cpu().numpy(), got_zi, zr, zi[:bw] if fmt == COMPLEX else np.zeros(bw)) <= TOL


def test_fly_plan_rejects_split_entry_points():
    import torch
    plan = api.Plan(64, fly=True)
    x = torch.zeros(1, 4 * 64 * 64, dtype=torch.float32, device="cuda")
    c = torch.zeros(1, 64 * 64, dtype=torch.float32, device="cuda")
    with pytest.raises(RuntimeError, match="on-the-fly plan"):
        plan.fst_real_f32(x, c, c.clone(), 1, api.PREC_BF16X3)
