"""COMPLEX data on the split-precision path (s2g_fst_complex_f32 / s2g_inv_fst_complex_f32)
against the oracle's COMPLEX FSTSemiMemo / InvFSTSemiMemo (FST_semi_memo.c:146-200, 290-333), the
reference-generated COMPLEX fixture, and the FP64 GPU path at larger bandwidths.

Error metric: normwise relative error max|x - x_ref| / max|x_ref| per function.  Tolerances as the
real-field split path: BF16X3 <= 1e-6, BF16X2 <= 1e-4, FP16X2 <= 2e-6 (bw <= 256).
"""
import ctypes as C

import numpy as np
import pytest

from s2kit_gb300 import api
from s2kit_gb300._lib import load
from tests._util import rel_err_norm

pytestmark = pytest.mark.gpu
S2G_ERR_ARG = 1
TOL = {api.PREC_BF16X3: 1e-6, api.PREC_BF16X2: 1e-4, api.PREC_FP16X2: 2e-6}


def _torch():
    import torch
    return torch


def _complex_coeffs(rng, bw, nb, p=1.0):
    """Independent complex coefficients for every (l, m): a band-limited complex field."""
    from tests._util import degree_of_index
    ls, _ = degree_of_index(bw)
    s = (1.0 + ls) ** (-p)
    return rng.standard_normal((nb, bw * bw)) * s, rng.standard_normal((nb, bw * bw)) * s


def _run(plan, gr, gi, cr, ci, nb, prec):
    """Split forward of the FP32 grids and split inverse of the FP32 coefficients."""
    torch = _torch()
    bw = plan.bw
    d = [torch.as_tensor(x).float().cuda().contiguous() for x in (gr, gi, cr, ci)]
    o_r = torch.full((nb, bw * bw), float("nan"), dtype=torch.float32, device="cuda")
    o_i = torch.full_like(o_r, float("nan"))
    plan.fst_complex_f32(d[0], d[1], o_r, o_i, nb, prec)
    s_r = torch.full((nb, 4 * bw * bw), float("nan"), dtype=torch.float32, device="cuda")
    s_i = torch.full_like(s_r, float("nan"))
    plan.inv_fst_complex_f32(d[2], d[3], s_r, s_i, nb, prec)
    torch.cuda.synchronize()
    return [x.double().cpu().numpy() for x in (o_r, o_i, s_r, s_i)]


@pytest.mark.parametrize("bw,nb", [(16, 3), (32, 2), (33, 2)])  # bw 33: chirp-z stages
@pytest.mark.parametrize("prec", [api.PREC_BF16X3, api.PREC_BF16X2, api.PREC_FP16X2])
def test_split_complex_vs_oracle(oracle, bw, nb, prec):
    rng = np.random.default_rng(1000 + bw)
    cr, ci = _complex_coeffs(rng, bw, nb)
    grids = [oracle.inv_fst(cr[f], ci[f], bw, api.COMPLEX, bw) for f in range(nb)]
    gr = np.stack([g[0] for g in grids])
    gi = np.stack([g[1] for g in grids])
    plan = api.Plan(bw, bw)
    o_r, o_i, s_r, s_i = _run(plan, gr, gi, cr, ci, nb, prec)
    for f in range(nb):
        assert rel_err_norm(o_r[f], o_i[f], cr[f], ci[f]) <= TOL[prec]
        assert rel_err_norm(s_r[f], s_i[f], gr[f], gi[f]) <= TOL[prec]


def test_split_complex_reference_fixture(golden):
    """bw 64 COMPLEX fixture made by the reference (cutoff 16; the coefficients do not depend on it)."""
    g = golden("ref_sht_bw64_cut16_complex")
    bw = int(g["bw"])
    plan = api.Plan(bw, bw)
    o_r, o_i, s_r, s_i = _run(plan, g["inv_r"][None], g["inv_i"][None], g["rcoeffs"][None], g["icoeffs"][None], 1,
                              api.PREC_BF16X3)
    assert rel_err_norm(o_r[0], o_i[0], g["rt_r"], g["rt_i"]) <= 1e-6
    assert rel_err_norm(s_r[0], s_i[0], g["inv_r"], g["inv_i"]) <= 1e-6
    # the noise grid is not band-limited: its forward transform is still the reference's
    torch = _torch()
    n_r = torch.from_numpy(g["noise_r"]).float().cuda()[None].contiguous()
    n_i = torch.from_numpy(g["noise_i"]).float().cuda()[None].contiguous()
    f_r = torch.zeros(1, bw * bw, dtype=torch.float32, device="cuda")
    f_i = torch.zeros_like(f_r)
    plan.fst_complex_f32(n_r, n_i, f_r, f_i, 1, api.PREC_BF16X3)
    torch.cuda.synchronize()
    assert rel_err_norm(f_r[0].double().cpu().numpy(), f_i[0].double().cpu().numpy(), g["fwd_noise_r"],
                        g["fwd_noise_i"]) <= 1e-6


@pytest.mark.parametrize("bw,nb", [(128, 5), (256, 3), (512, 2), (101, 3), (100, 2)])  # 100: 4 does not divide bw(bw+1)/2
def test_split_complex_vs_fp64_path(bw, nb):
    torch = _torch()
    rng = np.random.default_rng(7 + bw)
    cr, ci = _complex_coeffs(rng, bw, nb)
    plan = api.Plan(bw, bw)
    d_cr, d_ci = torch.from_numpy(cr).cuda(), torch.from_numpy(ci).cuda()
    gr = torch.zeros(nb, 4 * bw * bw, dtype=torch.float64, device="cuda")
    gi = torch.zeros_like(gr)
    plan.inv_fst(d_cr, d_ci, gr, gi, nb, api.COMPLEX)
    torch.cuda.synchronize()
    o_r, o_i, s_r, s_i = _run(plan, gr.cpu().numpy(), gi.cpu().numpy(), cr, ci, nb, api.PREC_BF16X3)
    tol = 1e-6 if bw <= 256 else 2e-6
    gr, gi = gr.cpu().numpy(), gi.cpu().numpy()
    for f in range(nb):
        assert rel_err_norm(o_r[f], o_i[f], cr[f], ci[f]) <= tol
        assert rel_err_norm(s_r[f], s_i[f], gr[f], gi[f]) <= tol


@pytest.mark.parametrize("prec", [api.PREC_BF16X3, api.PREC_FP16X2])
def test_split_complex_of_real_field_is_the_real_transform(prec):
    """With a zero imaginary field the combine reduces to the real path's symmetric fill: bit for bit."""
    torch = _torch()
    bw, nb = 64, 4
    g = torch.randn(nb, 4 * bw * bw, generator=torch.Generator().manual_seed(5)).float().cuda()
    z = torch.zeros_like(g)
    plan = api.Plan(bw, bw)
    a_r = torch.zeros(nb, bw * bw, dtype=torch.float32, device="cuda")
    a_i, b_r, b_i = torch.zeros_like(a_r), torch.zeros_like(a_r), torch.zeros_like(a_r)
    plan.fst_real_f32(g, a_r, a_i, nb, prec)
    plan.fst_complex_f32(g, z, b_r, b_i, nb, prec)
    torch.cuda.synchronize()
    assert torch.equal(a_r, b_r) and torch.equal(a_i, b_i)
    # inverse: the split gives g = f exactly and h = 0 exactly (f(l,-m) was written as (-1)^m conj f(l,m)),
    # so the real field comes back bit for bit and the imaginary field is exactly zero
    s_r, s_i = torch.zeros_like(g), torch.full_like(g, float("nan"))
    plan.inv_fst_complex_f32(a_r, a_i, s_r, s_i, nb, prec)
    t = torch.zeros_like(g)
    plan.inv_fst_real_f32(a_r, a_i, t, nb, prec)
    torch.cuda.synchronize()
    assert torch.count_nonzero(s_i).item() == 0
    assert torch.equal(s_r, t)


def test_split_complex_rejects_misaligned_pointers():
    torch = _torch()
    bw = 16
    plan = api.Plan(bw, bw)
    g = torch.zeros(4 * bw * bw + 4, dtype=torch.float32, device="cuda")
    c = torch.zeros(bw * bw, dtype=torch.float32, device="cuda")
    lib = load()
    rc = lib.s2g_fst_complex_f32(plan.h, C.c_void_p(g.data_ptr() + 4), C.c_void_p(g.data_ptr()),
                                 C.c_void_p(c.data_ptr()), C.c_void_p(c.data_ptr()), 1, api.PREC_BF16X3, None)
    assert rc == S2G_ERR_ARG
    assert b"aligned" in lib.s2g_last_error()
