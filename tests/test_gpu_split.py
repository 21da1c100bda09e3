"""Split-BF16 tensor-core path (tcgen05) vs the FP64 path and the oracle, through the C ABI.

Error metric: normwise relative error max|x - x_ref| / max|x_ref| per function (coefficients
for the forward, samples for the inverse), reference = FP64.  Stated tolerances:
  S2G_PREC_BF16X3 (6 split products, FP32 FFT/DCT): <= 1e-6   (the headline tolerance)
  S2G_PREC_BF16X2 (3 split products):               <= 1e-4
  S2G_PREC_FP16X2 (2-term FP16, 3 products):        <= 2e-6 for bw <= 256, <= 5e-6 at bw 512
    (two FP16 terms hold 22 bits: about 2^-22 per product before cancellation in the sums)
"""
import numpy as np
import pytest

from s2kit_gb300 import api
from tests._util import real_field_coeffs

pytestmark = pytest.mark.gpu
TOL = {api.PREC_BF16X3: 1e-6, api.PREC_BF16X2: 1e-4, api.PREC_FP16X2: 2e-6}


def _torch():
    import torch
    return torch


@pytest.mark.parametrize("n,k", [(16, 16), (64, 32), (128, 64), (256, 32), (32, 128)])
def test_tc_selftest_tile(n, k):
    torch = _torch()
    g = torch.Generator(device="cpu").manual_seed(n * 1000 + k)
    A = torch.randn(128, k, generator=g, dtype=torch.float32)
    B = torch.randn(n, k, generator=g, dtype=torch.float32)
    ref = A.double() @ B.double().T
    dA, dB = A.cuda(), B.cuda()
    scale = ref.abs().max().item()
    errs = {}
    for nprod in (1, 3, 6):
        D = torch.zeros(128, n, dtype=torch.float32, device="cuda")
        api.selftest_tc(dA, dB, D, nprod)
        torch.cuda.synchronize()
        errs[nprod] = (D.double().cpu() - ref).abs().max().item() / scale
    assert errs[1] < 3e-2
    assert errs[3] < 1e-4
    assert errs[6] < 2e-6, errs


def _fp64_pair(plan, rc, ic):
    """FP64 grid of the coefficients and FP64 forward of that grid (device API)."""
    torch = _torch()
    nb = rc.shape[0]
    d_rc, d_ic = torch.from_numpy(rc).cuda(), torch.from_numpy(ic).cuda()
    grid = torch.zeros(nb, 4 * plan.bw ** 2, dtype=torch.float64, device="cuda")
    plan.inv_fst(d_rc, d_ic, grid, None, nb, api.REAL)
    o_rc, o_ic = torch.zeros_like(d_rc), torch.zeros_like(d_ic)
    plan.fst(grid, None, o_rc, o_ic, nb, api.REAL)
    torch.cuda.synchronize()
    return grid, o_rc, o_ic


def _nerr(got, ref):
    torch = _torch()
    d = (got.double() - ref).abs().amax(dim=1)
    return (d / ref.abs().amax(dim=1)).max().item()


@pytest.mark.parametrize("bw,nb", [(16, 3), (32, 70), (64, 10), (128, 65), (256, 130), (512, 2),
                                   # multiples of 16 that are not powers of two (transform lengths
                                   # 32 R, R = 3 .. 15; bw 144 and 240 have a partial naive block)
                                   (48, 5), (80, 70), (112, 3), (144, 65), (192, 33), (208, 2), (240, 4),
                                   # chirp-z lengths (odd bw, and even bw that no warp FFT takes), one per
                                   # convolution length M = 128 .. 1024 at least
                                   (17, 3), (24, 5), (33, 66), (100, 2), (127, 65), (200, 3), (255, 33)])
@pytest.mark.parametrize("prec", [api.PREC_BF16X3, api.PREC_BF16X2, api.PREC_FP16X2])
def test_split_forward_inverse_vs_fp64(bw, nb, prec):
    torch = _torch()
    rng = np.random.default_rng(bw + nb)
    rc, ic = real_field_coeffs(rng, bw, 1.0, nfunc=nb)
    plan = api.Plan(bw, bw)
    grid64, frc64, fic64 = _fp64_pair(plan, rc, ic)
    # forward: FP32 samples of the FP64 grid
    g32 = grid64.float()
    s_rc = torch.full((nb, bw * bw), float("nan"), dtype=torch.float32, device="cuda")
    s_ic = torch.full_like(s_rc, float("nan"))
    plan.fst_real_f32(g32, s_rc, s_ic, nb, prec)
    # inverse: FP32 coefficients
    c32r, c32i = torch.from_numpy(rc).float().cuda(), torch.from_numpy(ic).float().cuda()
    s_grid = torch.full((nb, 4 * bw * bw), float("nan"), dtype=torch.float32, device="cuda")
    plan.inv_fst_real_f32(c32r, c32i, s_grid, nb, prec)
    plan.sync_status()
    assert torch.isfinite(s_rc).all() and torch.isfinite(s_ic).all() and torch.isfinite(s_grid).all()
    # coefficients compared as complex magnitudes
    ref_mag = torch.hypot(frc64, fic64).amax(dim=1)
    e_fwd = (torch.hypot(s_rc.double() - frc64, s_ic.double() - fic64).amax(dim=1) / ref_mag).max().item()
    e_inv = _nerr(s_grid, grid64)
    tol = 5e-6 if (prec == api.PREC_FP16X2 and bw > 256) else TOL[prec]
    assert e_fwd <= tol, e_fwd
    assert e_inv <= tol, e_inv


@pytest.mark.parametrize("bw", list(range(16, 257, 13)))
@pytest.mark.parametrize("prec", [api.PREC_BF16X3, api.PREC_FP16X2])
def test_split_bandwidth_sweep_vs_fp64(bw, prec):
    """Every 13th bandwidth from 16 to 250 (odd and even, warp-FFT and chirp-z lengths, full and
    partial naive blocks): two functions forward and inverse against the FP64 path, BF16X3 and
    FP16X2 at their stated tolerances."""
    torch = _torch()
    nb = 2
    rng = np.random.default_rng(1000 + bw)
    rc, ic = real_field_coeffs(rng, bw, 1.0, nfunc=nb)
    plan = api.Plan(bw, bw)
    grid64, frc64, fic64 = _fp64_pair(plan, rc, ic)
    s_rc = torch.full((nb, bw * bw), float("nan"), dtype=torch.float32, device="cuda")
    s_ic = torch.full_like(s_rc, float("nan"))
    plan.fst_real_f32(grid64.float(), s_rc, s_ic, nb, prec)
    s_grid = torch.full((nb, 4 * bw * bw), float("nan"), dtype=torch.float32, device="cuda")
    plan.inv_fst_real_f32(torch.from_numpy(rc).float().cuda(), torch.from_numpy(ic).float().cuda(), s_grid, nb,
                          prec)
    plan.sync_status()
    ref_mag = torch.hypot(frc64, fic64).amax(dim=1)
    e_fwd = (torch.hypot(s_rc.double() - frc64, s_ic.double() - fic64).amax(dim=1) / ref_mag).max().item()
    e_inv = _nerr(s_grid, grid64)
    assert e_fwd <= TOL[prec] and e_inv <= TOL[prec], (e_fwd, e_inv)


@pytest.mark.parametrize("bw", [96, 192, 31, 101, 255])
def test_split_non_power_of_two_vs_oracle(oracle, bw):
    """Bandwidths that are not powers of two on the split path against the oracle directly: lengths
    2 bw = 32 R (R = 6 and 12: the warp FFTs' direct register DFT) and odd bandwidths (chirp-z
    transforms), forward of the oracle's samples and inverse of the coefficients, BF16X3 tolerance.
    The reference's own inverse is wrong at odd bw (Transpose_RowSize, cospml.c:270-288); the
    oracle uses the true row counts and reproduces the reference's odd-bw forward known answers."""
    torch = _torch()
    nb = 2
    rng = np.random.default_rng(bw)
    rc, ic = real_field_coeffs(rng, bw, 1.0, nfunc=nb)
    grids = np.stack([oracle.inv_fst(rc[f], ic[f], bw, api.REAL, bw)[0] for f in range(nb)])
    plan = api.Plan(bw, bw)
    s_rc = torch.zeros(nb, bw * bw, dtype=torch.float32, device="cuda")
    s_ic = torch.zeros_like(s_rc)
    plan.fst_real_f32(torch.from_numpy(grids).float().cuda(), s_rc, s_ic, nb, api.PREC_BF16X3)
    s_grid = torch.zeros(nb, 4 * bw * bw, dtype=torch.float32, device="cuda")
    plan.inv_fst_real_f32(torch.from_numpy(rc).float().cuda(), torch.from_numpy(ic).float().cuda(), s_grid, nb,
                          api.PREC_BF16X3)
    plan.sync_status()
    mag = np.hypot(rc, ic).max(axis=1)
    e_f = (np.hypot(s_rc.double().cpu().numpy() - rc, s_ic.double().cpu().numpy() - ic).max(axis=1) / mag).max()
    e_i = (np.abs(s_grid.double().cpu().numpy() - grids).max(axis=1) / np.abs(grids).max(axis=1)).max()
    assert e_f <= TOL[api.PREC_BF16X3] and e_i <= TOL[api.PREC_BF16X3], (e_f, e_i)


def test_split_matches_oracle_and_roundtrip(oracle):
    torch = _torch()
    bw, nb = 64, 4
    rng = np.random.default_rng(5)
    rc, ic = real_field_coeffs(rng, bw, 1.5, nfunc=nb)
    plan = api.Plan(bw, bw)
    c32r, c32i = torch.from_numpy(rc).float().cuda(), torch.from_numpy(ic).float().cuda()
    grid = torch.zeros(nb, 4 * bw * bw, dtype=torch.float32, device="cuda")
    plan.inv_fst_real_f32(c32r, c32i, grid, nb, api.PREC_BF16X3)
    o_rc, o_ic = torch.zeros_like(c32r), torch.zeros_like(c32i)
    plan.fst_real_f32(grid, o_rc, o_ic, nb, api.PREC_BF16X3)
    plan.sync_status()
    g = grid.double().cpu().numpy()
    for f in range(nb):
        er, _ = oracle.inv_fst(rc[f], ic[f], bw, api.REAL, bw)
        assert np.abs(g[f] - er).max() <= 1e-6 * np.abs(er).max()
        mag = np.hypot(rc[f], ic[f]).max()
        d = np.hypot(o_rc[f].double().cpu().numpy() - rc[f], o_ic[f].double().cpu().numpy() - ic[f]).max()
        assert d <= 2e-6 * mag


@pytest.mark.parametrize("nb", [2, 17])
def test_split_bw1024_forward_inverse_vs_fp64(nb):
    """bw 1024 (2048-point transforms as two 1024-point four-step FFTs and a radix-2 step)."""
    torch = _torch()
    bw = 1024
    rng = np.random.default_rng(1024 + nb)
    rc, ic = real_field_coeffs(rng, bw, 1.0, nfunc=nb)
    plan = api.Plan(bw, bw)
    grid64, frc64, fic64 = _fp64_pair(plan, rc, ic)
    s_rc = torch.full((nb, bw * bw), float("nan"), dtype=torch.float32, device="cuda")
    s_ic = torch.full_like(s_rc, float("nan"))
    plan.fst_real_f32(grid64.float(), s_rc, s_ic, nb, api.PREC_BF16X3)
    s_grid = torch.full((nb, 4 * bw * bw), float("nan"), dtype=torch.float32, device="cuda")
    plan.inv_fst_real_f32(torch.from_numpy(rc).float().cuda(), torch.from_numpy(ic).float().cuda(), s_grid, nb,
                          api.PREC_BF16X3)
    torch.cuda.synchronize()
    plan.sync_status()
    mag = torch.hypot(frc64, fic64).amax(dim=1)
    e_f = (torch.hypot(s_rc.double() - frc64, s_ic.double() - fic64).amax(dim=1) / mag).max().item()
    e_i = _nerr(s_grid, grid64)
    assert e_f <= 2e-6 and e_i <= 2e-6, (e_f, e_i)


def test_split_repeated_runs_are_bit_identical():
    """40 forward and 40 inverse runs at bw 256 give identical bits: the pipelines have no ordering
    race (an unordered reuse of a staging buffer shows up as run-to-run differences in a few rows)."""
    torch = _torch()
    bw, nb = 256, 64
    rng = np.random.default_rng(40)
    rc, ic = real_field_coeffs(rng, bw, 1.0, nfunc=nb)
    plan = api.Plan(bw, bw)
    c_r, c_i = torch.from_numpy(rc).float().cuda(), torch.from_numpy(ic).float().cuda()
    g0 = torch.empty(nb, 4 * bw * bw, dtype=torch.float32, device="cuda")
    plan.inv_fst_real_f32(c_r, c_i, g0, nb, api.PREC_BF16X3)
    f0r, f0i = torch.empty_like(c_r), torch.empty_like(c_i)
    plan.fst_real_f32(g0, f0r, f0i, nb, api.PREC_BF16X3)
    g, fr, fi = torch.empty_like(g0), torch.empty_like(f0r), torch.empty_like(f0i)
    bad = 0
    for _ in range(40):
        plan.inv_fst_real_f32(c_r, c_i, g, nb, api.PREC_BF16X3)
        plan.fst_real_f32(g0, fr, fi, nb, api.PREC_BF16X3)
        bad += int(not torch.equal(g, g0)) + int(not (torch.equal(fr, f0r) and torch.equal(fi, f0i)))
    plan.sync_status()
    assert bad == 0, bad


def test_contraction_wait_timeout_is_reported_and_recoverable():
    """The failure path without a fault: with the test hook on, the contraction's scheduler publishes
    no work, every other role's bounded wait runs out (about half a second), the kernel records
    S2G_ERR_TIMEOUT and returns.  The status reaches the host, and the next transform is correct."""
    import s2kit_gb300 as s2
    torch = _torch()
    lib = s2.load()
    bw, nb = 64, 2
    rng = np.random.default_rng(77)
    rc, ic = real_field_coeffs(rng, bw, 1.0, nfunc=nb)
    plan = api.Plan(bw, bw)
    grid64, frc64, fic64 = _fp64_pair(plan, rc, ic)
    g32 = grid64.float()
    s_rc = torch.zeros(nb, bw * bw, dtype=torch.float32, device="cuda")
    s_ic = torch.zeros_like(s_rc)
    assert lib.s2g_test_stall_contraction(1) == 0
    try:
        plan.fst_real_f32(g32, s_rc, s_ic, nb, api.PREC_BF16X3)  # queued: returns at once
        status = lib.s2g_plan_sync_status(plan.h)
    finally:
        lib.s2g_test_stall_contraction(0)
    assert status == 5, status  # S2G_ERR_TIMEOUT, read and cleared
    assert lib.s2g_plan_sync_status(plan.h) == 0
    plan.fst_real_f32(g32, s_rc, s_ic, nb, api.PREC_BF16X3)
    plan.sync_status()
    mag = torch.hypot(frc64, fic64).amax(dim=1)
    e = (torch.hypot(s_rc.double() - frc64, s_ic.double() - fic64).amax(dim=1) / mag).max().item()
    assert e <= 1e-6, e


def test_split_host_api_matches_device_api():
    torch = _torch()
    bw, nb = 64, 150  # several pipeline chunks
    rng = np.random.default_rng(9)
    rc, ic = real_field_coeffs(rng, bw, 1.0, nfunc=nb)
    rc32, ic32 = rc.astype(np.float32), ic.astype(np.float32)
    plan = api.Plan(bw, bw)
    grid_h = np.zeros((nb, 4 * bw * bw), dtype=np.float32)
    plan.inv_fst_real_f32_host(rc32, ic32, grid_h, nb, api.PREC_BF16X3)
    orc_h, oic_h = np.zeros_like(rc32), np.zeros_like(ic32)
    plan.fst_real_f32_host(grid_h, orc_h, oic_h, nb, api.PREC_BF16X3)
    d_grid = torch.zeros(nb, 4 * bw * bw, dtype=torch.float32, device="cuda")
    plan.inv_fst_real_f32(torch.from_numpy(rc32).cuda(), torch.from_numpy(ic32).cuda(), d_grid, nb,
                          api.PREC_BF16X3)
    torch.cuda.synchronize()
    assert np.array_equal(d_grid.cpu().numpy(), grid_h)
    d_rc = torch.zeros(nb, bw * bw, dtype=torch.float32, device="cuda")
    d_ic = torch.zeros_like(d_rc)
    plan.fst_real_f32(torch.from_numpy(grid_h).cuda(), d_rc, d_ic, nb, api.PREC_BF16X3)
    torch.cuda.synchronize()
    assert np.array_equal(d_rc.cpu().numpy(), orc_h) and np.array_equal(d_ic.cpu().numpy(), oic_h)


def test_split_rejects_unsupported():
    import s2kit_gb300 as s2
    torch = _torch()
    for bw in (8, 272, 300):  # below 16, and above 256 without being a power of two
        plan = api.Plan(bw, bw)
        x = torch.zeros(4 * bw * bw, device="cuda")
        with pytest.raises(s2.S2GError):
            plan.fst_real_f32(x, x, x, 1, api.PREC_BF16X3)
    plan64 = api.Plan(64, 64)
    with pytest.raises(s2.S2GError):
        plan64.fst_real_f32(x, x, x, 1, 7)  # unknown precision


@pytest.mark.parametrize("bw,nb", [(16, 70), (64, 130), (192, 33), (256, 64), (512, 3)])
@pytest.mark.parametrize("prec", [api.PREC_BF16X3, api.PREC_FP16X2])
def test_contraction_kernels_agree_bitwise(bw, nb, prec):
    """The warp-specialised kernel's two data paths (tensor-map TMA and per-thread cp.async) do the
    same arithmetic per work item: forward and inverse outputs are identical bit for bit."""
    torch = _torch()
    lib = api.load()
    rng = np.random.default_rng(bw * 7 + nb)
    rc, ic = real_field_coeffs(rng, bw, 1.0, nfunc=nb)
    plan = api.Plan(bw, bw)
    c32r, c32i = torch.from_numpy(rc).float().cuda(), torch.from_numpy(ic).float().cuda()
    outs = []
    try:
        for which in (1, 2):
            assert lib.s2g_set_contraction_kernel(which) == 0
            g = torch.full((nb, 4 * bw * bw), float("nan"), dtype=torch.float32, device="cuda")
            plan.inv_fst_real_f32(c32r, c32i, g, nb, prec)
            o_r = torch.full((nb, bw * bw), float("nan"), dtype=torch.float32, device="cuda")
            o_i = torch.full_like(o_r, float("nan"))
            plan.fst_real_f32(g, o_r, o_i, nb, prec)
            plan.sync_status()
            outs.append((g, o_r, o_i))
    finally:
        lib.s2g_set_contraction_kernel(1)
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert torch.isfinite(a).all()
            assert torch.equal(a, b)


@pytest.mark.parametrize("prec", [api.PREC_BF16X3, api.PREC_FP16X2])
@pytest.mark.parametrize("bw", [32, 256])
def test_split_forward_zonal_imaginary_is_exact_zero(bw, prec):
    """For real samples the reference's order-0 imaginary coefficients are exact zeros (the
    REDFT10 of a zero row, FST_semi_memo.c:96-120); the split path must give the same zeros,
    not FP32 rounding residue (which an FP64 REAL inverse ignores, so no refinement fixes it)."""
    torch = _torch()
    from tests._util import harmonic_index
    rng = np.random.default_rng(bw + 7)
    rc, ic = real_field_coeffs(rng, bw, 1.0, nfunc=4)
    plan = api.Plan(bw, bw)
    grid, _, _ = _fp64_pair(plan, rc, ic)
    s_rc = torch.empty(4, bw * bw, dtype=torch.float32, device="cuda")
    s_ic = torch.empty_like(s_rc)
    plan.fst_real_f32(grid.float(), s_rc, s_ic, 4, prec)
    plan.sync_status()
    i0 = harmonic_index(0, np.arange(bw), bw)
    assert (s_ic.cpu().numpy()[:, i0] == 0.0).all()
    assert (s_rc.cpu().numpy()[:, i0] != 0.0).any()
