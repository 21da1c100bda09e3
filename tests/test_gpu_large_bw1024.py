"""The large single-function workload at bw 1024 (2048 x 2048 grid) pinned to the oracle and to
the reference itself.

The FP64 GPU path is compared with the oracle (oracle/s2oracle.c, built on the GPU host) on the
full outputs, and with the reference's own outputs (tests/golden/ref_bw1024.npz, written by
tests/golden/make_golden.py from the unmodified S2kit sources) at a seeded sample of positions
and through the L2 norm of every block of consecutive values (4096; 65536 for the tables),
which a systematic error anywhere in an output would move.  Covered: the FP64 seminaive tables
(generated on the GPU), InvFSTSemiMemo / FSTSemiMemo of a seeded real field with coefficients N(0,1)(1+l)^-1,
FSTSemiMemo of seeded noise, ConvOn2SphereSemiMemo with the zonal filter
h_l^0 = exp(-l(l+1)/(2*150^2)), and the split-BF16 forward with one FP64-residual refinement step.

Tolerances (normwise, max|got - ref| / max|ref|): 1e-11 for the FP64 path (the parity bar),
1e-12 of the largest entry for the tables, 1e-10 for the refined forward.
"""
import numpy as np
import pytest

from s2kit_gb300 import api
from tests._util import bw1024_inputs as _inputs
from tests._util import block_norms as _blocks
from tests._util import harmonic_index, rel_err_norm
from tests._util import vs_sampled_reference as _vs_reference

pytestmark = pytest.mark.gpu
BW = 1024
TOL = 1e-11
TOL_TABLE = 1e-12
TOL_REFINED = 1e-10


@pytest.fixture(scope="module")
def large(oracle, golden):
    g = golden("ref_bw1024")
    yield g
    oracle.drop_tables(BW, BW)


def test_bw1024_tables_vs_oracle_and_reference(oracle, large):
    g = large
    _, o_fwd, o_inv, o_off = oracle.tables(BW, BW)
    assert np.array_equal(o_off, g["table_offsets"])
    size = api.Reduced_Naive_TableSize(BW, BW) + api.Reduced_SpharmonicTableSize(BW, BW)
    fwd = np.zeros(size)
    inv = np.zeros(size)
    t = api.SemiNaive_Naive_Pml_Table(BW, BW, fwd, None)
    api.Transpose_SemiNaive_Naive_Pml_Table(t, BW, BW, inv, None)
    scale = np.abs(o_fwd).max()
    e_fwd = np.abs(fwd - o_fwd).max() / scale
    e_inv = np.abs(inv - o_inv).max() / scale
    assert e_fwd <= TOL_TABLE and e_inv <= TOL_TABLE, (e_fwd, e_inv)
    pos = g["table_pos"]
    for got, orc, ref in ((fwd, o_fwd, g["table_fwd"]), (inv, o_inv, g["table_inv"])):
        assert np.abs(got[pos] - ref).max() <= TOL_TABLE * scale
        assert np.abs(orc[pos] - ref).max() <= TOL_TABLE * scale
    blk = int(g["table_block"])
    for got, ref in ((fwd, g["table_fwd_blocks"]), (inv, g["table_inv_blocks"])):
        assert np.abs(_blocks(got, blk) - ref).max() <= TOL_TABLE * ref.max()
    print(f"bw 1024 tables: GPU vs oracle fwd {e_fwd:.2e}, inv {e_inv:.2e} (of the largest entry)")


def test_bw1024_fp64_transforms_and_conv_vs_oracle_and_reference(oracle, large):
    import torch
    g = large
    rc, ic, noise, hr = _inputs(g)
    plan = api.Plan(BW, BW)
    d_rc, d_ic = torch.from_numpy(rc)[None].cuda(), torch.from_numpy(ic)[None].cuda()
    grid = torch.empty(1, 4 * BW * BW, dtype=torch.float64, device="cuda")
    plan.inv_fst(d_rc, d_ic, grid, None, 1, api.REAL)
    o_rc, o_ic = torch.empty_like(d_rc), torch.empty_like(d_ic)
    plan.fst(grid, None, o_rc, o_ic, 1, api.REAL)
    d_noise = torch.from_numpy(noise)[None].cuda()
    n_rc, n_ic = torch.empty_like(d_rc), torch.empty_like(d_ic)
    plan.fst(d_noise, None, n_rc, n_ic, 1, api.REAL)
    fgrid = torch.empty_like(grid)
    plan.inv_fst(torch.from_numpy(hr)[None].cuda(), torch.zeros_like(d_rc), fgrid, None, 1, api.REAL)
    zero = torch.zeros_like(grid)
    cr, ci = torch.empty_like(grid), torch.empty_like(grid)
    plan.conv(grid, zero, fgrid, zero, cr, ci, 1)
    torch.cuda.synchronize()
    grid_h, fgrid_h = grid[0].cpu().numpy(), fgrid[0].cpu().numpy()
    z = np.zeros(4 * BW * BW)
    zc = np.zeros(BW * BW)

    # the oracle on the same inputs (tables of the oracle, built once)
    e_inv_r, _ = oracle.inv_fst(rc, ic, BW, api.REAL, BW)
    e_rt = oracle.fst(e_inv_r, z, BW, api.REAL, BW)
    e_noise = oracle.fst(noise, z, BW, api.REAL, BW)
    e_filt, _ = oracle.inv_fst(hr, zc, BW, api.REAL, BW)
    e_conv = oracle.conv(e_inv_r, z, e_filt, z, BW, cached_tables=True)
    errs = {
        "inv": rel_err_norm(grid_h, z, e_inv_r, z),
        "rt": rel_err_norm(o_rc[0].cpu().numpy(), o_ic[0].cpu().numpy(), *e_rt),
        "noise_fwd": rel_err_norm(n_rc[0].cpu().numpy(), n_ic[0].cpu().numpy(), *e_noise),
        "filter_grid": rel_err_norm(fgrid_h, z, e_filt, z),
        "conv": rel_err_norm(cr[0].cpu().numpy(), ci[0].cpu().numpy(), *e_conv),
    }
    # the oracle's own round trip (inverse then forward against the input coefficients)
    orc_rt = rel_err_norm(*e_rt, rc, ic)
    print("bw 1024 FP64 GPU vs oracle:", {k: f"{v:.2e}" for k, v in errs.items()}, f"oracle round trip {orc_rt:.2e}")
    assert max(errs.values()) <= TOL, errs

    # against the reference's own outputs (sampled values and block norms), GPU and oracle alike
    outs = {"inv": (grid_h, z), "rt": (o_rc[0].cpu().numpy(), o_ic[0].cpu().numpy()),
            "noise_fwd": (n_rc[0].cpu().numpy(), n_ic[0].cpu().numpy()), "filter_grid": (fgrid_h, z),
            "conv": (cr[0].cpu().numpy(), ci[0].cpu().numpy())}
    orcs = {"inv": (e_inv_r, z), "rt": e_rt, "noise_fwd": e_noise, "filter_grid": (e_filt, z), "conv": e_conv}
    ref_errs = {k: _vs_reference(g, k, *v, tol=TOL) for k, v in outs.items()}
    orc_errs = {k: _vs_reference(g, k, *v, tol=TOL) for k, v in orcs.items()}
    print("bw 1024 vs reference: GPU", {k: f"{v:.2e}" for k, v in ref_errs.items()},
          "oracle", {k: f"{v:.2e}" for k, v in orc_errs.items()})


def test_bw1024_refined_forward_vs_oracle(oracle, large):
    """The split-BF16 forward with one FP64-residual refinement step against the oracle's FP64
    forward of the same samples, for two functions: the seeded field (band-limited samples, the
    workload the refinement serves: <= 1e-10) and the noise grid.  Noise is not band-limited: its
    part outside the band lies in the null space of the forward transform, the FP64 residual
    f - I(a1) keeps it at full size, and the second split forward adds the split precision's error
    relative to it, so there the refined forward is held to the split bound (2e-6) only."""
    import torch
    rc, ic, noise, _ = _inputs(large)
    z = np.zeros(4 * BW * BW)
    e_inv_r, _ = oracle.inv_fst(rc, ic, BW, api.REAL, BW)
    grids = np.stack([e_inv_r, noise])
    plan = api.Plan(BW, BW)
    d_grid = torch.from_numpy(grids).cuda()
    r_rc = torch.empty(2, BW * BW, dtype=torch.float64, device="cuda")
    r_ic = torch.empty_like(r_rc)
    plan.fst_refined(d_grid, r_rc, r_ic, 2, api.PREC_BF16X3)
    plan.sync_status()
    errs = []
    for f in range(2):
        er, ei = oracle.fst(grids[f], z, BW, api.REAL, BW)
        errs.append(rel_err_norm(r_rc[f].cpu().numpy(), r_ic[f].cpu().numpy(), er, ei))
    print(f"bw 1024 refined forward vs oracle: field {errs[0]:.2e}, noise {errs[1]:.2e}")
    assert errs[0] <= TOL_REFINED, errs
    assert errs[1] <= 2e-6, errs


def test_bw1024_on_the_fly_memory_and_parity(oracle, large):
    """The on-the-fly plan at bw 1024: no Legendre table on the device (the memo tables of this
    bandwidth take 2 x 1.37 GiB), so the device memory the plan and its calls take is the
    workspace (the row DFTs of one function and the convolution's coefficient buffers, tens of
    MiB).  Its inverse, round trip, filter synthesis and convolution of the band-limited field
    match the reference's own outputs to the FP64 parity bar.

    The forward of noise is pinned order by order to the oracle's naive transform (DLTNaive on
    GeneratePmlTable, naive.c:34-63 and pml.c:41-79, the form the reference itself applies to the
    orders >= cutoff), which is the form the on-the-fly kernels compute.  Against the reference's
    memo output (seminaive at every order) it is held to 1e-10: on samples that are not
    band-limited the seminaive form's own FP64 rounding reaches 7e-11 of an order's largest
    coefficient at m = 1 (G = P / sin(theta) has large cosine coefficients), while the naive form
    stays near 1e-13 (both measured against a long-double naive transform)."""
    import torch
    g = large
    rc, ic, noise, hr = _inputs(g)
    d_rc, d_ic = torch.from_numpy(rc)[None].cuda(), torch.from_numpy(ic)[None].cuda()
    d_noise = torch.from_numpy(noise)[None].cuda()
    d_hr = torch.from_numpy(hr)[None].cuda()
    grid = torch.empty(1, 4 * BW * BW, dtype=torch.float64, device="cuda")
    fgrid, zero, cr, ci = (torch.empty_like(grid) for _ in range(4))
    zero.zero_()
    o_rc, o_ic, n_rc, n_ic = (torch.empty_like(d_rc) for _ in range(4))
    zc = torch.zeros_like(d_rc)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    plan = api.Plan(BW, fly=True)
    plan.inv_fst(d_rc, d_ic, grid, None, 1, api.REAL)
    plan.fst(grid, None, o_rc, o_ic, 1, api.REAL)
    plan.fst(d_noise, None, n_rc, n_ic, 1, api.REAL)
    plan.inv_fst(d_hr, zc, fgrid, None, 1, api.REAL)
    plan.conv(grid, zero, fgrid, zero, cr, ci, 1)
    torch.cuda.synchronize()
    used = free0 - torch.cuda.mem_get_info()[0]
    print(f"bw 1024 on-the-fly plan: {used / 2**20:.1f} MiB of device memory (memo tables: 2 x 1.37 GiB)")
    assert used <= 192 * 2 ** 20, used
    z = np.zeros(4 * BW * BW)
    outs = {"inv": (grid[0].cpu().numpy(), z), "rt": (o_rc[0].cpu().numpy(), o_ic[0].cpu().numpy()),
            "noise_fwd": (n_rc[0].cpu().numpy(), n_ic[0].cpu().numpy()), "filter_grid": (fgrid[0].cpu().numpy(), z),
            "conv": (cr[0].cpu().numpy(), ci[0].cpu().numpy())}
    ref_errs = {k: _vs_reference(g, k, *v, tol=1e-10 if k == "noise_fwd" else TOL) for k, v in outs.items()}
    e_inv_r, _ = oracle.inv_fst(rc, ic, BW, api.REAL, BW)
    errs = {"inv": rel_err_norm(outs["inv"][0], z, e_inv_r, z)}
    # noise, order by order against the oracle's naive transform of the same latitude rows
    S = 2 * BW
    rows = np.fft.fft(noise.reshape(S, S), axis=1) * (np.sqrt(2 * np.pi) / S)
    w = oracle.weights(BW)
    got_r, got_i = outs["noise_fwd"]
    scale = np.hypot(got_r, got_i).max()
    worst = 0.0
    for m in (0, 1, 2, 3, 17, 200, 777, 1023):
        pml = oracle.pml_table(BW, m)
        er = oracle.dlt_naive(np.ascontiguousarray(rows[:, m].real), BW, m, w, pml)
        ei = oracle.dlt_naive(np.ascontiguousarray(rows[:, m].imag), BW, m, w, pml)
        idx = harmonic_index(m, np.arange(m, BW), BW)
        worst = max(worst, float(np.hypot(got_r[idx] - er, got_i[idx] - ei).max() / scale))
    errs["noise_fwd_naive_orders"] = worst
    print("bw 1024 on-the-fly vs reference:", {k: f"{v:.2e}" for k, v in ref_errs.items()},
          "vs oracle:", {k: f"{v:.2e}" for k, v in errs.items()})
    assert max(errs.values()) <= TOL, errs
