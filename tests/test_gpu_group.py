"""Grouped uneven-bandwidth transforms (s2g_group_*): one persistent tensor-core contraction
launch over every bandwidth class, class FFT stages on parallel graph branches, CUDA-graph
replay and autotuned tile shapes.

Checks:
  * grouped results equal the uniform per-bandwidth path bit for bit (same arithmetic per item);
  * tile shape (N extent) and CTAs per SM do not change a single bit (K order is fixed);
  * graph replays equal the eager first call bit for bit;
  * the 512-function mix, bandwidths {16, 32, 64, 128, 256} with probabilities
    {.3, .3, .2, .15, .05}, coefficients N(0,1)(1+l)^-2, split FP16: per-bandwidth normwise
    error vs the FP64 path <= 2e-6 (forward and inverse).
"""
import numpy as np
import pytest

from s2kit_gb300 import api
from s2kit_gb300._lib import S2GError
from tests._util import real_field_coeffs

pytestmark = pytest.mark.gpu
TOL_FP16X2 = 2e-6


def _torch():
    import torch
    return torch


def _mix(rng, n):
    return rng.choice([16, 32, 64, 128, 256], size=n, p=[0.3, 0.3, 0.2, 0.15, 0.05]).tolist()


def _fp64_reference(bws, p, seed):
    """Per function: FP64 coefficients, FP64 grid (inverse) and FP64 forward of that grid."""
    torch = _torch()
    out = {}
    for B in sorted(set(bws)):
        idx = [i for i, b in enumerate(bws) if b == B]
        rng = np.random.default_rng(seed + B)
        rc, ic = real_field_coeffs(rng, B, p, nfunc=len(idx))
        plan = api.Plan(B, B)
        d_rc, d_ic = torch.from_numpy(rc).cuda(), torch.from_numpy(ic).cuda()
        grid = torch.zeros(len(idx), 4 * B * B, dtype=torch.float64, device="cuda")
        plan.inv_fst(d_rc, d_ic, grid, None, len(idx), api.REAL)
        f_rc, f_ic = torch.zeros_like(d_rc), torch.zeros_like(d_ic)
        plan.fst(grid, None, f_rc, f_ic, len(idx), api.REAL)
        torch.cuda.synchronize()
        out[B] = (idx, d_rc, d_ic, grid, f_rc, f_ic, plan)
    return out


def _pack(g, ref):
    """Flat FP32 device buffers in the group layout from the per-class FP64 arrays."""
    torch = _torch()
    grid = torch.zeros(g.grid_total, dtype=torch.float32, device="cuda")
    rc = torch.zeros(g.coeff_total, dtype=torch.float32, device="cuda")
    ic = torch.zeros_like(rc)
    for B, (idx, d_rc, d_ic, grid64, *_r) in ref.items():
        for j, f in enumerate(idx):
            go, co = int(g.grid_offsets[f]), int(g.coeff_offsets[f])
            grid[go:go + 4 * B * B] = grid64[j].float()
            rc[co:co + B * B] = d_rc[j].float()
            ic[co:co + B * B] = d_ic[j].float()
    return grid, rc, ic


def _gather(g, flat, idx, size, offsets):
    torch = _torch()
    return torch.stack([flat[int(offsets[f]):int(offsets[f]) + size] for f in idx])


@pytest.mark.parametrize("prec", [api.PREC_FP16X2, api.PREC_BF16X3])
@pytest.mark.parametrize("bws", [[16, 32, 16, 64, 128, 32, 256, 16, 64, 32, 128, 16],
                                 # any split-path bandwidth: warp-FFT lengths 32 R with R not a power of
                                 # two (48, 192) and chirp-z lengths (17, 33, 100, 127, 255) beside powers of two
                                 [17, 48, 100, 127, 192, 255, 64, 17, 100, 33, 16, 256]])
def test_group_equals_uniform_path_bitwise(prec, bws):
    torch = _torch()
    ref = _fp64_reference(bws, 2.0, 7)
    g = api.Group(bws, prec)
    grid, rc, ic = _pack(g, ref)
    o_rc = torch.full_like(rc, float("nan"))
    o_ic = torch.full_like(ic, float("nan"))
    o_grid = torch.full_like(grid, float("nan"))
    g.fst(grid, o_rc, o_ic)
    g.inv_fst(rc, ic, o_grid)
    g.sync_status()
    for B, (idx, d_rc, d_ic, grid64, f_rc, f_ic, plan) in ref.items():
        n = len(idx)
        u_rc = torch.zeros(n, B * B, dtype=torch.float32, device="cuda")
        u_ic = torch.zeros_like(u_rc)
        plan.fst_real_f32(grid64.float().contiguous(), u_rc, u_ic, n, prec)
        u_grid = torch.zeros(n, 4 * B * B, dtype=torch.float32, device="cuda")
        plan.inv_fst_real_f32(d_rc.float().contiguous(), d_ic.float().contiguous(), u_grid, n, prec)
        plan.sync_status()
        assert torch.equal(_gather(g, o_rc, idx, B * B, g.coeff_offsets), u_rc), B
        assert torch.equal(_gather(g, o_ic, idx, B * B, g.coeff_offsets), u_ic), B
        assert torch.equal(_gather(g, o_grid, idx, 4 * B * B, g.grid_offsets), u_grid), B


def test_group_config_mix_512_fp16():
    torch = _torch()
    rng = np.random.default_rng(2024)
    bws = _mix(rng, 512)
    ref = _fp64_reference(bws, 2.0, 11)
    g = api.Group(bws, api.PREC_FP16X2)
    grid, rc, ic = _pack(g, ref)
    o_rc, o_ic = torch.zeros_like(rc), torch.zeros_like(ic)
    o_grid = torch.zeros_like(grid)
    g.fst(grid, o_rc, o_ic)          # eager + capture
    g.inv_fst(rc, ic, o_grid)
    first = (o_rc.clone(), o_ic.clone(), o_grid.clone())
    for _ in range(2):               # graph replays
        o_rc.zero_(), o_ic.zero_(), o_grid.zero_()
        g.fst(grid, o_rc, o_ic)
        g.inv_fst(rc, ic, o_grid)
    g.sync_status()
    assert torch.equal(first[0], o_rc) and torch.equal(first[1], o_ic) and torch.equal(first[2], o_grid)
    d = g.describe()
    assert d["graph_kernels"][0] > 0 and d["graph_kernels"][1] > 0
    errs = {}
    for B, (idx, d_rc, d_ic, grid64, f_rc, f_ic, _p) in ref.items():
        s_rc = _gather(g, o_rc, idx, B * B, g.coeff_offsets).double()
        s_ic = _gather(g, o_ic, idx, B * B, g.coeff_offsets).double()
        mag = torch.hypot(f_rc, f_ic).amax(dim=1)
        e_f = (torch.hypot(s_rc - f_rc, s_ic - f_ic).amax(dim=1) / mag).max().item()
        s_g = _gather(g, o_grid, idx, 4 * B * B, g.grid_offsets).double()
        e_i = ((s_g - grid64).abs().amax(dim=1) / grid64.abs().amax(dim=1)).max().item()
        errs[B] = (len(idx), e_f, e_i)
    print("per-bandwidth (count, fwd err, inv err):", errs)
    for B, (n, e_f, e_i) in errs.items():
        assert e_f <= TOL_FP16X2 and e_i <= TOL_FP16X2, (B, e_f, e_i)


def test_group_tile_shapes_do_not_change_results():
    torch = _torch()
    rng = np.random.default_rng(5)
    bws = _mix(rng, 96)
    ref = _fp64_reference(bws, 2.0, 3)
    g = api.Group(bws, api.PREC_FP16X2)
    grid, rc, ic = _pack(g, ref)
    outs = []
    ncls = len(g.describe()["classes"])
    for ts, tiles, dct in [(0, None, 0), (2, [32] * ncls, 1), (3, [64] * ncls, 2), (0, [16] * ncls, 3)]:
        g.set_tiles(ts, tiles, dct)
        o_rc, o_ic, o_grid = torch.zeros_like(rc), torch.zeros_like(ic), torch.zeros_like(grid)
        g.fst_inv(grid, o_rc, o_ic, o_grid)
        g.sync_status()
        outs.append((o_rc, o_ic, o_grid))
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            assert torch.equal(a, b)
    g.autotune(force=True)
    t = g.describe()["tiles"]
    assert set(t) == {"table_stages", "dct_ctas_per_sm", "tile_n"}
    o_rc, o_ic, o_grid = torch.zeros_like(rc), torch.zeros_like(ic), torch.zeros_like(grid)
    g.fst_inv(grid, o_rc, o_ic, o_grid)
    g.sync_status()
    for a, b in zip(outs[0], (o_rc, o_ic, o_grid)):
        assert torch.equal(a, b)


def test_group_graph_replay_counts_launches():
    torch = _torch()
    g = api.Group([16, 32, 32, 64], api.PREC_BF16X3)
    grid = torch.zeros(g.grid_total, dtype=torch.float32, device="cuda")
    rc, ic = torch.zeros(g.coeff_total, device="cuda"), torch.zeros(g.coeff_total, device="cuda")
    g.fst(grid, rc, ic)
    torch.cuda.synchronize()
    nk = g.describe()["graph_kernels"][0]
    # every class here is in the short tier (bw <= 64): one rows-DFT, one DCT, one contraction
    assert nk == 3
    lib = api.load()
    before = lib.s2g_launch_count()
    g.fst(grid, rc, ic)
    torch.cuda.synchronize()
    assert lib.s2g_launch_count() - before == nk


def test_group_stage_launches_do_not_grow_with_classes():
    """Five bandwidth classes in both tiers: a forward is one rows-DFT and one DCT launch per tier
    and one contraction, five kernels, not two per class."""
    torch = _torch()
    g = api.Group([16, 32, 64, 128, 256, 256], api.PREC_FP16X2)
    grid = torch.zeros(g.grid_total, dtype=torch.float32, device="cuda")
    rc, ic = torch.zeros(g.coeff_total, device="cuda"), torch.zeros(g.coeff_total, device="cuda")
    og = torch.zeros_like(grid)
    g.fst(grid, rc, ic)
    g.inv_fst(rc, ic, og)
    torch.cuda.synchronize()
    d = g.describe()
    assert d["graph_kernels"][0] == 5 and d["graph_kernels"][1] == 5, d


def test_group_rejects_bad_arguments():
    with pytest.raises(S2GError):
        api.Group([16, 300], api.PREC_FP16X2)  # above 256 and not a power of two
    with pytest.raises(S2GError):
        api.Group(list(range(16, 33)), api.PREC_FP16X2)  # 17 distinct bandwidths
    with pytest.raises(S2GError):
        api.Group([16, 32], api.PREC_FP64)
    with pytest.raises(S2GError):
        api.Group([1024], api.PREC_BF16X3)
