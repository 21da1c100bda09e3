"""Queued host-buffer transforms (s2g_*_host_async, s2g_plan_wait): results equal the synchronous
calls bit for bit, and chained calls on aliased pinned buffers are ordered per chunk (a forward
that uploads the grid an inverse downloads into, an inverse that downloads into a grid a queued
forward still uploads from)."""
import numpy as np
import pytest

from s2kit_gb300 import api
from tests._util import real_field_coeffs

pytestmark = pytest.mark.gpu
PREC = api.PREC_BF16X3


def _pinned(shape):
    import torch
    return torch.zeros(shape, dtype=torch.float32).pin_memory().numpy()


def _sync_roundtrip(plan, rc, ic, nb):
    bw = plan.bw
    g = np.zeros((nb, 4 * bw * bw), dtype=np.float32)
    plan.inv_fst_real_f32_host(rc, ic, g, nb, PREC)
    orc, oic = np.zeros_like(rc), np.zeros_like(ic)
    plan.fst_real_f32_host(g, orc, oic, nb, PREC)
    return g, orc, oic


@pytest.mark.parametrize("bw,nb", [(64, 150), (256, 70), (101, 70)])
def test_async_chain_matches_sync(bw, nb):
    rng = np.random.default_rng(bw + nb)
    plan = api.Plan(bw, bw)
    steps = []
    for k in range(3):
        rc, ic = real_field_coeffs(rng, bw, 1.0, nfunc=nb)
        steps.append((rc.astype(np.float32), ic.astype(np.float32)))
    # three inverse -> forward round trips queued back to back through ONE pinned grid buffer
    h_rc, h_ic = [_pinned((nb, bw * bw)) for _ in range(3)], [_pinned((nb, bw * bw)) for _ in range(3)]
    h_grid = _pinned((nb, 4 * bw * bw))
    outs = [(_pinned((nb, bw * bw)), _pinned((nb, bw * bw))) for _ in range(3)]
    grids = [_pinned((nb, 4 * bw * bw)) for _ in range(3)]
    for k, (rc, ic) in enumerate(steps):
        h_rc[k][:] = rc
        h_ic[k][:] = ic
    for k in range(3):
        plan.inv_fst_real_f32_host_async(h_rc[k], h_ic[k], h_grid, nb, PREC)
        plan.fst_real_f32_host_async(h_grid, outs[k][0], outs[k][1], nb, PREC)
    plan.wait()
    for k in range(3):
        g, orc, oic = _sync_roundtrip(plan, steps[k][0], steps[k][1], nb)
        assert np.array_equal(orc, outs[k][0]) and np.array_equal(oic, outs[k][1]), k
        grids[k][:] = g
    assert np.array_equal(h_grid, grids[2])


def test_async_write_after_read_is_ordered():
    """A queued forward uploads grid A; the next queued inverse downloads a different field into the
    same buffer. The forward must see A."""
    bw, nb = 128, 96
    rng = np.random.default_rng(3)
    plan = api.Plan(bw, bw)
    rc1, ic1 = (x.astype(np.float32) for x in real_field_coeffs(rng, bw, 1.0, nfunc=nb))
    rc2, ic2 = (x.astype(np.float32) for x in real_field_coeffs(rng, bw, 1.0, nfunc=nb))
    gA, ref_rc, ref_ic = _sync_roundtrip(plan, rc1, ic1, nb)
    h_grid = _pinned((nb, 4 * bw * bw))
    h_grid[:] = gA
    h_rc2, h_ic2 = _pinned((nb, bw * bw)), _pinned((nb, bw * bw))
    h_rc2[:], h_ic2[:] = rc2, ic2
    o_rc, o_ic = _pinned((nb, bw * bw)), _pinned((nb, bw * bw))
    plan.fst_real_f32_host_async(h_grid, o_rc, o_ic, nb, PREC)
    plan.inv_fst_real_f32_host_async(h_rc2, h_ic2, h_grid, nb, PREC)
    plan.wait()
    assert np.array_equal(o_rc, ref_rc) and np.array_equal(o_ic, ref_ic)
    g2, _, _ = _sync_roundtrip(plan, rc2, ic2, nb)
    assert np.array_equal(h_grid, g2)


def test_device_call_waits_for_queued_host_work():
    import torch
    bw, nb = 64, 80
    rng = np.random.default_rng(4)
    plan = api.Plan(bw, bw)
    rc, ic = (x.astype(np.float32) for x in real_field_coeffs(rng, bw, 1.0, nfunc=nb))
    h_rc, h_ic, h_grid = _pinned((nb, bw * bw)), _pinned((nb, bw * bw)), _pinned((nb, 4 * bw * bw))
    h_rc[:], h_ic[:] = rc, ic
    plan.inv_fst_real_f32_host_async(h_rc, h_ic, h_grid, nb, PREC)
    # a device-buffer call on the same plan (shared scratch) right behind the queued host work
    d_grid = torch.zeros(nb, 4 * bw * bw, dtype=torch.float32, device="cuda")
    plan.inv_fst_real_f32(torch.from_numpy(rc).cuda(), torch.from_numpy(ic).cuda(), d_grid, nb, PREC)
    torch.cuda.synchronize()
    plan.wait()
    assert np.array_equal(d_grid.cpu().numpy(), h_grid)


def test_async_batch_change_and_pageable_buffers():
    """Consecutive queued calls with different batch sizes (a new staging layout) and pageable
    (non-pinned) host buffers, for which the copies block but stay ordered."""
    bw = 64
    rng = np.random.default_rng(5)
    plan = api.Plan(bw, bw)
    res = []
    for nb in (7, 40, 3):
        rc, ic = (x.astype(np.float32) for x in real_field_coeffs(rng, bw, 1.0, nfunc=nb))
        g = np.zeros((nb, 4 * bw * bw), dtype=np.float32)
        plan.inv_fst_real_f32_host_async(rc, ic, g, nb, PREC)
        o_rc, o_ic = np.zeros_like(rc), np.zeros_like(ic)
        plan.fst_real_f32_host_async(g, o_rc, o_ic, nb, PREC)
        res.append((rc, ic, g, o_rc, o_ic))
    plan.wait()
    for rc, ic, g, o_rc, o_ic in res:
        g2, r2, i2 = _sync_roundtrip(plan, rc, ic, rc.shape[0])
        assert np.array_equal(g, g2) and np.array_equal(o_rc, r2) and np.array_equal(o_ic, i2)
