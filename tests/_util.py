"""Shared helpers for the test suite: coefficient layout, seeded inputs, error metrics."""
from __future__ import annotations

import numpy as np


def harmonic_index(m, l, bw):
    """Vectorised IndexOfHarmonicCoeff (util.c:42-49)."""
    m = np.asarray(m)
    l = np.asarray(l)
    L = bw - 1
    am = np.abs(m)
    pos = m * bw - (m * (m - 1)) // 2 + (l - m)
    neg = (L * (L + 3)) // 2 + 1 + ((L - am) * (L - am + 1)) // 2 + (l - am)
    return np.where(m >= 0, pos, neg)


def degree_of_index(bw):
    """l (degree) and m (order) of every slot of the bw*bw coefficient array."""
    ls = np.empty(bw * bw, dtype=np.int64)
    ms = np.empty(bw * bw, dtype=np.int64)
    for m in range(-(bw - 1), bw):
        l = np.arange(abs(m), bw)
        idx = harmonic_index(m, l, bw)
        ls[idx] = l
        ms[idx] = m
    return ls, ms


def real_field_coeffs(rng, bw, p=0.0, nfunc=None):
    """Complex N(0,1)*(1+l)^-p with f(l,-m) = (-1)^m conj f(l,m) and f(l,0) real.
    Returns (rc, ic) of shape (bw*bw,) or (nfunc, bw*bw)."""
    n = 1 if nfunc is None else nfunc
    rc = np.zeros((n, bw * bw))
    ic = np.zeros((n, bw * bw))
    for m in range(bw):
        l = np.arange(m, bw)
        s = (1.0 + l) ** (-p)
        x = rng.standard_normal((n, l.size)) * s
        y = rng.standard_normal((n, l.size)) * s
        if m == 0:
            y[:] = 0.0
        i0 = harmonic_index(m, l, bw)
        rc[:, i0], ic[:, i0] = x, y
        if m:
            i1 = harmonic_index(-m, l, bw)
            sg = (-1.0) ** m
            rc[:, i1], ic[:, i1] = sg * x, -sg * y
    if nfunc is None:
        return rc[0], ic[0]
    return rc, ic


def rel_err_norm(got_r, got_i, ref_r, ref_i):
    """max |got - ref| / max |ref| (complex magnitudes)."""
    d = np.hypot(np.asarray(got_r) - ref_r, np.asarray(got_i) - ref_i)
    return float(d.max() / max(np.hypot(ref_r, ref_i).max(), 1e-300))


def max_abs(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))))


def block_norms(v, block):
    """L2 norm of every consecutive block of `block` values (the last one zero-padded)."""
    v = np.asarray(v, dtype=np.float64)
    v = np.pad(v, (0, -v.size % block))
    return np.sqrt((v.reshape(-1, block) ** 2).sum(axis=1))


def bw1024_inputs(g):
    """The seeded inputs of tests/golden/ref_bw1024.npz (a real field with coefficients
    N(0,1)(1+l)^-1, a noise grid, the zonal filter exp(-l(l+1)/(2*150^2))), regenerated and
    checked against the fixture's checksums."""
    bw = 1024
    rc, ic = real_field_coeffs(np.random.default_rng(1024), bw, 1.0)
    noise = np.random.default_rng(1025).standard_normal(4 * bw * bw)
    assert rc.sum() == g["rc_sum"] and ic.sum() == g["ic_sum"] and (rc ** 2).sum() == g["rc_sq"]
    assert noise.sum() == g["noise_sum"]
    l = np.arange(bw)
    hr = np.zeros(bw * bw)
    hr[harmonic_index(0, l, bw)] = np.exp(-l * (l + 1) / (2 * 150.0 ** 2))
    return rc, ic, noise, hr


def vs_sampled_reference(g, name, got_r, got_i, tol):
    """One full output (grid or coefficients) against the reference's values at the fixture's
    sample positions and its block norms; returns the larger normwise error."""
    bw = int(g["bw"])
    pos = g["grid_pos"] if np.asarray(got_r).size == 4 * bw * bw else g["coef_pos"]
    e_s = rel_err_norm(got_r[pos], got_i[pos], g[f"{name}_r"], g[f"{name}_i"])
    blk = int(g["block"])
    scale = max(g[f"{name}_r_blocks"].max(), g[f"{name}_i_blocks"].max())
    e_b = max(np.abs(block_norms(got_r, blk) - g[f"{name}_r_blocks"]).max(),
              np.abs(block_norms(got_i, blk) - g[f"{name}_i_blocks"]).max()) / scale
    assert e_s <= tol and e_b <= tol, (name, e_s, e_b)
    return max(e_s, e_b)
