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
