"""Pins the CPU oracle (oracle/s2oracle.c) against the reference's golden data and the
reference C sources, before it is trusted as the checker for the GPU path."""
import os

import numpy as np
import pytest

from oracle.oracle import COMPLEX, REAL
from tests._util import harmonic_index, real_field_coeffs, rel_err_norm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("n", [2, 4, 8, 16, 64, 512, 6, 10, 34])
def test_dct_fast_matches_definition(oracle, n):
    x = np.random.default_rng(n).standard_normal(n)
    y10 = oracle.redft10(x)
    y01 = oracle.redft01(x)
    tol = 1e-13 * np.abs(x).sum()
    assert np.abs(y10 - oracle.redft10(x, direct=True)).max() <= tol
    assert np.abs(y01 - oracle.redft01(x, direct=True)).max() <= tol
    # FFTW's REDFT01 is the inverse of REDFT10 up to 2n
    assert np.abs(oracle.redft01(y10) - 2 * n * x).max() <= 1e-12 * n * np.abs(x).max()


@pytest.mark.parametrize("n", [8, 128, 512, 12, 34])
def test_dft_matches_numpy(oracle, n):
    rng = np.random.default_rng(n)
    re, im = rng.standard_normal(n), rng.standard_normal(n)
    r, i = oracle.dft(re, im, -1)
    ref = np.fft.fft(re + 1j * im)
    assert np.abs(r + 1j * i - ref).max() <= 1e-13 * n
    r, i = oracle.dft(re, im, +1)
    ref = np.fft.ifft(re + 1j * im) * n
    assert np.abs(r + 1j * i - ref).max() <= 1e-13 * n


@pytest.mark.parametrize("bw", [64, 128])
def test_conv_golden(oracle, golden, bw):
    """data/o{64,128}_conv_semi_memo_original.dat were produced by the reference with FFTW3."""
    g = golden(f"conv_bw{bw}")
    z = np.zeros_like(g["signal"])
    rr, _ = oracle.conv(g["signal"], z, g["filter"], z, bw)
    assert np.abs(rr - g["golden"]).max() <= 2e-15


@pytest.mark.parametrize("name", ["y20_bw8", "y31_bw8", "y43_bw23", "yMix_bw17"])
def test_known_answers(oracle, golden, name):
    g = golden(f"ka_{name}")
    bw = int(g["bw"])
    rc, ic = oracle.fst(g["rdata"], g["idata"], bw, COMPLEX, bw)
    exp = np.zeros(bw * bw, dtype=complex)
    for m, l, re, im in g["expected"]:
        exp[harmonic_index(int(m), int(l), bw)] = re + 1j * im
    assert np.abs(rc + 1j * ic - exp).max() <= 1e-13


@pytest.mark.parametrize("case", ["bw8_cut8_complex", "bw16_cut4_complex", "bw32_cut32_real", "bw64_cut64_real",
                                  "bw64_cut16_complex"])
def test_reference_sht_fixtures(oracle, golden, case):
    g = golden(f"ref_sht_{case}")
    bw, cut, fmt = int(g["bw"]), int(g["cutoff"]), int(g["fmt"])
    gr, gi = oracle.inv_fst(g["rcoeffs"], g["icoeffs"], bw, fmt, cut)
    scale = np.abs(g["inv_r"]).max()
    assert np.abs(gr - g["inv_r"]).max() <= 1e-13 * scale
    assert np.abs(gi - g["inv_i"]).max() <= 1e-13 * scale
    fr, fi = oracle.fst(g["noise_r"], g["noise_i"], bw, fmt, cut)
    assert rel_err_norm(fr, fi, g["fwd_noise_r"], g["fwd_noise_i"]) <= 1e-13
    rr, ri = oracle.fst(g["inv_r"], g["inv_i"], bw, fmt, cut)
    assert rel_err_norm(rr, ri, g["rt_r"], g["rt_i"]) <= 1e-13
    # and the round trip recovers the coefficients (reference metric, test_s2_semi_memo.c:196-203)
    assert rel_err_norm(rr, ri, g["rcoeffs"], g["icoeffs"]) <= 1e-11


def test_reference_fzt_transmult(oracle, golden):
    g = golden("ref_fzt_transmult_bw16")
    bw = int(g["bw"])
    zr, zi = oracle.fzt(g["data_r"], g["data_i"], bw, COMPLEX)
    assert np.abs(zr - g["fzt_complex_r"]).max() <= 1e-14
    assert np.abs(zi[:bw] - g["fzt_complex_i"]).max() <= 1e-14
    zr, zi = oracle.fzt(g["data_r"], g["data_i"], bw, REAL)
    assert np.abs(zr - g["fzt_real_r"]).max() <= 1e-14
    assert np.all(zi == 0) and zi.size == 2 * bw
    tr, ti = oracle.transmult(g["tm_data_r"], g["tm_data_i"], g["tm_filter_r"], g["tm_filter_i"], bw)
    assert np.abs(tr - g["tm_out_r"]).max() <= 1e-14
    assert np.abs(ti - g["tm_out_i"]).max() <= 1e-14


@pytest.mark.parametrize("bw,cut", [(16, 16), (16, 5)])
def test_reference_tables(oracle, golden, bw, cut):
    g = golden(f"ref_tables_bw{bw}_cut{cut}")
    _, fwd, inv, _ = oracle.tables(bw, cut)
    assert np.abs(fwd - g["fwd"]).max() <= 1e-14
    assert np.abs(inv - g["inv"]).max() <= 1e-14


def test_reference_weights(oracle, golden):
    g = golden("ref_weights")
    for bw in (16, 64, 256):
        assert np.abs(oracle.weights(bw) - g[f"w{bw}"]).max() <= 1e-15


@pytest.mark.parametrize("bw", [9, 17, 23])
def test_odd_bandwidth_roundtrip(oracle, bw):
    """The restatement's transposed table is correct for odd bw (the reference v1.1 is not)."""
    rng = np.random.default_rng(bw)
    rc, ic = rng.standard_normal(bw * bw), rng.standard_normal(bw * bw)
    gr, gi = oracle.inv_fst(rc, ic, bw, COMPLEX, bw)
    fr, fi = oracle.fst(gr, gi, bw, COMPLEX, bw)
    assert rel_err_norm(fr, fi, rc, ic) <= 1e-12


def test_single_function_bw64_roundtrip(oracle):
    """B=64 real field, coefficients N(0,1) with conjugate symmetry, round trip <= 1e-11."""
    rng = np.random.default_rng(1)
    rc, ic = real_field_coeffs(rng, 64, 0.0)
    gr, gi = oracle.inv_fst(rc, ic, 64, REAL, 64)
    assert np.abs(gi).max() <= 1e-13 * np.abs(gr).max()
    fr, fi = oracle.fst(gr, gi, 64, REAL, 64)
    assert rel_err_norm(fr, fi, rc, ic) <= 1e-11


def test_bench_roundtrip_threads(oracle):
    rng = np.random.default_rng(3)
    rc, ic = real_field_coeffs(rng, 16, 1.0, nfunc=4)
    coeffs = np.stack([rc, ic], axis=1)
    secs, out = oracle.bench_roundtrip(16, coeffs, 2)
    assert secs > 0
    assert np.abs(out - coeffs).max() <= 1e-12


def test_oracle_matches_reference_build(oracle):
    """Restatement vs the unmodified reference sources (only where the checkout exists)."""
    from oracle.oracle import Reference
    try:
        ref = Reference()
    except Exception as e:  # not available on machines without the reference checkout
        pytest.skip(str(e))
    rng = np.random.default_rng(7)
    for bw, cut, fmt in [(32, 8, COMPLEX), (32, 32, REAL), (64, 20, REAL)]:
        n = 2 * bw
        rd = rng.standard_normal(n * n)
        idd = rng.standard_normal(n * n)
        a = oracle.fst(rd, idd, bw, fmt, cut)
        b = ref.fst(rd, idd, bw, fmt, cut)
        assert rel_err_norm(*a, *b) <= 1e-14
        c = oracle.inv_fst(*a, bw, fmt, cut)
        d = ref.inv_fst(*a, bw, fmt, cut)
        assert rel_err_norm(*c, *d) <= 1e-14
    for bw in (8, 17, 64):
        for m in range(bw):
            assert oracle.table_size(m, bw) == ref.lib.TableSize(m, bw)


FLY_CASES = [(16, 16, REAL), (16, 6, COMPLEX), (32, 32, REAL), (32, 20, COMPLEX)]


@pytest.mark.parametrize("bw,cut,fmt", FLY_CASES)
def test_oracle_matches_reference_fly(oracle, golden, bw, cut, fmt):
    """The on-the-fly family (FST_semi_fly.c) computes the memo family's transforms: the oracle's
    memo restatement reproduces the reference's FSTSemiFly / InvFSTSemiFly outputs (ref_fly.npz)."""
    g = golden("ref_fly")
    tag = f"bw{bw}_cut{cut}_{'real' if fmt else 'complex'}"
    a = oracle.fst(g[f"{tag}_grid_r"], g[f"{tag}_grid_i"], bw, fmt, cut)
    assert rel_err_norm(*a, g[f"{tag}_fst_r"], g[f"{tag}_fst_i"]) <= 1e-14
    b = oracle.inv_fst(g[f"{tag}_coef_r"], g[f"{tag}_coef_i"], bw, fmt, cut)
    assert rel_err_norm(*b, g[f"{tag}_inv_r"], g[f"{tag}_inv_i"]) <= 1e-14


def test_oracle_matches_reference_fly_fzt_conv(oracle, golden):
    g = golden("ref_fly")
    for fmt, key in ((COMPLEX, "complex"), (REAL, "real")):
        zr, zi = oracle.fzt(g["fzt_bw16_data_r"], g["fzt_bw16_data_i"], 16, fmt)
        assert rel_err_norm(zr, zi[:16], g[f"fzt_bw16_{key}_r"], g[f"fzt_bw16_{key}_i"][:16]) <= 1e-14
        # REAL: the reference zeroes 2*bw imaginary values (FST_semi_fly.c:424)
        if fmt == REAL:
            assert not g["fzt_bw16_real_i"].any()
    z = np.zeros(4 * 16 * 16)
    cr, ci = oracle.conv(g["conv_bw16_signal"], z, g["conv_bw16_filter"], z, 16)
    assert rel_err_norm(cr, ci, g["conv_bw16_out_r"], g["conv_bw16_out_i"]) <= 1e-14


def test_oracle_matches_reference_at_bw1024(oracle, golden):
    """The large single-function workload (bw 1024): the oracle's tables, inverse and forward
    transforms, forward of noise and convolution with the zonal filter exp(-l(l+1)/(2*150^2))
    against the reference's own outputs (sampled values and block norms, ref_bw1024.npz)."""
    from tests._util import block_norms, bw1024_inputs, vs_sampled_reference
    g = golden("ref_bw1024")
    bw = int(g["bw"])
    rc, ic, noise, hr = bw1024_inputs(g)
    try:
        _, fwd, inv, off = oracle.tables(bw, bw)
        assert np.array_equal(off, g["table_offsets"])
        pos = g["table_pos"]
        scale = np.abs(fwd).max()
        assert np.abs(fwd[pos] - g["table_fwd"]).max() <= 1e-13 * scale
        assert np.abs(inv[pos] - g["table_inv"]).max() <= 1e-13 * scale
        tb = int(g["table_block"])
        assert np.abs(block_norms(fwd, tb) - g["table_fwd_blocks"]).max() <= 1e-13 * g["table_fwd_blocks"].max()
        assert np.abs(block_norms(inv, tb) - g["table_inv_blocks"]).max() <= 1e-13 * g["table_inv_blocks"].max()
        z = np.zeros(4 * bw * bw)
        grid, _ = oracle.inv_fst(rc, ic, bw, REAL, bw)
        filt, _ = oracle.inv_fst(hr, np.zeros(bw * bw), bw, REAL, bw)
        outs = {"inv": (grid, z), "rt": oracle.fst(grid, z, bw, REAL, bw), "noise_fwd": oracle.fst(noise, z, bw, REAL, bw),
                "filter_grid": (filt, z), "conv": oracle.conv(grid, z, filt, z, bw, cached_tables=True)}
        for name, (a, b) in outs.items():
            vs_sampled_reference(g, name, a, b, tol=1e-13)
    finally:
        oracle.drop_tables(bw, bw)
