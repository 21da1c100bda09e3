"""Generate the committed golden fixtures in tests/golden/ from the S2kit reference.

Run where the reference checkout exists, naming it with $S2_REFERENCE_DIR:

    S2_REFERENCE_DIR=<S2kit checkout> python tests/golden/make_golden.py [--only bw1024]

Two kinds of fixture are written (all float64, np.savez_compressed):

* copied reference data (data/*.dat of the reference repository), converted to binary:
  - conv_bw64.npz / conv_bw128.npz : signal, filter and the golden real part of
    ConvOn2SphereSemiMemo produced by the reference with real FFTW3
    (data/s64.dat, f64.dat, o64_conv_semi_memo_original.dat and the 128 versions);
  - ka_<name>.npz : the analytic known-answer sample files y20_bw8, y31_bw8, y43_bw23,
    yMix_bw17 (interleaved re/im, latitude-major) with the expected coefficients
    documented for them (Y_2^0, Y_3^1, (sqrt2 + pi i) Y_4^3, Y_1^1 + (3-2i) Y_5^-2).
* outputs of the unmodified reference C sources compiled by `make -C oracle ref`
  (FSTSemiMemo, InvFSTSemiMemo, FZTSemiMemo, ConvOn2SphereSemiMemo, DLTSemi/InvDLTSemi,
  table generators, GenerateWeightsForDLT) on seeded inputs -> ref_*.npz, and of the
  on-the-fly family (FSTSemiFly, InvFSTSemiFly, FZTSemiFly, ConvOn2SphereSemiFly) -> ref_fly.npz.
* the large single-function workload at bw 1024 (ref_bw1024.npz): the reference's tables,
  InvFSTSemiMemo / FSTSemiMemo of a seeded real field (N(0,1)(1+l)^-1), FSTSemiMemo of seeded
  noise and ConvOn2SphereSemiMemo with the zonal filter exp(-l(l+1)/(2*150^2)).  The full
  outputs (16-32 MiB each) are too large to commit, so the fixture holds, for each output, the
  values at a seeded sample of positions (some in every order for the tables) and the L2 norm of
  every consecutive block of 4096 values (65536 for the tables); the inputs are regenerated from their seeds by the
  tests and checked against stored checksums.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.oracle import COMPLEX, REAL, Reference  # noqa: E402

REF = os.environ.get("S2_REFERENCE_DIR", "")

# sample sizes of the bw-1024 fixture
BW1024 = 1024
SAMPLE = 4096
BLOCK = 4096          # outputs (grids: 1024 blocks, coefficients: 256)
TABLE_BLOCK = 65536   # tables (2735 blocks each)


def real_field_coeffs(rng, bw, p=0.0):
    """Complex N(0,1)*(1+l)^-p coefficients with f(l,-m) = (-1)^m conj f(l,m), f(l,0) real."""
    from oracle.oracle import Oracle
    o = Oracle()
    rc = np.zeros(bw * bw)
    ic = np.zeros(bw * bw)
    for m in range(bw):
        for l in range(m, bw):
            s = (1.0 + l) ** (-p)
            x, y = rng.standard_normal(2) * s
            if m == 0:
                y = 0.0
            i0 = o.index(m, l, bw)
            rc[i0], ic[i0] = x, y
            if m:
                i1 = o.index(-m, l, bw)
                rc[i1], ic[i1] = (-1) ** m * x, -((-1) ** m) * y
    return rc, ic


def block_norms(v, block=BLOCK):
    """L2 norm of every consecutive block of `block` values (the last one zero-padded)."""
    v = np.asarray(v, dtype=np.float64)
    v = np.pad(v, (0, -v.size % block))
    return np.sqrt((v.reshape(-1, block) ** 2).sum(axis=1))


def bw1024_inputs():
    """The seeded inputs of ref_bw1024.npz: coefficients of a real field N(0,1)(1+l)^-1, a noise
    grid, the zonal filter's coefficients, and the sample positions.  tests/ regenerate them."""
    from tests._util import harmonic_index, real_field_coeffs
    bw = BW1024
    rc, ic = real_field_coeffs(np.random.default_rng(1024), bw, 1.0)
    noise = np.random.default_rng(1025).standard_normal(4 * bw * bw)
    l = np.arange(bw)
    hr = np.zeros(bw * bw)
    hr[harmonic_index(0, l, bw)] = np.exp(-l * (l + 1) / (2 * 150.0 ** 2))
    ps = np.random.default_rng(1026)
    return dict(rc=rc, ic=ic, noise=noise, filter_r=hr, coef_pos=np.sort(ps.choice(bw * bw, SAMPLE, replace=False)),
                grid_pos=np.sort(ps.choice(4 * bw * bw, SAMPLE, replace=False)))


def bw1024_table_positions(offsets, total, bw):
    """Sample positions in the packed tables: up to 8 entries of every order plus SAMPLE more."""
    ps = np.random.default_rng(1027)
    ends = np.append(offsets[1:], total)
    pos = [np.sort(ps.choice(np.arange(a, b), min(8, b - a), replace=False)) for a, b in zip(offsets, ends)]
    pos.append(ps.choice(total, SAMPLE, replace=False))
    return np.unique(np.concatenate(pos))


def make_bw1024(r, out):
    bw = BW1024
    x = bw1024_inputs()
    tf, ti, fwd, inv = r.tables(bw, bw)
    size = fwd.size
    # order offsets of the packed table (m < cutoff = bw: cosine tables back to back)
    offsets = np.cumsum([0] + [r.lib.TableSize(m, bw) for m in range(bw - 1)]).astype(np.int64)
    tpos = bw1024_table_positions(offsets, size, bw)
    grid_r, grid_i = r.inv_fst(x["rc"], x["ic"], bw, REAL, bw, tables=(tf, ti, fwd, inv))
    rt_r, rt_i = r.fst(grid_r, grid_i, bw, REAL, bw, tables=(tf, ti, fwd, inv))
    nz = np.zeros(4 * bw * bw)
    nf_r, nf_i = r.fst(x["noise"], nz, bw, REAL, bw, tables=(tf, ti, fwd, inv))
    filt_r, _ = r.inv_fst(x["filter_r"], np.zeros(bw * bw), bw, REAL, bw, tables=(tf, ti, fwd, inv))
    cv_r, cv_i = r.conv(grid_r, nz, filt_r, nz, bw)
    cp, gp = x["coef_pos"], x["grid_pos"]
    res = dict(bw=bw, block=BLOCK, table_block=TABLE_BLOCK, rc_sum=x["rc"].sum(), ic_sum=x["ic"].sum(),
               rc_sq=(x["rc"] ** 2).sum(), noise_sum=x["noise"].sum(), coef_pos=cp, grid_pos=gp, table_pos=tpos,
               table_offsets=offsets, table_fwd=fwd[tpos], table_inv=inv[tpos],
               table_fwd_blocks=block_norms(fwd, TABLE_BLOCK), table_inv_blocks=block_norms(inv, TABLE_BLOCK))
    for name, (a, b) in dict(inv=(grid_r, grid_i), rt=(rt_r, rt_i), noise_fwd=(nf_r, nf_i), filter_grid=(filt_r, nz),
                             conv=(cv_r, cv_i)).items():
        pos = gp if a.size == 4 * bw * bw else cp
        res[f"{name}_r"], res[f"{name}_i"] = a[pos], b[pos]
        res[f"{name}_r_blocks"], res[f"{name}_i_blocks"] = block_norms(a), block_norms(b)
    np.savez_compressed(os.path.join(out, "ref_bw1024.npz"), **res)


def main():
    if not os.path.isdir(os.path.join(REF, "src")):
        raise SystemExit("set S2_REFERENCE_DIR to the S2kit checkout")
    r = Reference(REF)
    out = HERE
    if "--only" in sys.argv:
        if sys.argv[sys.argv.index("--only") + 1] == "bw1024":
            make_bw1024(r, out)
            return
        raise SystemExit("--only takes: bw1024")

    # ---- copied reference data --------------------------------------------------------
    for bw in (64, 128):
        s = np.loadtxt(os.path.join(REF, "data", f"s{bw}.dat"))
        f = np.loadtxt(os.path.join(REF, "data", f"f{bw}.dat"))
        o = np.loadtxt(os.path.join(REF, "data", f"o{bw}_conv_semi_memo_original.dat"))
        np.savez_compressed(os.path.join(out, f"conv_bw{bw}.npz"), signal=s, filter=f, golden=o, bw=bw)

    ka = {
        "y20_bw8": (8, [(0, 2, 1.0)]),
        "y31_bw8": (8, [(1, 3, 1.0)]),
        "y43_bw23": (23, [(3, 4, np.sqrt(2.0) + np.pi * 1j)]),
        "yMix_bw17": (17, [(1, 1, 1.0), (-2, 5, 3.0 - 2.0j)]),
    }
    for name, (bw, terms) in ka.items():
        d = np.loadtxt(os.path.join(REF, "data", f"{name}.dat")).reshape(-1, 2)
        exp = np.array([(m, l, complex(v).real, complex(v).imag) for (m, l, v) in terms])
        np.savez_compressed(os.path.join(out, f"ka_{name}.npz"), rdata=d[:, 0], idata=d[:, 1], bw=bw,
                            expected=exp)

    # ---- reference outputs on seeded inputs ----------------------------------------
    rng = np.random.default_rng(20240601)
    # round trips through the reference API (the single-function workload uses B=64, p=0)
    cases = [(8, 8, COMPLEX, 0.0), (16, 4, COMPLEX, 0.0), (32, 32, REAL, 1.0), (64, 64, REAL, 0.0),
             (64, 16, COMPLEX, 1.0)]
    for bw, cut, fmt, p in cases:
        if fmt == REAL:
            rc, ic = real_field_coeffs(rng, bw, p)
        else:
            rc = rng.standard_normal(bw * bw)
            ic = rng.standard_normal(bw * bw)
        grid_r, grid_i = r.inv_fst(rc, ic, bw, fmt, cut)
        # forward on an independent (noisy) grid too, so FST is checked off the band-limited subspace
        nr = rng.standard_normal(4 * bw * bw)
        ni = rng.standard_normal(4 * bw * bw) if fmt == COMPLEX else np.zeros(4 * bw * bw)
        frc, fic = r.fst(nr, ni, bw, fmt, cut)
        brc, bic = r.fst(grid_r, grid_i, bw, fmt, cut)
        np.savez_compressed(os.path.join(out, f"ref_sht_bw{bw}_cut{cut}_{'real' if fmt else 'complex'}.npz"),
                            bw=bw, cutoff=cut, fmt=fmt, rcoeffs=rc, icoeffs=ic, inv_r=grid_r, inv_i=grid_i,
                            noise_r=nr, noise_i=ni, fwd_noise_r=frc, fwd_noise_i=fic, rt_r=brc, rt_i=bic)

    # FZT (REAL and COMPLEX) and TransMult at bw=16
    bw = 16
    dr = rng.standard_normal(4 * bw * bw)
    di = rng.standard_normal(4 * bw * bw)
    zr, zi = r.fzt(dr, di, bw, COMPLEX)
    zr2, zi2 = r.fzt(dr, di, bw, REAL)
    a = rng.standard_normal((4, bw * bw))
    fr = rng.standard_normal(bw)
    fi = np.zeros(bw)
    tr = np.zeros(bw * bw)
    ti = np.zeros(bw * bw)
    ptr = lambda x: x.ctypes.data_as(__import__("ctypes").POINTER(__import__("ctypes").c_double))  # noqa: E731
    ad, ai = a[0].copy(), a[1].copy()
    r.lib.TransMult(ptr(ad), ptr(ai), ptr(fr), ptr(fi), ptr(tr), ptr(ti), bw)
    np.savez_compressed(os.path.join(out, "ref_fzt_transmult_bw16.npz"), bw=bw, data_r=dr, data_i=di,
                        fzt_complex_r=zr, fzt_complex_i=zi[:bw], fzt_real_r=zr2, fzt_real_i=zi2,
                        tm_data_r=ad, tm_data_i=ai, tm_filter_r=fr, tm_filter_i=fi, tm_out_r=tr, tm_out_i=ti)

    # tables and weights at bw=16 (cutoff 16 and cutoff 5), weights at 64
    for bw, cut in ((16, 16), (16, 5)):
        _, _, fwd, inv = r.tables(bw, cut)
        np.savez_compressed(os.path.join(out, f"ref_tables_bw{bw}_cut{cut}.npz"), bw=bw, cutoff=cut, fwd=fwd,
                            inv=inv)
    np.savez_compressed(os.path.join(out, "ref_weights.npz"), w16=r.weights(16), w64=r.weights(64),
                        w256=r.weights(256))

    # on-the-fly family (FST_semi_fly.c) on seeded inputs: forward of a noisy grid, inverse of
    # random coefficients, FZT, and the convolution of a noisy signal with a zonal filter grid
    rng = np.random.default_rng(20261204)
    fly = {}
    for bw, cut, fmt in ((16, 16, REAL), (16, 6, COMPLEX), (32, 32, REAL), (32, 20, COMPLEX)):
        tag = f"bw{bw}_cut{cut}_{'real' if fmt else 'complex'}"
        nr = rng.standard_normal(4 * bw * bw)
        ni = rng.standard_normal(4 * bw * bw) if fmt == COMPLEX else np.zeros(4 * bw * bw)
        if fmt == REAL:
            rc, ic = real_field_coeffs(rng, bw, 1.0)
        else:
            rc, ic = rng.standard_normal(bw * bw), rng.standard_normal(bw * bw)
        fr_, fi_ = r.fst_fly(nr, ni, bw, fmt, cut)
        gr_, gi_ = r.inv_fst_fly(rc, ic, bw, fmt, cut)
        fly.update({f"{tag}_grid_r": nr, f"{tag}_grid_i": ni, f"{tag}_fst_r": fr_, f"{tag}_fst_i": fi_,
                    f"{tag}_coef_r": rc, f"{tag}_coef_i": ic, f"{tag}_inv_r": gr_, f"{tag}_inv_i": gi_})
    bw = 16
    zr_, zi_ = rng.standard_normal(4 * bw * bw), rng.standard_normal(4 * bw * bw)
    fly["fzt_bw16_data_r"], fly["fzt_bw16_data_i"] = zr_, zi_
    fly["fzt_bw16_complex_r"], fly["fzt_bw16_complex_i"] = r.fzt_fly(zr_, zi_, bw, COMPLEX)
    fly["fzt_bw16_real_r"], fly["fzt_bw16_real_i"] = r.fzt_fly(zr_, zi_, bw, REAL)
    hr = np.zeros(bw * bw)
    for l in range(bw):
        hr[r.lib.IndexOfHarmonicCoeff(0, l, bw)] = np.exp(-l * (l + 1) / (2 * 6.0 ** 2))
    filt_r, _ = r.inv_fst(hr, np.zeros(bw * bw), bw, REAL, bw)
    sig = rng.standard_normal(4 * bw * bw)
    fly["conv_bw16_signal"], fly["conv_bw16_filter"] = sig, filt_r
    fly["conv_bw16_out_r"], fly["conv_bw16_out_i"] = r.conv_fly(sig, np.zeros(4 * bw * bw), filt_r,
                                                                np.zeros(4 * bw * bw), bw)
    np.savez_compressed(os.path.join(out, "ref_fly.npz"), **fly)
    make_bw1024(r, out)

    print("fixtures written to", out)


if __name__ == "__main__":
    main()
