"""Command-line drivers (bin/test_s2_semi_memo_fwd and the reference's other test-program names,
s2kit_gb300/cli/s2kit_drivers.c): the reference programs' arguments, text input and output
formats, run through the library.  GPU tests feed them committed fixtures: the known-answer
sample files, a reference inverse fixture, the real-FFTW convolution goldens, plus the round-trip
and 1-D programs' own error reports.  Without a GPU the programs must fail loudly."""
import os
import re
import subprocess

import numpy as np
import pytest

import s2kit_gb300  # noqa: F401
from s2kit_gb300 import build as b
from tests._util import harmonic_index, rel_err_norm


def _bin(name):
    b.build()
    p = os.path.join(b.BIN_DIR, name)
    assert os.path.exists(p), p
    return p


def _run(name, *args, check=True):
    r = subprocess.run([_bin(name), *map(str, args)], capture_output=True, text=True, timeout=300)
    if check:
        assert r.returncode == 0, r.stdout + r.stderr
    return r


def _write_pairs(path, a, b_):
    with open(path, "w") as f:
        for x, y in zip(a, b_):
            f.write("%.17g %.17g\n" % (x, y))


def _gpu():
    import torch
    return torch.cuda.is_available()


def test_cli_usage_and_names():
    for n in b.CLI_NAMES:
        r = _run(n)
        assert r.stdout.startswith(f"Usage: {n} "), r.stdout
    r = _run("s2kit", check=False)
    assert r.returncode == 2 and "test_s2_semi_memo_fwd" in r.stdout


def test_cli_fails_loudly_without_gpu(tmp_path):
    if _gpu():
        pytest.skip("a GPU is present")
    f = tmp_path / "s.txt"
    _write_pairs(f, np.zeros(256), np.zeros(256))
    r = _run("test_s2_semi_memo_fwd", f, tmp_path / "o.txt", 8, check=False)
    assert r.returncode == 1 and "FSTSemiMemo" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["y20_bw8", "y31_bw8", "yMix_bw17"])
def test_cli_forward_known_answers(golden, tmp_path, name):
    g = golden("ka_" + name)
    bw = int(g["bw"])
    src = tmp_path / "samples.txt"
    _write_pairs(src, g["rdata"], g["idata"])
    out = tmp_path / "coeffs.txt"
    _run("test_s2_semi_memo_fwd", src, out, bw)
    v = np.loadtxt(out).reshape(-1, 2)
    rc, ic = v[:, 0], v[:, 1]
    er, ei = np.zeros(bw * bw), np.zeros(bw * bw)
    for m, l, re_, im_ in g["expected"]:
        k = int(harmonic_index(int(m), int(l), bw))
        er[k], ei[k] = re_, im_
    assert rel_err_norm(rc, ic, er, ei) <= 1e-11
    # human-readable format: "l = %d\t m = %d\t %.15f + %.15f I", l major, m from -l to l
    out2 = tmp_path / "coeffs_hr.txt"
    _run("test_s2_semi_memo_fwd", src, out2, bw, 1)
    lines = open(out2).read().splitlines()
    assert len(lines) == bw * bw
    pat = re.compile(r"^l = (\d+)\t m = (-?\d+)\t (\S+) \+ (\S+) I$")
    seen = [(int(pat.match(s).group(1)), int(pat.match(s).group(2))) for s in lines]
    assert seen == [(l, m) for l in range(bw) for m in range(-l, l + 1)]


@pytest.mark.gpu
def test_cli_inverse_vs_reference(golden, tmp_path):
    g = golden("ref_sht_bw8_cut8_complex")  # the reference's InvFSTSemiMemo, COMPLEX, cutoff = bw
    src = tmp_path / "coeffs.txt"
    _write_pairs(src, g["rcoeffs"], g["icoeffs"])
    out = tmp_path / "samples.txt"
    _run("test_s2_semi_memo_inv", src, out, 8)
    v = np.loadtxt(out).reshape(-1, 2)
    assert rel_err_norm(v[:, 0], v[:, 1], g["inv_r"], g["inv_i"]) <= 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("prog", ["test_conv_semi_memo", "test_conv_semi_fly"])
def test_cli_convolution_vs_fftw_golden(golden, tmp_path, prog):
    g = golden("conv_bw64")  # data/s64.dat, f64.dat and o64_conv_semi_memo_original.dat (real FFTW3)
    s, f = tmp_path / "s.txt", tmp_path / "f.txt"
    np.savetxt(s, g["signal"], fmt="%.17g")
    np.savetxt(f, g["filter"], fmt="%.17g")
    out = tmp_path / "o.txt"
    _run(prog, s, f, out, 64)
    got = np.loadtxt(out)
    gold = g["golden"]
    assert np.abs(got - gold).max() <= 1e-11 * np.abs(gold).max()


@pytest.mark.gpu
@pytest.mark.parametrize("prog", ["test_s2_semi_memo", "test_s2_semi_fly"])
def test_cli_roundtrip_reports(tmp_path, prog):
    err = tmp_path / "errors.txt"
    r = _run(prog, 16, 2, err)
    assert f"Program: {prog}" in r.stdout and "Bandwidth = 16" in r.stdout
    avg = float(re.search(r"Average r-o error:\s+(\S+)", r.stdout).group(1))
    assert avg <= 1e-12
    lines = open(err).read().splitlines()
    assert len(lines) == 2 * (16 * 17 // 2)
    assert lines[0].startswith("index = 0\t m = 0\tl = 0\t")


@pytest.mark.gpu
@pytest.mark.parametrize("prog", ["test_DLT_semi", "test_DLT_naive"])
def test_cli_dlt_reports(prog):
    r = _run(prog, 3, 32, 2)
    assert r.stdout.startswith("bw = 32\tm = 3\nloops = 2\n")
    avg = float(re.search(r"Average r-o error:\s+(\S+)", r.stdout).group(1))
    assert avg <= 1e-12
    assert "average forward time" in r.stdout and "average inverse time" in r.stdout
