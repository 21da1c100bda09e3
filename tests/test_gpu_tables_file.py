"""Table files (s2g_tables_save / s2g_tables_load): the device tables of one process, saved to
disk, reproduce that process's transforms bit for bit in another process that loads them instead
of generating; corrupt, truncated or mismatched files are rejected.  Each process is separate
because the table cache lives for the whole process."""
import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys, json, time, hashlib, ctypes as C
sys.path.insert(0, %r)
import numpy as np, torch
from s2kit_gb300 import api, load
lib = load()
mode, path, bw = sys.argv[1], sys.argv[2], int(sys.argv[3])
torch.cuda.init()
t0 = time.perf_counter()
if mode == "save":
    st = lib.s2g_tables_save(bw, bw, path.encode())
elif mode == "load":
    b, c = C.c_int(), C.c_int()
    st = lib.s2g_tables_load(path.encode(), C.byref(b), C.byref(c))
    assert st != 0 or (b.value, c.value) == (bw, bw)
else:
    st = 0
dt = time.perf_counter() - t0
if st != 0:
    print(json.dumps({"status": st, "error": lib.s2g_last_error().decode()})); sys.exit(0)
t1 = time.perf_counter()
plan = api.Plan(bw, bw)
torch.cuda.synchronize()
dplan = time.perf_counter() - t1
rng = np.random.default_rng(3)
n = 2 * bw
g = torch.from_numpy(rng.standard_normal((2, n * n))).cuda()
rc, ic = torch.zeros(2, bw * bw, dtype=torch.float64, device="cuda"), torch.zeros(2, bw * bw, dtype=torch.float64, device="cuda")
plan.fst(g, None, rc, ic, 2, api.REAL)
out = torch.zeros_like(g)
plan.inv_fst(rc, ic, out, None, 2, api.REAL)
torch.cuda.synchronize()
h = hashlib.sha256(rc.cpu().numpy().tobytes() + ic.cpu().numpy().tobytes() + out.cpu().numpy().tobytes()).hexdigest()
print(json.dumps({"status": 0, "hash": h, "seconds": dt, "plan_seconds": dplan}))
""" % ROOT


def _child(mode, path, bw):
    r = subprocess.run([sys.executable, "-c", CHILD, mode, str(path), str(bw)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("bw", [64, 256])
def test_saved_tables_reproduce_transforms(tmp_path, bw):
    f = tmp_path / f"tables_{bw}.s2gtab"
    saved = _child("save", f, bw)
    assert saved["status"] == 0
    loaded = _child("load", f, bw)
    fresh = _child("none", f, bw)
    assert loaded["status"] == 0
    assert loaded["hash"] == saved["hash"] == fresh["hash"]


def test_table_file_errors(tmp_path):
    f = tmp_path / "t.s2gtab"
    assert _child("save", f, 32)["status"] == 0
    data = bytearray(open(f, "rb").read())
    bad = tmp_path / "bad.s2gtab"
    data2 = bytearray(data)
    data2[len(data2) // 2] ^= 0x40
    open(bad, "wb").write(bytes(data2))
    r = _child("load", bad, 32)
    assert r["status"] != 0 and "hash mismatch" in r["error"]
    short = tmp_path / "short.s2gtab"
    open(short, "wb").write(bytes(data[: len(data) - 8]))
    r = _child("load", short, 32)
    assert r["status"] != 0 and "truncated" in r["error"]
    other = tmp_path / "other.s2gtab"
    d3 = bytearray(data)
    d3[8:16] = (16).to_bytes(4, "little") + (16).to_bytes(4, "little")  # claims bw 16, cutoff 16: sizes differ
    open(other, "wb").write(bytes(d3))
    r = _child("load", other, 16)
    assert r["status"] != 0 and "needs" in r["error"]
    # loading over tables that already exist in the process is refused
    from s2kit_gb300 import api, load
    lib = load()
    api.Plan(32, 32)
    st = lib.s2g_tables_load(str(f).encode(), None, None)
    assert st != 0 and b"already exist" in lib.s2g_last_error()


def test_table_file_timing_bw1024(tmp_path):
    """Records generation (GPU) against loading (disk) at bw 1024; both work, either may be faster."""
    f = tmp_path / "t1024.s2gtab"
    saved = _child("save", f, 1024)
    loaded = _child("load", f, 1024)
    assert loaded["status"] == 0 and loaded["hash"] == saved["hash"]
    size = os.path.getsize(f)
    print(f"bw 1024 tables: file {size / 2**30:.2f} GiB; generate+save {saved['seconds']:.2f} s, "
          f"load {loaded['seconds']:.2f} s")
