"""Builds libs2kit_gb300.so in-tree for sm_103a (nvcc, one -gencode, TUs compiled in parallel),
and the command-line drivers bin/s2kit (linked as bin/test_s2_semi_memo_fwd and the reference's
other test-program names) over its C ABI.

    python -m s2kit_gb300.build          # or __graft_entry__.build()

The library has no torch dependency: a plain C ABI (include/s2kit_gb300.h) over the CUDA
runtime, linked statically against cudart.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "libs2kit_gb300.so")
BUILD_DIR = os.path.join(PKG, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["capi.cu", "tables.cu", "sht_fp64.cu", "sht_split.cu", "czt_split.cu", "group.cu", "refine.cu",
           "noalloc.cu"]
CLI_SRC = os.path.join(PKG, "cli", "s2kit_drivers.c")
BIN_DIR = os.path.join(PKG, "bin")
CLI_NAMES = ["test_s2_semi_memo_fwd", "test_s2_semi_memo_inv", "test_s2_semi_memo", "test_s2_semi_fly",
             "test_conv_semi_memo", "test_conv_semi_fly", "test_DLT_semi", "test_DLT_naive"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
           "-I", os.path.join(ROOT, "include"), "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def _stale() -> bool:
    if not os.path.exists(OUT):
        return True
    t = os.path.getmtime(OUT)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "s2kit_gb300.h"),
                                                                 __file__]
    return any(os.path.getmtime(d) > t for d in deps)


def build_cli() -> str:
    """Compiles bin/s2kit (host C, gcc) against the in-tree library and links the program names."""
    exe = os.path.join(BIN_DIR, "s2kit")
    if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(CLI_SRC), os.path.getmtime(OUT)):
        return exe
    os.makedirs(BIN_DIR, exist_ok=True)
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the command-line drivers")
    cmd = [cc, "-O2", "-std=c11", "-I", os.path.join(ROOT, "include"), CLI_SRC, "-o", exe + ".tmp", "-L", PKG,
           "-ls2kit_gb300", "-Wl,-rpath,$ORIGIN/..", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command-line drivers failed to build:\n{r.stderr}")
    os.replace(exe + ".tmp", exe)
    for n in CLI_NAMES:
        link = os.path.join(BIN_DIR, n)
        if os.path.lexists(link):
            os.remove(link)
        os.symlink("s2kit", link)
    return exe


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        build_cli()
        return OUT
    os.makedirs(BUILD_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = OUT + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, OUT)
    build_cli()
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
