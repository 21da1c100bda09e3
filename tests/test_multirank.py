"""The N>1 path of bench.py on CPU: gloo ranks (world size 2), no GPU.

Functions are independent, so each rank transforms its own batch (weak scaling) and the only
communication is the max-over-ranks reduction of the step time.  These tests run that
reduction and the throughput aggregation with gloo, and launch the reference arm under
torchrun (rank 0 alone prints the JSON line, the other rank exits 0).
"""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    # each rank: its own seeded batch, a transform through the oracle, a local "step time"
    from oracle.oracle import Oracle
    orc = Oracle()
    rc, ic = bench.real_field_coeffs(np.random.default_rng(100 + rank), 8, 1.0, 2)
    out = []
    for f in range(2):
        g, _ = orc.inv_fst(rc[f], ic[f], 8, 1, 8)
        a, b = orc.fst(g, np.zeros_like(g), 8, 1, 8)
        out.append(max(np.abs(a - rc[f]).max(), np.abs(b - ic[f]).max()))
    ms_local = 10.0 + 5.0 * rank
    ms = bench.reduce_max(ms_local, dist, "cpu")
    value = bench.weak_scaling_value(2, ws, ms)
    q.put((rank, ms, value, max(out)))
    dist.destroy_process_group()


def test_gloo_two_ranks_reduce_and_aggregate():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value, err in res:
        assert ms == 15.0                      # the slowest rank
        assert value == pytest.approx(2 * 2 / 0.015)
        assert err < 1e-12                     # each rank's shard transformed correctly


def test_reference_arm_under_torchrun():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--bw", "16"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port"
