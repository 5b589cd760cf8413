"""The N > 1 launch path of bench.py on CPU (gloo, world size 2).

The solve path does not shard (replicas only), so what N > 1 adds is the
launcher plumbing: rank discovery, the barrier, the max over ranks of the
timed region, and "rank 0 alone prints the line".  Checked here with two gloo
ranks on 127.0.0.1, and end to end through torch.distributed.run with the
CPU reference arm (rank 0 runs the oracle port and prints one JSON line, the
other rank exits 0 without work).
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    import torch.distributed as dist
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        got_ws, got_rank, got_local = bench.dist_setup()
        bench.barrier(ws)
        m = bench.max_over_ranks(10.0 + rank, ws)
        q.put((got_ws, got_rank, got_local, m))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_max_and_barrier():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [0, 1] and all(r[0] == 2 for r in res)
    assert all(r[3] == 11.0 for r in res)  # max over ranks seen by both


def test_torchrun_reference_arm_two_ranks():
    pytest.importorskip("torch")
    oracle_lib = [f for f in os.listdir(os.path.join(ROOT, "oracle")) if f.endswith(".so")]
    if not oracle_lib:
        pytest.skip("oracle library not built")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--cube-n", "4", "--steps", "1", "--warmup", "3"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout  # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0
