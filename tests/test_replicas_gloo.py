"""The replica path of bench.py under torch.distributed (gloo, world size 2, CPU only).

A single solve does not shard: under torchrun every rank advances its own replica, and
the ranks meet only at the barriers around the timed region and in the max-over-ranks
reduction of the elapsed time.  These tests run that host logic as two CPU processes;
no GPU is involved.
"""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=2)
    ws, r, _ = bench.dist_env()
    assert (ws, r) == (2, rank)
    bench.barrier(ws)
    out[rank] = bench.reduce_max(1.5 + rank, ws)
    bench.barrier(ws)
    dist.destroy_process_group()


def test_timed_region_reduces_to_the_slowest_rank():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    out = ctx.Array("d", 2)
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert [p.exitcode for p in procs] == [0, 0]
    assert list(out) == [2.5, 2.5]


def test_reference_arm_prints_one_line_from_rank_zero():
    """`bench.py --impl reference` under torchrun with two ranks: rank 0 times the CPU
    path and prints the only JSON line; rank 1 exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", "--master-port=%d" % _free_port(), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--workload", "ch2d-256", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
