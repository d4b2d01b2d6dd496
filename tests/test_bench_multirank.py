"""The multi-rank side of bench.py on CPU (gloo, two ranks): each rank runs a replica, the slowest
rank's time is taken (max over ranks) and the whole-job rate counts every rank's units; the
reference arm (the reference's own time loop on the host cores) prints one line, from rank 0."""
import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = [3.0, 5.0][rank]                       # rank 1 is the slow one
        t = bench.max_over_ranks(local, world, device="cpu")
        out[rank] = (t, bench.whole_job_rate(1000.0, world, t))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_on_two_gloo_ranks():
    port = free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        res = dict(out)
    assert res[0] == res[1] == (5.0, 400.0)


def test_one_rank_is_the_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(2.5, 1, device="cpu") == 2.5
    assert bench.whole_job_rate(100.0, 1, 2.0) == 50.0


def test_reference_arm_prints_once_on_two_ranks():
    import oracle_lib as O

    O.lib(fast=True)                                    # built here, not by both ranks at once
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--size", "64", "--steps", "2", "--warmup", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0
    # the reference's own sources when their tree is staged (baseline/_ref), else the oracle port
    staged = os.path.isdir(os.path.join(ROOT, "baseline", "_ref", "src", "kernels"))
    assert d["cpu_baseline"]["kind"] == ("reference" if staged else "port")
