"""Multi-process paths of bench.py on CPU with gloo (world size 2): the
max-over-ranks clock and the reference arm under torchrun (rank 0 alone
measures and prints one line; the other rank exits 0 without work)."""
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


def _worker(rank, port, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    dist.barrier()
    v = bench.max_over_ranks(dist, 1.5 + rank)
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
        f.write(repr(v))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_with_gloo(tmp_path):
    import torch.multiprocessing as mp

    mp.start_processes(_worker, args=(_free_port(), str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    vals = [float(open(tmp_path / f"r{r}.txt").read()) for r in range(2)]
    assert vals == [2.5, 2.5]


def test_reference_arm_under_torchrun(oracle_lib):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "3", "--workload", "tiny"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0


def _replica_worker(rank, port, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench
    from ocean_gb300 import workloads as WL

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    # each replica builds its own problem, as run_ours does (seed = rank)
    w = WL.make("tiny", seed=rank)
    # rank 1 is the slower one: the job's clock is its time
    rate, ms = bench.replica_rate(dist, 2, 100.0 + 50.0 * rank, 3000)
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"rate": rate, "ms": ms, "psi0": float(w.psi_r[0])}, f)
    dist.barrier()
    dist.destroy_process_group()


def test_repo_arm_replica_rate_with_gloo(tmp_path):
    """The repo arm's replica bookkeeping over two gloo ranks: each rank's own
    problem, the job's H*psi/s = all ranks' work over the slowest rank's time."""
    import torch.multiprocessing as mp

    mp.start_processes(_replica_worker, args=(_free_port(), str(tmp_path)), nprocs=2, start_method="spawn",
                       join=True)
    r = [json.load(open(tmp_path / f"r{k}.json")) for k in range(2)]
    assert r[0]["ms"] == r[1]["ms"] == 150.0
    assert r[0]["rate"] == r[1]["rate"] == 2 * 3000 / 0.150
    assert r[0]["psi0"] != r[1]["psi0"]  # different problems per replica
