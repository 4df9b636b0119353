"""The N > 1 host path of bench.py on CPU with the gloo backend, world size 2: the barrier and the
max-over-ranks timing reduction, and the reference arm under torchrun (rank 0 alone prints one JSON
line, the other rank exits 0 without output).  The data path has no collective (replicas)."""
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


def _worker(rank, world, port, out_path):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist()
    d.barrier()
    m = d.max(1.5 + rank)  # per-rank "times"; the job time is the slowest rank's
    d.barrier()
    if rank == 0:
        with open(out_path, "w") as f:
            json.dump({"world": d.world, "max": m}, f)
    d.close()


def test_dist_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp

    out = str(tmp_path / "dist.json")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    r = json.load(open(out))
    assert r == {"world": 2, "max": 2.5}


def test_reference_arm_under_torchrun_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--workload", "h2o16", "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-seconds", "1"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


def test_gpu_arm_cpu_baseline_runs_in_a_clean_child(monkeypatch):
    """The GPU arm's cpu_baseline is the reference arm run as a child process: it must not inherit the
    torchrun rendezvous variables (the child would try to join the process group) and it reports the
    measured sample."""
    import bench

    for k, v in (("RANK", "0"), ("WORLD_SIZE", "2"), ("LOCAL_RANK", "0"), ("MASTER_ADDR", "127.0.0.1"),
                 ("MASTER_PORT", str(_free_port()))):
        monkeypatch.setenv(k, v)
    cpu = bench.cpu_baseline("h2o16", 1.0)
    assert cpu["kind"] == "port" and cpu["unit"] == "Fock builds/s"
    assert cpu["value"] > 0 and cpu["cores"] >= 1
    assert "measured" in cpu["sample"] and "child process" in cpu["how"]
