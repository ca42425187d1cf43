"""The N>1 form of the benchmark without a GPU: replicas timed with a
barrier and the job time taken as the max over ranks, over gloo with two
processes on the CPU, and the reference arm under torchrun (rank 0 alone
runs and prints; the other rank exits 0 without work)."""
import json
import os
import pathlib
import socket
import subprocess
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r timed 100 + 50 r ms for 10 steps of 1000 particles
    value, job_ms = bench.replica_throughput(1000, 10, 100.0 + 50.0 * rank, world, "cpu")
    dist.barrier()
    out.put((rank, value, job_ms))
    dist.destroy_process_group()


def test_replica_throughput_max_over_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, job_ms in got:
        assert job_ms == pytest.approx(150.0)  # the slower rank's time
        # whole-job particle-steps/s: both replicas' work over the job time
        assert value == pytest.approx(2 * 1000 * 10 / 0.150)


def test_single_rank_is_its_own_max():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(12.5, 1, "cpu") == 12.5
    value, job_ms = bench.replica_throughput(500, 4, 20.0, 1, "cpu")
    assert job_ms == 20.0 and value == pytest.approx(500 * 4 / 0.020)


def test_reference_arm_under_torchrun():
    """Two ranks of `bench.py --impl reference`: one JSON line, from rank 0."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--workload", "dam_break_16k",
           "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
