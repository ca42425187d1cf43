"""Scene-sharded serving over several devices (fluidsim.dispatch) without a
GPU: the placement by free HBM budget, a dispatcher over a fake device set
whose backends step each request with the oracle on the CPU (results equal
each request run alone), and two gloo ranks that each serve their own share
of one stream -- the same placement computed on both, every request served
exactly once, nothing exchanged but the results gathered for the check."""
import hashlib
import os
import pathlib
import socket
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
BPP = 1000  # state bytes per particle of the fake devices


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def small_requests(count=6, seed=3):
    """Small dam-break requests (200-600 particles, 2-4 steps of 1/180 s)."""
    sys.path[:0] = [str(ROOT), str(ROOT / "fluid-simulation-3d_gb300")]
    from fluidsim import scenes, server
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(rng.integers(200, 600))
        pos, vel, bound = scenes.fill_box_scene(rng, n, 0.4, (1.0, 0.75, 1.0))
        p = scenes.SimParams(radius=0.35, bound=bound, **scenes.DAM_CONSTANTS)
        out.append(server.Request(k, p, pos, vel, 1.0 / 180.0, 1, int(rng.integers(2, 5)),
                                  arrival=0.01 * k))
    return out


def run_alone(req):
    """The request stepped on its own with the oracle (Jacobi, FP32)."""
    import oracle
    pos, vel = req.pos.copy(), req.vel.copy()
    d = {}
    for _ in range(req.steps):
        for _ in range(req.substeps):
            pos, vel, d = oracle.substep_f32(req.params, pos, vel,
                                             np.float32(req.dt / req.substeps), nthreads=1)
    return pos, vel, d["dens"]


class OracleBackend:
    """A fake device: serves requests with the oracle when collected."""

    def __init__(self, device):
        self.device = device
        self.jobs = {}
        self.closed = False

    def submit(self, req):
        self.jobs[req.rid] = req
        return req.rid

    def wait(self, job, timeout=600.0):
        return run_alone(self.jobs.pop(job))

    def close(self):
        self.closed = True


def digest(result):
    return hashlib.sha256(b"".join(np.ascontiguousarray(a).tobytes() for a in result)).hexdigest()


def test_place_by_free_budget():
    from fluidsim.dispatch import place
    # budgets 10k, 10k, 4k bytes at 1000 B a particle
    assert place([5, 3, 4, 2, 6], [10_000, 10_000, 4_000], 1000) == [0, 1, 1, 0, 2]
    assert place([1, 1, 1], [5_000] * 3, 1000) == [0, 1, 2]  # ties: lowest index
    # over budget everywhere: the least loaded device still takes it
    assert place([9, 9, 9], [5_000, 5_000], 1000) == [0, 1, 0]
    sizes = list(np.random.default_rng(0).integers(1, 50, 40))
    assert place(sizes, [30_000] * 4, 1000) == place(sizes, [30_000] * 4, 1000)


def test_dispatcher_fake_devices_match_alone(oracle_mod):
    from fluidsim.dispatch import Dispatcher, place
    reqs = small_requests()
    backs = [OracleBackend(d) for d in range(3)]
    disp = Dispatcher(backs, [600 * BPP] * 3, BPP)
    done, placed = disp.run(reqs)
    disp.close()
    assert all(b.closed for b in backs)
    assert [placed[r.rid] for r in reqs] == place([r.n for r in reqs], [600 * BPP] * 3, BPP)
    assert len(set(placed.values())) == 3  # the stream spread over every device
    assert disp.used == [0, 0, 0]  # collected requests free their budget
    for r in reqs:
        for g, w in zip(done[r.rid], run_alone(r)):
            assert np.array_equal(g, w)


def _shard_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path[:0] = [str(ROOT), str(ROOT / "fluid-simulation-3d_gb300")]
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from fluidsim.dispatch import Dispatcher, shard
    reqs = small_requests()
    mine = shard(reqs, rank, world, 600 * BPP, BPP)
    disp = Dispatcher([OracleBackend(rank)], [600 * BPP], BPP)
    done, _ = disp.run(mine)
    disp.close()
    got = [None] * world
    dist.all_gather_object(got, {rid: digest(r) for rid, r in done.items()})
    out.put((rank, got))
    dist.destroy_process_group()


def test_two_ranks_serve_disjoint_shares(oracle_mod):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    shares = res[0][1]
    assert shares == res[1][1]
    rids = [rid for s in shares for rid in s]
    reqs = small_requests()
    assert sorted(rids) == [r.rid for r in reqs]  # each request served exactly once
    assert all(len(s) > 0 for s in shares)
    merged = {rid: h for s in shares for rid, h in s.items()}
    for r in reqs:
        assert merged[r.rid] == digest(run_alone(r))


def test_failed_wait_keeps_the_budget_until_forgotten():
    from fluidsim.dispatch import Dispatcher

    class Slow(OracleBackend):
        def wait(self, job, timeout=600.0):
            raise TimeoutError("still running")

    reqs = small_requests(2)
    disp = Dispatcher([Slow(0)], [10_000 * BPP], BPP)
    pl = disp.submit(reqs[0])
    with pytest.raises(TimeoutError):
        disp.wait(pl.rid)
    assert disp.used == [reqs[0].n * BPP]  # still running: still placed
    disp.forget(pl.rid)
    assert disp.used == [0]
