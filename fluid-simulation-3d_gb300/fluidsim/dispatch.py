"""Scene-sharded serving over several GPUs of one node.

Batched and served scenes are independent: a request's particles only ever
interact with each other, so requests shard across GPUs with no exchange
between them. The dispatcher owns one serving backend per device (by default
the library's native serving loop, sph_server_*, created with that device
current) and places every request, as it arrives, on the device with the
most free HBM budget: budget minus the state bytes (particles x
sph_bytes_per_particle) of the requests placed there and not yet collected.
Ties go to the lowest device index, so the placement of a stream depends on
the stream alone. A request that fits no device's free budget still goes to
the least loaded one, whose serving loop queues it until room frees up.

The same placement runs in every rank of a multi-process job (one process
per GPU, `shard`): each rank serves the requests placed on its own device,
so the ranks need no collective on the data path. The reference has no
distributed form; its only parallelism is the std::execution::par loops of
engine/physics/physicsWorld.cc:42,63,72,81 inside one scene.
"""
from __future__ import annotations

import dataclasses


@dataclasses.dataclass
class Placement:
    rid: int
    device: int
    job: object = None


def place(sizes, budgets, bytes_per_particle):
    """Device of each request for request sizes `sizes` (particles, in
    arrival order) over devices with HBM budgets `budgets` (bytes), when no
    request finishes in between: greedy on the most free budget, ties to the
    lowest index. Pure function of its inputs (every rank computes the same
    placement)."""
    free = [int(b) for b in budgets]
    out = []
    for n in sizes:
        need = int(n) * int(bytes_per_particle)
        d = max(range(len(free)), key=lambda k: (free[k], -k))
        free[d] -= need
        out.append(d)
    return out


class NativeBackend:
    """The library's serving loop on one device."""

    def __init__(self, device, budget_bytes, max_scenes=8192, substeps=3):
        import torch

        from .server import NativeServer
        torch.cuda.set_device(device)  # the server takes the current device
        self.device = device
        self.server = NativeServer(budget_bytes, max_scenes=max_scenes, substeps=substeps)

    def submit(self, req):
        return self.server.submit(req.params, req.pos, req.vel, req.dt, req.steps)

    def wait(self, job, timeout=600.0):
        return self.server.wait(job, timeout)

    def close(self):
        self.server.close()


class Dispatcher:
    """One backend per device; requests placed by free HBM budget.

    backends: list of objects with submit(request) -> job, wait(job) ->
    (pos, vel, dens) and close(); budgets: bytes per device; the state of a
    request is request.n * bytes_per_particle bytes."""

    def __init__(self, backends, budgets, bytes_per_particle):
        if len(backends) != len(budgets) or not backends:
            raise ValueError("one budget per backend, at least one")
        self.backends = list(backends)
        self.budgets = [int(b) for b in budgets]
        self.bpp = int(bytes_per_particle)
        self.used = [0] * len(backends)
        self._live = {}  # rid -> Placement

    @classmethod
    def native(cls, devices, budget_bytes, max_scenes=8192, substeps=3):
        from .server import bytes_per_particle
        backs = [NativeBackend(d, budget_bytes, max_scenes, substeps) for d in devices]
        return cls(backs, [budget_bytes] * len(backs), bytes_per_particle())

    def choose(self, n):
        free = [b - u for b, u in zip(self.budgets, self.used)]
        return max(range(len(free)), key=lambda k: (free[k], -k))

    def submit(self, req):
        d = self.choose(req.n)
        self.used[d] += req.n * self.bpp
        pl = Placement(req.rid, d, self.backends[d].submit(req))
        self._live[req.rid] = (pl, req.n)
        return pl

    def wait(self, rid, timeout=600.0):
        """The result of request `rid`; its budget is released once collected.
        A wait that raises (still running after `timeout`, cancelled, failed)
        keeps it placed: wait again, or forget() it."""
        pl, n = self._live[rid]
        res = self.backends[pl.device].wait(pl.job, timeout)
        self.forget(rid)
        return res

    def forget(self, rid):
        """Drop request `rid` from the placement accounting (its budget is
        free again), e.g. after it was cancelled or failed."""
        pl, n = self._live.pop(rid)
        self.used[pl.device] -= n * self.bpp

    def run(self, requests):
        """Submit every request (arrival order), then collect: results by
        rid and the device each request ran on."""
        placed = {r.rid: self.submit(r).device for r in sorted(requests, key=lambda q: q.arrival)}
        done = {rid: self.wait(rid) for rid in list(placed)}
        return done, placed

    def close(self):
        for b in self.backends:
            b.close()


def shard(requests, rank, world, budget_bytes, bytes_per_particle):
    """The requests a rank of a `world`-rank job serves: the same placement
    computed on every rank (place() over equal budgets, arrival order), this
    rank's share kept."""
    reqs = sorted(requests, key=lambda q: q.arrival)
    dev = place([r.n for r in reqs], [budget_bytes] * world, bytes_per_particle)
    return [r for r, d in zip(reqs, dev) if d == rank]
