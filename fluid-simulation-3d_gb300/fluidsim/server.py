"""Serving form: a continuous-batching request loop over the batched engine.

Requests (a scene of N particles to advance K steps) arrive over time. The
loop admits them, first come first served, with smaller later requests
allowed to backfill. A request is admitted while the HBM state budget
(capacity = budget / device bytes per particle) and the scene slots have
room. Admitted state stays resident on the device, and every resident scene
advances one step per batched launch, so requests that arrive while others
run share the device with them. A request leaves, with its final state read
back, after its K-th step. A request can be withdrawn with cancel() (for
instance from the per-step callback): it is dropped if it has not been
admitted, and a resident one leaves the batch at the next step boundary,
freeing its capacity for the requests still waiting. checkpoint() persists
the loop between steps (scene snapshots of the resident requests, the queue,
the finished results); resume() turns that into requests for a new loop.
The loop records each request's per-step latency: the wall time of the
batched step it took part in, measured with a stream sync around the step.

The batched step runs the same per-particle arithmetic in the same order as a
scene stepped alone, so every result is the same alone and in the mix (the
GPU tests check it bit for bit).
"""
from __future__ import annotations

import dataclasses
import json
import os
import time

import numpy as np

from . import _lib, snapshot
from .simulation import Batch, FluidSimulation, to_params


@dataclasses.dataclass
class Request:
    rid: int
    params: object
    pos: np.ndarray
    vel: np.ndarray
    dt: float
    substeps: int
    steps: int
    arrival: float = 0.0  # seconds after the loop starts
    snapshot: str | None = None  # resumed: admitted from this scene snapshot

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])


@dataclasses.dataclass
class Done:
    rid: int
    pos: np.ndarray
    vel: np.ndarray
    dens: np.ndarray
    admitted: float
    finished: float
    step_ms: list


def bytes_per_particle() -> int:
    return int(_lib.load().sph_bytes_per_particle())


class Server:
    """Continuous batching under an HBM budget (bytes of resident state)."""

    def __init__(self, budget_bytes: int, max_scenes: int = 4096, stream=None,
                 tuning=None):
        self.capacity = max(1, int(budget_bytes) // bytes_per_particle())
        self.batch = Batch(self.capacity, max_scenes, stream)
        if tuning:
            self.batch.set_tuning(**tuning)
        self.resident = {}  # scene id -> [request, steps left, admitted, step_ms]
        self._cancel = set()  # request ids to withdraw at the next boundary

    def close(self):
        self.batch.close()

    def cancel(self, rid: int) -> None:
        """Withdraw request `rid` at the next step boundary of run(); it
        returns no result. Ids of requests already finished are ignored."""
        self._cancel.add(int(rid))

    def _apply_cancels(self, pending, waiting, cancelled):
        if not self._cancel:
            return
        for queue in (pending, waiting):
            for req in [r for r in queue if r.rid in self._cancel]:
                queue.remove(req)
                cancelled.append(req.rid)
        for sid in [s for s, v in self.resident.items() if v[0].rid in self._cancel]:
            req = self.resident.pop(sid)[0]
            self.batch.remove(sid)
            cancelled.append(req.rid)
        self._cancel.clear()

    def _try_add(self, req):
        if req.snapshot is None:
            return self.batch.try_add(req.params, req.pos, req.vel, req.dt)
        try:
            return self.batch.add_snapshot(req.snapshot)
        except _lib.SphError as e:
            if e.code == -3:
                return None
            raise

    def _admit(self, waiting, now):
        admitted = []
        for req in list(waiting):
            sid = self._try_add(req)
            if sid is None:
                continue  # does not fit now; a smaller later one may
            self.resident[sid] = [req, req.steps, now, []]
            waiting.remove(req)
            admitted.append(req.rid)
        return admitted

    def run(self, requests, realtime=True, on_step=None):
        """Serve `requests` (sorted by arrival). Returns (results by rid,
        stats dict). With realtime the loop waits for arrivals on the wall
        clock; otherwise time jumps to the next arrival when idle."""
        pending = sorted(requests, key=lambda r: r.arrival)
        substeps = {r.substeps for r in pending}
        if len(substeps) > 1:
            raise ValueError("one substep count per server")
        substeps = substeps.pop() if substeps else 1
        waiting, done, cancelled = [], {}, []
        self._run_state = dict(pending=pending, waiting=waiting, done=done,
                               substeps=substeps, t0=time.perf_counter(), offset=0.0)
        t0 = time.perf_counter()
        offset = 0.0  # time skipped while idle (realtime=False)
        lat, steps, pstep = [], 0, 0
        peak_resident = 0
        while pending or waiting or self.resident:
            self._apply_cancels(pending, waiting, cancelled)
            now = time.perf_counter() - t0 + offset
            while pending and pending[0].arrival <= now:
                waiting.append(pending.pop(0))
            self._admit(waiting, now)
            if not self.resident:
                if pending:
                    gap = pending[0].arrival - now
                    if realtime:
                        time.sleep(max(0.0, gap))
                    else:
                        offset += max(0.0, gap)
                        self._run_state["offset"] = offset
                    continue
                if waiting:
                    raise RuntimeError(f"request {waiting[0].rid} ({waiting[0].n} particles) "
                                       f"exceeds the capacity of {self.capacity}")
                break
            peak_resident = max(peak_resident, sum(v[0].n for v in self.resident.values()))
            ts = time.perf_counter()
            self.batch.step(substeps)
            self.batch.sync()
            ms = 1000.0 * (time.perf_counter() - ts)
            steps += 1
            finished = []
            for sid, v in self.resident.items():
                v[1] -= 1
                v[3].append(ms)
                lat.append(ms)
                pstep += v[0].n
                if v[1] == 0:
                    finished.append(sid)
            for sid in finished:
                req, _, adm, sm = self.resident.pop(sid)
                pos, vel, dens = self.batch.download(sid)
                self.batch.remove(sid)
                done[req.rid] = Done(req.rid, pos, vel, dens, adm,
                                     time.perf_counter() - t0 + offset, sm)
            if on_step:
                on_step(steps, ms, len(self.resident))
        wall = time.perf_counter() - t0
        lat = np.asarray(lat) if lat else np.zeros(1)
        stats = dict(
            requests=len(done), cancelled=sorted(cancelled),
            batched_steps=steps, particle_steps=int(pstep),
            wall_s=wall, particle_steps_per_s=pstep / max(wall, 1e-9),
            p50_step_ms=float(np.percentile(lat, 50)),
            p99_step_ms=float(np.percentile(lat, 99)),
            peak_resident_particles=int(peak_resident),
            capacity_particles=int(self.capacity),
        )
        return done, stats


    def checkpoint(self, directory) -> None:
        """Persist the loop between two steps (call it from run()'s on_step):
        every resident request's scene as a snapshot file with its steps left,
        the requests not admitted yet (initial state and settings), and the
        finished results, under `directory` with a manifest.json. resume()
        turns it back into requests and results; a new Server run on them
        finishes every request exactly as the uninterrupted loop would."""
        st = getattr(self, "_run_state", None)
        if st is None:
            raise RuntimeError("checkpoint() is called from inside run()")
        os.makedirs(directory, exist_ok=True)
        now = time.perf_counter() - st["t0"] + st["offset"]
        man = dict(version=1, substeps=st["substeps"], time=now, resident=[], queued=[],
                   done=[])
        for sid, (req, left, adm, sm) in self.resident.items():
            name = f"r{req.rid}.sph"
            self.batch.save(sid, os.path.join(directory, name))
            man["resident"].append(dict(rid=req.rid, steps=left, file=name, step_ms=sm))
        for req in list(st["waiting"]) + list(st["pending"]):
            name = f"q{req.rid}.npz"
            p = to_params(req.params)
            np.savez(os.path.join(directory, name), pos=req.pos, vel=req.vel)
            man["queued"].append(dict(
                rid=req.rid, steps=req.steps, file=name, dt=req.dt, arrival=req.arrival,
                params={k: (list(getattr(p, k)) if k == "bound" else getattr(p, k))
                        for k, _ in p._fields_}))
        for rid, d in st["done"].items():
            name = f"d{rid}.npz"
            np.savez(os.path.join(directory, name), pos=d.pos, vel=d.vel, dens=d.dens)
            man["done"].append(dict(rid=rid, file=name, admitted=d.admitted,
                                    finished=d.finished, step_ms=d.step_ms))
        with open(os.path.join(directory, "manifest.json"), "w") as f:
            json.dump(man, f)


def resume(directory):
    """The requests and results of a Server.checkpoint(): (requests, done)
    -- resident requests resume from their scene snapshots with their steps
    left, queued ones keep their arrival offset relative to the checkpoint."""
    with open(os.path.join(directory, "manifest.json")) as f:
        man = json.load(f)
    S = man["substeps"]
    reqs, done = [], {}
    for r in man["resident"]:
        path = os.path.join(directory, r["file"])
        snap = snapshot.read(path)
        reqs.append(Request(r["rid"], snap["params"], snap["pos"], snap["vel"], snap["dt"],
                            S, r["steps"], arrival=0.0, snapshot=path))
    for q in man["queued"]:
        a = np.load(os.path.join(directory, q["file"]))
        p = _lib.Params()
        for k, v in q["params"].items():
            if k == "bound":
                for i in range(3):
                    p.bound[i] = v[i]
            else:
                setattr(p, k, v)
        reqs.append(Request(q["rid"], p, a["pos"], a["vel"], q["dt"], S, q["steps"],
                            arrival=max(0.0, q["arrival"] - man["time"])))
    for d in man["done"]:
        a = np.load(os.path.join(directory, d["file"]))
        done[d["rid"]] = Done(d["rid"], a["pos"], a["vel"], a["dens"], d["admitted"],
                              d["finished"], d["step_ms"])
    return reqs, done


def run_alone(req: Request, stream=None, tuning=None):
    """The same request on its own single-scene handle (the comparison path
    and the serial baseline)."""
    sim = FluidSimulation(req.params, stream=stream)
    sim.InitializeData(req.n, req.pos, req.vel)
    if tuning:
        sim.set_tuning(**tuning)
    for _ in range(req.steps):
        sim.step_async(req.dt, req.substeps)
    out = sim.download()
    sim.close()
    return out


class NativeServer:
    """The library's own serving loop (sph_server_*): a worker thread in the
    library admits jobs by the HBM budget, steps every resident job per
    batched launch and retires finished ones; submit() returns at once and
    wait() blocks for a job's result. Same admission rule and results as
    Server, without Python in the loop."""

    def __init__(self, budget_bytes: int, max_scenes: int = 4096, substeps: int = 3):
        import ctypes
        self._ct = ctypes
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        rc = self._lib.sph_server_create(int(budget_bytes), int(max_scenes), int(substeps),
                                         ctypes.byref(h))
        if rc != 0:
            raise _lib.SphError(rc, (self._lib.sph_global_error() or b"").decode())
        self._h = h
        self.substeps = int(substeps)
        self._sizes = {}

    def _raise(self, rc):
        msg = self._lib.sph_server_last_error(self._h) or b""
        raise _lib.SphError(rc, msg.decode(errors="replace"))

    def submit(self, params, pos, vel, dt, steps) -> int:
        ct = self._ct
        pos = np.ascontiguousarray(pos, np.float32)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32)
        job = ct.c_uint64()
        rc = self._lib.sph_server_submit(
            self._h, ct.byref(to_params(params)), pos.shape[0], pos.ctypes.data,
            None if v is None else v.ctypes.data, float(np.float32(dt)), int(steps),
            ct.byref(job))
        if rc != 0:
            self._raise(rc)
        self._sizes[job.value] = pos.shape[0]
        return int(job.value)

    def cancel(self, job: int) -> None:
        rc = self._lib.sph_server_cancel(self._h, int(job))
        if rc != 0:
            self._raise(rc)

    def wait(self, job: int, timeout: float = 600.0):
        """(pos, vel, dens) of a finished job; SphError if it was cancelled,
        failed or is still running after `timeout` seconds."""
        n = self._sizes[int(job)]
        pos = np.empty((n, 3), np.float32)
        vel = np.empty((n, 3), np.float32)
        dens = np.empty((n, 2), np.float32)
        rc = self._lib.sph_server_wait(self._h, int(job), pos.ctypes.data, vel.ctypes.data,
                                       dens.ctypes.data, float(timeout))
        if rc != 0:
            self._raise(rc)
        self._sizes.pop(int(job), None)
        return pos, vel, dens

    def stats(self) -> dict:
        s = _lib.ServerStats()
        rc = self._lib.sph_server_get_stats(self._h, self._ct.byref(s))
        if rc != 0:
            self._raise(rc)
        return {k: getattr(s, k) for k, _ in s._fields_}

    def run(self, requests, realtime=True):
        """Submit `requests` at their arrival times (all at once with
        realtime=False) and collect every result: (results by rid, stats)."""
        t0 = time.perf_counter()
        jobs = {}
        for r in sorted(requests, key=lambda q: q.arrival):
            if realtime:
                time.sleep(max(0.0, r.arrival - (time.perf_counter() - t0)))
            if r.substeps != self.substeps:
                raise ValueError("one substep count per server")
            jobs[r.rid] = self.submit(r.params, r.pos, r.vel, r.dt, r.steps)
        done = {}
        for rid, job in jobs.items():
            pos, vel, dens = self.wait(job)
            done[rid] = Done(rid, pos, vel, dens, 0.0, time.perf_counter() - t0, [])
        st = self.stats()
        stats = dict(requests=len(done), batched_steps=st["steps"],
                     particle_steps=st["particle_steps"], wall_s=st["wall_s"],
                     particle_steps_per_s=st["particle_steps_per_s"],
                     p50_step_ms=st["p50_step_ms"], p99_step_ms=st["p99_step_ms"],
                     capacity_particles=st["capacity_particles"])
        return done, stats

    def close(self):
        if self._h is not None:
            self._lib.sph_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
