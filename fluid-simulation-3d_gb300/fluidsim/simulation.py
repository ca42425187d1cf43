"""Host mirror of the reference's simulation class and plug-in interface.

`FluidSimulation` keeps the method names, defaults and argument meaning of
Physics::Fluid::FluidSimulation (engine/physics/physicsWorld.h:28-155) on top
of the C ABI; `FluidSimCUDA` is the FluidSimBase plug-in
(projects/Simulation/code/simulations/fluidSimBase.h:5-14) whose render()
becomes a headless device buffer. `Batch` wraps the batched form.

Differences from the reference, all deliberate:
  * not a singleton: any number of simulations can live side by side;
  * viscosity is Jacobi (post-pressure snapshot) instead of the reference's
    serial in-place sweep;
  * Update(dt, substeps) runs `substeps` reference Updates of dt/substeps.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._lib import Params, Tuning, check


def _f32(x):
    return float(np.float32(x))


def to_params(p) -> Params:
    """Params from a scenes.SimParams-like object (or a Params)."""
    if isinstance(p, Params):
        return p
    o = Params()
    o.radius = p.radius
    o.cutoff_sq = p.cutoff_sq
    o.target_density = p.target_density
    o.pressure_mult = p.pressure_mult
    o.near_pressure_mult = p.near_pressure_mult
    o.viscosity = p.viscosity
    o.gravity_scale = p.gravity_scale
    o.gravity_on = 1 if p.gravity_on else 0
    for a in range(3):
        o.bound[a] = p.bound[a]
    o.damping = p.damping
    o.predict_dt = p.predict_dt
    return o


def default_params() -> Params:
    o = Params()
    _lib.load().sph_default_params(ctypes.byref(o))
    return o


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _stream(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return ctypes.c_void_p(stream)
    return ctypes.c_void_p(int(getattr(stream, "cuda_stream", stream)))


def key_table(params, n: int, table: int = 0):
    """(grid, entries) of the key table the engine gives a scene of n
    particles stepped alone under tuning.table = `table`: one entry per cell
    of its internal grid (grid = True) when the grid has at most four cells per
    particle -- or, with table 2, when its excess over n fits the 65,536-entry
    allowance -- else n bucket entries. Mirrors the engine's GridAxis and
    UploadScenes (csrc/sph_engine.cu)."""
    p = to_params(params)
    r = float(np.float32(p.radius))

    def axis(b):
        h = float(np.float32(b) * np.float32(0.5))
        a, c = -h / r, h / r
        if not (math.isfinite(a) and math.isfinite(c)):
            return 1024
        lo, hi = min(math.floor(a), math.floor(c)) - 2, max(math.floor(a), math.floor(c)) + 2
        if lo < -1e9 or hi > 1e9:
            return 1024
        return int(min(hi - lo + 1, 32768))

    cells = axis(p.bound[0]) * axis(p.bound[1]) * axis(p.bound[2])
    if table != 1 and cells <= 4 * n:
        return True, cells
    if table == 2 and cells - n <= 65536:
        return True, cells
    return False, n


def grid_arrangement(n: int, gap: float = 0.215):
    """Default lattice of InitializeData / GridArrangement
    (physicsWorld.cc:139-142, 518-557), in float32 like the reference."""
    f = np.float32
    # RowSize = ceil(powf(n, 1.0f / 3.0f)): powf is correctly rounded, so the
    # double-precision power rounded to float32 reproduces it (numpy's own
    # float32 power differs for n = 27 and n = 1000)
    row = int(math.ceil(f(float(n) ** float(f(1.0) / f(3.0)))))
    g = f(gap)
    tot = f(row) * g
    ox = f(0) - ((tot - g) / f(2.0))
    oy = f(0) + (tot - g) / f(2.0)
    oz = f(0) - (tot - g) / f(2.0)
    out = np.zeros((n, 3), np.float32)
    i = 0
    for ly in range(row):
        for lx in range(row):
            for lz in range(row):
                if i >= n:
                    return out
                out[i] = (ox + f(lx) * g, oy - f(ly) * g, oz + f(lz) * g)
                i += 1
    return out


def speed_of(vel):
    """getSpeed (physicsWorld.cc:172-176) of velocities [..., 3] in float32:
    glm::length, sqrt((x*x + y*y) + z*z), each step rounded."""
    v = np.asarray(vel, np.float32)
    return np.sqrt((v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1]) + v[..., 2] * v[..., 2])


def speed_normalized(vel):
    """getSpeedNormalzied (physicsWorld.cc:178-182) in float32:
    clamp(|v|, 0, 1.5) / 1.5."""
    f = np.float32
    return (np.minimum(np.maximum(speed_of(vel), f(0.0)), f(1.5)) / f(1.5)).astype(np.float32)


class FluidSimulation:
    """GB300 drop-in for Physics::Fluid::FluidSimulation.

    Settings take effect at the next Update. Getters of per-particle state
    read from the last download (refreshed lazily after each Update).
    """

    def __init__(self, params=None, stream=None):
        self._lib = _lib.load()
        self._params = to_params(params) if params is not None else default_params()
        self._h = None
        self._n = 0
        self._stream = _stream(stream)
        self._cache = None
        self.simTime = 0.0
        self._timers = dict(gravity=0.0, spatial=0.0, density=0.0,
                            pressure=0.0, viscosity=0.0, posncoll=0.0)

    # ---------------------------------------------------------- lifecycle
    def InitializeData(self, particleAmmount: int, positions=None,
                       velocities=None):
        """physicsWorld.cc:112-147: sizes the buffers, zeroes velocity, lays
        out the default lattice (or the given positions)."""
        self.close()
        n = int(particleAmmount)
        h = ctypes.c_void_p()
        check(self._lib.sph_create(ctypes.byref(self._params), n, ctypes.byref(h)))
        self._h = h
        self._n = n
        pos = grid_arrangement(n) if positions is None else positions
        self.upload(pos, velocities)

    def close(self):
        if self._h is not None:
            self._lib.sph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- data
    def upload(self, pos, vel=None):
        pos = np.ascontiguousarray(pos, np.float32).reshape(self._n, 3)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(self._n, 3)
        check(self._lib.sph_upload(self._h, _ptr(pos), _ptr(v), self._stream), self._h)
        self._cache = None

    def download(self):
        n = self._n
        pos = np.empty((n, 3), np.float32)
        vel = np.empty((n, 3), np.float32)
        dens = np.empty((n, 2), np.float32)
        check(self._lib.sph_download(self._h, _ptr(pos), _ptr(vel), _ptr(dens),
                                     self._stream), self._h)
        self._cache = (pos, vel, dens)
        return pos, vel, dens

    def _state(self):
        if self._cache is None:
            self.download()
        return self._cache

    @property
    def positions(self):
        """The reference's public `positions` buffer (physicsWorld.h:79)."""
        return self._state()[0]

    @property
    def OutPositions(self):
        """(position, 0.34) per particle (physicsWorld.h:80, :107)."""
        p = self._state()[0]
        return np.concatenate([p, np.full((self._n, 1), 0.34, np.float32)], axis=1)

    def save(self, path):
        """Snapshot the state and settings to `path` (sph_save)."""
        check(self._lib.sph_save(self._h, str(path).encode(), self._stream), self._h)

    def load(self, path):
        """Replace the state and settings with a snapshot of the same
        particle count (sph_load)."""
        check(self._lib.sph_load(self._h, str(path).encode(), self._stream), self._h)
        check(self._lib.sph_get_params(self._h, ctypes.byref(self._params)), self._h)
        self._cache = None

    def render(self, view):
        """Headless render of the current state (sph_render): `view` is a
        fluidsim.render.view(...). Returns (rgba uint8 [H, W, 4], depth
        float32 [H, W]), rows bottom to top as glReadPixels gives them."""
        rgba = np.empty((view.height, view.width, 4), np.uint8)
        depth = np.empty((view.height, view.width), np.float32)
        check(self._lib.sph_render(self._h, ctypes.byref(view), _ptr(rgba), _ptr(depth),
                                   self._stream), self._h)
        return rgba, depth

    def out_positions_device_ptr(self) -> int:
        """Device address of the headless float4 OutPositions buffer."""
        ptr = ctypes.c_void_p()
        check(self._lib.sph_out_positions(self._h, ctypes.byref(ptr)), self._h)
        return int(ptr.value or 0)

    # -------------------------------------------------------------- update
    def Update(self, deltatime: float, substeps: int = 1):
        """physicsWorld.cc:39-111, `substeps` times with dt/substeps."""
        check(self._lib.sph_step(self._h, _f32(deltatime), int(substeps),
                                 self._stream), self._h)
        self._cache = None

    def step_async(self, deltatime: float, substeps: int = 1, stream=None):
        s = self._stream if stream is None else _stream(stream)
        check(self._lib.sph_step(self._h, _f32(deltatime), int(substeps), s), self._h)
        self._cache = None

    def status(self) -> int:
        f = ctypes.c_uint32()
        check(self._lib.sph_status(self._h, ctypes.byref(f), self._stream), self._h)
        return int(f.value)

    def profile_enable(self, on=True):
        check(self._lib.sph_profile_enable(self._h, 1 if on else 0), self._h)

    def phase_times(self):
        """ms per phase of the last Update (gravity, spatial, density,
        pressure, viscosity, posncoll) from CUDA events; also refreshes the
        getElapsedTime* getters."""
        out = (ctypes.c_double * 6)()
        check(self._lib.sph_phase_times(self._h, out), self._h)
        vals = [float(x) for x in out]
        for k, v in zip(("gravity", "spatial", "density", "pressure",
                         "viscosity", "posncoll"), vals):
            self._timers[k] = v
        return vals

    def kernel_launches(self) -> int:
        return int(self._lib.sph_kernel_launches(self._h))

    def set_tuning(self, block=128, cell_tile=1, particles_per_warp=32, gather=2,
                   force_block=0, table=0):
        t = Tuning(block, cell_tile, particles_per_warp, gather, force_block, table)
        check(self._lib.sph_set_tuning(self._h, ctypes.byref(t)), self._h)

    def tuning(self):
        t = Tuning()
        check(self._lib.sph_get_tuning(self._h, ctypes.byref(t)), self._h)
        return dict(block=t.block, cell_tile=t.cell_tile,
                    particles_per_warp=t.particles_per_warp, gather=t.gather,
                    force_block=t.force_block, table=t.table)

    def autotune(self, deltatime, substeps=1, steps_per_trial=2):
        """Sweep the launch configuration on real steps and keep the fastest;
        the state is saved before the sweep and restored after it. Returns
        (tuning dict, ms per step)."""
        t = Tuning()
        ms = ctypes.c_float()
        check(self._lib.sph_autotune(self._h, _f32(deltatime), int(substeps),
                                     int(steps_per_trial), ctypes.byref(t),
                                     ctypes.byref(ms), self._stream), self._h)
        self._cache = None
        return dict(block=t.block, cell_tile=t.cell_tile,
                    particles_per_warp=t.particles_per_warp, gather=t.gather,
                    force_block=t.force_block, table=t.table), float(ms.value)

    @property
    def handle(self):
        return self._h

    # ------------------------------------------------------------ getters
    def _in(self, i):
        return 0 <= int(i) < self._n

    def getPosition(self, i):
        return self._state()[0][i].copy() if self._in(i) else np.zeros(3, np.float32)

    def getVelocity(self, i):
        return self._state()[1][i].copy() if self._in(i) else np.zeros(3, np.float32)

    def getDensity(self, i):
        return float(self._state()[2][i, 0]) if self._in(i) else 0.0

    def getNearDensity(self, i):
        return float(self._state()[2][i, 1]) if self._in(i) else 0.0

    def getSpeed(self, i):
        return float(speed_of(self._state()[1][i])) if self._in(i) else 0.0

    def getSpeedNormalzied(self, i):
        return float(speed_normalized(self._state()[1][i])) if self._in(i) else 0.0

    def getElapsedTimeGravity(self): return self._timers["gravity"]
    def getElapsedTimeSpatial(self): return self._timers["spatial"]
    def getElapsedTimeDensity(self): return self._timers["density"]
    def getElapsedTimePressure(self): return self._timers["pressure"]
    def getElapsedTimeViscosity(self): return self._timers["viscosity"]
    def getElapsedTimePosNColl(self): return self._timers["posncoll"]

    # ----------------------------------------------------------- settings
    def _set(self, name, value):
        setattr(self._params, name, value)
        if self._h is not None:
            check(self._lib.sph_set_params(self._h, ctypes.byref(self._params)), self._h)

    def setSimulationTime(self, t): self.simTime = float(t)
    def getSimulationTime(self): return self.simTime
    def setGravity(self, status): self._set("gravity_on", 1 if status else 0)
    def getGravityStatus(self): return bool(self._params.gravity_on)
    def setInteractionRadius(self, v): self._set("radius", _f32(v))
    def getInteractionRadius(self): return self._params.radius
    def setDensityTarget(self, v): self._set("target_density", _f32(v))
    def getDensityTarget(self): return self._params.target_density
    def setPressureMultiplier(self, v): self._set("pressure_mult", _f32(v))
    def getPressureMultiplier(self): return self._params.pressure_mult
    def setNearPressureMultiplier(self, v): self._set("near_pressure_mult", _f32(v))
    def getNearPressureMultiplier(self): return self._params.near_pressure_mult
    def setViscosityStrength(self, v): self._set("viscosity", _f32(v))
    def getViscosityStrength(self): return self._params.viscosity
    def setGravityScale(self, v): self._set("gravity_scale", _f32(v))
    def getGravityScale(self): return self._params.gravity_scale

    def setBound(self, v):
        b = (ctypes.c_float * 3)(*[_f32(x) for x in v])
        self._set("bound", b)

    def getBounds(self): return np.array(list(self._params.bound), np.float32)
    def setCollisionDamping(self, v): self._set("damping", _f32(v))
    def setPredictionDt(self, v): self._set("predict_dt", _f32(v))

    # -------------------------------------------------------------- parity
    def debug_enable(self, on=True):
        check(self._lib.sph_debug_enable(self._h, 1 if on else 0), self._h)

    def debug_export(self):
        n = self._n
        d = dict(hash=np.empty(n, np.uint32), key=np.empty(n, np.uint32),
                 sorted_ids=np.empty(n, np.uint32), start=np.empty(n, np.uint32),
                 dens=np.empty((n, 2), np.float32), acc_p=np.empty((n, 3), np.float32),
                 vel_p=np.empty((n, 3), np.float32), vel_v=np.empty((n, 3), np.float32))
        check(self._lib.sph_debug_export(
            self._h, _ptr(d["hash"]), _ptr(d["key"]), _ptr(d["sorted_ids"]),
            _ptr(d["start"]), _ptr(d["dens"]), _ptr(d["acc_p"]), _ptr(d["vel_p"]),
            _ptr(d["vel_v"]), self._stream), self._h)
        return d

    def debug_export_layout(self):
        """The timed sort's own layout of the captured substep
        (sph_debug_export_layout): per particle its internal cell index and
        key-table entry, the caller index at each slot, the key table's
        start offsets and whether it is a grid table."""
        n = self._n
        tl, direct = ctypes.c_uint32(), ctypes.c_int()
        d = dict(cell=np.empty(n, np.uint32), key=np.empty(n, np.uint32),
                 slot_ids=np.empty(n, np.uint32))
        check(self._lib.sph_debug_export_layout(
            self._h, _ptr(d["cell"]), _ptr(d["key"]), _ptr(d["slot_ids"]), None, 0,
            ctypes.byref(tl), ctypes.byref(direct), self._stream), self._h)
        start = np.empty(tl.value + 1, np.uint32)
        check(self._lib.sph_debug_export_layout(
            self._h, None, None, None, _ptr(start), start.shape[0], None, None,
            self._stream), self._h)
        d["start"] = start
        d["direct"] = bool(direct.value)
        return d

    @property
    def num_particles(self):
        return self._n


class FluidSimCUDA:
    """FluidSimBase plug-in (fluidSimBase.h:5-14) driving FluidSimulation on
    the GPU. render() without a camera hands back the headless OutPositions
    device buffer; with a camera view (fluidsim.render.view) it draws the
    frame FluidSimCPU::render draws (fluidSimCPU.cc:53-93) headlessly."""

    def __init__(self, params=None, substeps: int = 1):
        self.sim = FluidSimulation(params)
        self.substeps = substeps
        self.nrParticles = 0

    def initialize(self, particleAmount: int):
        self.nrParticles = int(particleAmount)
        self.sim.InitializeData(self.nrParticles)

    def update(self, dt: float):
        self.sim.Update(dt, self.substeps)

    def reset(self):
        self.sim.InitializeData(self.nrParticles)

    def cleanup(self):
        self.sim.close()

    def render(self, view=None):
        """Headless: (device pointer of float4[n] (pos, 0.34), n) without a
        view; (rgba, depth) images of the frame with one."""
        if view is not None:
            return self.sim.render(view)
        return self.sim.out_positions_device_ptr(), self.nrParticles


class Batch:
    """Batched form: many independent scenes stepped by one set of segmented
    launches per substep (see sph_batch_* in include/sph_gb300.h)."""

    def __init__(self, capacity: int, max_scenes: int, stream=None):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        check(self._lib.sph_batch_create(int(capacity), int(max_scenes), ctypes.byref(h)))
        self._h = h
        self._stream = _stream(stream)
        self.sizes = {}

    def close(self):
        if self._h is not None:
            self._lib.sph_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        check(rc, self._h, batch=True)

    def add(self, params, pos, vel=None, dt=1.0 / 60.0) -> int:
        pos = np.ascontiguousarray(pos, np.float32)
        n = pos.shape[0]
        v = None if vel is None else np.ascontiguousarray(vel, np.float32)
        sid = ctypes.c_uint32()
        self._check(self._lib.sph_batch_add(self._h, ctypes.byref(to_params(params)), n,
                                            _ptr(pos), _ptr(v), _f32(dt),
                                            ctypes.byref(sid), self._stream))
        self.sizes[int(sid.value)] = n
        return int(sid.value)

    def try_add(self, params, pos, vel=None, dt=1.0 / 60.0):
        """add(), returning None instead of raising when it does not fit."""
        try:
            return self.add(params, pos, vel, dt)
        except _lib.SphError as e:
            if e.code == -3:
                return None
            raise

    def remove(self, sid: int):
        self._check(self._lib.sph_batch_remove(self._h, int(sid)))
        self.sizes.pop(int(sid), None)

    def save(self, sid: int, path):
        """Snapshot scene `sid` to `path` (sph_batch_save)."""
        self._check(self._lib.sph_batch_save(self._h, int(sid), str(path).encode(),
                                             self._stream))

    def add_snapshot(self, path) -> int:
        """Add a saved scene (sph_batch_add_snapshot); returns its id."""
        with open(path, "rb") as f:
            head = f.read(16)
        n = int(np.frombuffer(head[12:16], np.uint32)[0]) if len(head) == 16 else 0
        sid = ctypes.c_uint32()
        self._check(self._lib.sph_batch_add_snapshot(self._h, str(path).encode(),
                                                     ctypes.byref(sid), self._stream))
        self.sizes[int(sid.value)] = n
        return int(sid.value)

    def step(self, substeps: int):
        self._check(self._lib.sph_batch_step(self._h, int(substeps), self._stream))

    def sync(self):
        self._check(self._lib.sph_batch_sync(self._h, self._stream))

    def status(self) -> int:
        """Device status flags of the batch's kernels since the last read
        (SPH_STATUS_NONFINITE | SPH_STATUS_RANGE; cleared by the read)."""
        f = ctypes.c_uint32()
        self._check(self._lib.sph_batch_status(self._h, ctypes.byref(f), self._stream))
        return int(f.value)

    def download(self, sid: int):
        n = self.sizes[int(sid)]
        pos = np.empty((n, 3), np.float32)
        vel = np.empty((n, 3), np.float32)
        dens = np.empty((n, 2), np.float32)
        self._check(self._lib.sph_batch_download(self._h, int(sid), _ptr(pos), _ptr(vel),
                                                 _ptr(dens), self._stream))
        return pos, vel, dens

    def render(self, sid: int, view):
        """sph_batch_render of scene `sid`; see FluidSimulation.render."""
        rgba = np.empty((view.height, view.width, 4), np.uint8)
        depth = np.empty((view.height, view.width), np.float32)
        self._check(self._lib.sph_batch_render(self._h, int(sid), ctypes.byref(view),
                                               _ptr(rgba), _ptr(depth), self._stream))
        return rgba, depth

    def set_tuning(self, block=128, cell_tile=1, particles_per_warp=32, gather=2,
                   force_block=0, table=0):
        t = Tuning(block, cell_tile, particles_per_warp, gather, force_block, table)
        self._check(self._lib.sph_batch_set_tuning(self._h, ctypes.byref(t)))

    def tuning(self):
        t = Tuning()
        self._check(self._lib.sph_batch_get_tuning(self._h, ctypes.byref(t)))
        return dict(block=t.block, cell_tile=t.cell_tile,
                    particles_per_warp=t.particles_per_warp, gather=t.gather,
                    force_block=t.force_block, table=t.table)

    def autotune(self, substeps: int, steps_per_trial: int = 2):
        """Sweep the launch configuration on real steps of the resident
        scenes and keep the fastest; every scene's state is saved before the
        sweep and restored after it. Returns (tuning dict, ms per step)."""
        t = Tuning()
        ms = ctypes.c_float()
        self._check(self._lib.sph_batch_autotune(self._h, int(substeps), int(steps_per_trial),
                                                 ctypes.byref(t), ctypes.byref(ms),
                                                 self._stream))
        return dict(block=t.block, cell_tile=t.cell_tile,
                    particles_per_warp=t.particles_per_warp, gather=t.gather,
                    force_block=t.force_block, table=t.table), float(ms.value)

    def profile_enable(self, on=True):
        self._check(self._lib.sph_batch_profile_enable(self._h, 1 if on else 0))

    def phase_times(self):
        out = (ctypes.c_double * 6)()
        self._check(self._lib.sph_batch_phase_times(self._h, out))
        return [float(x) for x in out]

    def kernel_launches(self) -> int:
        return int(self._lib.sph_batch_kernel_launches(self._h))

    @property
    def num_scenes(self):
        return int(self._lib.sph_batch_num_scenes(self._h))

    @property
    def num_particles(self):
        return int(self._lib.sph_batch_num_particles(self._h))
