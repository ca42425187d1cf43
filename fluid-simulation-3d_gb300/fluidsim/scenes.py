"""Seeded synthetic scenes for the SPH substep.

The reference has no scene files: its app lays particles on a cube lattice
(InitializeData / GridArrangement, engine/physics/physicsWorld.cc:112-147,
518-557) and the user tunes settings with sliders (projects/Simulation/code/
gameApp.cc:364-411). These generators build the dam-break / falling-block
layouts the benchmark workloads are quoted on, from a numpy PCG64 seed, so the
same float32 arrays come out on every host (only IEEE +,*,/ on float64 and a
final cast; no transcendental calls on positions).

Each scene is a dict: pos (n,3) f32, vel (n,3) f32, params (SimParams), dt,
substeps, name.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class SimParams:
    """Settings surface of FluidSimulation (physicsWorld.h:96-106, 145) plus the
    two constants the reference hard-codes: collision damping 0.95
    (physicsWorld.cc:87) and the 1/120 s prediction look-ahead (:47)."""

    radius: float = 0.35
    cutoff_sq: float = float(np.float32(0.35) * np.float32(0.35))
    target_density: float = 99.7
    pressure_mult: float = 300.0
    near_pressure_mult: float = 20.0
    viscosity: float = 0.5
    gravity_scale: float = 10.0
    gravity_on: bool = False
    bound: tuple = (20.0, 20.0, 20.0)
    damping: float = 0.95
    predict_dt: float = float(np.float32(1.0) / np.float32(120.0))


# Physical constants shared by every benchmark workload.
DAM_CONSTANTS = dict(target_density=55.0, pressure_mult=500.0,
                     near_pressure_mult=18.0, viscosity=0.06,
                     gravity_scale=9.81, gravity_on=True)


def lattice_block(counts, spacing, origin, jitter, rng, n=None):
    """Cube lattice of counts=(nx,ny,nz) points at `spacing` starting at
    `origin` (the first point), each coordinate jittered U[-jitter, jitter].
    Points are emitted y-layer by y-layer from the floor up (x fastest), so a
    truncated block (n < nx*ny*nz) keeps a flat top. float32 (n,3)."""
    nx, ny, nz = (int(c) for c in counts)
    total = nx * ny * nz
    n = total if n is None else int(n)
    if n > total:
        raise ValueError(f"block {counts} holds {total} < {n} particles")
    idx = np.arange(n, dtype=np.int64)
    ix = idx % nx
    iz = (idx // nx) % nz
    iy = idx // (nx * nz)
    base = np.stack([ix, iy, iz], axis=1).astype(np.float64) * spacing
    base += np.asarray(origin, dtype=np.float64)[None, :]
    jit = rng.uniform(-jitter, jitter, size=(n, 3))
    return (base + jit).astype(np.float32)


def _corner_origin(bound, spacing, corner=(-1, -1, -1), counts=None):
    """First lattice point of a block flush with a box corner (half a spacing
    away from the walls)."""
    o = []
    for a in range(3):
        half = 0.5 * bound[a]
        if corner[a] < 0:
            o.append(-half + 0.5 * spacing)
        else:
            o.append(half - 0.5 * spacing - (counts[a] - 1) * spacing)
    return o


def dam_break_16k(seed: int = 0):
    """16,384 particles: a 32x32x16 (x,y,z) lattice at spacing 0.2 in the
    floor corner of a 12x8x6 box, jitter +-0.02, at rest. r 0.35, rho0 55,
    k 500, kn 18, mu 0.06, g 9.81 down; dt 1/60 in 3 substeps."""
    rng = np.random.default_rng(seed)
    bound = (12.0, 8.0, 6.0)
    counts = (32, 32, 16)
    pos = lattice_block(counts, 0.2, _corner_origin(bound, 0.2), 0.02, rng)
    p = SimParams(radius=0.35, bound=bound, **DAM_CONSTANTS)
    return dict(name="dam_break_16k", pos=pos, vel=np.zeros_like(pos),
                params=p, dt=1.0 / 60.0, substeps=3)


def dam_break_1m(seed: int = 1):
    """1,048,576 particles: a 128x64x128 (x,y,z) lattice at spacing 0.1 in the
    floor corner of a 25.6x12.8x25.6 box (a quarter of the lower half), jitter
    +-0.02, at rest; the dam-break constants with r scaled to 0.175;
    dt 1/120 in 2 substeps."""
    rng = np.random.default_rng(seed)
    bound = (25.6, 12.8, 25.6)
    counts = (128, 64, 128)
    pos = lattice_block(counts, 0.1, _corner_origin(bound, 0.1), 0.02, rng)
    p = SimParams(radius=0.175, bound=bound, **DAM_CONSTANTS)
    return dict(name="dam_break_1m", pos=pos, vel=np.zeros_like(pos),
                params=p, dt=1.0 / 120.0, substeps=2)


def opposing_blocks_8m(seed: int = 4, trim_overlap: bool = True):
    """Two 256x128x128 (x,y,z) blocks at spacing 0.08, jitter +-0.008, one
    flush with the (-x,-y,-z) corner and one with the (+x,+y,+z) corner of a
    40x20x20 box. The long axis only fits along x and the blocks then overlap
    by 0.96x0.48x0.48; with trim_overlap the second block drops its particles
    inside the first block's hull (so n is a little under 8,388,608).
    r 0.14, dt 1/240 in 2 substeps."""
    rng = np.random.default_rng(seed)
    bound = (40.0, 20.0, 20.0)
    counts = (256, 128, 128)
    s = 0.08
    a = lattice_block(counts, s, _corner_origin(bound, s, (-1, -1, -1), counts),
                      0.008, rng)
    b = lattice_block(counts, s, _corner_origin(bound, s, (1, 1, 1), counts),
                      0.008, rng)
    if trim_overlap:
        hi = a.max(axis=0) + 0.5 * s
        inside = np.all(b < hi[None, :], axis=1)
        b = b[~inside]
    pos = np.concatenate([a, b], axis=0)
    p = SimParams(radius=0.14, bound=bound, **DAM_CONSTANTS)
    return dict(name="opposing_blocks_8m", pos=pos, vel=np.zeros_like(pos),
                params=p, dt=1.0 / 240.0, substeps=2)


def fill_box_scene(rng, n, fill, aspect, spacing=0.2, jitter=0.02,
                   layout="dam", v_down=0.0):
    """A box of aspect `aspect` sized so a block of n particles at `spacing`
    fills `fill` of its volume; the block has the box's shape scaled by
    fill^(1/3). layout "dam": the block sits in the floor corner; "fall": the
    block's centre is uniform in the upper half of the box (clamped inside)
    and it starts moving down at v_down."""
    aspect = np.asarray(aspect, dtype=np.float64)
    vol_block = n * spacing ** 3
    vol_box = vol_block / fill
    scale = (vol_box / float(np.prod(aspect))) ** (1.0 / 3.0)
    box = aspect * scale
    blk = box * fill ** (1.0 / 3.0)
    counts = np.maximum(1, np.floor(blk / spacing)).astype(np.int64)
    # grow the lattice until it holds n particles (the top layer is partial)
    while int(np.prod(counts)) < n:
        counts[1] += 1
    extent = (counts - 1) * spacing
    box = np.maximum(box, extent + 2.0 * spacing)
    bound = tuple(float(x) for x in box)
    if layout == "dam":
        origin = _corner_origin(bound, spacing)
    else:
        origin = []
        for a in range(3):
            half = 0.5 * box[a]
            lo, hi = -half + 0.5 * spacing, half - 0.5 * spacing - extent[a]
            if a == 1:
                c = rng.uniform(0.0, half)
                o = c - 0.5 * extent[a]
            else:
                o = rng.uniform(lo, max(lo, hi))
            origin.append(min(max(o, lo), max(lo, hi)))
    pos = lattice_block(tuple(counts), spacing, origin, jitter, rng, n=n)
    vel = np.zeros_like(pos)
    if layout == "fall":
        vel[:, 1] = np.float32(-v_down)
    return pos, vel, bound


def batched_scenes(count: int = 256, seed: int = 2, lo: int = 4096,
                   hi: int = 131072):
    """Independent scenes: n log-uniform in [lo, hi], box aspect U[0.5, 2] per
    axis, the fluid block filling U[0.2, 0.6] of the box volume at spacing 0.2
    +-0.02, dam-break constants with r 0.35; dt 1/60 in 3 substeps."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        aspect = rng.uniform(0.5, 2.0, size=3)
        fill = rng.uniform(0.2, 0.6)
        pos, vel, bound = fill_box_scene(rng, n, fill, aspect)
        p = SimParams(radius=0.35, bound=bound, **DAM_CONSTANTS)
        out.append(dict(name=f"batch{s}", pos=pos, vel=vel, params=p,
                        dt=1.0 / 60.0, substeps=3))
    return out


def request_size(rng, lo: int = 8192, hi: int = 524288, kmin: int = 60,
                 kmax: int = 600):
    """(n, K) of a served request: the first two draws of request_scene, so a
    request's size is known without building its scene."""
    n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
    k = int(rng.integers(kmin, kmax + 1))
    return n, k


def request_scene(rng, lo: int = 8192, hi: int = 524288, kmin: int = 60,
                  kmax: int = 600):
    """One served request: n log-uniform in [lo, hi], K steps uniform in
    [kmin, kmax], a dam-break or a falling block (centre uniform in the upper
    half of the box, downward speed U[0, 3]); box aspect (1, 0.75, 1) at 30%
    fill; dam-break constants, r 0.35, dt 1/60 in 3 substeps."""
    n, k = request_size(rng, lo, hi, kmin, kmax)
    layout = "dam" if rng.uniform() < 0.5 else "fall"
    v = float(rng.uniform(0.0, 3.0)) if layout == "fall" else 0.0
    pos, vel, bound = fill_box_scene(rng, n, 0.3, (1.0, 0.75, 1.0),
                                     layout=layout, v_down=v)
    p = SimParams(radius=0.35, bound=bound, **DAM_CONSTANTS)
    return dict(name=f"req_{layout}", pos=pos, vel=vel, params=p,
                dt=1.0 / 60.0, substeps=3, steps=k)


WORKLOADS = {
    "dam_break_16k": dam_break_16k,
    "dam_break_1m": dam_break_1m,
    "opposing_blocks_8m": opposing_blocks_8m,
}
