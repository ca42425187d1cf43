"""Seeded random scenes against the oracle, one captured substep each, under
the parity contract of the golden scenes (tests/parity.py): random particle
counts (1 to 3000), radii (the stale 0.35^2 cut-off active or not), box
shapes, clustered or uniform placement with particles outside the box,
random velocities and gravity. Complements the fixed golden cases with
corner cases nobody wrote down."""
import numpy as np
import pytest

from parity import compare_substep

pytestmark = pytest.mark.gpu


def random_scene(seed, speed=None):
    from fluidsim import scenes
    rng = np.random.default_rng(seed)
    n = int(rng.choice([1, 2, 3, 31, 32, 33, 500, int(rng.integers(100, 3000))]))
    radius = float(np.float32(rng.uniform(0.1, 0.5)))
    bound = tuple(float(np.float32(x)) for x in rng.uniform(1.0, 8.0, 3))
    half = np.array(bound) / 2
    if rng.uniform() < 0.5:   # a few dense clusters, some straddling a wall
        centres = rng.uniform(-half, half, (int(rng.integers(1, 5)), 3))
        pos = centres[rng.integers(0, len(centres), n)] + rng.normal(0, radius, (n, 3))
    else:                     # uniform, 10% of the box width outside it
        pos = rng.uniform(-1.1 * half, 1.1 * half, (n, 3))
    vel = rng.normal(0, rng.uniform(0.0, 3.0) if speed is None else speed, (n, 3))
    p = scenes.SimParams(radius=radius, bound=bound, **scenes.DAM_CONSTANTS)
    if rng.uniform() < 0.3:
        import dataclasses
        p = dataclasses.replace(p, gravity_on=False)
    dt = float(np.float32(rng.choice([1 / 60, 1 / 120, 1 / 240])))
    return p, pos.astype(np.float32), vel.astype(np.float32), dt


@pytest.mark.parametrize("table", [0, 2])
@pytest.mark.parametrize("seed", range(24))
def test_random_scene_substep(gpu_lib, oracle_mod, seed, table):
    """Each scene with its automatic key table and with a grid table wherever
    the allowance reaches (most of these small scenes)."""
    check_scene(oracle_mod, *random_scene(seed), table)


@pytest.mark.parametrize("table", [1, 2])
@pytest.mark.parametrize("seed", range(100, 108))
def test_random_scene_fast_particles(gpu_lib, oracle_mod, seed, table):
    """Speeds of ~150 (predictions 1-2 box lengths away at dt 1/120, many
    cells beyond the walls): a grid table clamps those predictions onto its
    edge cells, a bucket table wraps the cell index; both must still find
    exactly the pairs within the cutoff."""
    check_scene(oracle_mod, *random_scene(seed, speed=150.0), table)


def check_scene(oracle_mod, p, pos, vel, dt, table):
    import fluidsim
    sim = fluidsim.FluidSimulation(p)
    sim.InitializeData(pos.shape[0], pos, vel)
    sim.set_tuning(table=table)
    sim.debug_enable(True)
    sim.Update(dt, 1)
    got = sim.debug_export()
    gpos, gvel, _ = sim.download()
    assert sim.status() == 0
    sim.close()
    opos, ovel, ref = oracle_mod.substep_f32(p, pos, vel, dt)
    fx = dict(ref, pos=opos, vel=ovel, bound=np.array(p.bound, np.float64))
    print(pos.shape[0], table, compare_substep(got, fx, dt, gpos, gvel))
