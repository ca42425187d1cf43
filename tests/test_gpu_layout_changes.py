"""The GPU orders particles by an internal cell grid derived from the radius
and the box, so settings changed between steps re-shape that grid, and
particles far outside the box land in cells beyond it, whose indices wrap
onto it. In each case one captured substep must match the oracle -- the
reference's algorithm, pinned to it bit for bit -- run from the same state,
under the parity contract of the golden scenes (tests/parity.py)."""
import dataclasses

import numpy as np
import pytest

from parity import compare_substep

pytestmark = pytest.mark.gpu


def captured_vs_oracle(sim, params, dt, oracle_mod):
    pos0, vel0, _ = sim.download()
    sim.debug_enable(True)
    sim.Update(dt, 1)
    got = sim.debug_export()
    pos, vel, _ = sim.download()
    assert sim.status() == 0
    sim.debug_enable(False)
    opos, ovel, ref = oracle_mod.substep_f32(params, pos0, vel0, dt)
    fx = dict(ref, pos=opos, vel=ovel, bound=np.array(params.bound, np.float64))
    return compare_substep(got, fx, dt, pos, vel)


def dam_break_16k():
    from fluidsim import scenes
    sc = scenes.dam_break_16k()
    dt = float(np.float32(np.float32(sc["dt"]) / np.float32(sc["substeps"])))
    return sc, dt


def test_radius_change_between_steps(gpu_lib, oracle_mod):
    import fluidsim
    sc, dt = dam_break_16k()
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(sc["pos"].shape[0], sc["pos"], sc["vel"])
    for _ in range(3):
        sim.Update(dt, 1)
    sim.setInteractionRadius(0.3)
    p = dataclasses.replace(sc["params"], radius=float(np.float32(0.3)))
    print(captured_vs_oracle(sim, p, dt, oracle_mod))
    sim.close()


def test_bound_change_between_steps(gpu_lib, oracle_mod):
    import fluidsim
    sc, dt = dam_break_16k()
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(sc["pos"].shape[0], sc["pos"], sc["vel"])
    for _ in range(3):
        sim.Update(dt, 1)
    bound = (7.0, 5.0, 9.0)  # narrower in x and y, wider in z
    sim.setBound(bound)
    p = dataclasses.replace(sc["params"], bound=bound)
    print(captured_vs_oracle(sim, p, dt, oracle_mod))
    sim.close()


def test_particles_far_outside_the_box(gpu_lib, oracle_mod):
    """Clusters 100+ cells beyond a 4^3 box (and its grid margin): their
    cells' indices wrap onto the grid and may share buckets with cells
    inside it."""
    import fluidsim
    from fluidsim import scenes
    rng = np.random.default_rng(23)
    p = scenes.SimParams(radius=0.35, bound=(4.0, 4.0, 4.0), **scenes.DAM_CONSTANTS)
    parts = [rng.uniform(-1.5, 1.5, (1500, 3)),
             rng.uniform(-0.4, 0.4, (300, 3)) + np.array([60.0, 0.0, 0.0]),
             rng.uniform(-0.4, 0.4, (300, 3)) + np.array([-45.0, 30.0, 10.0]),
             rng.uniform(-0.4, 0.4, (300, 3)) + np.array([0.0, -2.3, 200.0])]
    pos = np.concatenate(parts).astype(np.float32)
    vel = rng.uniform(-1.0, 1.0, pos.shape).astype(np.float32)
    dt = float(np.float32(1.0 / 180.0))
    sim = fluidsim.FluidSimulation(p)
    sim.InitializeData(pos.shape[0], pos, vel)
    print(captured_vs_oracle(sim, p, dt, oracle_mod))
    sim.close()
