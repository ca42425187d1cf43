"""The last substep of a step also predicts the next step's first substep;
the next step uses that prediction only if nothing changed in between. A
handle stepped through a change of dt, of a setting and of its state, and
then through plain steps, must give bit for bit what fresh handles give from
the same state and settings (the physics does not depend on the handle's
previous layout)."""
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def fresh(params, pos, vel, dt, steps, substeps=3):
    import fluidsim
    sim = fluidsim.FluidSimulation(params)
    sim.InitializeData(pos.shape[0], pos, vel)
    for _ in range(steps):
        sim.Update(dt, substeps)
    out = sim.download()
    assert sim.status() == 0
    sim.close()
    return out


def same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_carried_prediction_follows_changes(gpu_lib):
    import fluidsim
    from fluidsim import scenes
    sc = scenes.dam_break_16k()
    p, dt = sc["params"], sc["dt"]
    sim = fluidsim.FluidSimulation(p)
    sim.InitializeData(sc["pos"].shape[0], sc["pos"], sc["vel"])

    for _ in range(2):
        sim.Update(dt, 3)
    s1 = sim.download()
    assert same(s1, fresh(p, sc["pos"], sc["vel"], dt, 2))

    dt2 = dt * 0.5                                  # new dt
    sim.Update(dt2, 3)
    s2 = sim.download()
    assert same(s2, fresh(p, s1[0], s1[1], dt2, 1))

    sim.setGravityScale(5.0)                        # new setting
    p3 = dataclasses.replace(p, gravity_scale=5.0)
    sim.Update(dt2, 3)
    s3 = sim.download()
    assert same(s3, fresh(p3, s2[0], s2[1], dt2, 1))

    rng = np.random.default_rng(4)                  # new state
    pos4 = (s3[0] + rng.uniform(-0.01, 0.01, s3[0].shape)).astype(np.float32)
    sim.upload(pos4, s3[1])
    sim.Update(dt2, 3)
    s4 = sim.download()
    assert same(s4, fresh(p3, pos4, s3[1], dt2, 1))

    for _ in range(3):                              # carried predictions
        sim.Update(dt2, 3)
    s5 = sim.download()
    assert sim.status() == 0
    sim.close()
    assert same(s5, fresh(p3, s4[0], s4[1], dt2, 3))
