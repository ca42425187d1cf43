"""GPU rollouts: the 120-step 16k dam break against the reference's own
Update (aggregates: the flow is chaotic, and the reference's viscosity is a
serial Gauss-Seidel sweep while this path is Jacobi), and short rollouts per
particle against the FP64 oracle."""
import json

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

# Aggregate tolerances. The restatement's own Jacobi rollout differs from the
# reference's Gauss-Seidel rollout by <0.1% mean density, ~1.5% kinetic
# energy and ~0.01 in centre of mass at step 120 (stored in the fixture).
TOL = dict(mean_density=0.01, max_density=0.06, kinetic=0.06, com=0.05,
           hist_l1=0.05)


def aggregates(pos, vel, dens):
    rho = dens[:, 0].astype(np.float64)
    v = vel.astype(np.float64)
    hist, _ = np.histogram(rho, bins=12, range=(0.0, 240.0))
    return dict(mean_density=float(rho.mean()), max_density=float(rho.max()),
                kinetic=float(0.5 * np.mean(np.sum(v * v, axis=1))),
                com=[float(x) for x in pos.astype(np.float64).mean(axis=0)],
                hist=[float(x) / rho.size for x in hist])


def test_rollout_120_steps_vs_reference(gpu_lib):
    import fluidsim
    from fluidsim import scenes
    with open(GOLDEN / "rollout_dam_break_16k.json") as f:
        fx = json.load(f)
    ref = fx["reference_gauss_seidel"]
    sc = scenes.dam_break_16k()
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(sc["pos"].shape[0], sc["pos"], sc["vel"])
    done = 0
    for c in sorted(int(k) for k in ref):
        for _ in range(c - done):
            sim.Update(sc["dt"], sc["substeps"])
        done = c
        got = aggregates(*sim.download())
        r = ref[str(c)]
        rep = {k: (got[k], r[k]) for k in ("mean_density", "max_density", "kinetic")}
        print(c, rep)
        assert abs(got["mean_density"] - r["mean_density"]) <= TOL["mean_density"] * r["mean_density"]
        assert abs(got["max_density"] - r["max_density"]) <= TOL["max_density"] * r["max_density"]
        assert abs(got["kinetic"] - r["kinetic"]) <= TOL["kinetic"] * max(r["kinetic"], 1.0)
        assert np.abs(np.subtract(got["com"], r["com"])).max() <= TOL["com"]
        assert np.abs(np.subtract(got["hist"], r["hist"])).sum() <= TOL["hist_l1"]
    assert sim.status() == 0
    sim.close()


@pytest.mark.parametrize("substeps", [1, 5])
def test_short_rollout_vs_fp64(gpu_lib, oracle_mod, substeps):
    """Per-particle state after a few substeps against the FP64 oracle."""
    import fluidsim
    from fluidsim import scenes
    sc = scenes.dam_break_16k()
    dt = np.float32(np.float32(sc["dt"]) / np.float32(sc["substeps"]))
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(sc["pos"].shape[0], sc["pos"], sc["vel"])
    p64, v64 = sc["pos"].astype(np.float64), sc["vel"].astype(np.float64)
    for _ in range(substeps):
        sim.Update(float(dt), 1)
        p64, v64, d64 = oracle_mod.substep_f64(sc["params"], p64, v64, float(dt))
    pos, vel, dens = sim.download()
    drel = np.abs(dens - d64["dens"]) / d64["dens"]
    print("density rel vs fp64", drel.max(), "pos abs", np.abs(pos - p64).max(),
          "vel abs", np.abs(vel - v64).max())
    assert drel.max() <= 1e-4
    assert np.abs(pos - p64).max() <= 1e-4
    vscale = max(1.0, np.abs(v64).max())
    assert np.abs(vel - v64).max() <= 1e-3 * vscale
    sim.close()


def test_long_run_1m_stays_physical(gpu_lib):
    """300 steps (2.5 s of simulated time) of the 1M dam break: no device
    status flag (non-finite state, index out of range), every particle
    inside the box, densities positive, and the block gone from its hull.
    (With the dam constants at r = 0.175 and spacing 0.1 the lattice's SPH
    density starts near 1150 against the target 55 -- the kernel scales as
    1/r^5 -- so it bursts outward rather than slump.)"""
    import fluidsim
    from fluidsim import scenes
    sc = scenes.dam_break_1m()
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(sc["pos"].shape[0], sc["pos"], sc["vel"])
    lo0, hi0 = sc["pos"].min(axis=0), sc["pos"].max(axis=0)
    for k in range(300):
        sim.step_async(sc["dt"], sc["substeps"])
        if k % 100 == 99:
            assert sim.status() == 0, k
    pos, vel, dens = sim.download()
    sim.close()
    half = np.array(sc["params"].bound, np.float32) / 2
    assert np.isfinite(pos).all() and np.isfinite(vel).all()
    assert np.all(np.abs(pos) <= half + 1e-5)
    assert np.all(dens[:, 0] > 0)
    outside = np.any((pos < lo0 - 0.5) | (pos > hi0 + 0.5), axis=1).mean()
    assert outside > 0.1                   # the fluid has left its initial hull
