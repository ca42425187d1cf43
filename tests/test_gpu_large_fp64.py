"""The heavily non-uniform 8.4M-particle scene (two opposing 256x128x128
blocks at spacing 0.08 in a 40x20x20 box, r 0.14, dt 1/240 in 2 substeps):
after 1, 10 and 20 steps (the blocks meet and splash), one captured
substep's density, near density, pressure acceleration and Jacobi viscosity
velocity increment against an FP64 recomputation on a 65,536-particle
random subset, reported per step.
Tolerances: density 1e-4 relative; acceleration 1e-4 of the particle's sum
of |pressure terms| (the sum cancels in the interior), plus
the acceleration's own sensitivity to FP32 rounding of the densities:
pressure is (rho - rho0) * k, which cancels for rho near rho0 in the
reference's FP32 formula itself, so a density exact to a few dozen ulp
(2^-18 relative) moves it by up to sens * 2^-18 (sens from the FP64 oracle);
and its sensitivity to the FP32 rounding of the distance: a spray particle
whose only neighbour sits just inside the support has a term linear in
r - dist, with r - dist as small as the rounding of dist itself, so an FP32
dist (squared sum and square root, about 2 ulp of r) moves it by up to
dsens * r * 2^-21 (dsens = sum of |d term / d dist| from the oracle).
The viscosity increment (velocity after the viscosity pass minus the
post-pressure velocity, physicsWorld.cc:424-464) is recomputed in FP64 from
the GPU's own FP32 predicted positions and post-pressure velocities, which
isolates the viscosity pass: |error| <= 1e-4 of mu * dt * sum|terms|, plus
the rounding of the final FP32 sum v + dv (2^-22 |v|), plus the distance
rounding term as above with the poly6 derivative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def predict_f32(p, pos, vel, dt):
    """physicsWorld.cc:45-47 in float32 without FMA (the GPU's prediction)."""
    f = np.float32
    dt = f(dt)
    gy = f(-p.gravity_scale) if p.gravity_on else f(0.0)
    v = vel.astype(np.float32).copy()
    v[:, 0] = v[:, 0] + f(0.0) * dt
    v[:, 1] = v[:, 1] + gy * dt
    v[:, 2] = v[:, 2] + f(0.0) * dt
    return (pos.astype(np.float32) + v * f(p.predict_dt)).astype(np.float32)


def check_against_fp64(oracle_mod, p, pos0, vel0, d, sub_dt, step):
    n = pos0.shape[0]
    pred = predict_f32(p, pos0, vel0, sub_dt)
    rng = np.random.default_rng(65536 + step)
    subset = np.sort(rng.choice(n, 65536, replace=False)).astype(np.uint32)
    dens64, acc64, abs64, sens64, dsens64 = oracle_mod.subset_f64(
        p, pred, subset, with_abs=True)
    drel = np.abs(d["dens"][subset].astype(np.float64) - dens64) / dens64
    da = np.linalg.norm(d["acc_p"][subset].astype(np.float64) - acc64, axis=1)
    scale = np.maximum(np.linalg.norm(acc64, axis=1), abs64)
    arel = da / np.maximum(scale, 1e-30)
    bound = (1e-4 * scale + sens64 * 2.0 ** -18 +
             dsens64 * float(np.float32(p.radius)) * 2.0 ** -21)
    over = np.where(bound > 0, da / np.where(bound > 0, bound, 1.0), 0.0)
    print(f"step {step}: n={n} density rel err max {drel.max():.3e} "
          f"mean {drel.mean():.3e}; accel err / sum|terms| max {arel.max():.3e} "
          f"mean {arel.mean():.3e} p99.9 {np.percentile(arel, 99.9):.3e}; "
          f"max err / bound {over.max():.3f}")
    assert drel.max() <= 1e-4
    assert np.all(da <= bound)
    # viscosity pass: GPU's vel_v against vel_p + FP64 increment
    dv64, absv, dsv = oracle_mod.subset_visc_f64(p, pred, d["vel_p"], subset, sub_dt)
    vp = d["vel_p"][subset].astype(np.float64)
    vv = d["vel_v"][subset].astype(np.float64)
    ev = np.linalg.norm(vv - (vp + dv64), axis=1)
    vbound = (1e-4 * absv + 2.0 ** -22 * np.linalg.norm(vv, axis=1) +
              dsv * float(np.float32(p.radius)) * 2.0 ** -21)
    vrel = ev / np.maximum(absv, 1e-30)
    vover = np.where(vbound > 0, ev / np.where(vbound > 0, vbound, 1.0), 0.0)
    # where the increment's terms stand well above the rounding of v itself
    # (else v + dv in FP32 cannot carry them)
    res = absv > 1e3 * 2.0 ** -22 * np.linalg.norm(vv, axis=1)
    vres = vrel[res] if res.any() else np.zeros(1)
    print(f"step {step}: viscosity increment err / sum|terms| max {vrel.max():.3e} "
          f"mean {vrel.mean():.3e}; where resolvable ({res.mean():.1%} of the subset) "
          f"max {vres.max():.3e} p99.9 {np.percentile(vres, 99.9):.3e}; "
          f"max err / bound {vover.max():.3f}; "
          f"max |dv| {np.linalg.norm(dv64, axis=1).max():.3e}")
    assert np.all(ev <= vbound)


def test_opposing_blocks_8m_vs_fp64(gpu_lib, oracle_mod):
    import fluidsim
    from fluidsim import scenes
    sc = scenes.opposing_blocks_8m()
    p = sc["params"]
    n = sc["pos"].shape[0]
    sub_dt = float(np.float32(np.float32(sc["dt"]) / np.float32(sc["substeps"])))
    sim = fluidsim.FluidSimulation(p)
    sim.InitializeData(n, sc["pos"], sc["vel"])
    done = 0
    for step in (1, 10, 20):
        for _ in range(step - done):
            sim.Update(sc["dt"], sc["substeps"])
        done = step
        pos0, vel0, _ = sim.download()
        sim.debug_enable(True)
        sim.Update(sub_dt, 1)  # the captured substep (advances the state)
        d = sim.debug_export()
        sim.debug_enable(False)
        assert sim.status() == 0
        check_against_fp64(oracle_mod, p, pos0, vel0, d, sub_dt, step)
    sim.close()
