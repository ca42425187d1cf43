"""The oracle's smoothing kernels and pair forces against their closed forms
(engine/physics/kernels.h:25-82, physicsWorld.cc:325-464), evaluated in
float64 for two particles whose substep can be written out by hand:

- density  rho  = W2(0) + W2(d),  W2(x) = 15 (r-x)^2 / (2 pi r^5)   (x < r)
- near     rhon = W3(0) + W3(d),  W3(x) = 15 (r-x)^3 / (pi r^6)     (x < r)
- pressure a_i  = dir * (D2(d) P/rho + D3(d) Pn/rhon) / rho, where dir
  points from i to its neighbour, D2(x) = -15 (r-x) / (pi r^5),
  D3(x) = -45 (r-x)^2 / (pi r^6), P = (rho - rho0) k, Pn = rhon kn; the
  shared pressures equal the particle's own since both densities agree
- coincident particles: dir = (0, 1, 0)                              (:414)
- viscosity (Jacobi) v_i += (v_j - v_i) V(d) mu dt, V(x) = 315 (r^2-x^2)^3
  / (64 pi r^9), on the post-pressure velocities.
The FP32 oracle must agree to FP32 rounding (2e-6 relative here)."""
import math

import numpy as np
import pytest

RTOL = 2e-6


def params(radius):
    from fluidsim import scenes
    return scenes.SimParams(radius=radius, bound=(8.0, 8.0, 8.0),
                            target_density=55.0, pressure_mult=500.0,
                            near_pressure_mult=18.0, viscosity=0.06,
                            gravity_scale=9.81, gravity_on=False)


def w2(x, r):
    return 15.0 * (r - x) ** 2 / (2.0 * math.pi * r ** 5) if x < r else 0.0


def w3(x, r):
    return 15.0 * (r - x) ** 3 / (math.pi * r ** 6) if x < r else 0.0


def d2(x, r):
    return -15.0 * (r - x) / (math.pi * r ** 5) if x <= r else 0.0


def d3(x, r):
    return -45.0 * (r - x) ** 2 / (math.pi * r ** 6) if x <= r else 0.0


def visc(x, r):
    return 315.0 * (r * r - x * x) ** 3 / (64.0 * math.pi * r ** 9) if x < r else 0.0


def pair_state(d, vy):
    """Two particles on the x axis, d apart after prediction, moving in y
    with +vy / -vy (their prediction offsets cancel in the x separation but
    add 2 vy / 120 in y)."""
    pos = np.array([[0.1, 0.2, 0.3], [0.1 + d, 0.2, 0.3]], np.float32)
    vel = np.array([[0.0, vy, 0.0], [0.0, -vy, 0.0]], np.float32)
    return pos, vel


@pytest.mark.parametrize("radius", [0.35, 0.2])
@pytest.mark.parametrize("frac", [0.0, 0.3, 0.7, 0.95])
def test_pair_matches_closed_form(oracle_mod, radius, frac):
    r = float(np.float32(radius))
    p = params(radius)
    dt = float(np.float32(1.0 / 180.0))
    vy = 0.4 if frac > 0.0 else 0.0
    pos, vel = pair_state(np.float32(frac * r), vy)
    _, _, dbg = oracle_mod.substep_f32(p, pos, vel, dt)
    pred = dbg["pred"].astype(np.float64)
    off = pred[1] - pred[0]
    d = float(np.sqrt(off @ off))

    rho = w2(0.0, r) + w2(d, r)
    rhon = w3(0.0, r) + w3(d, r)
    for k in range(2):
        assert dbg["dens"][k, 0] == pytest.approx(rho, rel=RTOL)
        assert dbg["dens"][k, 1] == pytest.approx(rhon, rel=RTOL)

    P = (rho - p.target_density) * p.pressure_mult
    Pn = rhon * p.near_pressure_mult
    mag = (d2(d, r) * P / rho + d3(d, r) * Pn / rhon) / rho
    if d > 0.0:
        dirs = [off / d, -off / d]
    else:
        dirs = [np.array([0.0, 1.0, 0.0])] * 2
    scale = abs(mag)
    for k in range(2):
        want = dirs[k] * mag
        got = dbg["acc_p"][k].astype(np.float64)
        assert np.allclose(got, want, rtol=RTOL, atol=RTOL * scale), (k, got, want)

    # Jacobi viscosity on the post-pressure velocities
    vp = dbg["vel_p"].astype(np.float64)
    for k in range(2):
        want = vp[k] + (vp[1 - k] - vp[k]) * visc(d, r) * p.viscosity * dt
        got = dbg["vel_v"][k].astype(np.float64)
        assert np.allclose(got, want, rtol=RTOL, atol=RTOL * np.abs(vp).max()), (k, got, want)


def test_pair_beyond_radius_does_not_interact(oracle_mod):
    r = float(np.float32(0.35))
    p = params(0.35)
    pos, vel = pair_state(np.float32(1.02 * r), 0.0)
    _, _, dbg = oracle_mod.substep_f32(p, pos, vel, float(np.float32(1.0 / 180.0)))
    for k in range(2):
        assert dbg["dens"][k, 0] == pytest.approx(w2(0.0, r), rel=RTOL)
        assert dbg["dens"][k, 1] == pytest.approx(w3(0.0, r), rel=RTOL)
        assert np.all(dbg["acc_p"][k] == 0.0)


def test_subset_viscosity_f64_matches_reference_fp32():
    """The FP64 viscosity evaluator the 8.4M test uses, fed the reference's
    own FP32 predicted positions and post-pressure velocities of every
    golden scene, reproduces the reference's FP32 post-viscosity velocity
    within 1e-5 of the increment's sum of |terms| (plus the rounding of the
    final sum and of the distances)."""
    import oracle
    from conftest import fixture_params, load_fixture, substep_fixtures
    for name in substep_fixtures():
        fx = load_fixture(name)
        p = fixture_params(fx)
        n = fx["pred"].shape[0]
        dv, absv, dsens = oracle.subset_visc_f64(
            p, fx["pred"], fx["vel_p"], np.arange(n, dtype=np.uint32), float(fx["dt"]))
        err = np.linalg.norm(fx["vel_v"] - (fx["vel_p"].astype(np.float64) + dv), axis=1)
        bound = (1e-5 * absv + 2.0 ** -22 * np.linalg.norm(fx["vel_v"], axis=1) +
                 dsens * float(np.float32(p.radius)) * 2.0 ** -21)
        assert np.all(err <= bound), name
