"""Comparison helpers shared by the GPU parity tests.

Tolerances (FP32, summation order differs from the reference):
  * hash, key, start table, sorted order: bit-exact;
  * density / near density: relative 1e-5;
  * pressure acceleration: conditioning-aware relative 1e-5,
    |da| / max(|a_ref|, sum|terms|) with sum|terms| = sum over neighbours of
    |pressure term| / density (interior sums cancel, so |a_ref| alone is an
    ill-conditioned denominator); the plain relative error is reported;
  * velocities after the pressure / viscosity passes: |dv| <= 1e-5 * (|v| +
    dt * (sum|pressure terms| + sum|viscosity terms|));
  * positions / velocities after integration: the velocity bound above
    (times dt for positions) plus 2 ulp; particles whose position ends within
    1e-5 of a wall may take the other collision branch and are counted, not
    compared.
"""
from __future__ import annotations

import numpy as np

TOL = 1e-5


def norm(a):
    return np.sqrt(np.sum(np.asarray(a, np.float64) ** 2, axis=-1))


def rel_err(got, ref, floor=0.0):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    return np.abs(got - ref) / np.maximum(np.abs(ref), floor)


def compare_substep(got: dict, fx: dict, dt: float, pos=None, vel=None,
                    tol=TOL):
    """Asserts the parity contract; returns a dict of the worst errors."""
    rep = {}
    for k in ("hash", "key", "start", "sorted_ids"):
        if k in got and k in fx:
            mism = int(np.sum(got[k] != fx[k]))
            rep[f"{k}_mismatch"] = mism
            assert mism == 0, f"{k}: {mism} mismatches"
    idx = got.get("_idx")
    dref = fx["dens"]
    de = rel_err(got["dens"], dref, floor=1e-30)
    rep["dens_rel"] = float(de.max())
    assert de.max() <= tol, f"density rel err {de.max():.3e}"

    absp = np.asarray(fx["abs_p"], np.float64)
    absv = np.asarray(fx["abs_v"], np.float64)
    da = norm(np.asarray(got["acc_p"], np.float64) - fx["acc_p"])
    aref = norm(fx["acc_p"])
    cond = da / np.maximum(np.maximum(aref, absp), 1e-30)
    rep["acc_p_cond"] = float(cond.max())
    well = aref >= 0.1 * absp
    rep["acc_p_rel_well_conditioned"] = float((da / np.maximum(aref, 1e-30))[well].max()) if well.any() else 0.0
    assert cond.max() <= tol, f"pressure accel cond err {cond.max():.3e}"

    scale_v = norm(fx["vel_v"]) + dt * (absp + absv) + norm(fx["vel_p"])
    for k in ("vel_p", "vel_v"):
        dv = norm(np.asarray(got[k], np.float64) - fx[k])
        e = dv / np.maximum(scale_v, 1e-30)
        rep[f"{k}_err"] = float(e.max())
        assert e.max() <= tol, f"{k} err {e.max():.3e}"

    if pos is not None:
        bound = np.asarray(fx["bound"], np.float64) if "bound" in fx else None
        half = 0.5 * bound if bound is not None else None
        near = np.zeros(pos.shape[0], bool)
        if half is not None:
            near = np.any(np.abs(half[None, :] - np.abs(fx["pos"].astype(np.float64))) < 1e-5, axis=1)
        rep["near_wall"] = int(near.sum())
        ok = ~near
        dx = np.abs(np.asarray(pos, np.float64) - fx["pos"])
        ulp = np.spacing(np.abs(fx["pos"]).astype(np.float32)).astype(np.float64)
        tol_x = 2 * ulp + dt * tol * scale_v[:, None] + 1e-12
        bad = np.any(dx > tol_x, axis=1) & ok
        rep["pos_bad"] = int(bad.sum())
        assert bad.sum() == 0, f"{bad.sum()} positions out of tolerance"
        dvv = norm(np.asarray(vel, np.float64) - fx["vel"])
        ev = dvv / np.maximum(scale_v, 1e-30)
        rep["vel_err"] = float(ev[ok].max()) if ok.any() else 0.0
        assert (ev[ok] <= tol).all(), f"final vel err {ev[ok].max():.3e}"
    return rep
