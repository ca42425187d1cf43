"""Generates the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own engine/physics code (oracle/_ref/ref_driver, built
by `make -C oracle ref` from the reference sources) on seeded scenes and
stores its outputs. Needs the reference sources, so it runs only where they
are mounted (an x86-64 host: the reference's float->uint32 hash cast wraps
there, see the oracle's header). The committed .npz files are what the tests
read; nothing at test time touches the reference.

    REF=<reference checkout> python tests/golden/make_golden.py   # all fixtures
    REF=<reference checkout> python tests/golden/make_golden.py --only substep
"""
from __future__ import annotations

import argparse
import hashlib
import json
import pathlib
import subprocess
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "fluid-simulation-3d_gb300"))

import oracle  # noqa: E402
from fluidsim import scenes  # noqa: E402
from fluidsim.simulation import grid_arrangement  # noqa: E402

F32 = np.float32


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def sub_dt(sc):
    return F32(F32(sc["dt"]) / F32(sc["substeps"]))


def edge_scenes():
    """Small scenes covering the edge cases of the reference's path."""
    out = []
    rng = np.random.default_rng(7)
    base = scenes.SimParams(radius=0.35, bound=(4.0, 4.0, 4.0),
                            **scenes.DAM_CONSTANTS)

    def add(name, pos, vel=None, params=base, dt=1.0 / 180.0):
        pos = np.asarray(pos, np.float32).reshape(-1, 3)
        vel = np.zeros_like(pos) if vel is None else np.asarray(vel, np.float32)
        out.append(dict(name=name, pos=pos, vel=vel, params=params, dt=dt,
                        substeps=1))

    add("n1", [[0.0, 0.0, 0.0]], [[0.5, -0.25, 0.125]])
    add("n2", [[0.0, 0.0, 0.0], [0.1, 0.02, -0.03]])
    g = np.stack(np.meshgrid(*[np.arange(3)] * 3, indexing="ij"), -1).reshape(-1, 3)
    add("n27_negative", (g - 1.5) * 0.2 - 0.07)
    add("n100_cloud", rng.uniform(-0.6, 0.6, (100, 3)),
        rng.uniform(-1, 1, (100, 3)))
    add("n1000_cloud", rng.uniform(-1.0, 1.0, (1000, 3)),
        rng.uniform(-2, 2, (1000, 3)))
    coinc = np.concatenate([np.zeros((8, 3)), rng.uniform(-0.3, 0.3, (24, 3))])
    add("coincident", coinc)
    r = F32(0.35)
    k = np.stack(np.meshgrid(*[np.arange(-2, 3)] * 3, indexing="ij"), -1).reshape(-1, 3)
    add("cell_boundaries", k.astype(np.float32) * r)
    # particles at / beyond the walls of a 4^3 box, moving outwards
    w = np.array([[2.0, 0, 0], [-2.0, 0.1, 0], [0, 2.0, 0], [0, -2.0, 0.2],
                  [0.3, 0, 2.0], [0, 0.4, -2.0], [1.99, 1.99, 1.99],
                  [-1.999, -1.999, -1.999], [2.5, -2.5, 0.0], [0.0, 0.0, 0.0]])
    add("walls", w, np.sign(w) * 3.0 + np.array([0, 0, 0.1]))
    add("single_cell", rng.uniform(0.01, 0.34, (64, 3)))
    dflt = scenes.SimParams()
    add("default_lattice_1000", grid_arrangement(1000), params=dflt, dt=1.0 / 60.0)
    grav = scenes.SimParams(radius=0.175, bound=(3.0, 3.0, 3.0),
                            **scenes.DAM_CONSTANTS)
    add("n2000_r0175", rng.uniform(-1.2, 1.2, (2000, 3)),
        rng.uniform(-0.5, 0.5, (2000, 3)), params=grav, dt=1.0 / 240.0)
    # A box 40,000 cells long (r 0.05): a cell grid over it has to wrap, so
    # two clusters 32768 cells apart along x land on the same cell indices
    # of a 32768-cell grid row -- far cells in one bucket, as HashCell
    # collisions put them in the reference.
    wide = scenes.SimParams(radius=0.05, bound=(2000.0, 4.0, 4.0),
                            **scenes.DAM_CONSTANTS)
    a = rng.uniform(-0.15, 0.15, (300, 3)) + np.array([-799.9, 0.0, 0.0])
    b = rng.uniform(-0.15, 0.15, (300, 3)) + np.array([-799.9 + 32768 * 0.05, 0.05, 0.0])
    add("wrapped_grid", np.concatenate([a, b]), rng.uniform(-0.2, 0.2, (600, 3)),
        params=wide, dt=1.0 / 240.0)
    return out


def params_dict(p):
    return dict(radius=p.radius, cutoff_sq=p.cutoff_sq,
                target_density=p.target_density, pressure_mult=p.pressure_mult,
                near_pressure_mult=p.near_pressure_mult, viscosity=p.viscosity,
                gravity_scale=p.gravity_scale, gravity_on=bool(p.gravity_on),
                bound=list(p.bound), damping=p.damping, predict_dt=p.predict_dt)


def substep_fixture(sc, path):
    dt = sub_dt(sc)
    R = oracle.ref_substep(sc["params"], sc["pos"], sc["vel"], dt, canonical=True)
    # pin the restatement against the reference on the way
    pos, vel, D = oracle.substep_f32(sc["params"], sc["pos"], sc["vel"], dt)
    same = all(np.array_equal(R[a], D[b]) for a, b in
               [("hash", "hash"), ("key", "key"), ("start", "start"),
                ("lookup_id", "sorted_ids"), ("pred", "pred"), ("dens", "dens"),
                ("acc_p", "acc_p"), ("vel_p", "vel_p"), ("vel_v", "vel_v")])
    same = same and np.array_equal(R["pos"], pos) and np.array_equal(R["vel"], vel)
    np.savez_compressed(
        path, pos_in=sc["pos"], vel_in=sc["vel"], dt=np.float32(dt),
        params=json.dumps(params_dict(sc["params"])), hash=R["hash"], key=R["key"],
        start=R["start"], sorted_ids=R["lookup_id"], pred=R["pred"],
        dens=R["dens"], acc_p=R["acc_p"], vel_p=R["vel_p"], vel_v=R["vel_v"],
        pos=R["pos"], vel=R["vel"], abs_p=D["abs_p"], abs_v=D["abs_v"],
        raw_lookup_keys_sorted=np.all(np.diff(R["lookup_raw"][:, 2]) >= 0))
    return same


def large_fixture(path, sample=4096):
    """1M-particle dam break, one substep: subsample + digests of the full
    integer outputs (the fixture stays small; the test regenerates the input
    from the seed)."""
    sc = scenes.dam_break_1m()
    dt = sub_dt(sc)
    R = oracle.ref_substep(sc["params"], sc["pos"], sc["vel"], dt, canonical=True)
    _, _, D = oracle.substep_f32(sc["params"], sc["pos"], sc["vel"], dt)
    rng = np.random.default_rng(11)
    idx = np.sort(rng.choice(sc["pos"].shape[0], sample, replace=False)).astype(np.uint32)
    np.savez_compressed(
        path, idx=idx, pos_in_digest=sha(sc["pos"]), hash_digest=sha(R["hash"]),
        key_digest=sha(R["key"]), start_digest=sha(R["start"]),
        sorted_digest=sha(R["lookup_id"]), hash=R["hash"][idx], key=R["key"][idx],
        dens=R["dens"][idx], acc_p=R["acc_p"][idx], vel_p=R["vel_p"][idx],
        vel_v=R["vel_v"][idx], pos=R["pos"][idx], vel=R["vel"][idx],
        abs_p=D["abs_p"][idx], abs_v=D["abs_v"][idx], dt=np.float32(dt),
        n_occupied=int(np.sum(R["start"] != 0x7FFFFFFF)))
    same = (np.array_equal(R["hash"], D["hash"]) and np.array_equal(R["start"], D["start"])
            and np.array_equal(R["lookup_id"], D["sorted_ids"])
            and np.array_equal(R["dens"], D["dens"]))
    return same


def aggregates(pos, vel, dens):
    rho = dens[:, 0].astype(np.float64)
    v = vel.astype(np.float64)
    hist, _ = np.histogram(rho, bins=12, range=(0.0, 240.0))
    return dict(mean_density=float(rho.mean()), max_density=float(rho.max()),
                kinetic=float(0.5 * np.mean(np.sum(v * v, axis=1))),
                com=[float(x) for x in pos.astype(np.float64).mean(axis=0)],
                max_speed=float(np.sqrt(np.sum(v * v, axis=1)).max()),
                hist=[float(x) / rho.size for x in hist])


def rollout_fixture(path, checkpoints=(1, 5, 10, 30, 60, 120)):
    """The reference's own Update (Gauss-Seidel viscosity, its own sort) over
    120 steps of the 16k dam break; aggregates at the checkpoints. The
    restatement's Jacobi rollout is stored beside it for scale."""
    sc = scenes.dam_break_16k()
    dt = sub_dt(sc)
    pos, vel = sc["pos"], sc["vel"]
    ref, jac = {}, {}
    done = 0
    pj, vj = pos.copy(), vel.copy()
    for c in checkpoints:
        k = (c - done) * sc["substeps"]
        pos, vel, dens, _, _ = oracle.ref_update(sc["params"], pos, vel, dt, k)
        ref[str(c)] = aggregates(pos, vel, dens)
        for _ in range(k):
            pj, vj, d = oracle.substep_f32(sc["params"], pj, vj, dt)
        jac[str(c)] = aggregates(pj, vj, d["dens"])
        done = c
        print(f"  step {c}: ref rho {ref[str(c)]['mean_density']:.3f} "
              f"KE {ref[str(c)]['kinetic']:.4f} | jacobi rho "
              f"{jac[str(c)]['mean_density']:.3f} KE {jac[str(c)]['kinetic']:.4f}")
    with open(path, "w") as f:
        json.dump(dict(scene="dam_break_16k", seed=0, substeps=sc["substeps"],
                       dt=float(sc["dt"]), reference_gauss_seidel=ref,
                       restatement_jacobi=jac), f, indent=1)


LATTICE_SIZES = (1, 2, 27, 64, 100, 343, 1000, 16384, 50000)


def lattice_fixture(path):
    """The reference's own InitializeData(n) lattice (RowSize = ceil(n^(1/3)),
    GridArrangement, gap 0.215) for several n: full positions up to 1000
    particles, digests and a 512-point sample beyond; OutPositions.w."""
    out = {}
    rng = np.random.default_rng(17)
    for n in LATTICE_SIZES:
        pos, w = oracle.ref_init(scenes.SimParams(), n)
        if n <= 1000:
            out[f"pos_{n}"] = pos
        else:
            idx = np.sort(rng.choice(n, 512, replace=False)).astype(np.uint32)
            out[f"idx_{n}"] = idx
            out[f"sample_{n}"] = pos[idx]
            out[f"digest_{n}"] = sha(pos)
        out[f"w_{n}"] = np.unique(w)
    np.savez_compressed(path, sizes=np.array(LATTICE_SIZES), **out)


def speed_fixture(path):
    """getSpeed / getSpeedNormalzied of the reference for the velocities of
    a stepped scene (the first 4096 particles of the 16k dam break after 30
    of the reference's own Updates, i.e. 10 steps of dt = 1/60 in 3
    substeps) and of hand-picked edge cases (rest, exactly 1.5, just above,
    large, negative components); index n is out of range (0)."""
    sc = scenes.dam_break_16k()
    dt = sub_dt(sc)
    _, vel, _, _, _ = oracle.ref_update(sc["params"], sc["pos"], sc["vel"], dt, 30)
    edge = np.array([[0, 0, 0], [1.5, 0, 0], [0, -1.5, 0], [0, 0, 1.5000001],
                     [1e-20, 0, 0], [3, -4, 0], [1e6, 1e6, 1e6], [-0.3, 0.4, -1.2],
                     [0.86602540, 0.86602540, 0.86602540]], np.float32)
    v = np.concatenate([vel[:4096], edge]).astype(np.float32)
    sp, nrm = oracle.ref_speed(sc["params"], v)
    np.savez_compressed(path, vel=v, speed=sp, speed_normalized=nrm)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=["substep", "large", "rollout", "lattice", "speed"],
                    default=None)
    a = ap.parse_args()
    # REF (the reference checkout) comes from the environment
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "oracle", "ref"], check=True)
    if a.only in (None, "lattice"):
        lattice_fixture(HERE / "lattice_init.npz")
        print("lattice_init: reference InitializeData lattices", LATTICE_SIZES)
    if a.only in (None, "speed"):
        speed_fixture(HERE / "speed_normalized.npz")
        print("speed_normalized: reference getSpeed / getSpeedNormalzied")
    if a.only in (None, "substep"):
        for sc in [scenes.dam_break_16k()] + edge_scenes():
            ok = substep_fixture(sc, HERE / f"substep_{sc['name']}.npz")
            print(f"substep_{sc['name']}: n={sc['pos'].shape[0]} restatement "
                  f"{'bit-exact' if ok else 'DIFFERS'}")
    if a.only in (None, "large"):
        ok = large_fixture(HERE / "substep_dam_break_1m_sample.npz")
        print(f"dam_break_1m: restatement {'bit-exact' if ok else 'DIFFERS'}")
    if a.only in (None, "rollout"):
        rollout_fixture(HERE / "rollout_dam_break_16k.json")


if __name__ == "__main__":
    main()
