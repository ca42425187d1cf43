"""The oracle (CPU restatement) against the golden fixtures generated from the
reference's own code -- bit-exact on every output, since both keep the
reference's float operation order and the canonical bucket order."""
import hashlib
import json

import numpy as np
import pytest

from conftest import GOLDEN, fixture_params, load_fixture, substep_fixtures


@pytest.mark.parametrize("name", substep_fixtures())
def test_restatement_bit_exact(oracle_mod, name):
    fx = load_fixture(name)
    p = fixture_params(fx)
    pos, vel, d = oracle_mod.substep_f32(p, fx["pos_in"], fx["vel_in"], fx["dt"])
    for k in ("hash", "key", "start", "sorted_ids", "pred", "dens", "acc_p",
              "vel_p", "vel_v"):
        assert np.array_equal(d[k], fx[k]), k
    assert np.array_equal(pos, fx["pos"])
    assert np.array_equal(vel, fx["vel"])


@pytest.mark.parametrize("name", substep_fixtures())
def test_fixture_invariants(name):
    """Properties of the reference lookup itself: keys = hash % n, sorted
    order ascending by (key, index), start[] points at each key's first
    entry and is INT_MAX elsewhere (physicsWorld.cc:466-498)."""
    fx = load_fixture(name)
    n = fx["hash"].shape[0]
    assert np.array_equal(fx["key"], fx["hash"] % np.uint32(n))
    ids = fx["sorted_ids"]
    assert np.array_equal(np.sort(ids), np.arange(n))
    ks = fx["key"][ids]
    assert np.all((np.diff(ks.astype(np.int64)) > 0) |
                  ((np.diff(ks.astype(np.int64)) == 0) & (np.diff(ids.astype(np.int64)) > 0)))
    start = fx["start"]
    first = np.full(n, 0x7FFFFFFF, np.uint32)
    for s in range(n - 1, -1, -1):
        first[ks[s]] = s
    assert np.array_equal(start, first)
    assert bool(fx["raw_lookup_keys_sorted"])


def test_hash_wraps_negative_cells(oracle_mod):
    """The float->uint32 cast of HashCell wraps (x86-64 semantics) on every
    host: cell (-1,0,0) hashes to 2^32 - 15823."""
    from fluidsim.scenes import SimParams
    p = SimParams(radius=0.35)
    pos = np.array([[-0.1, 0.1, 0.1]], np.float32)
    _, _, d = oracle_mod.substep_f32(p, pos, np.zeros_like(pos), 0.0)
    assert int(d["hash"][0]) == (2 ** 32 - 15823)


def test_large_fixture_input_digest():
    """The 1M-particle scene regenerates bit-identically from its seed."""
    from fluidsim import scenes
    fx = load_fixture("substep_dam_break_1m_sample.npz")
    sc = scenes.dam_break_1m()
    got = hashlib.sha256(np.ascontiguousarray(sc["pos"]).tobytes()).hexdigest()
    assert got == str(fx["pos_in_digest"])


def test_oracle_jacobi_vs_gauss_seidel_differ_only_in_viscosity(oracle_mod):
    fx = load_fixture("substep_dam_break_16k.npz")
    p = fixture_params(fx)
    _, _, dj = oracle_mod.substep_f32(p, fx["pos_in"], fx["vel_in"], fx["dt"])
    _, _, dg = oracle_mod.substep_f32(p, fx["pos_in"], fx["vel_in"], fx["dt"],
                                      gauss_seidel=True)
    assert np.array_equal(dj["vel_p"], dg["vel_p"])
    assert np.array_equal(dj["dens"], dg["dens"])


def test_fp64_oracle_close_to_fp32(oracle_mod):
    fx = load_fixture("substep_dam_break_16k.npz")
    p = fixture_params(fx)
    _, _, d64 = oracle_mod.substep_f64(p, fx["pos_in"], fx["vel_in"], fx["dt"])
    rel = np.abs(d64["dens"] - fx["dens"]) / np.abs(d64["dens"])
    assert rel.max() < 1e-5


def test_fp64_subset_matches_full(oracle_mod):
    fx = load_fixture("substep_n2000_r0175.npz")
    p = fixture_params(fx)
    _, _, d64 = oracle_mod.substep_f64(p, fx["pos_in"], fx["vel_in"], fx["dt"])
    sub = np.arange(0, 2000, 7, dtype=np.uint32)
    dens, acc = oracle_mod.subset_f64(p, fx["pred"], sub)
    assert np.allclose(dens, d64["dens"][sub], rtol=1e-6)
    scale = np.abs(d64["acc_p"][sub]).max()
    assert np.abs(acc - d64["acc_p"][sub]).max() < 1e-4 * scale


def test_rollout_fixture_present():
    with open(GOLDEN / "rollout_dam_break_16k.json") as f:
        r = json.load(f)
    assert set(r["reference_gauss_seidel"]) == {"1", "5", "10", "30", "60", "120"}
