"""The timed spatial sort, bit for bit: the layout the substep's kernels read
(internal cell index and key-table entry per particle, the particle at every
slot, the key table's start offsets) exported from a captured substep
(sph_debug_export_layout) against the oracle's restatement of the sort's
contract (oracle/layout.py) from the same predicted positions. The
reference's own lookup (HashCell keys, startIndices) is compared by
test_gpu_parity; this checks the sort the bench times, under both key-table
forms: every golden scene, the 1M dam break, and scenes at the edge of the
grid-table allowance."""
import numpy as np
import pytest

from conftest import fixture_params, load_fixture, substep_fixtures

pytestmark = pytest.mark.gpu


def captured_layout(params, pos, vel, dt, table):
    import fluidsim
    sim = fluidsim.FluidSimulation(params)
    sim.InitializeData(pos.shape[0], pos, vel)
    sim.set_tuning(table=table)
    sim.debug_enable(True)
    sim.Update(float(dt), 1)
    got = sim.debug_export_layout()
    assert sim.status() == 0
    sim.close()
    return got


def check(got, want):
    assert got["direct"] == want["direct"]
    for k in ("cell", "key", "slot_ids", "start"):
        assert got[k].shape == want[k].shape, k
        bad = int(np.sum(got[k] != want[k]))
        assert bad == 0, f"{k}: {bad} mismatches"


@pytest.mark.parametrize("table", [0, 1, 2])
@pytest.mark.parametrize("name", substep_fixtures())
def test_sort_layout_goldens(gpu_lib, oracle_mod, name, table):
    from oracle import layout
    fx = load_fixture(name)
    p = fixture_params(fx)
    got = captured_layout(p, fx["pos_in"], fx["vel_in"], fx["dt"], table)
    # the reference's own prediction (the fixture), which the GPU's matches
    want = layout.sort_layout(p, fx["pred"], table)
    check(got, want)


@pytest.mark.parametrize("table", [0, 1])
def test_sort_layout_1m(gpu_lib, oracle_mod, table):
    from fluidsim import scenes
    from oracle import layout
    sc = scenes.dam_break_1m()
    p = sc["params"]
    sub_dt = np.float32(np.float32(sc["dt"]) / np.float32(sc["substeps"]))
    got = captured_layout(p, sc["pos"], sc["vel"], sub_dt, table)
    want = layout.sort_layout(p, layout.predict(p, sc["pos"], sc["vel"], sub_dt), table)
    assert want["direct"] == (table == 0)
    check(got, want)


def allowance_scene(fits):
    """1000 particles in a cube box: with fits, the largest box whose grid
    exceeds n by at most the 65,536-entry allowance (tuning.table = 2 gives
    it a grid table); otherwise the next box size up (n buckets)."""
    import dataclasses

    from fluidsim.scenes import DAM_CONSTANTS, SimParams
    from oracle import layout
    prev = None
    for side in np.arange(4.0, 40.0, 0.05):
        p = SimParams(radius=0.35, bound=(float(side),) * 3, **DAM_CONSTANTS)
        _, cnt, _, _ = layout.grid(p)
        cells = cnt[0] * cnt[1] * cnt[2]
        if cells - 1000 > 65536:
            if fits:
                p, cells = prev
            rng = np.random.default_rng(11)
            h = 0.45 * p.bound[0]
            pos = rng.uniform(-h, h, (1000, 3)).astype(np.float32)
            return dataclasses.replace(p), pos, cells
        prev = (p, cells)
    raise AssertionError("no box found")


@pytest.mark.parametrize("fits", [True, False])
def test_sort_layout_allowance_edge(gpu_lib, oracle_mod, fits):
    """The largest grid within the allowance takes a grid table (table = 2);
    the next box size up falls back to n buckets."""
    from oracle import layout
    p, pos, cells = allowance_scene(fits)
    vel = np.zeros_like(pos)
    want = layout.sort_layout(p, layout.predict(p, pos, vel, 1 / 180), table=2)
    assert want["direct"] == fits
    assert (cells - 1000 <= 65536) == fits
    got = captured_layout(p, pos, vel, 1 / 180, table=2)
    check(got, want)
