"""The largest scene a handle takes: 2^24 - 1 particles (the reference keeps
particle indices and keys in floats, exact below 2^24; sph_create refuses
2^24, test_abi). A 256^3 lattice at spacing 0.1 minus its last point, jitter
+-0.01, in the floor corner of a 30^3 box, r 0.175, the dam-break constants,
one step of 1/120 s in 2 substeps first so that it moves. Then one captured
substep per key-table form checks, against the oracle from the same state:
  * the timed sort's layout (cell index, key-table entry, slot order, start
    table) bit for bit (oracle/layout.py sort_layout), grid table and bucket
    table (key = cell mod (2^24 - 1));
  * the reference's own lookup (HashCell, key = hash % (2^24 - 1), the
    (key, index) order, startIndices) bit for bit (oracle/layout.py
    reference_lookup);
  * density, pressure acceleration and the viscosity increment on a 65,536
    particle subset against FP64, with the bounds of the 8.4M test."""
import numpy as np
import pytest

from test_gpu_large_fp64 import check_against_fp64
from test_gpu_sort_layout import check

pytestmark = pytest.mark.gpu

N_MAX = (1 << 24) - 1


def max_scene():
    from fluidsim import scenes
    rng = np.random.default_rng(24)
    bound = (30.0, 30.0, 30.0)
    counts = (256, 256, 256)
    pos = scenes.lattice_block(counts, 0.1, scenes._corner_origin(bound, 0.1), 0.01, rng,
                               n=N_MAX)
    p = scenes.SimParams(radius=0.175, bound=bound, **scenes.DAM_CONSTANTS)
    return p, pos, np.zeros_like(pos)


def test_max_particles(gpu_lib, oracle_mod):
    import fluidsim
    from oracle import layout
    p, pos, vel = max_scene()
    assert pos.shape[0] == N_MAX
    sub_dt = float(np.float32(np.float32(1.0 / 120.0) / np.float32(2)))
    sim = fluidsim.FluidSimulation(p)
    try:
        sim.InitializeData(N_MAX, pos, vel)
        sim.Update(1.0 / 120.0, 2)
        for step, table in enumerate((0, 1)):
            pos0, vel0, _ = sim.download()
            sim.set_tuning(table=table)
            sim.debug_enable(True)
            sim.Update(sub_dt, 1)  # the captured substep (advances the state)
            got = sim.debug_export_layout()
            d = sim.debug_export()
            sim.debug_enable(False)
            assert sim.status() == 0
            pred = layout.predict(p, pos0, vel0, sub_dt)
            want = layout.sort_layout(p, pred, table)
            assert want["direct"] == (table == 0)
            check(got, want)
            del got, want
            ref = layout.reference_lookup(pred, p.radius)
            for k in ("hash", "key", "sorted_ids", "start"):
                bad = int(np.sum(d[k] != ref[k]))
                assert bad == 0, f"{k}: {bad} mismatches"
            del ref
            check_against_fp64(oracle_mod, p, pos0, vel0, d, sub_dt, step)
    finally:
        sim.close()
