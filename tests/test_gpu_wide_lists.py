"""Neighbour-list offsets past 2^32: entry k of slot i's list sits at
k * capacity + i, so in an engine of 80M slots a particle's 54th neighbour
lies beyond 2^32 elements. A small dense scene (about 60 neighbours per
particle, r / spacing = 2.4) stepped in such an engine must give exactly
what it gives in an engine of its own size (the offsets change, the
arithmetic does not). The big engine allocates about 55 GB of HBM."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CAPACITY = 80_000_000


def dense_scene():
    from fluidsim import scenes
    rng = np.random.default_rng(11)
    counts = (40, 40, 40)
    pos = scenes.lattice_block(counts, 0.1, (-2.0, -2.0, -2.0), 0.01, rng)
    p = scenes.SimParams(radius=0.24, bound=(8.0, 8.0, 8.0), **scenes.DAM_CONSTANTS)
    return dict(pos=pos, vel=np.zeros_like(pos), params=p, dt=1.0 / 240.0)


def test_list_offsets_past_2_32(gpu_lib):
    import fluidsim
    sc = dense_scene()
    n = sc["pos"].shape[0]
    # the small engine: the scene alone
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(n, sc["pos"], sc["vel"])
    for _ in range(2):
        sim.Update(sc["dt"], 2)
    ref = sim.download()
    assert sim.status() == 0
    sim.close()
    # the same scene in an engine of CAPACITY slots
    b = fluidsim.Batch(CAPACITY, 1)
    sid = b.add(sc["params"], sc["pos"], sc["vel"], sc["dt"])
    for _ in range(2):
        b.step(2)
    got = b.download(sid)
    b.close()
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)
    # the lists reach past entry 2^32 / CAPACITY = 53.7: check that the
    # scene is as dense as intended
    spatial = pytest.importorskip("scipy.spatial")
    tree = spatial.cKDTree(sc["pos"].astype(np.float64))
    inner = np.all(np.abs(sc["pos"]) < 1.5, axis=1)
    nb = np.array([len(v) - 1 for v in tree.query_ball_point(
        sc["pos"][inner].astype(np.float64), sc["params"].radius)])
    assert (nb >= 54).mean() > 0.5
