"""Failure detection without a GPU fault: bad input made on the host. A
particle whose position or velocity is NaN must raise the non-finite status
flag (read and cleared by sph_status); its NaN cell coordinate converts to
a valid cell (0), so no index leaves its buffer (no range flag), and it
interacts with nobody:
every other particle ends the step exactly as in the same scene without it
(all its distance tests are false, and the in-cell order of the others is
unchanged)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def step(params, pos, vel, dt, substeps):
    import fluidsim
    sim = fluidsim.FluidSimulation(params)
    sim.InitializeData(pos.shape[0], pos, vel)
    sim.Update(dt, substeps)
    out = sim.download()
    flags = sim.status()
    again = sim.status()
    sim.close()
    return out, flags, again


@pytest.mark.parametrize("field,k", [("pos", 123), ("vel", 4000)])
def test_nonfinite_particle_is_flagged_and_isolated(gpu_lib, field, k):
    """(An infinite position is not an error: the reference's collision
    clamps it onto the wall, physicsWorld.cc:84-107.)"""
    from fluidsim import _lib, scenes
    sc = scenes.dam_break_16k()
    pos, vel = sc["pos"].copy(), sc["vel"].copy()
    (pos if field == "pos" else vel)[k, 1] = np.nan
    (p1, v1, d1), flags, again = step(sc["params"], pos, vel, sc["dt"], 3)
    assert flags & _lib.STATUS_NONFINITE
    assert not flags & _lib.STATUS_RANGE
    assert again == 0  # the read cleared it
    keep = np.arange(pos.shape[0]) != k
    (p0, v0, d0), flags0, _ = step(sc["params"], pos[keep], vel[keep], sc["dt"], 3)
    assert flags0 == 0
    assert np.array_equal(p1[keep], p0)
    assert np.array_equal(v1[keep], v0)
    assert np.array_equal(d1[keep], d0)


def test_batch_and_server_report_the_flag(gpu_lib):
    """The batched form reads the same flags over all its scenes
    (sph_batch_status), and the native serving loop keeps the flags of
    every step in its statistics; a clean batch and a clean server raise
    none."""
    import fluidsim
    from fluidsim import _lib, scenes, server
    scs = scenes.batched_scenes(count=3, seed=31, lo=500, hi=2000)
    bad_pos = scs[1]["pos"].copy()
    bad_pos[7, 0] = np.nan
    for poison in (False, True):
        b = fluidsim.Batch(sum(s["pos"].shape[0] for s in scs), 4)
        for k, s in enumerate(scs):
            b.add(s["params"], bad_pos if (poison and k == 1) else s["pos"], s["vel"], s["dt"])
        b.step(3)
        flags = b.status()
        assert bool(flags & _lib.STATUS_NONFINITE) == poison
        assert not flags & _lib.STATUS_RANGE
        assert b.status() == 0  # the read cleared it
        b.close()
    for poison in (False, True):
        srv = server.NativeServer(4000 * server.bytes_per_particle(), 4, substeps=3)
        s = scs[1]
        job = srv.submit(s["params"], bad_pos if poison else s["pos"], s["vel"], s["dt"], 2)
        srv.wait(job)
        flags = srv.stats()["status_flags"]
        assert bool(flags & _lib.STATUS_NONFINITE) == poison
        srv.close()
