"""Batched and served forms: every scene's result is the same alone and in
the mix (bit for bit: the segmented launches run the same per-particle
arithmetic in the same order), scenes come and go between steps, and the
autotuner returns a valid configuration."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_scenes(count, seed=5, lo=500, hi=6000):
    from fluidsim import scenes
    return scenes.batched_scenes(count=count, seed=seed, lo=lo, hi=hi)


def alone(sc, steps, substeps=3):
    import fluidsim
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(sc["pos"].shape[0], sc["pos"], sc["vel"])
    for _ in range(steps):
        sim.Update(sc["dt"], substeps)
    out = sim.download()
    assert sim.status() == 0
    sim.close()
    return out


def test_batch_equals_alone(gpu_lib):
    import fluidsim
    scs = small_scenes(6)
    b = fluidsim.Batch(sum(s["pos"].shape[0] for s in scs), 16)
    ids = [b.add(s["params"], s["pos"], s["vel"], s["dt"]) for s in scs]
    for _ in range(4):
        b.step(3)
    for sid, sc in zip(ids, scs):
        got = b.download(sid)
        ref = alone(sc, 4)
        for g, r in zip(got, ref):
            assert np.array_equal(g, r)
    b.close()


def test_mixed_key_tables_batch_equals_alone(gpu_lib):
    """Scenes with grid key tables next to one with a bucket table (its box
    three times wider along each axis, so its grid has far more cells than
    particles): the batch runs the kernels that choose the table per scene,
    each scene alone the single-form ones, and the results agree bit for
    bit."""
    import dataclasses
    import fluidsim
    from fluidsim.simulation import key_table
    scs = small_scenes(4, seed=11)
    wide = dict(scs[0])
    wide["params"] = dataclasses.replace(
        scs[0]["params"], bound=tuple(3.0 * b for b in scs[0]["params"].bound))
    scs = [wide] + scs[1:]
    forms = [key_table(s["params"], s["pos"].shape[0])[0] for s in scs]
    assert forms[0] is False and all(forms[1:])
    b = fluidsim.Batch(sum(s["pos"].shape[0] for s in scs), 8)
    ids = [b.add(s["params"], s["pos"], s["vel"], s["dt"]) for s in scs]
    for _ in range(4):
        b.step(3)
    for sid, sc in zip(ids, scs):
        got = b.download(sid)
        ref = alone(sc, 4)
        for g, r in zip(got, ref):
            assert np.array_equal(g, r)
    b.close()


def test_scenes_join_and_leave_between_steps(gpu_lib):
    import fluidsim
    scs = small_scenes(5, seed=9)
    cap = sum(s["pos"].shape[0] for s in scs)
    b = fluidsim.Batch(cap, 8)
    a = [b.add(s["params"], s["pos"], s["vel"], s["dt"]) for s in scs[:3]]
    b.step(3); b.step(3)
    late = b.add(scs[3]["params"], scs[3]["pos"], scs[3]["vel"], scs[3]["dt"])
    b.step(3)
    b.remove(a[1])                       # leaves after 3 steps
    later = b.add(scs[4]["params"], scs[4]["pos"], scs[4]["vel"], scs[4]["dt"])
    b.step(3); b.step(3)
    expect = {a[0]: (scs[0], 5), a[2]: (scs[2], 5), late: (scs[3], 3),
              later: (scs[4], 2)}
    for sid, (sc, k) in expect.items():
        got = b.download(sid)
        ref = alone(sc, k)
        for g, r in zip(got, ref):
            assert np.array_equal(g, r), sid
    assert b.num_scenes == 4
    b.close()


def test_capacity_refusal_is_clean(gpu_lib):
    import fluidsim
    scs = small_scenes(2, seed=3)
    b = fluidsim.Batch(scs[0]["pos"].shape[0], 4)
    b.add(scs[0]["params"], scs[0]["pos"], scs[0]["vel"], scs[0]["dt"])
    assert b.try_add(scs[1]["params"], scs[1]["pos"], scs[1]["vel"]) is None
    b.step(3)
    b.close()


def test_batch_autotune(gpu_lib):
    import fluidsim
    scs = small_scenes(4, seed=11)
    b = fluidsim.Batch(sum(s["pos"].shape[0] for s in scs), 8)
    ids = [b.add(s["params"], s["pos"], s["vel"], s["dt"]) for s in scs]
    b.step(3)
    before = [b.download(i) for i in ids]
    best, ms = b.autotune(3, steps_per_trial=1)
    assert best["block"] in (64, 128, 256, 512)
    assert best["cell_tile"] in (1, 64, 128, 256)
    assert best["force_block"] in (0, 64, 128, 256, 512)  # 0: same as block
    assert best["gather"] in (2, 3, 4, 8)
    assert best["particles_per_warp"] in (16, 32)
    assert ms > 0.0
    assert b.tuning() == best
    # the sweep's trial steps leave no trace in the scenes' state
    for i, was in zip(ids, before):
        for g, e in zip(b.download(i), was):
            assert np.array_equal(g, e), i
    b.close()


def out_positions(sim, n):
    import ctypes
    host = np.empty((n, 4), np.float32)
    rt = ctypes.CDLL("libcudart.so.13")  # the runtime the library loaded
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                              ctypes.c_int]
    assert rt.cudaMemcpy(host.ctypes.data, sim.out_positions_device_ptr(), n * 16, 2) == 0
    return host


def test_single_scene_autotune_restores_state(gpu_lib):
    import fluidsim
    sc = small_scenes(1, seed=12, lo=3000, hi=4000)[0]
    n = sc["pos"].shape[0]
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(n, sc["pos"], sc["vel"])
    sim.Update(sc["dt"], 3)
    before = sim.download()
    out_before = out_positions(sim, n)
    best, ms = sim.autotune(sc["dt"], 3, steps_per_trial=1)
    assert ms > 0.0 and sim.tuning() == best
    for g, e in zip(sim.download(), before):
        assert np.array_equal(g, e)
    assert np.array_equal(out_positions(sim, n), out_before)
    sim.Update(sc["dt"], 3)  # and it steps on from there
    assert sim.status() == 0
    sim.close()


def test_served_results_match_alone(gpu_lib):
    """Requests arriving while others run: each result equals the request
    run alone."""
    from fluidsim import scenes, server
    rng = np.random.default_rng(21)
    reqs = []
    for k in range(6):
        sc = scenes.request_scene(rng, lo=800, hi=5000, kmin=2, kmax=6)
        reqs.append(server.Request(k, sc["params"], sc["pos"], sc["vel"], sc["dt"],
                                   sc["substeps"], sc["steps"], arrival=0.002 * k))
    budget = 3 * 5000 * server.bytes_per_particle()  # about 3 scenes at once
    srv = server.Server(budget, max_scenes=16)
    done, stats = srv.run(reqs, realtime=False)
    srv.close()
    assert stats["requests"] == len(reqs)
    for r in reqs:
        ref = server.run_alone(r)
        for g, e in zip((done[r.rid].pos, done[r.rid].vel, done[r.rid].dens), ref):
            assert np.array_equal(g, e), r.rid
    assert stats["p99_step_ms"] >= stats["p50_step_ms"] > 0


def served_requests(count, seed, steps, lo=2100, hi=2900):
    from fluidsim import scenes, server
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(count):
        sc = scenes.request_scene(rng, lo=lo, hi=hi, kmin=3, kmax=3)
        reqs.append(server.Request(k, sc["params"], sc["pos"], sc["vel"], sc["dt"],
                                   sc["substeps"], steps[k], arrival=0.0))
    return reqs


def test_served_cancellation_frees_capacity(gpu_lib):
    """A budget of two requests at a time: cancelling a long resident request
    admits a waiting one in its place, a cancelled waiting request never
    runs, and every finished request still equals its run alone."""
    from fluidsim import server
    reqs = served_requests(4, seed=31, steps=[40, 3, 3, 3])
    srv = server.Server(2 * 2900 * server.bytes_per_particle(), max_scenes=8)

    def on_step(step, ms, resident):
        if step == 2:
            srv.cancel(0)  # resident, 38 steps left
            srv.cancel(3)  # still waiting for room

    done, stats = srv.run(reqs, realtime=False, on_step=on_step)
    srv.close()
    assert stats["cancelled"] == [0, 3]
    assert sorted(done) == [1, 2]
    # request 2 only fits once request 0 has left: it runs steps 3..5
    assert stats["batched_steps"] == 5
    for rid in (1, 2):
        ref = server.run_alone(reqs[rid])
        for g, e in zip((done[rid].pos, done[rid].vel, done[rid].dens), ref):
            assert np.array_equal(g, e), rid


def test_served_request_beyond_budget_is_refused(gpu_lib):
    from fluidsim import server
    reqs = served_requests(1, seed=32, steps=[2])
    srv = server.Server(1000 * server.bytes_per_particle(), max_scenes=4)
    with pytest.raises(RuntimeError, match="exceeds the capacity"):
        srv.run(reqs, realtime=False)
    srv.close()


def test_removed_scene_room_is_reused_before_the_next_step(gpu_lib):
    """A scene added right after another was removed takes over its room in
    the current layout (no step in between needed); with every scene
    removed the whole capacity is free again. Results equal each scene run
    alone."""
    import fluidsim
    scs = sorted(small_scenes(3, seed=13), key=lambda s: -s["pos"].shape[0])
    big, mid, small = scs
    n = [s["pos"].shape[0] for s in scs]
    assert n[2] < n[0]
    b = fluidsim.Batch(n[0] + n[1], 8)
    a = b.add(big["params"], big["pos"], big["vel"], big["dt"])
    m = b.add(mid["params"], mid["pos"], mid["vel"], mid["dt"])
    b.step(3)
    b.remove(a)
    s = b.try_add(small["params"], small["pos"], small["vel"], small["dt"])
    assert s is not None
    # what is left of the big scene's room and the layout's end is too small
    assert b.try_add(big["params"], big["pos"], big["vel"], big["dt"]) is None
    b.step(3); b.step(3)
    for sid, sc, k in ((m, mid, 3), (s, small, 2)):
        got = b.download(sid)
        for g, r in zip(got, alone(sc, k)):
            assert np.array_equal(g, r), sid
    b.remove(m)
    b.remove(s)
    a2 = b.add(big["params"], big["pos"], big["vel"], big["dt"])
    m2 = b.add(mid["params"], mid["pos"], mid["vel"], mid["dt"])
    b.step(3)
    for sid, sc in ((a2, big), (m2, mid)):
        for g, r in zip(b.download(sid), alone(sc, 1)):
            assert np.array_equal(g, r), sid
    b.close()


def test_batch_equals_alone_two_lanes_per_particle(gpu_lib):
    """With 16 particles per warp (two lanes a particle in the force
    kernels) a batch still equals each scene stepped alone bit for bit."""
    import fluidsim
    scs = small_scenes(3, seed=31)
    b = fluidsim.Batch(sum(s["pos"].shape[0] for s in scs), 4)
    b.set_tuning(particles_per_warp=16, gather=3)
    ids = [b.add(s["params"], s["pos"], s["vel"], s["dt"]) for s in scs]
    for _ in range(3):
        b.step(3)
    got = [b.download(i) for i in ids]
    b.close()
    for s, g in zip(scs, got):
        sim = fluidsim.FluidSimulation(s["params"])
        sim.InitializeData(s["pos"].shape[0], s["pos"], s["vel"])
        sim.set_tuning(particles_per_warp=16, gather=3)
        for _ in range(3):
            sim.Update(s["dt"], 3)
        for a, w in zip(g, sim.download()):
            assert np.array_equal(a, w)
        sim.close()


def test_many_tiny_scenes_equal_alone(gpu_lib):
    """8,192 ragged scenes of 1 to 40 particles (every tile partial, many
    scenes of a single particle, 8,192 key tables of one launch): a sample of
    48, the smallest and largest among them, equals each scene stepped alone
    bit for bit, and every scene stays finite."""
    import fluidsim
    from fluidsim import scenes
    rng = np.random.default_rng(8192)
    scs = []
    for s in range(8192):
        n = int(rng.integers(1, 41))
        pos, vel, bound = scenes.fill_box_scene(rng, n, rng.uniform(0.2, 0.6),
                                                rng.uniform(0.5, 2.0, size=3))
        p = scenes.SimParams(radius=0.35, bound=bound, **scenes.DAM_CONSTANTS)
        scs.append(dict(pos=pos, vel=vel, params=p, dt=1.0 / 60.0))
    sizes = np.array([s["pos"].shape[0] for s in scs])
    assert sizes.min() == 1 and sizes.max() == 40
    b = fluidsim.Batch(int(sizes.sum()), 8192)
    ids = [b.add(s["params"], s["pos"], s["vel"], s["dt"]) for s in scs]
    for _ in range(3):
        b.step(3)
    sample = set(np.random.default_rng(1).choice(8192, 44, replace=False).tolist())
    sample |= {int(np.argmin(sizes)), int(np.argmax(sizes)),
               int(np.flatnonzero(sizes == 1)[-1]), int(np.flatnonzero(sizes == 33)[0])}
    for k, (sid, sc) in enumerate(zip(ids, scs)):
        got = b.download(sid)
        assert all(np.isfinite(g).all() for g in got), k
        if k in sample:
            for g, r in zip(got, alone(sc, 3)):
                assert np.array_equal(g, r), k
    assert b.status() == 0
    b.close()
