"""Snapshots through the C ABI (sph_save / sph_load / sph_batch_save /
sph_batch_add_snapshot): a saved scene continues bit for bit as if it had
never been saved (the physics does not depend on the layout, and the next
step recomputes its prediction from the stored state); damaged or
mismatched files are refused with an error; a served request loop
checkpointed mid-stream and resumed by a new server finishes every request
exactly as the uninterrupted loop does."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def sim_16k(steps):
    import fluidsim
    from fluidsim import scenes
    sc = scenes.dam_break_16k()
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(sc["pos"].shape[0], sc["pos"], sc["vel"])
    for _ in range(steps):
        sim.Update(sc["dt"], 3)
    return sim, sc


def test_save_load_continues_bit_for_bit(gpu_lib, tmp_path):
    import fluidsim
    from fluidsim import scenes
    sim, sc = sim_16k(4)
    before = sim.download()
    sim.save(tmp_path / "s.sph")
    for _ in range(4):
        sim.Update(sc["dt"], 3)
    straight = sim.download()
    sim.close()
    # a handle of the same size with other settings and state
    other = fluidsim.FluidSimulation(scenes.SimParams(radius=0.5, bound=(5.0, 5.0, 5.0)))
    other.InitializeData(sc["pos"].shape[0])
    other.load(tmp_path / "s.sph")
    assert same(other.download(), before)         # densities included
    assert np.float32(other.getInteractionRadius()) == np.float32(sc["params"].radius)
    for _ in range(4):
        other.Update(sc["dt"], 3)
    assert same(other.download(), straight)
    assert other.status() == 0
    other.close()


def test_damaged_or_mismatched_snapshots_are_refused(gpu_lib, tmp_path):
    import fluidsim
    sim, sc = sim_16k(1)
    f = tmp_path / "s.sph"
    sim.save(f)
    blob = bytearray(f.read_bytes())
    cases = {"flip": bytes(blob[:1000] + bytes([blob[1000] ^ 1]) + blob[1001:]),
             "short": bytes(blob[:-8]), "magic": b"X" + bytes(blob[1:]),
             # a flipped bit of the radius (header byte 16): refused, not read
             # as another plausible scene
             "setting": bytes(blob[:16] + bytes([blob[16] ^ 1]) + blob[17:])}
    for name, data in cases.items():
        g = tmp_path / f"{name}.sph"
        g.write_bytes(data)
        with pytest.raises(fluidsim.SphError):
            sim.load(g)
    small = fluidsim.FluidSimulation(sc["params"])
    small.InitializeData(1000)
    with pytest.raises(fluidsim.SphError):
        small.load(f)                             # other particle count
    small.close()
    with pytest.raises(fluidsim.SphError):
        sim.load(tmp_path / "missing.sph")
    sim.close()


def test_batch_scene_moves_between_batches(gpu_lib, tmp_path):
    import fluidsim
    from fluidsim import scenes
    scs = scenes.batched_scenes(count=3, seed=41, lo=1500, hi=4000)
    a = fluidsim.Batch(sum(s["pos"].shape[0] for s in scs), 4)
    ids = [a.add(s["params"], s["pos"], s["vel"], s["dt"]) for s in scs]
    for _ in range(3):
        a.step(3)
    a.save(ids[1], tmp_path / "mid.sph")
    for _ in range(2):
        a.step(3)
    want = a.download(ids[1])
    a.close()
    b = fluidsim.Batch(10000, 4)
    sid = b.add_snapshot(tmp_path / "mid.sph")
    for _ in range(2):
        b.step(3)
    assert same(b.download(sid), want)
    b.close()


def test_served_checkpoint_and_resume(gpu_lib, tmp_path):
    from fluidsim import scenes, server
    rng = np.random.default_rng(77)
    reqs = []
    for k in range(5):
        sc = scenes.request_scene(rng, lo=900, hi=3000, kmin=3, kmax=9)
        reqs.append(server.Request(k, sc["params"], sc["pos"], sc["vel"], sc["dt"],
                                   sc["substeps"], sc["steps"], arrival=0.003 * k))
    budget = 2 * 3000 * server.bytes_per_particle()   # two at a time: a queue forms
    srv = server.Server(budget, max_scenes=8)
    whole, _ = srv.run(reqs, realtime=False)
    srv.close()

    class Crash(Exception):
        pass

    srv = server.Server(budget, max_scenes=8)

    def on_step(step, ms, resident):
        if step == 4:
            srv.checkpoint(tmp_path / "ckpt")
            raise Crash()

    with pytest.raises(Crash):
        srv.run(reqs, realtime=False, on_step=on_step)
    srv.close()
    again, done = server.resume(tmp_path / "ckpt")
    assert sorted([r.rid for r in again] + list(done)) == list(range(5))
    srv = server.Server(budget, max_scenes=8)
    rest, _ = srv.run(again, realtime=False)
    srv.close()
    done.update(rest)
    for rid, d in whole.items():
        got = done[rid]
        assert np.array_equal(got.pos, d.pos) and np.array_equal(got.vel, d.vel), rid
        assert np.array_equal(got.dens, d.dens), rid
