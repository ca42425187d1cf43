"""Headless render through the C ABI (sph_render) against the oracle's CPU
restatement (oracle/sph_render_oracle.cc) on the same state: the RGBA8 image
and the depth buffer must match bit for bit -- both evaluate the splat
coverage, depth, depth test (ties to the lower particle index) and colour
gradient with the same rounded operations in the same order."""
import numpy as np
import pytest

from fluidsim import render

pytestmark = pytest.mark.gpu

CAMERAS = {
    "outside": ((2.0, 3.0, 9.0), (-2.0, -1.5, -1.0)),   # the whole box in view
    "inside": ((-3.0, -2.5, -1.5), (3.0, -2.0, 2.0)),  # within the fluid: near clipping
    "above": ((0.0, 7.5, 0.01), (0.0, -4.0, 0.0)),
}


@pytest.fixture(scope="module")
def evolved_16k(gpu_lib):
    import fluidsim
    from fluidsim import scenes
    sc = scenes.dam_break_16k()
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(sc["pos"].shape[0], sc["pos"], sc["vel"])
    for _ in range(12):
        sim.Update(sc["dt"], sc["substeps"])
    yield sim
    sim.close()


@pytest.mark.parametrize("size", [(320, 240), (1280, 720)])
@pytest.mark.parametrize("camera", sorted(CAMERAS))
def test_render_matches_oracle(evolved_16k, oracle_mod, camera, size):
    sim = evolved_16k
    eye, center = CAMERAS[camera]
    v = render.view(eye, center, *size)
    img, depth = sim.render(v)
    pos, vel, _ = sim.download()
    want_img, want_depth = oracle_mod.render(pos, vel, v)
    drawn = (want_depth < 1.0).mean()
    assert drawn > 0.001, "the camera should see particles"
    assert np.array_equal(depth, want_depth)
    assert np.array_equal(img, want_img)
    print(camera, size, f"covered {drawn:.3f}")


def test_batch_scene_render_equals_single(gpu_lib, oracle_mod):
    import fluidsim
    from fluidsim import scenes
    scs = scenes.batched_scenes(count=3, seed=8, lo=2000, hi=5000)
    b = fluidsim.Batch(sum(s["pos"].shape[0] for s in scs), 4)
    ids = [b.add(s["params"], s["pos"], s["vel"], s["dt"]) for s in scs]
    for _ in range(3):
        b.step(3)
    for sid, sc in zip(ids, scs):
        hx, hy, hz = (0.5 * x for x in sc["params"].bound)
        v = render.view((hx * 1.2, hy * 1.5, hz * 2.5), (0.0, 0.0, 0.0), 400, 300)
        img, depth = b.render(sid, v)
        pos, vel, _ = b.download(sid)
        want_img, want_depth = oracle_mod.render(pos, vel, v)
        assert (want_depth < 1.0).any()
        assert np.array_equal(img, want_img) and np.array_equal(depth, want_depth), sid
    b.close()


def test_coincident_particles_tie_to_the_lower_index(gpu_lib, oracle_mod):
    import fluidsim
    from fluidsim import scenes
    p = scenes.SimParams(radius=0.35, bound=(4.0, 4.0, 4.0), **scenes.DAM_CONSTANTS)
    rng = np.random.default_rng(5)
    base = rng.uniform(-1.0, 1.0, (200, 3)).astype(np.float32)
    pos = np.concatenate([base, base])            # every position twice
    vel = np.concatenate([np.zeros_like(base), np.full_like(base, 2.0)])
    sim = fluidsim.FluidSimulation(p)
    sim.InitializeData(pos.shape[0], pos, vel)    # rendered before any step
    v = render.view((0.0, 0.0, 4.0), (0.0, 0.0, 0.0), 300, 300)
    img, depth = sim.render(v)
    want_img, want_depth = oracle_mod.render(pos, vel, v)
    sim.close()
    assert np.array_equal(img, want_img) and np.array_equal(depth, want_depth)
    drawn = img[want_depth < 1.0]
    assert np.all(drawn[:, 0] == 0)  # the zero-velocity first copies win (Color1)


def test_invalid_views_are_rejected(gpu_lib):
    import fluidsim
    from fluidsim import scenes
    sc = scenes.dam_break_16k()
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(1000, sc["pos"][:1000], sc["vel"][:1000])
    v = render.view((0.0, 0.0, 5.0), (0.0, 0.0, 0.0), 64, 64)
    v.proj[4] = 0.1  # a sheared projection
    with pytest.raises(fluidsim.SphError):
        sim.render(v)
    v = render.view((0.0, 0.0, 5.0), (0.0, 0.0, 0.0), 64, 64)
    v.width = 0
    with pytest.raises(fluidsim.SphError):
        sim.render(v)
    sim.close()
