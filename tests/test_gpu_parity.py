"""GPU parity: one substep through the C ABI against the reference's own
outputs (golden fixtures), plus run-to-run determinism."""
import hashlib

import numpy as np
import pytest

from conftest import fixture_params, load_fixture, substep_fixtures
from parity import compare_substep

pytestmark = pytest.mark.gpu


def run_substep(fx, params, debug=True, tuning=None):
    import fluidsim
    sim = fluidsim.FluidSimulation(params)
    n = fx["pos_in"].shape[0]
    sim.InitializeData(n, fx["pos_in"], fx["vel_in"])
    if tuning:
        sim.set_tuning(**tuning)
    if debug:
        sim.debug_enable(True)
    sim.Update(float(fx["dt"]), 1)
    got = sim.debug_export() if debug else {}
    pos, vel, dens = sim.download()
    assert sim.status() == 0
    sim.close()
    return got, pos, vel, dens


@pytest.mark.parametrize("table", [0, 1, 2])
@pytest.mark.parametrize("name", substep_fixtures())
def test_substep_parity(gpu_lib, name, table):
    """Every fixture under each key-table form: automatic, n buckets
    (cell index mod n), and one entry per grid cell wherever the table
    buffers have room (the small fixtures' 16^3 grids included)."""
    fx = load_fixture(name)
    p = fixture_params(fx)
    fx["bound"] = np.array(p.bound, np.float64)
    got, pos, vel, dens = run_substep(fx, p, tuning=dict(table=table))
    assert np.array_equal(got["dens"], dens)
    rep = compare_substep(got, fx, float(fx["dt"]), pos, vel)
    print(name, table, rep)


@pytest.mark.parametrize("tile", [64, 128, 192, 256])
@pytest.mark.parametrize("name", ["substep_dam_break_16k.npz", "substep_wrapped_grid.npz",
                                  "substep_single_cell.npz", "substep_n1000_cloud.npz",
                                  "substep_coincident.npz"])
def test_substep_parity_cooperative_density(gpu_lib, name, tile):
    """The autotuner's other density form (a warp per cell, candidates of
    the cell's runs held in registers, `tile` at a time) under the same
    contract."""
    fx = load_fixture(name)
    p = fixture_params(fx)
    fx["bound"] = np.array(p.bound, np.float64)
    got, pos, vel, dens = run_substep(fx, p, tuning=dict(cell_tile=tile))
    assert np.array_equal(got["dens"], dens)
    rep = compare_substep(got, fx, float(fx["dt"]), pos, vel)
    print(name, tile, rep)


@pytest.mark.parametrize("table", [0, 1])
def test_large_scene_parity(gpu_lib, table):
    """1M-particle dam break: full keys / hashes / start table / sorted order
    bit-exact (digests), sampled particles within tolerance; with its grid
    table (automatic) and with n buckets."""
    from fluidsim import scenes
    fx = load_fixture("substep_dam_break_1m_sample.npz")
    sc = scenes.dam_break_1m()
    full = dict(pos_in=sc["pos"], vel_in=sc["vel"], dt=fx["dt"])
    got, pos, vel, dens = run_substep(full, sc["params"], tuning=dict(table=table))
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    assert sha(got["hash"]) == str(fx["hash_digest"])
    assert sha(got["key"]) == str(fx["key_digest"])
    assert sha(got["start"]) == str(fx["start_digest"])
    assert sha(got["sorted_ids"]) == str(fx["sorted_digest"])
    idx = fx["idx"]
    sub = {k: got[k][idx] for k in ("dens", "acc_p", "vel_p", "vel_v")}
    fx["bound"] = np.array(sc["params"].bound, np.float64)
    rep = compare_substep(sub, fx, float(fx["dt"]), pos[idx], vel[idx])
    print(rep)


def test_deterministic(gpu_lib):
    """Two runs of several substeps give bit-identical state (the bucket order
    is canonical, no atomics decide a summation order)."""
    import fluidsim
    from fluidsim import scenes
    sc = scenes.dam_break_16k()
    outs = []
    for _ in range(2):
        sim = fluidsim.FluidSimulation(sc["params"])
        sim.InitializeData(sc["pos"].shape[0], sc["pos"], sc["vel"])
        for _ in range(4):
            sim.Update(sc["dt"], sc["substeps"])
        outs.append(sim.download())
        sim.close()
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_table_forms_agree(gpu_lib):
    """The 16k dam break (a grid table by default) stepped with each key
    table form: the walks visit the same particles in the same order, so the
    states are bit-identical."""
    import fluidsim
    from fluidsim import scenes
    sc = scenes.dam_break_16k()
    outs = []
    for table in (0, 1, 2):
        sim = fluidsim.FluidSimulation(sc["params"])
        sim.InitializeData(sc["pos"].shape[0], sc["pos"], sc["vel"])
        sim.set_tuning(table=table)
        assert sim.tuning()["table"] == table
        for _ in range(6):
            sim.Update(sc["dt"], sc["substeps"])
        assert sim.status() == 0
        outs.append(sim.download())
        sim.close()
    # switching forms between steps (new keys, a new table length, the
    # captured graphs and the carried prediction dropped) changes nothing
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(sc["pos"].shape[0], sc["pos"], sc["vel"])
    for k in range(6):
        sim.set_tuning(table=(0, 1, 2)[k % 3])
        sim.Update(sc["dt"], sc["substeps"])
    assert sim.status() == 0
    outs.append(sim.download())
    sim.close()
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("scene,table", [("dam_break_16k", 0), ("dam_break_16k", 1),
                                         ("substep_cell_boundaries.npz", 0),
                                         ("substep_cell_boundaries.npz", 2)])
def test_key_table_choice(gpu_lib, scene, table):
    """fluidsim.simulation.key_table predicts the engine's table form: a
    substep over a grid table launches no cell-table kernel, so it runs one
    kernel fewer (a carried prediction: no prediction kernel either)."""
    import fluidsim
    from fluidsim import scenes
    from fluidsim.simulation import key_table
    if scene.endswith(".npz"):
        fx = load_fixture(scene)
        params, pos, vel = fixture_params(fx), fx["pos_in"], fx["vel_in"]
    else:
        sc = getattr(scenes, scene)()
        params, pos, vel = sc["params"], sc["pos"], sc["vel"]
    n = pos.shape[0]
    grid, entries = key_table(params, n, table)
    sim = fluidsim.FluidSimulation(params)
    sim.InitializeData(n, pos, vel)
    sim.set_tuning(table=table)
    sim.Update(1 / 120, 1)
    k0 = sim.kernel_launches()
    sim.Update(1 / 120, 1)
    scan = 2 if (entries + 2047) // 2048 <= 4096 else 3
    assert sim.kernel_launches() - k0 == scan + 6 - (1 if grid else 0)
    assert sim.status() == 0
    sim.close()


def test_out_positions_buffer(gpu_lib):
    """OutPositions (physicsWorld.cc:107): float4 (pos, 0.34) in caller order."""
    import ctypes
    import fluidsim
    from fluidsim import scenes
    sc = scenes.dam_break_16k()
    sim = fluidsim.FluidSimulation(sc["params"])
    n = sc["pos"].shape[0]
    sim.InitializeData(n, sc["pos"], sc["vel"])
    sim.Update(sc["dt"], sc["substeps"])
    pos, _, _ = sim.download()
    ptr = sim.out_positions_device_ptr()
    host = np.empty((n, 4), np.float32)
    # the CUDA runtime the library itself loaded (same soname)
    rt = ctypes.CDLL("libcudart.so.13")
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                              ctypes.c_int]
    assert rt.cudaMemcpy(host.ctypes.data, ptr, n * 16, 2) == 0  # D2H
    assert np.array_equal(host[:, :3], pos)
    assert np.all(host[:, 3] == np.float32(0.34))
    sim.close()


def test_settings_surface_roundtrip(gpu_lib):
    import fluidsim
    sim = fluidsim.FluidSimulation()
    sim.InitializeData(64)
    sim.setGravity(True)
    sim.setGravityScale(9.81)
    sim.setInteractionRadius(0.2)
    sim.setDensityTarget(55)
    sim.setPressureMultiplier(500)
    sim.setNearPressureMultiplier(18)
    sim.setViscosityStrength(0.06)
    sim.setBound((12, 8, 6))
    assert sim.getGravityStatus()
    assert sim.getInteractionRadius() == np.float32(0.2)
    assert list(sim.getBounds()) == [12, 8, 6]
    sim.Update(1 / 60, 3)
    assert sim.status() == 0
    assert sim.getDensity(10**6) == 0.0  # out of range -> 0 (physicsWorld.cc:163)
    assert sim.getDensity(0) > 0.0
    sim.close()


@pytest.mark.parametrize("gather", [2, 3, 4, 8])
@pytest.mark.parametrize("name", ["substep_dam_break_16k.npz", "substep_n2000_r0175.npz",
                                  "substep_coincident.npz", "substep_single_cell.npz"])
def test_substep_parity_gather(gpu_lib, name, gather):
    """Every gather batch of the force kernels (the autotuner may pick any)
    under the parity contract: predicated batch loads at the end of a list
    and the padding of a partial batch."""
    fx = load_fixture(name)
    p = fixture_params(fx)
    fx["bound"] = np.array(p.bound, np.float64)
    got, pos, vel, dens = run_substep(fx, p, tuning=dict(gather=gather))
    rep = compare_substep(got, fx, float(fx["dt"]), pos, vel)
    print(name, gather, rep)


@pytest.mark.parametrize("gather", [3, 4, 8])
def test_full_lists_gather_bit_equal(gpu_lib, gather):
    """A dense scene (r / spacing = 2.4, about 60 neighbours a particle, so
    lists fill their 64 entries and some overflow to the walk) gives the
    same bits under every gather batch as under batches of 2: the batch only
    changes which loads are in flight, not the summation order."""
    import fluidsim
    from test_gpu_wide_lists import dense_scene
    sc = dense_scene()
    n = sc["pos"].shape[0]
    outs = []
    for g in (2, gather):
        sim = fluidsim.FluidSimulation(sc["params"])
        sim.InitializeData(n, sc["pos"], sc["vel"])
        sim.set_tuning(gather=g)
        for _ in range(2):
            sim.Update(sc["dt"], 2)
        assert sim.status() == 0
        outs.append(sim.download())
        sim.close()
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("gather", [2, 3, 8])
@pytest.mark.parametrize("name", ["substep_dam_break_16k.npz", "substep_n2000_r0175.npz",
                                  "substep_coincident.npz", "substep_walls.npz",
                                  "substep_n1.npz", "substep_wrapped_grid.npz"])
def test_substep_parity_two_lanes_per_particle(gpu_lib, name, gather):
    """16 particles per warp: two lanes share each particle's list in the
    pressure and viscosity kernels (odd and even entries, then a shuffle):
    the same parity contract as one lane a particle."""
    fx = load_fixture(name)
    p = fixture_params(fx)
    fx["bound"] = np.array(p.bound, np.float64)
    got, pos, vel, dens = run_substep(fx, p, tuning=dict(particles_per_warp=16, gather=gather))
    rep = compare_substep(got, fx, float(fx["dt"]), pos, vel)
    print(name, gather, rep)


def test_two_lanes_per_particle_full_lists(gpu_lib):
    """The dense scene (full and overflowing lists) under 16 particles per
    warp agrees with 32 to the FP32 tolerance of the force sums."""
    import fluidsim
    from test_gpu_wide_lists import dense_scene
    sc = dense_scene()
    n = sc["pos"].shape[0]
    outs = []
    for ppw in (32, 16):
        sim = fluidsim.FluidSimulation(sc["params"])
        sim.InitializeData(n, sc["pos"], sc["vel"])
        sim.set_tuning(particles_per_warp=ppw)
        sim.Update(sc["dt"], 1)
        assert sim.status() == 0
        outs.append(sim.download())
        sim.close()
    (p1, v1, d1), (p2, v2, d2) = outs
    assert np.array_equal(d1, d2)  # densities come before the force kernels
    dv = np.linalg.norm(v1.astype(np.float64) - v2, axis=1)
    scale = np.linalg.norm(v1.astype(np.float64), axis=1) + 1.0
    assert (dv / scale).max() < 1e-4
