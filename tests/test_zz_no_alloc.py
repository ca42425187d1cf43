"""sph_spatial_lookup_static: the spatial lookup for callers that cannot
allocate device memory (a render loop that must not stall on cudaMalloc's
device-wide synchronisation, an engine with a fixed memory pool). It works
in a fixed array inside the library, so the test checks that two calls in a
row -- the second on a different scene, over whatever the first left in
that array -- give exactly what the main entry point (sph_step with parity
capture) gives, and that a scene whose 65,536 particles share one cell (one
key) takes milliseconds, not the quadratic time an in-bucket ranking would.

Named to be collected last: a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

from conftest import fixture_params, load_fixture

SCENES = ["substep_dam_break_16k.npz", "substep_n2000_r0175.npz"]


def main_path_lookup(name):
    """hash, key, sorted ids, start table of the main entry point."""
    import fluidsim
    fx = load_fixture(name)
    sim = fluidsim.FluidSimulation(fixture_params(fx))
    sim.InitializeData(fx["pos_in"].shape[0], fx["pos_in"], fx["vel_in"])
    sim.debug_enable(True)
    sim.Update(float(fx["dt"]), 1)
    d = sim.debug_export()
    sim.close()
    return fx, d


def test_rejects_sizes_beyond_the_limit(built_lib):
    import fluidsim
    L = fluidsim.load()
    rc = L.sph_spatial_lookup_static(None, 65537, 0.35, None, None, None, None, None)
    assert rc == -1
    assert b"65536" in L.sph_static_error()


@pytest.mark.gpu
def test_static_lookup_matches_main_entry_point_twice(gpu_lib):
    import torch
    import fluidsim
    L = fluidsim.load()
    for name in SCENES:  # two calls in a row, different n
        fx, ref = main_path_lookup(name)
        n = fx["pred"].shape[0]
        pred = torch.from_numpy(np.ascontiguousarray(fx["pred"])).cuda()
        outs = [torch.empty(n, dtype=torch.int32, device="cuda") for _ in range(4)]
        torch.cuda.synchronize()
        p = fixture_params(fx)
        rc = L.sph_spatial_lookup_static(
            ctypes.c_void_p(pred.data_ptr()), n, ctypes.c_float(p.radius),
            *[ctypes.c_void_p(o.data_ptr()) for o in outs],
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == 0, L.sph_static_error()
        torch.cuda.synchronize()
        got = [o.cpu().numpy().view(np.uint32) for o in outs]
        for g, k in zip(got, ("hash", "key", "sorted_ids", "start")):
            assert np.array_equal(g, ref[k]), (name, k)
            assert np.array_equal(g, fx[k]), (name, k)  # and the reference's


@pytest.mark.gpu
def test_static_lookup_one_key_is_linear(gpu_lib, oracle_mod):
    """All SPH_STATIC_LOOKUP_MAX particles in one cell (one key, one bucket
    of 65,536), then a scene of random cells: each matches the reference's
    lookup restated in numpy, and the one-key call finishes in milliseconds."""
    import time

    import torch
    import fluidsim
    from oracle import layout
    L = fluidsim.load()
    n = 65536
    rng = np.random.default_rng(5)
    scenes = [rng.uniform(0.01, 0.3, (n, 3)).astype(np.float32),      # one cell
              rng.uniform(-3.0, 3.0, (n, 3)).astype(np.float32)]
    warm = torch.zeros((1, 3), dtype=torch.float32, device="cuda")
    wout = [torch.empty(1, dtype=torch.int32, device="cuda") for _ in range(4)]
    assert L.sph_spatial_lookup_static(  # module load and set-up outside the timing
        ctypes.c_void_p(warm.data_ptr()), 1, ctypes.c_float(0.35),
        *[ctypes.c_void_p(o.data_ptr()) for o in wout],
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    for pred in scenes:
        want = layout.reference_lookup(pred, np.float32(0.35))
        d = torch.from_numpy(pred).cuda()
        outs = [torch.empty(n, dtype=torch.int32, device="cuda") for _ in range(4)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = L.sph_spatial_lookup_static(
            ctypes.c_void_p(d.data_ptr()), n, ctypes.c_float(0.35),
            *[ctypes.c_void_p(o.data_ptr()) for o in outs],
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == 0, L.sph_static_error()
        torch.cuda.synchronize()
        ms = 1000.0 * (time.perf_counter() - t0)
        got = [o.cpu().numpy().view(np.uint32) for o in outs]
        for g, k in zip(got, ("hash", "key", "sorted_ids", "start")):
            assert np.array_equal(g, want[k]), k
        print(f"static lookup of {n}: {ms:.2f} ms")
        assert ms < 100.0
