"""sph_spatial_lookup_static: the spatial lookup for callers that cannot
allocate device memory (a render loop that must not stall on cudaMalloc's
device-wide synchronisation, an engine with a fixed memory pool, code inside
another library's captured region). It works in a fixed array inside the
library, so the test checks that two calls in a row -- the second on a
different scene, over whatever the first left in that array -- give exactly
what the main entry point (sph_step with parity capture) gives.

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
