"""Host transfers through page-locked memory: sph_upload reads 16-byte
aligned pinned rows with the import kernel itself (over the host link),
everything else through staged copies. Both routes must give the same bits:
the same state uploaded either way steps to the same result, for sizes with
a partial last 32-particle chunk and for a pinned view that is not 16-byte
aligned (staged route); downloads into pinned arrays, any subset of the
outputs, equal the pageable ones."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class Pinned:
    """Page-locked host memory from the CUDA runtime the library loaded."""

    def __init__(self):
        self.rt = ctypes.CDLL("libcudart.so.13")
        self.rt.cudaHostAlloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t,
                                          ctypes.c_uint]
        self.rt.cudaFreeHost.argtypes = [ctypes.c_void_p]
        self.ptrs = []

    def array(self, shape, offset_floats=0):
        count = int(np.prod(shape)) + offset_floats
        p = ctypes.c_void_p()
        assert self.rt.cudaHostAlloc(ctypes.byref(p), 4 * count, 0) == 0
        self.ptrs.append(p)
        flat = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_float)),
                                     shape=(count,))
        return flat[offset_floats:].reshape(shape)

    def free(self):
        for p in self.ptrs:
            self.rt.cudaFreeHost(p)
        self.ptrs = []


def run(sc, pos, vel, out_pos, out_vel, out_dens, steps=2):
    import fluidsim
    n = sc["pos"].shape[0]
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(n, sc["pos"], sc["vel"])
    lib, h = sim._lib, sim.handle
    ptr = (lambda a: None if a is None else a.ctypes.data)
    for _ in range(steps):
        assert lib.sph_upload(h, ptr(pos), ptr(vel), sim._stream) == 0
        sim.step_async(sc["dt"], 3)
        assert lib.sph_download(h, ptr(out_pos), ptr(out_vel), ptr(out_dens), sim._stream) == 0
        pos, vel = out_pos, out_vel
    assert sim.status() == 0
    sim.close()


@pytest.mark.parametrize("n,offset", [(2000, 0), (1000 + 7, 0), (1000 + 7, 1)])
def test_pinned_rows_match_pageable(gpu_lib, n, offset):
    from fluidsim import scenes
    sc = scenes.batched_scenes(count=1, seed=17, lo=n, hi=n)[0]
    n = sc["pos"].shape[0]
    pg = [sc["pos"].copy(), sc["vel"].copy(), np.empty((n, 3), np.float32),
          np.empty((n, 3), np.float32), np.empty((n, 2), np.float32)]
    # pageable: upload the scene, step, download into separate arrays; then
    # those arrays are uploaded again (the loop of run())
    run(sc, pg[0], pg[1], pg[2], pg[3], pg[4])
    pin = Pinned()
    try:
        pp = pin.array((n, 3), offset)
        pv = pin.array((n, 3), offset)
        op = pin.array((n, 3), offset)
        ov = pin.array((n, 3), offset)
        od = pin.array((n, 2), offset)
        pp[:] = sc["pos"]
        pv[:] = sc["vel"]
        run(sc, pp, pv, op, ov, od)
        assert np.array_equal(op, pg[2])
        assert np.array_equal(ov, pg[3])
        assert np.array_equal(od, pg[4])
    finally:
        pin.free()


def test_pinned_download_subsets(gpu_lib):
    import fluidsim
    from fluidsim import scenes
    sc = scenes.batched_scenes(count=1, seed=18, lo=3000, hi=3000)[0]
    n = sc["pos"].shape[0]
    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(n, sc["pos"], sc["vel"])
    sim.Update(sc["dt"], 3)
    want = sim.download()
    pin = Pinned()
    try:
        lib, h, st = sim._lib, sim.handle, sim._stream
        for mask in range(1, 8):
            outs = [pin.array((n, 3)) if mask & 1 else None,
                    pin.array((n, 3)) if mask & 2 else None,
                    pin.array((n, 2)) if mask & 4 else None]
            for o in outs:
                if o is not None:
                    o[:] = -1.0
            assert lib.sph_download(h, *[None if o is None else o.ctypes.data for o in outs],
                                    st) == 0
            for o, w in zip(outs, want):
                if o is not None:
                    assert np.array_equal(o, w), mask
    finally:
        pin.free()
        sim.close()


def test_pinned_upload_prediction_follows_dt_and_substeps(gpu_lib):
    """A pinned upload into a handle that has stepped predicts the next step
    with its last dt and substeps; a step with another dt or substep count
    must discard that prediction. Pinned and pageable uploads give the same
    bits through a sequence that changes both."""
    import fluidsim
    from fluidsim import scenes
    sc = scenes.batched_scenes(count=1, seed=19, lo=3000, hi=3000)[0]
    n = sc["pos"].shape[0]
    plan = [(sc["dt"], 3), (sc["dt"], 3), (sc["dt"] * 0.5, 3), (sc["dt"] * 0.5, 2),
            (sc["dt"] * 0.5, 2), (sc["dt"], 3)]

    def run(make):
        sim = fluidsim.FluidSimulation(sc["params"])
        sim.InitializeData(n, sc["pos"], sc["vel"])
        lib, h = sim._lib, sim.handle
        pos, vel = make((n, 3)), make((n, 3))
        pos[:] = sc["pos"]
        vel[:] = sc["vel"]
        for dt, ss in plan:
            assert lib.sph_upload(h, pos.ctypes.data, vel.ctypes.data, sim._stream) == 0
            sim.step_async(dt, ss)
            assert lib.sph_download(h, pos.ctypes.data, vel.ctypes.data, None, sim._stream) == 0
        assert sim.status() == 0
        sim.close()
        return pos.copy(), vel.copy()

    pin = Pinned()
    try:
        got = run(lambda shape: pin.array(shape))
    finally:
        pin.free()
    want = run(lambda shape: np.empty(shape, np.float32))
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


@pytest.mark.parametrize("pinned", [False, True])
def test_upload_into_last_layout_changes_nothing(gpu_lib, pinned):
    """An upload between steps replaces the whole state: a simulation that
    has stepped and is then given another state (moved particles, pageable
    or pinned rows) continues exactly as a fresh simulation given that
    state -- the carried prediction, the layout and the sort's canonical
    (cell, caller index) order leave no trace of the earlier steps."""
    import fluidsim
    from fluidsim import scenes
    sc = scenes.dam_break_16k()
    n = sc["pos"].shape[0]
    pin = Pinned()
    host = (lambda a: (lambda b: (b.__setitem__(slice(None), a), b)[1])(pin.array(a.shape))
            if pinned else a.copy())

    sim = fluidsim.FluidSimulation(sc["params"])
    sim.InitializeData(n, sc["pos"], sc["vel"])
    for _ in range(3):
        sim.Update(sc["dt"], 3)
    p3, v3, _ = sim.download()
    rng = np.random.default_rng(4)
    p3m = (p3 + rng.normal(0, 0.01, p3.shape)).astype(np.float32)  # another state
    sim.upload(host(p3m), host(v3))
    for _ in range(2):
        sim.Update(sc["dt"], 3)
    a = sim.download()
    assert sim.status() == 0
    sim.close()

    fresh = fluidsim.FluidSimulation(sc["params"])
    fresh.InitializeData(n, p3m, v3)
    for _ in range(2):
        fresh.Update(sc["dt"], 3)
    b = fresh.download()
    fresh.close()
    pin.free()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
