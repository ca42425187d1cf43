"""C ABI checks that need no GPU: the library loads, exports exactly what
include/sph_gb300.h declares, reports the reference defaults, and fails
loudly (an error code and message, no fallback) when no device is usable."""
import ctypes
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    text = (ROOT / "include" / "sph_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sph_[a-z0-9_]+)\s*\(", text)))


def test_header_matches_binding_list():
    from fluidsim import _lib
    assert declared_symbols() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(str(built_lib))
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_default_params_are_reference_defaults(built_lib):
    """physicsWorld.h:96-106,145 and physicsWorld.cc:47,87."""
    import fluidsim
    p = fluidsim.default_params()
    f = np.float32
    assert p.radius == f(0.35)
    assert p.cutoff_sq == f(0.35) * f(0.35)
    assert p.target_density == f(99.7)
    assert p.pressure_mult == 300.0
    assert p.near_pressure_mult == 20.0
    assert p.viscosity == 0.5
    assert p.gravity_scale == 10.0
    assert p.gravity_on == 0
    assert list(p.bound) == [20.0, 20.0, 20.0]
    assert p.damping == f(0.95)
    assert p.predict_dt == f(1.0) / f(120.0)


def test_create_without_device_fails_loudly(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    import fluidsim
    with pytest.raises(fluidsim.SphError) as e:
        s = fluidsim.FluidSimulation()
        s.InitializeData(16)
    assert e.value.code == -2


def test_invalid_sizes_rejected(built_lib):
    import fluidsim
    L = fluidsim.load()
    p = fluidsim.default_params()
    h = ctypes.c_void_p()
    assert L.sph_create(ctypes.byref(p), 0, ctypes.byref(h)) == -1
    assert L.sph_create(ctypes.byref(p), 1 << 24, ctypes.byref(h)) == -1
    assert b"2^24" in L.sph_global_error()


def test_grid_arrangement_matches_reference_layout():
    """GridArrangement (physicsWorld.cc:518-557): rows of ceil(powf(N, 1/3)),
    gap 0.215, y descending from the top, x then z ascending. powf(1000,
    1/3) rounds to 10.000001, so 1000 particles take rows of 11 (the
    reference's own output, tests/test_reference_pins.py)."""
    from fluidsim import grid_arrangement
    g = grid_arrangement(1000)
    assert g.shape == (1000, 3)
    f = np.float32
    off = (f(11) * f(0.215) - f(0.215)) / f(2.0)
    assert np.array_equal(g[0], np.array([-off, off, -off], np.float32))
    assert g[1, 2] == g[0, 2] + f(0.215)
    assert g[11, 0] == g[0, 0] + f(0.215)
    assert g[121, 1] == g[0, 1] - f(0.215)
