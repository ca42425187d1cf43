"""Host-side restatements pinned to the reference's own outputs
(tests/golden/lattice_init.npz and speed_normalized.npz, made by
tests/golden/make_golden.py from the reference compiled by oracle/Makefile):

- the default lattice of InitializeData / GridArrangement
  (physicsWorld.cc:112-147, 518-557) as fluidsim.simulation.grid_arrangement
  and the C++ mirror's sph::GridArrangement lay it out;
- getSpeed / getSpeedNormalzied (physicsWorld.cc:172-182) as the Python
  binding, the C++ mirror and the render oracle (whose colours the GPU
  render matches bit for bit) compute them.
Bit for bit, in float32."""
import hashlib
import shutil
import struct
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def lattice():
    return np.load(GOLDEN / "lattice_init.npz")


def speeds():
    return np.load(GOLDEN / "speed_normalized.npz")


def check_lattice(L, n, pos):
    assert pos.shape == (n, 3) and pos.dtype == np.float32
    if f"pos_{n}" in L.files:
        assert np.array_equal(pos, L[f"pos_{n}"])
    else:
        assert np.array_equal(pos[L[f"idx_{n}"]], L[f"sample_{n}"])
        assert hashlib.sha256(np.ascontiguousarray(pos).tobytes()).hexdigest() == str(L[f"digest_{n}"])


@pytest.fixture(scope="module")
def mirror_exe(tmp_path_factory):
    exe = tmp_path_factory.mktemp("pins") / "mirror_pins"
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}",
           str(ROOT / "tests" / "cpp" / "mirror_pins.cc"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_python_lattice_matches_reference():
    from fluidsim.simulation import grid_arrangement
    L = lattice()
    for n in L["sizes"]:
        check_lattice(L, int(n), grid_arrangement(int(n)))
        assert np.array_equal(L[f"w_{int(n)}"], np.array([0.34], np.float32))


def test_cpp_mirror_lattice_matches_reference(mirror_exe):
    L = lattice()
    for n in L["sizes"]:
        out = subprocess.run([str(mirror_exe), "lattice", str(int(n))], capture_output=True,
                             check=True).stdout
        check_lattice(L, int(n), np.frombuffer(out, np.float32).reshape(-1, 3))


def test_python_speed_matches_reference():
    from fluidsim.simulation import speed_normalized, speed_of
    S = speeds()
    v = S["vel"]
    assert np.array_equal(speed_of(v), S["speed"][:-1])
    assert np.array_equal(speed_normalized(v), S["speed_normalized"][:-1])
    assert S["speed"][-1] == 0.0 and S["speed_normalized"][-1] == 0.0  # out of range


def test_cpp_mirror_speed_matches_reference(mirror_exe):
    S = speeds()
    v = np.ascontiguousarray(S["vel"], np.float32)
    n = v.shape[0]
    out = subprocess.run([str(mirror_exe), "speed"], input=struct.pack("<I", n) + v.tobytes(),
                         capture_output=True, check=True).stdout
    got = np.frombuffer(out, np.float32)
    assert np.array_equal(got[:n], S["speed"][:-1])
    assert np.array_equal(got[n:], S["speed_normalized"][:-1])


def test_render_oracle_speed_matches_reference(oracle_mod):
    S = speeds()
    assert np.array_equal(oracle_mod.speed_normalized(S["vel"]), S["speed_normalized"][:-1])
