"""The snapshot file format (csrc/sph_snapshot.cu) as the host-side reader
fluidsim.snapshot parses it: a file laid out by hand here -- magic, version,
n, the 13 settings fields, dt, FNV-1a 64 of the header's first 72 bytes and
the payload (version 2; version 1 covered the payload alone), then
positions, velocities and densities -- reads back field for field, and
damaged files, a flipped setting included, are refused."""
import struct

import numpy as np
import pytest


def make_file(path, n=5, seed=1, bad_digest=False, version=2):
    rng = np.random.default_rng(seed)
    pos = rng.normal(size=(n, 3)).astype(np.float32)
    vel = rng.normal(size=(n, 3)).astype(np.float32)
    dens = rng.uniform(1, 50, size=(n, 2)).astype(np.float32)
    payload = pos.tobytes() + vel.tobytes() + dens.tobytes()
    head72 = (b"SPHSNAP1" + struct.pack("<II", version, n) +
              struct.pack("<7f", 0.35, 0.1225, 55.0, 500.0, 18.0, 0.06, 9.81) +
              struct.pack("<i", 1) + struct.pack("<5f", 12.0, 8.0, 6.0, 0.95, 1 / 120) +
              struct.pack("<f", 1 / 60))
    assert len(head72) == 72
    h = 14695981039346656037
    for b in (payload if version == 1 else head72 + payload):
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    if bad_digest:
        h ^= 1
    path.write_bytes(head72 + struct.pack("<Q", h) + payload)
    return pos, vel, dens


def test_reader_parses_every_field(tmp_path):
    from fluidsim import snapshot
    f = tmp_path / "a.sph"
    pos, vel, dens = make_file(f)
    s = snapshot.read(f, verify=True)
    p = s["params"]
    assert np.float32(p.radius) == np.float32(0.35)
    assert np.float32(p.target_density) == np.float32(55.0) and p.gravity_on == 1
    assert [np.float32(x) for x in p.bound] == [12.0, 8.0, 6.0]
    assert np.float32(p.predict_dt) == np.float32(1 / 120)
    assert np.float32(s["dt"]) == np.float32(1 / 60)
    assert np.array_equal(s["pos"], pos) and np.array_equal(s["vel"], vel)
    assert np.array_equal(s["dens"], dens)


def test_version_1_files_still_read(tmp_path):
    from fluidsim import snapshot
    f = tmp_path / "v1.sph"
    pos, _, _ = make_file(f, version=1)
    assert np.array_equal(snapshot.read(f, verify=True)["pos"], pos)


@pytest.mark.parametrize("damage", ["digest", "truncated", "magic", "version", "setting"])
def test_damaged_files_are_refused(tmp_path, damage):
    from fluidsim import snapshot
    f = tmp_path / "b.sph"
    make_file(f, bad_digest=(damage == "digest"))
    blob = bytearray(f.read_bytes())
    if damage == "truncated":
        blob = blob[:-4]
    elif damage == "magic":
        blob[0] ^= 0xFF
    elif damage == "version":
        blob[8] = 7
    elif damage == "setting":
        blob[16] ^= 0x01  # a bit of the radius
    f.write_bytes(bytes(blob))
    with pytest.raises(ValueError):
        snapshot.read(f, verify=True)
