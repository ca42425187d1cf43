"""Reader of the scene snapshot files sph_save / sph_batch_save write
(layout in csrc/sph_snapshot.cu), for host-side tools such as the request
server's resume: the settings, step dt and caller-order state of a scene,
without a GPU."""
from __future__ import annotations

import struct

import numpy as np

from ._lib import Params

MAGIC = b"SPHSNAP1"
HEADER = 80


def _fnv1a(data: bytes) -> int:
    h = 14695981039346656037
    for b in data:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def read(path, verify: bool = False) -> dict:
    """Returns dict(params=Params, dt, pos [n,3], vel [n,3], dens [n,2]).
    verify: also check the checksum here (a byte loop in Python; the
    library checks it whenever it loads a snapshot)."""
    with open(path, "rb") as f:
        blob = f.read()
    if len(blob) < HEADER or blob[:8] != MAGIC:
        raise ValueError(f"{path}: not a snapshot")
    version, n = struct.unpack_from("<II", blob, 8)
    if version not in (1, 2):
        raise ValueError(f"{path}: unknown snapshot version {version}")
    if len(blob) != HEADER + 32 * n:
        raise ValueError(f"{path}: {len(blob)} bytes, expected {HEADER + 32 * n}")
    f7 = struct.unpack_from("<7f", blob, 16)
    (gravity_on,) = struct.unpack_from("<i", blob, 44)
    f5 = struct.unpack_from("<5f", blob, 48)
    (dt,) = struct.unpack_from("<f", blob, 68)
    (digest,) = struct.unpack_from("<Q", blob, 72)
    # version 2: the checksum covers header bytes 0-71 and the payload;
    # version 1: the payload alone
    covered = blob[HEADER:] if version == 1 else blob[:72] + blob[HEADER:]
    if verify and _fnv1a(covered) != digest:
        raise ValueError(f"{path}: checksum mismatch")
    p = Params()
    (p.radius, p.cutoff_sq, p.target_density, p.pressure_mult, p.near_pressure_mult,
     p.viscosity, p.gravity_scale) = f7
    p.gravity_on = gravity_on
    p.bound[0], p.bound[1], p.bound[2], p.damping, p.predict_dt = f5
    arr = np.frombuffer(blob, np.float32, offset=HEADER)
    pos = arr[:3 * n].reshape(n, 3).copy()
    vel = arr[3 * n:6 * n].reshape(n, 3).copy()
    dens = arr[6 * n:].reshape(n, 2).copy()
    return dict(params=p, dt=float(dt), pos=pos, vel=vel, dens=dens)
