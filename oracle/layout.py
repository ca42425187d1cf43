"""Restatement of the timed spatial sort's contract -- TEST INFRASTRUCTURE ONLY.

The GPU path replaces the reference's UpdateSpatialLookup
(engine/physics/physicsWorld.cc:466-498: key = HashCell(cell) % n, std::sort
by key, startIndices) with a counting sort by an internal cell index of the
same cells (cell = floor(pred / radius), physicsWorld.cc:499-503). This
module restates, in numpy and from the predicted positions alone, what that
sort must produce, so that the layout the timed kernels read can be checked
bit for bit (tests/test_gpu_sort_layout.py):

  * the internal grid around the box: per axis the cells of [-h, h] plus two
    cells each side, h = bound / 2 (in double precision, at most 2^15 cells);
  * the cell index cx' + cy' * gnx + cz' * gnx * gny (mod 2^32), with c' the
    cell coordinate clamped to the grid's inner cells (grid key table) or
    minus the grid origin (bucket table);
  * the key: the cell index itself (grid table, one entry per grid cell) or
    the cell index mod n (bucket table, n entries); a grid table is used when
    the grid has at most four cells per particle, or, with tuning.table = 2,
    when its excess over n fits a 65,536-entry allowance (never with
    tuning.table = 1);
  * the order: stable by (key, cell index, caller index);
  * start[k]: the number of particles with a smaller key (exclusive prefix
    of the key counts), start[table_len] = n.
"""
from __future__ import annotations

import math

import numpy as np

F32 = np.float32
U32 = 0xFFFFFFFF
DIRECT_CELLS_PER_PARTICLE = 4
TABLE_ALLOWANCE = 65536


def predict(params, pos, vel, sub_dt):
    """physicsWorld.cc:45-47 in float32, each product and sum rounded (no
    FMA): v += (0, -gScale*gravity, 0) * dt; pred = pos + v * (1/120)."""
    dt = F32(sub_dt)
    gy = F32(-params.gravity_scale) if params.gravity_on else F32(0.0)
    v = np.asarray(vel, np.float32).copy()
    v[:, 0] = v[:, 0] + F32(0.0) * dt
    v[:, 1] = v[:, 1] + gy * dt
    v[:, 2] = v[:, 2] + F32(0.0) * dt
    return (np.asarray(pos, np.float32) + v * F32(params.predict_dt)).astype(np.float32)


def grid_axis(bound, radius):
    """(origin, cells) of the internal grid along one axis."""
    h = float(F32(bound) * F32(0.5))
    r = float(F32(radius))
    a, b = -h / r, h / r
    lo = hi = None
    if math.isfinite(a) and math.isfinite(b):
        lo = min(math.floor(a), math.floor(b)) - 2.0
        hi = max(math.floor(a), math.floor(b)) + 2.0
    if lo is None or lo < -1e9 or hi > 1e9:
        lo, hi = 0.0, 1023.0
    return int(lo), int(min(hi - lo + 1.0, 32768.0))


def grid(params):
    """Origins, cell counts and strides (wy, wz mod 2^32) of the scene's grid."""
    ax = [grid_axis(params.bound[a], params.radius) for a in range(3)]
    org = [o for o, _ in ax]
    cnt = [c for _, c in ax]
    return org, cnt, cnt[0], (cnt[0] * cnt[1]) & U32


def uses_grid_table(params, n, table=0):
    _, cnt, _, _ = grid(params)
    cells = cnt[0] * cnt[1] * cnt[2]
    if table != 1 and cells <= DIRECT_CELLS_PER_PARTICLE * n:
        return True, cells
    if table == 2 and cells - n <= TABLE_ALLOWANCE:
        return True, cells
    return False, n


def cell_coords(pred, radius):
    """floor of the correctly rounded quotient, converted to int32 as the
    device's float-to-int conversion does (saturating, NaN -> 0)."""
    q = np.floor(np.asarray(pred, np.float32) / F32(radius)).astype(np.float64)
    q = np.where(np.isnan(q), 0.0, q)
    return np.clip(q, -2.0 ** 31, 2.0 ** 31 - 1).astype(np.int64)


def cell_index(params, pred, direct):
    org, cnt, wy, wz = grid(params)
    c = cell_coords(pred, params.radius)
    if direct:
        g = []
        for a in range(3):
            lo = org[a] + 1
            hi = lo + cnt[a] - 3
            g.append(np.clip(c[:, a], lo, hi) - lo + 1)
    else:
        g = [(c[:, a] - org[a]) & U32 for a in range(3)]
    return ((g[0] + g[1] * wy + g[2] * wz) & U32).astype(np.uint32)


def sort_layout(params, pred, table=0):
    """What the timed sort must produce for predicted positions `pred`
    (n x 3 float32): dict of cell[n], key[n] (caller order), slot_ids[n]
    (caller index at each slot), start[table_len + 1] and direct."""
    n = pred.shape[0]
    direct, table_len = uses_grid_table(params, n, table)
    cell = cell_index(params, pred, direct)
    key = cell.copy() if direct else (cell % np.uint32(n)).astype(np.uint32)
    ids = np.arange(n, dtype=np.uint32)
    slot_ids = ids[np.lexsort((ids, cell, key))].astype(np.uint32)
    counts = np.bincount(key.astype(np.int64), minlength=table_len)
    start = np.zeros(table_len + 1, np.uint32)
    start[1:] = np.cumsum(counts, dtype=np.uint64).astype(np.uint32)
    return dict(cell=cell, key=key, slot_ids=slot_ids, start=start, direct=direct)


def reference_lookup(pred, radius):
    """The reference's own spatial lookup (UpdateSpatialLookup,
    physicsWorld.cc:466-498) for predicted positions `pred`: HashCell of each
    particle's cell (physicsWorld.cc:505-511, the float->uint32 cast wrapping
    as on x86-64), key = hash % n, the (key, index) order, and startIndices
    (0x7fffffff for an empty key)."""
    n = pred.shape[0]
    c = cell_coords(pred, radius) & U32
    h = ((c[:, 0] * 15823 + c[:, 1] * 9737333 + c[:, 2] * 440817757) & U32).astype(np.uint32)
    key = (h % np.uint32(n)).astype(np.uint32)
    ids = np.arange(n, dtype=np.uint32)
    order = ids[np.lexsort((ids, key))].astype(np.uint32)
    start = np.full(n, 0x7FFFFFFF, np.uint32)
    ks = key[order]
    first = np.ones(n, bool)
    first[1:] = ks[1:] != ks[:-1]
    start[ks[first]] = np.nonzero(first)[0].astype(np.uint32)
    return dict(hash=h, key=key, sorted_ids=order, start=start)
