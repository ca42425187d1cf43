"""Oracle for the SPH substep -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
may import this package. It wraps

  * oracle/_build/libsph_oracle.so -- the CPU restatement (sph_oracle.cc) of
    engine/physics/physicsWorld.cc:39-111,304-516 and kernels.h:25-82 of
    Allkams/Fluid-Simulation-3D, and of the frame its CPU plug-in draws
    (sph_render_oracle.cc: fluidSimCPU.cc:53-124 with the particleRender
    shaders), built by `make -C oracle oracle`;
  * oracle/_ref/ref_driver -- the reference's own physicsWorld.cc compiled
    unmodified with a stepwise driver (`make -C oracle ref`), present only
    where the reference sources exist (used to pin the restatement and to
    generate tests/golden/).
"""
from __future__ import annotations

import ctypes
import os
import pathlib
import struct
import subprocess
import tempfile

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libsph_oracle.so"
REF_DRIVER = HERE / "_ref" / "ref_driver"


class OracleParams(ctypes.Structure):
    _fields_ = [
        ("radius", ctypes.c_float),
        ("cutoff_sq", ctypes.c_float),
        ("target_density", ctypes.c_float),
        ("pressure_mult", ctypes.c_float),
        ("near_pressure_mult", ctypes.c_float),
        ("viscosity", ctypes.c_float),
        ("gravity_scale", ctypes.c_float),
        ("gravity_on", ctypes.c_int32),
        ("bound", ctypes.c_float * 3),
        ("damping", ctypes.c_float),
        ("predict_dt", ctypes.c_float),
    ]


_P = ctypes.c_void_p


class DebugF32(ctypes.Structure):
    _fields_ = [(k, _P) for k in ("hash", "key", "sorted_ids", "start", "pred",
                                  "dens", "acc_p", "vel_p", "vel_v", "abs_p",
                                  "abs_v")]


class DebugF64(ctypes.Structure):
    _fields_ = [(k, _P) for k in ("dens", "acc_p", "vel_p", "vel_v")]


_lib = None


def build(quiet: bool = True) -> None:
    """Compile the restatement (make -C oracle oracle)."""
    out = subprocess.run(["make", "-s", "-C", str(HERE), "oracle"],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        L.sph_oracle_substep_f32.argtypes = [
            ctypes.POINTER(OracleParams), ctypes.c_uint32, _P, _P,
            ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.POINTER(DebugF32)]
        L.sph_oracle_substep_f64.argtypes = [
            ctypes.POINTER(OracleParams), ctypes.c_uint32, _P, _P,
            ctypes.c_double, ctypes.c_int, ctypes.POINTER(DebugF64)]
        L.sph_oracle_subset_f64.argtypes = [
            ctypes.POINTER(OracleParams), ctypes.c_uint32, _P, ctypes.c_uint32,
            _P, ctypes.c_int, _P, _P, _P, _P, _P]
        L.sph_oracle_subset_visc_f64.argtypes = [
            ctypes.POINTER(OracleParams), ctypes.c_uint32, _P, _P, ctypes.c_uint32, _P,
            ctypes.c_double, ctypes.c_int, _P, _P, _P]
        L.sph_oracle_hw_threads.restype = ctypes.c_int
        L.sph_oracle_speed_normalized.argtypes = [_P, ctypes.c_uint32, _P]
        L.sph_oracle_render.argtypes = [_P, _P, ctypes.c_uint32, _P, _P, ctypes.c_uint32,
                                        ctypes.c_uint32, ctypes.c_float, _P, _P, _P]
        _lib = L
    return _lib


def make_params(p) -> OracleParams:
    """OracleParams from a fluidsim.scenes.SimParams-like object."""
    o = OracleParams()
    o.radius = p.radius
    o.cutoff_sq = p.cutoff_sq
    o.target_density = p.target_density
    o.pressure_mult = p.pressure_mult
    o.near_pressure_mult = p.near_pressure_mult
    o.viscosity = p.viscosity
    o.gravity_scale = p.gravity_scale
    o.gravity_on = 1 if p.gravity_on else 0
    for a in range(3):
        o.bound[a] = p.bound[a]
    o.damping = p.damping
    o.predict_dt = p.predict_dt
    return o


def _ptr(a):
    return None if a is None else a.ctypes.data


def substep_f32(params, pos, vel, dt, gauss_seidel=False, nthreads=0,
                debug=True):
    """One FP32 substep. Returns (pos, vel, dbg dict) with pos/vel updated
    copies; dbg holds per-particle intermediates when debug is True."""
    pos = np.ascontiguousarray(pos, dtype=np.float32).copy()
    vel = np.ascontiguousarray(vel, dtype=np.float32).copy()
    n = pos.shape[0]
    d = {}
    dbg = DebugF32()
    if debug:
        d = dict(hash=np.empty(n, np.uint32), key=np.empty(n, np.uint32),
                 sorted_ids=np.empty(n, np.uint32), start=np.empty(n, np.uint32),
                 pred=np.empty((n, 3), np.float32), dens=np.empty((n, 2), np.float32),
                 acc_p=np.empty((n, 3), np.float32), vel_p=np.empty((n, 3), np.float32),
                 vel_v=np.empty((n, 3), np.float32), abs_p=np.empty(n, np.float32),
                 abs_v=np.empty(n, np.float32))
        for k, v in d.items():
            setattr(dbg, k, v.ctypes.data)
    prm = make_params(params)
    rc = lib().sph_oracle_substep_f32(ctypes.byref(prm), n, pos.ctypes.data,
                                      vel.ctypes.data, np.float32(dt),
                                      1 if gauss_seidel else 0, nthreads,
                                      ctypes.byref(dbg))
    if rc != 0:
        raise ValueError(f"oracle substep failed: {rc}")
    return pos, vel, d


def substep_f64(params, pos, vel, dt, nthreads=0):
    pos = np.ascontiguousarray(pos, dtype=np.float64).copy()
    vel = np.ascontiguousarray(vel, dtype=np.float64).copy()
    n = pos.shape[0]
    d = dict(dens=np.empty((n, 2)), acc_p=np.empty((n, 3)),
             vel_p=np.empty((n, 3)), vel_v=np.empty((n, 3)))
    dbg = DebugF64()
    for k, v in d.items():
        setattr(dbg, k, v.ctypes.data)
    prm = make_params(params)
    rc = lib().sph_oracle_substep_f64(ctypes.byref(prm), n, pos.ctypes.data,
                                      vel.ctypes.data, float(dt), nthreads,
                                      ctypes.byref(dbg))
    if rc != 0:
        raise ValueError(f"oracle f64 substep failed: {rc}")
    return pos, vel, d


def subset_f64(params, pred, subset, nthreads=0, with_abs=False):
    pred = np.ascontiguousarray(pred, dtype=np.float32)
    subset = np.ascontiguousarray(subset, dtype=np.uint32)
    m = subset.shape[0]
    dens = np.empty((m, 2))
    acc = np.empty((m, 3))
    absp = np.empty(m)
    sens = np.empty(m)
    dsens = np.empty(m)
    prm = make_params(params)
    rc = lib().sph_oracle_subset_f64(ctypes.byref(prm), pred.shape[0],
                                     pred.ctypes.data, m, subset.ctypes.data,
                                     nthreads, dens.ctypes.data, acc.ctypes.data,
                                     absp.ctypes.data, sens.ctypes.data,
                                     dsens.ctypes.data)
    if rc != 0:
        raise ValueError(f"oracle subset failed: {rc}")
    return (dens, acc, absp, sens, dsens) if with_abs else (dens, acc)


def subset_visc_f64(params, pred, velp, subset, dt, nthreads=0):
    """FP64 Jacobi viscosity velocity increment of the listed particles from
    FP32 predicted positions and post-pressure velocities (all n): returns
    (dv [m, 3], sum|terms| [m], sensitivity to the distance [m])."""
    pred = np.ascontiguousarray(pred, dtype=np.float32)
    velp = np.ascontiguousarray(velp, dtype=np.float32)
    subset = np.ascontiguousarray(subset, dtype=np.uint32)
    m = subset.shape[0]
    dv = np.empty((m, 3))
    absv = np.empty(m)
    dsens = np.empty(m)
    prm = make_params(params)
    rc = lib().sph_oracle_subset_visc_f64(ctypes.byref(prm), pred.shape[0], pred.ctypes.data,
                                          velp.ctypes.data, m, subset.ctypes.data,
                                          float(dt), nthreads, dv.ctypes.data,
                                          absv.ctypes.data, dsens.ctypes.data)
    if rc != 0:
        raise ValueError(f"oracle viscosity subset failed: {rc}")
    return dv, absv, dsens


def speed_normalized(vel):
    """The render restatement's speed normalisation of velocities [n, 3]."""
    vel = np.ascontiguousarray(vel, dtype=np.float32)
    out = np.empty(vel.shape[0], np.float32)
    if lib().sph_oracle_speed_normalized(vel.ctypes.data, vel.shape[0], out.ctypes.data) != 0:
        raise ValueError("oracle speed normalisation failed")
    return out


def hw_threads() -> int:
    return int(lib().sph_oracle_hw_threads())


# ---------------------------------------------------------------- reference
def ref_available() -> bool:
    return REF_DRIVER.exists()


def _write_input(path, params, pos, vel, dt, steps, flags):
    n = pos.shape[0]
    hdr = struct.pack("<4I11f", 0x49485053, n, steps, flags, params.radius,
                      params.target_density, params.pressure_mult,
                      params.near_pressure_mult, params.viscosity,
                      params.gravity_scale, 1.0 if params.gravity_on else 0.0,
                      params.bound[0], params.bound[1], params.bound[2],
                      float(np.float32(dt)))
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(np.ascontiguousarray(pos, np.float32).tobytes())
        f.write(np.ascontiguousarray(vel, np.float32).tobytes())


def ref_substep(params, pos, vel, dt, canonical=True):
    """Run one decomposed substep through the reference's own code."""
    if not ref_available():
        raise RuntimeError("reference driver not built (make -C oracle ref)")
    n = pos.shape[0]
    with tempfile.TemporaryDirectory() as td:
        fi, fo = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        _write_input(fi, params, pos, vel, dt, 1, 1 if canonical else 0)
        subprocess.run([str(REF_DRIVER), "substep", fi, fo], check=True)
        raw = open(fo, "rb").read()
    off = 0
    out = {}

    def take(name, dtype, shape):
        nonlocal off
        cnt = int(np.prod(shape))
        a = np.frombuffer(raw, dtype=dtype, count=cnt, offset=off).reshape(shape)
        off += cnt * np.dtype(dtype).itemsize
        out[name] = a.copy()

    for k in ("hash", "key", "start", "lookup_id"):
        take(k, np.uint32, (n,))
    take("lookup_raw", np.float32, (n, 3))
    take("pred", np.float32, (n, 3))
    take("dens", np.float32, (n, 2))
    for k in ("acc_p", "vel_p", "vel_v", "pos", "vel"):
        take(k, np.float32, (n, 3))
    assert off == len(raw)
    return out


def ref_update(params, pos, vel, dt, steps):
    """`steps` calls of the reference's Update(dt). Returns pos, vel, dens,
    per-call ms and the last call's six phase timers."""
    if not ref_available():
        raise RuntimeError("reference driver not built (make -C oracle ref)")
    n = pos.shape[0]
    with tempfile.TemporaryDirectory() as td:
        fi, fo = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        _write_input(fi, params, pos, vel, dt, steps, 0)
        subprocess.run([str(REF_DRIVER), "update", fi, fo], check=True)
        raw = open(fo, "rb").read()
    o = 0
    posF = np.frombuffer(raw, np.float32, 3 * n, o).reshape(n, 3).copy(); o += 12 * n
    velF = np.frombuffer(raw, np.float32, 3 * n, o).reshape(n, 3).copy(); o += 12 * n
    dens = np.frombuffer(raw, np.float32, 2 * n, o).reshape(n, 2).copy(); o += 8 * n
    ms = np.frombuffer(raw, np.float64, steps, o).copy(); o += 8 * steps
    phase = np.frombuffer(raw, np.float64, 6, o).copy()
    return posF, velF, dens, ms, phase


def _ref_run(mode, params, pos, vel, dt=0.0, steps=1):
    n = pos.shape[0]
    with tempfile.TemporaryDirectory() as td:
        fi, fo = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        _write_input(fi, params, pos, vel, dt, steps, 0)
        subprocess.run([str(REF_DRIVER), mode, fi, fo], check=True)
        return open(fo, "rb").read()


def ref_init(params, n):
    """The reference's own InitializeData(n) lattice: (positions [n, 3],
    OutPositions.w [n])."""
    if not ref_available():
        raise RuntimeError("reference driver not built (make -C oracle ref)")
    z = np.zeros((n, 3), np.float32)
    raw = _ref_run("init", params, z, z)
    pos = np.frombuffer(raw, np.float32, 3 * n, 0).reshape(n, 3).copy()
    w = np.frombuffer(raw, np.float32, n, 12 * n).copy()
    return pos, w


def ref_speed(params, vel):
    """The reference's getSpeed / getSpeedNormalzied for velocities `vel`
    [n, 3] at indices 0..n (index n is out of range): two float32 [n + 1]."""
    if not ref_available():
        raise RuntimeError("reference driver not built (make -C oracle ref)")
    n = vel.shape[0]
    raw = _ref_run("speed", params, np.zeros((n, 3), np.float32), vel)
    sp = np.frombuffer(raw, np.float32, n + 1, 0).copy()
    nrm = np.frombuffer(raw, np.float32, n + 1, 4 * (n + 1)).copy()
    return sp, nrm


def render(pos, vel, view):
    """The frame sph_render draws, on the CPU: pos/vel (n, 3) in caller
    order, `view` a fluidsim.render View. Returns (rgba [H, W, 4] uint8,
    depth [H, W] float32)."""
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    vel = np.ascontiguousarray(vel, dtype=np.float32)
    vp = np.array(list(view.view_proj), np.float32)
    pr = np.array(list(view.proj), np.float32)
    clear = np.array(list(view.clear), np.float32)
    rgba = np.empty((view.height, view.width, 4), np.uint8)
    depth = np.empty((view.height, view.width), np.float32)
    rc = lib().sph_oracle_render(_ptr(pos), _ptr(vel), pos.shape[0], _ptr(vp), _ptr(pr),
                                 view.width, view.height, float(view.scale), _ptr(clear),
                                 _ptr(rgba), _ptr(depth))
    if rc != 0:
        raise ValueError(f"oracle render failed: {rc}")
    return rgba, depth
