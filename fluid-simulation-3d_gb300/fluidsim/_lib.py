"""ctypes binding of libsph_gb300.so (the C ABI in include/sph_gb300.h).

There is no fallback: if the library is missing or no CUDA device is usable
the calls raise.
"""
from __future__ import annotations

import ctypes
import pathlib

PKG = pathlib.Path(__file__).resolve().parent.parent
LIB_PATH = PKG / "_build" / "libsph_gb300.so"

SPH_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of memory",
          -4: "invalid state", -5: "device status"}
STATUS_NONFINITE = 0x1
STATUS_RANGE = 0x2

# Every entry point declared in include/sph_gb300.h.
EXPORTS = (
    "sph_default_params", "sph_create", "sph_destroy", "sph_set_params",
    "sph_get_params", "sph_num_particles", "sph_upload", "sph_step",
    "sph_download", "sph_out_positions", "sph_upload_device",
    "sph_download_device", "sph_debug_enable", "sph_debug_export",
    "sph_debug_export_layout",
    "sph_status", "sph_last_error", "sph_global_error", "sph_batch_create",
    "sph_batch_destroy", "sph_batch_add", "sph_batch_remove", "sph_batch_step",
    "sph_batch_download", "sph_batch_set_tuning", "sph_batch_get_tuning",
    "sph_batch_autotune", "sph_batch_num_scenes", "sph_batch_num_particles",
    "sph_batch_last_error", "sph_profile_enable", "sph_phase_times",
    "sph_kernel_launches", "sph_batch_kernel_launches",
    "sph_batch_profile_enable", "sph_batch_phase_times", "sph_set_tuning",
    "sph_get_tuning", "sph_autotune", "sph_spatial_lookup_static",
    "sph_static_error", "sph_bytes_per_particle", "sph_batch_sync", "sph_batch_status",
    "sph_render", "sph_batch_render", "sph_save", "sph_load", "sph_batch_save",
    "sph_batch_add_snapshot", "sph_server_create", "sph_server_destroy",
    "sph_server_submit", "sph_server_cancel", "sph_server_wait", "sph_server_get_stats",
    "sph_server_last_error",
)
STATIC_LOOKUP_MAX = 65536


class Params(ctypes.Structure):
    """struct sph_params."""
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


class Tuning(ctypes.Structure):
    """struct sph_tuning."""
    _fields_ = [("block", ctypes.c_int32), ("cell_tile", ctypes.c_int32),
                ("particles_per_warp", ctypes.c_int32), ("gather", ctypes.c_int32),
                ("force_block", ctypes.c_int32), ("table", ctypes.c_int32)]


class View(ctypes.Structure):
    """struct sph_view."""
    _fields_ = [("view_proj", ctypes.c_float * 16), ("proj", ctypes.c_float * 16),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("scale", ctypes.c_float), ("clear", ctypes.c_float * 4)]


class ServerStats(ctypes.Structure):
    """struct sph_server_stats."""
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("cancelled", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("queued", ctypes.c_uint32), ("resident", ctypes.c_uint32),
                ("steps", ctypes.c_uint64), ("particle_steps", ctypes.c_uint64),
                ("capacity_particles", ctypes.c_uint64), ("wall_s", ctypes.c_double),
                ("particle_steps_per_s", ctypes.c_double),
                ("p50_step_ms", ctypes.c_double), ("p99_step_ms", ctypes.c_double),
                ("step_s", ctypes.c_double), ("admit_s", ctypes.c_double),
                ("retire_s", ctypes.c_double), ("status_flags", ctypes.c_uint32)]


_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_lib = None


def _sig(L):
    i, u32, u64, f = ctypes.c_int, _U32, ctypes.c_uint64, ctypes.c_float
    pp = ctypes.POINTER(Params)
    sigs = {
        "sph_default_params": (None, [pp]),
        "sph_create": (i, [pp, u32, ctypes.POINTER(_P)]),
        "sph_destroy": (i, [_P]),
        "sph_set_params": (i, [_P, pp]),
        "sph_get_params": (i, [_P, pp]),
        "sph_num_particles": (u32, [_P]),
        "sph_upload": (i, [_P, _P, _P, _P]),
        "sph_upload_device": (i, [_P, _P, _P, _P]),
        "sph_step": (i, [_P, f, i, _P]),
        "sph_download": (i, [_P, _P, _P, _P, _P]),
        "sph_download_device": (i, [_P, _P, _P, _P, _P]),
        "sph_out_positions": (i, [_P, ctypes.POINTER(_P)]),
        "sph_render": (i, [_P, ctypes.POINTER(View), _P, _P, _P]),
        "sph_batch_render": (i, [_P, u32, ctypes.POINTER(View), _P, _P, _P]),
        "sph_server_create": (i, [u64, u32, i, ctypes.POINTER(_P)]),
        "sph_server_destroy": (i, [_P]),
        "sph_server_submit": (i, [_P, pp, u32, _P, _P, f, u32, ctypes.POINTER(u64)]),
        "sph_server_cancel": (i, [_P, u64]),
        "sph_server_wait": (i, [_P, u64, _P, _P, _P, ctypes.c_double]),
        "sph_server_get_stats": (i, [_P, ctypes.POINTER(ServerStats)]),
        "sph_server_last_error": (ctypes.c_char_p, [_P]),
        "sph_save": (i, [_P, ctypes.c_char_p, _P]),
        "sph_load": (i, [_P, ctypes.c_char_p, _P]),
        "sph_batch_save": (i, [_P, u32, ctypes.c_char_p, _P]),
        "sph_batch_add_snapshot": (i, [_P, ctypes.c_char_p, ctypes.POINTER(u32), _P]),
        "sph_debug_enable": (i, [_P, i]),
        "sph_debug_export": (i, [_P] + [_P] * 8 + [_P]),
        "sph_debug_export_layout": (i, [_P, _P, _P, _P, _P, u64, ctypes.POINTER(u32),
                                        ctypes.POINTER(i), _P]),
        "sph_status": (i, [_P, ctypes.POINTER(u32), _P]),
        "sph_last_error": (ctypes.c_char_p, [_P]),
        "sph_global_error": (ctypes.c_char_p, []),
        "sph_batch_create": (i, [u64, u32, ctypes.POINTER(_P)]),
        "sph_batch_destroy": (i, [_P]),
        "sph_batch_add": (i, [_P, pp, u32, _P, _P, f, ctypes.POINTER(u32), _P]),
        "sph_batch_remove": (i, [_P, u32]),
        "sph_batch_step": (i, [_P, i, _P]),
        "sph_batch_download": (i, [_P, u32, _P, _P, _P, _P]),
        "sph_batch_set_tuning": (i, [_P, ctypes.POINTER(Tuning)]),
        "sph_batch_get_tuning": (i, [_P, ctypes.POINTER(Tuning)]),
        "sph_batch_autotune": (i, [_P, i, i, ctypes.POINTER(Tuning),
                                   ctypes.POINTER(f), _P]),
        "sph_batch_num_scenes": (u32, [_P]),
        "sph_batch_num_particles": (u64, [_P]),
        "sph_batch_last_error": (ctypes.c_char_p, [_P]),
        "sph_profile_enable": (i, [_P, i]),
        "sph_phase_times": (i, [_P, ctypes.POINTER(ctypes.c_double)]),
        "sph_kernel_launches": (u64, [_P]),
        "sph_batch_kernel_launches": (u64, [_P]),
        "sph_batch_profile_enable": (i, [_P, i]),
        "sph_batch_phase_times": (i, [_P, ctypes.POINTER(ctypes.c_double)]),
        "sph_set_tuning": (i, [_P, ctypes.POINTER(Tuning)]),
        "sph_get_tuning": (i, [_P, ctypes.POINTER(Tuning)]),
        "sph_autotune": (i, [_P, f, i, i, ctypes.POINTER(Tuning),
                             ctypes.POINTER(f), _P]),
        "sph_spatial_lookup_static": (i, [_P, u32, f, _P, _P, _P, _P, _P]),
        "sph_static_error": (ctypes.c_char_p, []),
        "sph_bytes_per_particle": (u64, []),
        "sph_batch_sync": (i, [_P, _P]),
        "sph_batch_status": (i, [_P, ctypes.POINTER(u32), _P]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def load():
    """Load the in-tree library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with build_lib.build() "
                "(there is no CPU fallback)")
        L = ctypes.CDLL(str(LIB_PATH))
        _sig(L)
        _lib = L
    return _lib


class SphError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def check(rc, handle=None, batch=False):
    if rc == SPH_OK:
        return
    L = load()
    if handle is None:
        msg = L.sph_global_error()
    elif batch:
        msg = L.sph_batch_last_error(handle)
    else:
        msg = L.sph_last_error(handle)
    raise SphError(rc, (msg or b"").decode(errors="replace"))
