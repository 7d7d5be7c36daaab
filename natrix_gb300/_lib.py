"""ctypes binding of libnatrix_gb300.so (the C ABI declared in include/natrix.h).

The library is built in-tree by ``natrix_gb300.build`` (or
``__graft_entry__.build()``).  There is no fallback: if the library is missing
or cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libnatrix_gb300.so"

NATRIX_OK = 0
NATRIX_EINVAL = -1
NATRIX_ECUDA = -2
NATRIX_ENOMEM = -3
NATRIX_EDEVICE = -4
NATRIX_ERANGE = -5

FIELD_VELOCITY = 0
FIELD_PRESSURE = 1
FIELD_DIVERGENCE = 2
FIELD_VORTICITY = 3
FIELD_OBSTACLES = 4
FIELD_DENSITY = 5

SPLAT_FLOATS = 6


class NatrixError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"natrix error {code}: {message}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [("speed", ctypes.c_float), ("iterations", ctypes.c_int32),
                ("dissipation", ctypes.c_float), ("vorticity", ctypes.c_float),
                ("viscosity", ctypes.c_float), ("has_borders", ctypes.c_int32),
                ("simulate", ctypes.c_int32), ("sweeps_per_launch", ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [("kernel_launches", ctypes.c_int64), ("jacobi_launches", ctypes.c_int64),
                ("jacobi_sweeps", ctypes.c_int64), ("timed_phases", ctypes.c_int64),
                ("timed_launches", ctypes.c_int64), ("timed_sweeps", ctypes.c_int64),
                ("jacobi_ms", ctypes.c_double),
                ("timed_fused", ctypes.c_int64)]


_vp = ctypes.c_void_p
_f = ctypes.c_float
_i = ctypes.c_int32
_i64p = ctypes.POINTER(ctypes.c_int64)
_vpp = ctypes.POINTER(ctypes.c_void_p)

# name -> argtypes (restype int unless listed in _RESTYPES)
SIGNATURES = {
    "natrix_create": [_i, _i, _vpp],
    "natrix_destroy": [_vp],
    "natrix_set_params": [_vp, ctypes.POINTER(Params)],
    "natrix_get_params": [_vp, ctypes.POINTER(Params)],
    "natrix_add_velocity": [_vp, _f, _f, _f, _f, _f],
    "natrix_add_circle_obstacle": [_vp, _f, _f, _f, _i],
    "natrix_add_triangle_obstacle": [_vp, _f, _f, _f, _f, _f, _f, _i],
    "natrix_add_splats": [_vp, _vp, _vp, _i],
    "natrix_step": [_vp, _f, _vp],
    "natrix_field": [_vp, _i, _vpp, _i64p],
    "natrix_upload": [_vp, _i, _vp, _vp],
    "natrix_download": [_vp, _i, _vp, _vp],
    "natrix_residual": [_vp, ctypes.POINTER(ctypes.c_double), _vp],
    "natrix_jacobi": [_vp, _i, _vp],
    "natrix_residual_regions": [_vp, _vp, _i, _vp, _vp],
    "natrix_sync": [_vp, _vp],
    "natrix_inject_status": [_vp, _i, _vp],
    "natrix_set_timing": [_vp, _i],
    "natrix_get_stats": [_vp, ctypes.POINTER(Stats), _i],
    "natrix_density_create": [_vp, _i, _i, _vpp],
    "natrix_density_destroy": [_vp],
    "natrix_density_set_params": [_vp, _f, _f, _i],
    "natrix_density_add": [_vp, _f, _f, _f, _f],
    "natrix_density_step": [_vp, _f, _vp],
    "natrix_density_field": [_vp, _vpp, _i64p],
    "natrix_density_upload": [_vp, _vp, _vp],
    "natrix_density_download": [_vp, _vp, _vp],
    "natrix_particles_create": [_vp, ctypes.c_int64, _vpp],
    "natrix_particles_destroy": [_vp],
    "natrix_particles_upload": [_vp, _vp, _vp],
    "natrix_particles_download": [_vp, _vp, _vp],
    "natrix_particles_step": [_vp, _f, _i, _vp],
    "natrix_particles_cells": [_vp, _vp, _vp],
    "natrix_particles_field": [_vp, _vpp, _vpp, _i64p],
    "natrix_batch_create": [_i, _vp, _vp, _vpp],
    "natrix_batch_destroy": [_vp],
    "natrix_batch_set_params": [_vp, _i, ctypes.POINTER(Params)],
    "natrix_batch_set_density_params": [_vp, _i, _f, _f],
    "natrix_batch_set_tuning": [_vp, _i, _i, _i],
    "natrix_batch_set_graph": [_vp, _i],
    "natrix_batch_set_persistent": [_vp, _i],
    "natrix_batch_add_velocity": [_vp, _i, _f, _f, _f, _f, _f],
    "natrix_batch_add_splats": [_vp, _i, _vp, _i],
    "natrix_batch_add_circle_obstacle": [_vp, _i, _f, _f, _f, _i],
    "natrix_batch_add_splats_bulk": [_vp, _vp, _vp],
    "natrix_batch_add_circles_bulk": [_vp, _vp, _vp],
    "natrix_batch_step": [_vp, _f, _vp],
    "natrix_batch_field": [_vp, _i, _i, _vpp, _i64p],
    "natrix_batch_download": [_vp, _i, _i, _vp, _vp],
    "natrix_batch_launches": [_vp, _i64p, ctypes.POINTER(ctypes.c_int32)],
    "natrix_batch_sync": [_vp, _vp],
    "natrix_residual_noalloc": [_vp, _vp, _vp, _i, _i, ctypes.c_int64, _vp, _vp],
    "natrix_render_density": [_vp, _i, _i, ctypes.c_int64, _vp, _vp, ctypes.c_int64, _vp],
    "natrix_quiver_tiles": [_i, _i, _f, ctypes.POINTER(ctypes.c_int32),
                            ctypes.POINTER(ctypes.c_int32)],
    "natrix_quiver": [_vp, _i, _i, ctypes.c_int64, _i, _i, _f, _vp, _vp, ctypes.c_int64, _vp],
    "natrix_last_error": [],
    "natrix_version": [],
}
_RESTYPES = {"natrix_last_error": ctypes.c_char_p, "natrix_version": ctypes.c_char_p}

_lib = None


def load() -> ctypes.CDLL:
    """Load the library (once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m natrix_gb300.build` "
                "(or __graft_entry__.build()); there is no CPU fallback")
        lib = ctypes.CDLL(str(LIB_PATH))
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        _lib = lib
    return _lib


def check(rc: int) -> None:
    if rc != NATRIX_OK:
        msg = load().natrix_last_error().decode(errors="replace")
        if rc == NATRIX_EINVAL:
            raise ValueError(msg)
        raise NatrixError(rc, msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))
