"""Drop-in ``FluidSimulator`` (natrix/core/fluid_simulator.py:15-515) on GB300.

Same constructor, properties, validation messages, flags and methods as the
reference; the fields live in device memory owned by libnatrix_gb300 and every
call goes through the C ABI (include/natrix.h) on torch's current CUDA stream.
The bgfx ``vertex_layout`` argument is accepted and ignored.

Differences a user can observe:
* ``get_velocity_buffer()`` returns a torch CUDA tensor view (H, W, 2) of the
  current velocity instead of a bgfx buffer handle; re-fetch it after each
  ``update`` (the view always points at the live state buffer).
* ``add_*`` calls are queued and applied by one fused kernel before the next
  step or field access (same results as applying them one by one).
* Extensions with no reference counterpart: ``add_density`` (the density cone
  splat on the attached density grids), ``add_splats`` (Gaussian splat
  forcing), ``residual``, ``jacobi``, field accessors and host copies.
"""
from __future__ import annotations

import ctypes
import weakref
from typing import Optional

import numpy as np
import torch

from .. import _lib
from .._lib import Params, call, load


class _DeviceArray:
    """Minimal ``__cuda_array_interface__`` holder for a pitched device field."""

    def __init__(self, ptr: int, shape, typestr: str, strides):
        self.__cuda_array_interface__ = {
            "shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
            "strides": tuple(strides), "version": 3,
        }


def _view(ptr: int, pitch: int, height: int, width: int, kind: str) -> torch.Tensor:
    if kind == "float2":
        arr = _DeviceArray(ptr, (height, width, 2), "<f4", (pitch * 8, 8, 4))
    elif kind == "float":
        arr = _DeviceArray(ptr, (height, width), "<f4", (pitch * 4, 4))
    else:
        arr = _DeviceArray(ptr, (height, width), "|u1", (pitch, 1))
    return torch.as_tensor(arr, device="cuda")


# The current stream's raw handle without building a torch.cuda.Stream object
# (a step calls this every frame; torch keeps the accessor in its C module)
_raw_stream = getattr(torch._C, "_cuda_getCurrentRawStream", None)


def _stream() -> ctypes.c_void_p:
    if _raw_stream is not None:
        return ctypes.c_void_p(_raw_stream(torch.cuda.current_device()))
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class FluidSimulator:
    VELOCITY_READ = 0
    VELOCITY_WRITE = 1

    PRESSURE_READ = 0
    PRESSURE_WRITE = 1

    _width = 512
    _height = 512

    # defaults, natrix/core/fluid_simulator.py:28-32
    _speed = 500.0
    _iterations = 50
    _dissipation = 1.0
    _vorticity = 0.0
    _viscosity = 0.1

    has_borders = True
    simulate = True

    # Jacobi sweeps fused per launch (temporal blocking); 0 = library default
    sweeps_per_launch = 0

    def __init__(self, width: int, height: int, vertex_layout=None):
        torch.cuda.init()
        self._width = int(width)
        self._height = int(height)
        self.vertex_layout = vertex_layout
        self._handle = ctypes.c_void_p()
        call("natrix_create", self._width, self._height, ctypes.byref(self._handle))
        self._pushed: Optional[tuple] = None
        # density grids advected by this simulator (SmoothParticlesArea
        # registers itself here); add_density splats into them
        self._density_grids: list = []

    # ------------------------------------------------------------ properties
    @property
    def width(self):
        return self._width

    @property
    def height(self):
        return self._height

    @property
    def speed(self):
        return self._speed

    @speed.setter
    def speed(self, value):
        if value > 0:
            self._speed = value
        else:
            raise ValueError("'Speed' should be greater than zero")

    @property
    def iterations(self):
        return self._iterations

    @iterations.setter
    def iterations(self, value):
        if value > 0:
            self._iterations = value
        else:
            raise ValueError("'Iterations' should be grater than zero")

    @property
    def dissipation(self):
        return self._dissipation

    @dissipation.setter
    def dissipation(self, value):
        if value > 0:
            self._dissipation = value
        else:
            raise ValueError("'Dissipation' should be grater than zero")

    @property
    def vorticity(self):
        return self._vorticity

    @vorticity.setter
    def vorticity(self, value):
        if value >= 0:
            self._vorticity = value
        else:
            raise ValueError("'Vorticity' should be grater or equal than zero")

    @property
    def viscosity(self):
        return self._viscosity

    @viscosity.setter
    def viscosity(self, value):
        if value >= 0.0:
            self._viscosity = value
        else:
            raise ValueError("'Viscosity' should be greater or equal than zero")

    # --------------------------------------------------------------- helpers
    @property
    def handle(self) -> ctypes.c_void_p:
        if not self._handle:
            raise RuntimeError("simulator has been destroyed")
        return self._handle

    def _sync_params(self) -> None:
        # compared as given (the frame's common case is "unchanged"), converted
        # only when pushed
        key = (self._speed, self._iterations, self._dissipation, self._vorticity,
               self._viscosity, self.has_borders, self.simulate, self.sweeps_per_launch)
        if key != self._pushed:
            p = Params(float(key[0]), int(key[1]), float(key[2]), float(key[3]), float(key[4]),
                       int(bool(key[5])), int(bool(key[6])), int(key[7]))
            call("natrix_set_params", self.handle, ctypes.byref(p))
            self._pushed = key

    def _field(self, field: int):
        ptr = ctypes.c_void_p()
        pitch = ctypes.c_int64()
        self._sync_params()
        call("natrix_field", self.handle, field, ctypes.byref(ptr), ctypes.byref(pitch))
        return ptr.value, pitch.value

    # ------------------------------------------------------------ reference API
    def get_velocity_buffer(self) -> torch.Tensor:
        """Velocity (H, W, 2) float32 CUDA view (stored units, clamped to [-1, 1])."""
        ptr, pitch = self._field(_lib.FIELD_VELOCITY)
        return _view(ptr, pitch, self._height, self._width, "float2")

    def add_velocity(self, position: tuple, velocity: tuple, radius: float):
        if self.simulate:
            self._sync_params()
            call("natrix_add_velocity", self.handle, position[0], position[1], velocity[0],
                 velocity[1], radius)

    # position in normalised local space, radius in cells
    def add_circle_obstacle(self, position: tuple, radius: float, static=False):
        if self.simulate:
            self._sync_params()
            call("natrix_add_circle_obstacle", self.handle, position[0], position[1], radius,
                 1 if static else 0)

    # points in normalised local space
    def add_triangle_obstacle(self, p1: tuple, p2: tuple, p3: tuple, static=False):
        if self.simulate:
            self._sync_params()
            call("natrix_add_triangle_obstacle", self.handle, p1[0], p1[1], p2[0], p2[1],
                 p3[0], p3[1], 1 if static else 0)

    def update(self, time_delta: float):
        if self.simulate:
            self._sync_params()
            call("natrix_step", self.handle, time_delta, _stream())

    def destroy(self):
        if self._handle:
            call("natrix_destroy", self._handle)
            self._handle = ctypes.c_void_p()

    # ------------------------------------------------------------- extensions
    step = update

    def density_grids(self) -> list:
        """Live density grids (SmoothParticlesArea) attached to this simulator."""
        live = [r() for r in self._density_grids]
        live = [d for d in live if d is not None and d._handle]
        self._density_grids = [weakref.ref(d) for d in live]
        return live

    def add_density(self, position: tuple, value: float, radius: float):
        """Cone splat of density (demo/shaders/shader.AddParticle.comp:18-36):
        cells within ``radius`` cells of ``position`` (normalised) gain
        ``value * (radius - d) / radius``, clamped to [0, 255].  Applied to
        every density grid attached to this simulator, in its own resolution
        (``SmoothParticlesArea.add_particles(position, radius, value)`` on
        each); raises RuntimeError when none is attached."""
        if not self.simulate:
            return
        grids = self.density_grids()
        if not grids:
            raise RuntimeError("add_density: no density grid (SmoothParticlesArea) is "
                               "attached to this simulator")
        for d in grids:
            d.add_particles(position, radius, value)

    def add_splats(self, splats, density=None):
        """Gaussian splats: (n, 6) float32 {px, py, radius_cells, vx, vy, density},
        applied to the velocity and, if given, to ``density`` (a SmoothParticlesArea)."""
        if not self.simulate:
            return
        arr = np.ascontiguousarray(splats, dtype=np.float32).reshape(-1, _lib.SPLAT_FLOATS)
        self._sync_params()
        dh = density.handle if density is not None else None
        call("natrix_add_splats", self.handle, dh, arr.ctypes.data,
             arr.shape[0])

    @property
    def velocity(self) -> torch.Tensor:
        return self.get_velocity_buffer()

    @property
    def pressure(self) -> torch.Tensor:
        ptr, pitch = self._field(_lib.FIELD_PRESSURE)
        return _view(ptr, pitch, self._height, self._width, "float")

    @property
    def divergence(self) -> torch.Tensor:
        ptr, pitch = self._field(_lib.FIELD_DIVERGENCE)
        return _view(ptr, pitch, self._height, self._width, "float")

    @property
    def vorticity_field(self) -> torch.Tensor:
        """Vorticity of the last step (computed only when ``vorticity`` > 0)."""
        ptr, pitch = self._field(_lib.FIELD_VORTICITY)
        return _view(ptr, pitch, self._height, self._width, "float")

    @property
    def obstacles(self) -> torch.Tensor:
        """uint8 mask: bit0 = obstacle, bit1 = static triangle (the reference's vec2)."""
        ptr, pitch = self._field(_lib.FIELD_OBSTACLES)
        return _view(ptr, pitch, self._height, self._width, "u8")

    def download(self, field: int, out: Optional[np.ndarray] = None) -> np.ndarray:
        """Copy a field to a dense host array (synchronises the current stream)."""
        shape = (self._height, self._width)
        dtype = np.uint8 if field == _lib.FIELD_OBSTACLES else np.float32
        if field == _lib.FIELD_VELOCITY:
            shape = shape + (2,)
        if out is None:
            out = np.empty(shape, dtype)
        self._sync_params()
        call("natrix_download", self.handle, field, out.ctypes.data_as(ctypes.c_void_p),
             _stream())
        torch.cuda.current_stream().synchronize()
        return out

    def upload(self, field: int, host: np.ndarray) -> None:
        dtype = np.uint8 if field == _lib.FIELD_OBSTACLES else np.float32
        arr = np.ascontiguousarray(host, dtype=dtype)
        self._sync_params()
        call("natrix_upload", self.handle, field, arr.ctypes.data_as(ctypes.c_void_p),
             _stream())
        torch.cuda.current_stream().synchronize()

    def residual_sums(self) -> np.ndarray:
        out = (ctypes.c_double * 5)()
        call("natrix_residual", self.handle, out, _stream())
        return np.array(out[:], np.float64)

    def residual(self) -> float:
        """||r - mean r|| / ||b - mean b|| over fluid cells of the last step's system."""
        n, sr, srr, sb, sbb = self.residual_sums()
        if n <= 0:
            return 0.0
        num = max(srr - sr * sr / n, 0.0)
        den = max(sbb - sb * sb / n, 0.0)
        return float(np.sqrt(num / den)) if den > 0 else 0.0

    def residual_regions(self, labels: torch.Tensor, n_labels: int) -> float:
        """Relative residual with the mean removed per connected fluid region
        (``labels``: int32 CUDA tensor H x W, region id per fluid cell, < 0 on
        obstacles; ``warmstart.Regions`` builds them)."""
        sums = torch.empty(n_labels, 5, dtype=torch.float64, device="cuda")
        call("natrix_residual_regions", self.handle, ctypes.c_void_p(labels.data_ptr()),
             int(n_labels), ctypes.c_void_p(sums.data_ptr()), _stream())
        s = sums.cpu().numpy()
        n = np.maximum(s[:, 0], 1.0)
        num = np.maximum(s[:, 2] - s[:, 1] ** 2 / n, 0.0).sum()
        den = np.maximum(s[:, 4] - s[:, 3] ** 2 / n, 0.0).sum()
        return float(np.sqrt(num / den)) if den > 0 else 0.0

    def jacobi(self, sweeps: int) -> None:
        """Run more Jacobi sweeps on the current pressure (no reset)."""
        self._sync_params()
        call("natrix_jacobi", self.handle, int(sweeps), _stream())

    def sync(self) -> None:
        call("natrix_sync", self.handle, _stream())

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def version() -> str:
    return load().natrix_version().decode()

