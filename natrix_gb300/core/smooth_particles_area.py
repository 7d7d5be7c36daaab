"""Drop-in ``SmoothParticlesArea`` (demo/smooth_particles_area.py:15-211) on GB300.

A density grid of its own size, advected semi-Lagrangianly by the fluid's
velocity (demo/shaders/shader.AdvectParticle.comp) and fed by cone splats
(demo/shaders/shader.AddParticle.comp).  The bgfx ``vertex_layout`` argument
is accepted and ignored.
"""
from __future__ import annotations

import ctypes
import weakref
from typing import Optional

import numpy as np
import torch

from .._lib import call
from .fluid_simulator import FluidSimulator, _stream, _view


class SmoothParticlesArea:
    PARTICLES_IN = 0
    PARTICLES_OUT = 1

    _width = 512
    _height = 512

    _speed = 500.0
    _dissipation = 1.0

    simulate = True

    def __init__(self, width: int, height: int, fluid_simulation: FluidSimulator,
                 vertex_layout=None):
        self.fluid_simulation = fluid_simulation
        self.vertex_layout = vertex_layout
        self._width = int(width)
        self._height = int(height)
        self._handle = ctypes.c_void_p()
        call("natrix_density_create", fluid_simulation.handle, self._width, self._height,
             ctypes.byref(self._handle))
        self._pushed: Optional[tuple] = None
        fluid_simulation._density_grids.append(weakref.ref(self))

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
    def dissipation(self):
        return self._dissipation

    @dissipation.setter
    def dissipation(self, value):
        if value > 0:
            self._dissipation = value
        else:
            raise ValueError("'Dissipation' should be grater than zero")

    @property
    def handle(self) -> ctypes.c_void_p:
        if not self._handle:
            raise RuntimeError("density grid has been destroyed")
        return self._handle

    def _sync_params(self) -> None:
        key = (self._speed, self._dissipation, self.simulate)
        if key != self._pushed:
            call("natrix_density_set_params", self.handle, float(key[0]), float(key[1]),
                 int(bool(key[2])))
            self._pushed = key

    def add_particles(self, position: tuple, radius: float, strength: float):
        if self.simulate:
            self._sync_params()
            call("natrix_density_add", self.handle, position[0], position[1], radius, strength)

    def update(self, time_delta: float):
        if self.simulate:
            self._sync_params()
            self.fluid_simulation._sync_params()
            call("natrix_density_step", self.handle, time_delta, _stream())

    def get_particles_buffer(self) -> torch.Tensor:
        """Density (H, W) float32 CUDA view of the current buffer."""
        ptr = ctypes.c_void_p()
        pitch = ctypes.c_int64()
        self._sync_params()
        call("natrix_density_field", self.handle, ctypes.byref(ptr), ctypes.byref(pitch))
        return _view(ptr.value, pitch.value, self._height, self._width, "float")

    @property
    def density(self) -> torch.Tensor:
        return self.get_particles_buffer()

    def download(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.empty((self._height, self._width), np.float32)
        call("natrix_density_download", self.handle, out.ctypes.data_as(ctypes.c_void_p),
             _stream())
        torch.cuda.current_stream().synchronize()
        return out

    def upload(self, host: np.ndarray) -> None:
        arr = np.ascontiguousarray(host, dtype=np.float32)
        call("natrix_density_upload", self.handle, arr.ctypes.data_as(ctypes.c_void_p),
             _stream())
        torch.cuda.current_stream().synchronize()

    def destroy(self):
        if self._handle:
            call("natrix_density_destroy", self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
