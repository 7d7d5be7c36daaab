"""Lagrangian particles advected by a FluidSimulator's velocity field.

No reference counterpart (the reference's "particles" are the Eulerian
density grid of SmoothParticlesArea).  Positions are in cells (x, y);
each ``step`` moves every particle by RK2 (midpoint) with the solver's
bilinear velocity sampler and displacement ``v * dt * speed``, clamps it to
the grid, and splats unit mass into a density grid of the simulator's size
with a 3x3 normalised linear hat around the nearest cell centre.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .._lib import call
from .fluid_simulator import FluidSimulator, _stream, _view


class LagrangianParticles:
    def __init__(self, fluid: FluidSimulator, positions: np.ndarray):
        pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 2)
        self.fluid = fluid
        self.n = pos.shape[0]
        self._handle = ctypes.c_void_p()
        call("natrix_particles_create", fluid.handle, self.n, ctypes.byref(self._handle))
        self.upload(pos)

    @property
    def handle(self) -> ctypes.c_void_p:
        if not self._handle:
            raise RuntimeError("particles have been destroyed")
        return self._handle

    def step(self, dt: float, splat: bool = True) -> None:
        self.fluid._sync_params()
        call("natrix_particles_step", self.handle, dt, 1 if splat else 0, _stream())

    def _ptrs(self):
        pos, rho = ctypes.c_void_p(), ctypes.c_void_p()
        pitch = ctypes.c_int64()
        call("natrix_particles_field", self.handle, ctypes.byref(pos), ctypes.byref(rho),
             ctypes.byref(pitch))
        return pos.value, rho.value, pitch.value

    @property
    def density(self) -> torch.Tensor:
        _, rho, pitch = self._ptrs()
        return _view(rho, pitch, self.fluid.height, self.fluid.width, "float")

    def upload(self, positions: np.ndarray) -> None:
        pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(self.n, 2)
        call("natrix_particles_upload", self.handle, pos.ctypes.data_as(ctypes.c_void_p),
             _stream())
        torch.cuda.current_stream().synchronize()

    def download(self) -> np.ndarray:
        out = np.empty((self.n, 2), np.float32)
        call("natrix_particles_download", self.handle, out.ctypes.data_as(ctypes.c_void_p),
             _stream())
        torch.cuda.current_stream().synchronize()
        return out

    def cells(self) -> np.ndarray:
        out = np.empty((self.n, 2), np.int32)
        call("natrix_particles_cells", self.handle, out.ctypes.data_as(ctypes.c_void_p),
             _stream())
        torch.cuda.current_stream().synchronize()
        return out

    def destroy(self) -> None:
        if self._handle:
            call("natrix_particles_destroy", self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
