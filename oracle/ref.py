"""Bindings for the reference's own compute shaders compiled on the CPU
(oracle/_ref/libnatrix_ref.so, built by oracle/build_ref.sh from the
reference checkout) — TEST INFRASTRUCTURE ONLY.

The shaders keep the reference's buffer layouts: velocity, pressure and
obstacles are vec2 per cell, everything else is float per cell.  The helpers
here convert to and from the oracle's layouts (pressure scalar per cell,
obstacles as a uint8 bit mask) so tests can compare kernel by kernel.
``RefFluid`` / ``RefDensity`` replay the host order of
natrix/core/fluid_simulator.py:174-280 and demo/smooth_particles_area.py:70-104
with the shaders, buffer flips included.

The library exists only where the reference sources are present (this
container); on other machines ``available()`` is False and the golden
vectors in tests/golden/ stand in for it.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB = _HERE / "_ref" / "libnatrix_ref.so"
_lib = None


def build(reference_root: str | None = None) -> bool:
    """Compile the reference shaders with oracle/build_ref.sh (which locates the
    checkout: `reference_root`, else NATRIX_REFERENCE_ROOT, else its default)."""
    subprocess.run(["bash", str(_HERE / "build_ref.sh")] +
                   ([reference_root] if reference_root else []), check=True,
                   stdout=subprocess.DEVNULL)
    return _LIB.exists()


def available() -> bool:
    return _LIB.exists()


def lib():
    global _lib
    if _lib is None:
        if not _LIB.exists():
            raise FileNotFoundError(f"{_LIB} not built (reference sources absent)")
        _lib = ctypes.CDLL(str(_LIB))
    return _lib


def _p(a):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.c_void_p)


F = ctypes.c_float


def obs_to_vec2(mask: np.ndarray) -> np.ndarray:
    """uint8 bit mask (bit0 -> .x, bit1 -> .y) to the reference's vec2 buffer."""
    out = np.zeros(mask.shape + (2,), np.float32)
    out[..., 0] = (mask & 1).astype(np.float32)
    out[..., 1] = ((mask >> 1) & 1).astype(np.float32)
    return out


def vec2_to_obs(buf: np.ndarray) -> np.ndarray:
    return ((buf[..., 0] > 0).astype(np.uint8) | ((buf[..., 1] > 0).astype(np.uint8) << 1))


def scalar_to_vec2(p: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.repeat(p[..., None], 2, axis=-1), np.float32)


class RefFluid:
    """FluidSimulator's host order driving the compiled reference shaders."""

    def __init__(self, width: int, height: int):
        self.width, self.height = W, H = int(width), int(height)
        self.vel = [np.zeros((H, W, 2), np.float32) for _ in range(2)]
        self.prs = [np.zeros((H, W, 2), np.float32) for _ in range(2)]
        self.vr = 0
        self.pr = 0
        self.divergence = np.zeros((H, W), np.float32)
        self.vorticity_field = np.zeros((H, W), np.float32)
        self.obs = np.zeros((H, W, 2), np.float32)
        self.speed = 500.0
        self.iterations = 50
        self.dissipation = 1.0
        self.vorticity = 0.0
        self.viscosity = 0.1
        self.has_borders = True

    @property
    def velocity(self):
        return self.vel[self.vr]

    @property
    def pressure(self):
        return self.prs[self.pr][..., 0]

    @property
    def obstacles(self):
        return vec2_to_obs(self.obs)

    def add_velocity(self, position, velocity, radius):
        lib().ref_add_velocity(_p(self.vel[self.vr]), _p(self.vel[self.vr ^ 1]), self.width,
                               self.height, F(position[0]), F(position[1]), F(velocity[0]),
                               F(velocity[1]), F(radius))
        self.vr ^= 1

    def add_circle_obstacle(self, position, radius, static=False):
        lib().ref_add_circle_obstacle(_p(self.obs), self.width, self.height, F(position[0]),
                                      F(position[1]), F(radius), int(bool(static)))

    def add_triangle_obstacle(self, p1, p2, p3, static=False):
        lib().ref_add_triangle_obstacle(_p(self.obs), self.width, self.height, F(p1[0]),
                                        F(p1[1]), F(p2[0]), F(p2[1]), F(p3[0]), F(p3[1]),
                                        int(bool(static)))

    def update(self, dt: float):
        L, W, H = lib(), self.width, self.height
        if self.has_borders:
            L.ref_init_boundaries(_p(self.vel[self.vr]), W, H)
        L.ref_advect_velocity(_p(self.vel[self.vr]), _p(self.vel[self.vr ^ 1]), _p(self.obs),
                              W, H, F(dt), F(self.speed), F(self.dissipation))
        self.vr ^= 1
        L.ref_calc_vorticity(_p(self.vel[self.vr]), _p(self.vorticity_field), W, H)
        L.ref_apply_vorticity(_p(self.vel[self.vr]), _p(self.vel[self.vr ^ 1]),
                              _p(self.vorticity_field), W, H, F(dt), F(self.vorticity))
        self.vr ^= 1
        if self.viscosity > 0.0:
            alpha = 1.0 / self.viscosity
            rbeta = 1.0 / (4.0 + alpha)
            L.ref_viscosity(_p(self.vel[self.vr]), _p(self.vel[self.vr ^ 1]), W, H, F(alpha),
                            F(rbeta))
            self.vr ^= 1
        L.ref_divergence(_p(self.vel[self.vr]), _p(self.obs), _p(self.divergence), W, H)
        L.ref_clear_buffer(_p(self.prs[self.pr]), W, H)
        for _ in range(self.iterations):
            L.ref_poisson(_p(self.prs[self.pr]), _p(self.prs[self.pr ^ 1]),
                          _p(self.divergence), _p(self.obs), W, H)
            self.pr ^= 1
        L.ref_subtract_gradient(_p(self.vel[self.vr]), _p(self.vel[self.vr ^ 1]),
                                _p(self.prs[self.pr]), _p(self.obs), W, H)
        self.vr ^= 1
        L.ref_clear_buffer(_p(self.obs), W, H)


class RefDensity:
    """SmoothParticlesArea's host order driving the compiled demo shaders."""

    def __init__(self, width: int, height: int, fluid: RefFluid):
        self.width, self.height = int(width), int(height)
        self.fluid = fluid
        self.buf = [np.zeros((height, width), np.float32) for _ in range(2)]
        self.r = 0
        self.speed = 500.0
        self.dissipation = 1.0

    @property
    def field(self):
        return self.buf[self.r]

    def add_particles(self, position, radius, strength):
        # the reference launches ceil(W/16) groups in both dimensions
        gy = (self.width + 15) // 16
        # cells the dispatch does not reach keep the input value (instead of
        # the stale contents of the output buffer): copy first
        self.buf[self.r ^ 1][:] = self.buf[self.r]
        lib().ref_add_particle(_p(self.buf[self.r]), _p(self.buf[self.r ^ 1]), self.width,
                               self.height, F(position[0]), F(position[1]), F(radius),
                               F(strength), gy)
        self.r ^= 1

    def update(self, dt: float):
        f = self.fluid
        lib().ref_advect_particle(_p(self.buf[self.r]), _p(self.buf[self.r ^ 1]),
                                  _p(f.velocity), _p(f.obs), self.width, self.height,
                                  f.width, f.height, F(dt), F(self.speed),
                                  F(self.dissipation))
        self.r ^= 1
