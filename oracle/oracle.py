"""CPU oracle of the per-step fluid solver — TEST INFRASTRUCTURE ONLY.

Python side of oracle/oracle.c: ctypes bindings for every kernel and two
classes that replay the reference's host orchestration on numpy arrays:

* ``OracleFluid`` follows ``FluidSimulator.update``
  (natrix/core/fluid_simulator.py:174-280, buffer flips :444-474, uniforms
  :315-336) and the mutating calls ``add_velocity`` (:116-131),
  ``add_circle_obstacle`` (:135-153), ``add_triangle_obstacle`` (:156-172);
* ``OracleDensity`` follows ``SmoothParticlesArea`` (demo/smooth_particles_area.py:
  ``add_particles`` :70-83, ``update`` :85-104).

``dtype`` float32 reproduces the shader arithmetic; float64 is the ground
truth.  Uniforms are rounded to float32 first in both cases, as the reference
passes them through ``c_float``.  Only the tests, ``__graft_entry__.smoke()``
and bench.py's CPU-baseline leg use this module, as the checker.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB_PATH = _HERE / "_build" / "liboracle.so"
_lib = None

_u8p = ctypes.POINTER(ctypes.c_uint8)
_i32p = ctypes.POINTER(ctypes.c_int32)
_dblp = ctypes.POINTER(ctypes.c_double)


def build(force: bool = False) -> Path:
    """Compile oracle.c and render.c (gcc, OpenMP) if the library is missing or stale."""
    src = [_HERE / "oracle.c", _HERE / "oracle_impl.h", _HERE / "render.c"]
    if force or not _LIB_PATH.exists() or any(
            s.stat().st_mtime > _LIB_PATH.stat().st_mtime for s in src):
        subprocess.run(["bash", str(_HERE / "build_oracle.sh")], check=True,
                       stdout=subprocess.DEVNULL)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(str(_LIB_PATH))
        _lib.nx_expf.restype = ctypes.c_float
        _lib.nx_expf.argtypes = [ctypes.c_float]
        _lib.orc_num_threads.restype = ctypes.c_int
    return _lib


def num_threads() -> int:
    return int(lib().orc_num_threads())


def set_num_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


def _sfx(dtype) -> str:
    dtype = np.dtype(dtype)
    if dtype == np.float32:
        return "_f32"
    if dtype == np.float64:
        return "_f64"
    raise TypeError(f"oracle dtype must be float32 or float64, not {dtype}")


def _p(a: np.ndarray):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.c_void_p)


def _real(dtype):
    return ctypes.c_float if np.dtype(dtype) == np.float32 else ctypes.c_double


def f32(x: float) -> float:
    """Round a Python float to float32 (the reference's c_float uniforms)."""
    return float(np.float32(x))


# ----------------------------------------------------------------- kernels
def init_boundaries(v):
    getattr(lib(), "orc_init_boundaries" + _sfx(v.dtype))(_p(v), v.shape[1], v.shape[0])


def add_velocity(vin, vout, px, py, vx, vy, radius):
    H, W = vin.shape[:2]
    F = ctypes.c_float
    getattr(lib(), "orc_add_velocity" + _sfx(vin.dtype))(
        _p(vin), _p(vout), W, H, F(px), F(py), F(vx), F(vy), F(radius))


def advect_velocity(vin, vout, obs, dt, speed, diss):
    H, W = vin.shape[:2]
    R = _real(vin.dtype)
    getattr(lib(), "orc_advect_velocity" + _sfx(vin.dtype))(
        _p(vin), _p(vout), _p(obs), W, H, R(f32(dt)), R(f32(speed)), R(f32(diss)))


def calc_vorticity(v, w):
    H, W = v.shape[:2]
    getattr(lib(), "orc_calc_vorticity" + _sfx(v.dtype))(_p(v), _p(w), W, H)


def apply_vorticity(vin, vout, w, dt, scale):
    H, W = vin.shape[:2]
    R = _real(vin.dtype)
    getattr(lib(), "orc_apply_vorticity" + _sfx(vin.dtype))(
        _p(vin), _p(vout), _p(w), W, H, R(f32(dt)), R(f32(scale)))


def viscosity_coeffs(nu: float) -> tuple[float, float]:
    """alpha = 1/nu and rbeta = 1/(4 + alpha) in double, then c_float
    (natrix/core/fluid_simulator.py:327-336)."""
    alpha = 1.0 / nu
    return f32(alpha), f32(1.0 / (4.0 + alpha))


def viscosity(vin, vout, nu):
    H, W = vin.shape[:2]
    R = _real(vin.dtype)
    a, rb = viscosity_coeffs(nu)
    getattr(lib(), "orc_viscosity" + _sfx(vin.dtype))(_p(vin), _p(vout), W, H, R(a), R(rb))


def divergence(v, obs, div):
    H, W = v.shape[:2]
    getattr(lib(), "orc_divergence" + _sfx(v.dtype))(_p(v), _p(obs), _p(div), W, H)


def jacobi(pin, pout, div, obs):
    H, W = pin.shape
    getattr(lib(), "orc_jacobi" + _sfx(pin.dtype))(_p(pin), _p(pout), _p(div), _p(obs), W, H)


def jacobi_n(pin, div, obs, sweeps):
    H, W = pin.shape
    pout = np.empty_like(pin)
    scratch = np.empty_like(pin)
    getattr(lib(), "orc_jacobi_n" + _sfx(pin.dtype))(
        _p(pin), _p(pout), _p(scratch), _p(div), _p(obs), W, H, int(sweeps))
    return pout


def subtract_gradient(vin, vout, p, obs):
    H, W = vin.shape[:2]
    getattr(lib(), "orc_subtract_gradient" + _sfx(vin.dtype))(
        _p(vin), _p(vout), _p(p), _p(obs), W, H)


def add_circle_obstacle(obs, px, py, radius):
    H, W = obs.shape
    F = ctypes.c_float
    lib().orc_add_circle_obstacle_f32(_p(obs), W, H, F(px), F(py), F(radius))


def add_triangle_obstacle(obs, p1, p2, p3, is_static=False):
    H, W = obs.shape
    F = ctypes.c_float
    lib().orc_add_triangle_obstacle_f32(_p(obs), W, H, F(p1[0]), F(p1[1]), F(p2[0]),
                                        F(p2[1]), F(p3[0]), F(p3[1]), int(bool(is_static)))


def add_particle_rows(width: int, height: int) -> int:
    """Rows the reference's AddParticle dispatch reaches: it launches
    ceil(W/16) groups in y as well as x (demo/smooth_particles_area.py:80-81)."""
    return min(height, 16 * ((width + 15) // 16))


def add_particle(rin, rout, px, py, radius, value):
    Hp, Wp = rin.shape
    F = ctypes.c_float
    getattr(lib(), "orc_add_particle" + _sfx(rin.dtype))(
        _p(rin), _p(rout), Wp, Hp, F(px), F(py), F(radius), F(value),
        add_particle_rows(Wp, Hp))


def advect_particle(rin, rout, v, obs, dt, speed, diss):
    Hp, Wp = rin.shape
    Hv, Wv = v.shape[:2]
    R = _real(rin.dtype)
    obs_p = _p(obs) if obs is not None else None
    getattr(lib(), "orc_advect_particle" + _sfx(rin.dtype))(
        _p(rin), _p(rout), _p(v), obs_p, Wp, Hp, Wv, Hv, R(f32(dt)), R(f32(speed)),
        R(f32(diss)))


def gauss_splats(v, rho, splats):
    """Apply (n, 6) float32 splats in place to velocity ``v`` and/or density ``rho``."""
    splats = np.ascontiguousarray(splats, np.float32)
    dt = v.dtype if v is not None else rho.dtype
    H, W = (v.shape[:2] if v is not None else (0, 0))
    Hp, Wp = (rho.shape if rho is not None else (0, 0))
    getattr(lib(), "orc_gauss_splats" + _sfx(dt))(
        _p(v) if v is not None else None, W, H, _p(rho) if rho is not None else None,
        Wp, Hp, _p(splats), int(splats.shape[0]))


def residual_sums(p, div, obs) -> np.ndarray:
    """{n, sum r, sum r^2, sum b, sum b^2} over fluid cells (r in double)."""
    H, W = p.shape
    out = np.zeros(5, np.float64)
    getattr(lib(), "orc_residual" + _sfx(p.dtype))(_p(p), _p(div), _p(obs), W, H, _p(out))
    return out


def relative_residual(p, div, obs) -> float:
    """||r - mean r|| / ||b - mean b|| over the fluid cells (the constant mode
    of the pure-Neumann system is removed from both)."""
    return rel_from_sums(residual_sums(p, div, obs))


def fluid_labels(obs) -> tuple:
    """4-connected fluid regions of an obstacle mask: int32 labels (-1 on
    obstacles) and their number."""
    from scipy import ndimage

    lab, n = ndimage.label(np.asarray(obs) == 0)
    return (lab.astype(np.int32) - 1), max(int(n), 1)


def residual_sums_regions(p, div, obs, labels, n_labels) -> np.ndarray:
    """{n, sum r, sum r^2, sum b, sum b^2} per connected fluid region."""
    H, W = p.shape
    out = np.zeros((n_labels, 5), np.float64)
    labels = np.ascontiguousarray(labels, np.int32)
    getattr(lib(), "orc_residual_regions" + _sfx(p.dtype))(
        _p(p), _p(div), _p(obs), _p(labels), n_labels, W, H, _p(out))
    return out


def rel_from_region_sums(s) -> float:
    """sqrt(sum ||r - mean r||^2 / sum ||b - mean b||^2), means per region."""
    s = np.asarray(s, np.float64).reshape(-1, 5)
    n = np.maximum(s[:, 0], 1.0)
    num = np.maximum(s[:, 2] - s[:, 1] ** 2 / n, 0.0).sum()
    den = np.maximum(s[:, 4] - s[:, 3] ** 2 / n, 0.0).sum()
    return float(math.sqrt(num / den)) if den > 0 else 0.0


def relative_residual_regions(p, div, obs) -> float:
    """Relative residual over the fluid cells with each connected region's
    mean removed (the null space of the pure-Neumann system on the fluid)."""
    labels, n = fluid_labels(obs)
    return rel_from_region_sums(residual_sums_regions(p, div, np.ascontiguousarray(obs), labels, n))


def rel_from_sums(s) -> float:
    n, sr, srr, sb, sbb = (float(x) for x in s)
    if n <= 0:
        return 0.0
    num = max(srr - sr * sr / n, 0.0)
    den = max(sbb - sb * sb / n, 0.0)
    return math.sqrt(num / den) if den > 0 else 0.0


def particles_advect(pos, v, dt, speed):
    """RK2 midpoint advection of float32 positions (n, 2) in place."""
    H, W = v.shape[:2]
    getattr(lib(), "orc_particles_advect" + _sfx(v.dtype))(
        _p(pos), ctypes.c_long(pos.shape[0]), _p(v), W, H, ctypes.c_float(dt),
        ctypes.c_float(speed))


def particle_cells(pos) -> np.ndarray:
    cells = np.empty(pos.shape, np.int32)
    lib().orc_particle_cells(_p(pos), ctypes.c_long(pos.shape[0]), _p(cells))
    return cells


def particles_splat(pos, W, H) -> np.ndarray:
    rho = np.zeros((H, W), np.float64)
    lib().orc_particles_splat(_p(pos), ctypes.c_long(pos.shape[0]), _p(rho), W, H)
    return rho


def expf(x: float) -> float:
    return float(lib().nx_expf(ctypes.c_float(x)))


# ------------------------------------------------------------ simulators
class OracleFluid:
    """FluidSimulator (natrix/core/fluid_simulator.py:15-515) on numpy arrays."""

    def __init__(self, width: int, height: int, dtype=np.float64):
        self.width, self.height = int(width), int(height)
        self.dtype = np.dtype(dtype)
        H, W = self.height, self.width
        self.vel = [np.zeros((H, W, 2), dtype), np.zeros((H, W, 2), dtype)]
        self.vr = 0  # VELOCITY_READ
        self.pressure = np.zeros((H, W), dtype)
        self.divergence = np.zeros((H, W), dtype)
        self.vorticity_field = np.zeros((H, W), dtype)
        self.obstacles = np.zeros((H, W), np.uint8)
        # defaults, natrix/core/fluid_simulator.py:28-35
        self.speed = 500.0
        self.iterations = 50
        self.dissipation = 1.0
        self.vorticity = 0.0
        self.viscosity = 0.1
        self.has_borders = True
        self.simulate = True

    @property
    def velocity(self) -> np.ndarray:
        return self.vel[self.vr]

    def _flip(self):
        self.vr ^= 1

    def add_velocity(self, position, velocity, radius):
        if self.simulate:
            add_velocity(self.vel[self.vr], self.vel[self.vr ^ 1], position[0], position[1],
                         velocity[0], velocity[1], radius)
            self._flip()

    def add_circle_obstacle(self, position, radius, static=False):
        if self.simulate:
            add_circle_obstacle(self.obstacles, position[0], position[1], radius)

    def add_triangle_obstacle(self, p1, p2, p3, static=False):
        if self.simulate:
            add_triangle_obstacle(self.obstacles, p1, p2, p3, static)

    def add_splats(self, splats, density: "OracleDensity | None" = None):
        if self.simulate:
            gauss_splats(self.vel[self.vr], density.field if density is not None else None,
                         splats)

    def update(self, dt: float):
        if not self.simulate:
            return
        if self.has_borders:
            init_boundaries(self.vel[self.vr])
        advect_velocity(self.vel[self.vr], self.vel[self.vr ^ 1], self.obstacles, dt,
                        self.speed, self.dissipation)
        self._flip()
        calc_vorticity(self.vel[self.vr], self.vorticity_field)
        apply_vorticity(self.vel[self.vr], self.vel[self.vr ^ 1], self.vorticity_field, dt,
                        self.vorticity)
        self._flip()
        if self.viscosity > 0.0:
            viscosity(self.vel[self.vr], self.vel[self.vr ^ 1], self.viscosity)
            self._flip()
        divergence(self.vel[self.vr], self.obstacles, self.divergence)
        p0 = np.zeros_like(self.pressure)
        self.pressure = jacobi_n(p0, self.divergence, self.obstacles, self.iterations)
        subtract_gradient(self.vel[self.vr], self.vel[self.vr ^ 1], self.pressure,
                          self.obstacles)
        self._flip()
        self.obstacles[:] = 0


class OracleDensity:
    """SmoothParticlesArea (demo/smooth_particles_area.py:15-211) on numpy arrays."""

    def __init__(self, width: int, height: int, fluid: OracleFluid):
        self.width, self.height = int(width), int(height)
        self.fluid = fluid
        self.buf = [np.zeros((height, width), fluid.dtype) for _ in range(2)]
        self.r = 0
        self.speed = 500.0
        self.dissipation = 1.0
        self.simulate = True

    @property
    def field(self) -> np.ndarray:
        return self.buf[self.r]

    def add_particles(self, position, radius, strength):
        if self.simulate:
            add_particle(self.buf[self.r], self.buf[self.r ^ 1], position[0], position[1],
                         radius, strength)
            self.r ^= 1

    def update(self, dt: float):
        if self.simulate:
            advect_particle(self.buf[self.r], self.buf[self.r ^ 1], self.fluid.velocity,
                            self.fluid.obstacles, dt, self.speed, self.dissipation)
            self.r ^= 1


# ---- headless visualisation (oracle/render.c) ----
def plasma_palette() -> np.ndarray:
    """(256, 4) uint8: the field shader's colour for each texel byte."""
    pal = np.empty((256, 4), np.uint8)
    lib().orc_plasma_palette(_p(pal))
    return pal


def render_density(rho) -> tuple:
    """float32 (H, W) density -> (texture, colour), each (H, W, 4) uint8."""
    rho = np.ascontiguousarray(rho, np.float32)
    H, W = rho.shape
    tex = np.empty((H, W, 4), np.uint8)
    col = np.empty((H, W, 4), np.uint8)
    lib().orc_render_density(_p(rho), W, H, _p(tex), _p(col))
    return tex, col


def quiver_tiles(win_w: int, win_h: int, tile: float) -> tuple:
    t = np.float32(tile)
    nx = int(np.floor((np.float32(win_w) - np.float32(0.5)) / t)) + 1
    ny = int(np.floor((np.float32(win_h) - np.float32(0.5)) / t)) + 1
    return nx, ny


def quiver(v, win_w: int, win_h: int, tile: float, overlay: bool = True) -> tuple:
    """float32 velocity (H, W, 2) -> (arrows (ny, nx, 2) float32, overlay
    (win_h, win_w, 4) uint8 or None)."""
    v = np.ascontiguousarray(v, np.float32)
    VH, VW = v.shape[:2]
    nx, ny = quiver_tiles(win_w, win_h, tile)
    arrows = np.empty((ny, nx, 2), np.float32)
    lib().orc_quiver_arrows(_p(v), VW, VH, win_w, win_h, ctypes.c_float(tile), _p(arrows), nx, ny)
    out = None
    if overlay:
        out = np.empty((win_h, win_w, 4), np.uint8)
        lib().orc_quiver_overlay(_p(arrows), nx, win_w, win_h, ctypes.c_float(tile), _p(out))
    return arrows, out
