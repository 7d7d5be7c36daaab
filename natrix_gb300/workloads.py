"""Seeded synthetic workloads for the solver (numpy only, no device code).

The reference publishes no benchmark inputs, so the workloads are generated
from a seed: Gaussian splat forcing and circular obstacles with the sizes and
distributions below.  Everything is returned as float32 host arrays in the
reference API's units:

* positions are normalised to [0, 1) (as ``add_velocity`` / ``add_circle_obstacle``
  take them, natrix/core/fluid_simulator.py:116-153);
* radii are in cells of the grid they act on;
* splat velocities are in *stored* units: the solver keeps velocity clamped to
  [-1, 1] and displaces by ``v * dt * speed`` (shader.AdvectVelocity.comp:37,49),
  so an amplitude of A cells/s is stored as A / speed.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

SPLAT_FIELDS = 6  # px, py, radius_cells, vx_stored, vy_stored, density


@dataclass(frozen=True)
class Workload:
    """One named solver workload (grid, sweeps, forcing, obstacles, steps)."""

    name: str
    width: int
    height: int
    iterations: int
    vorticity: float
    viscosity: float
    dissipation: float
    speed: float
    dt: float
    steps: int
    splats_per_step: int
    n_obstacles: int
    seed: int = 0


# Plain solver, 256x256, eps = 0, 40 sweeps, 8 splats/step, no obstacles, 200 steps.
SMALL_256 = Workload("plain-256x256-K40", 256, 256, 40, 0.0, 0.0, 0.99, 5.0, 1.0 / 60.0,
                     200, 8, 0)
# Large solver, 2048x2048, eps = 0.35, 80 sweeps, 16 splats/step, 12 discs, 500 steps.
LARGE_2048 = Workload("plain-2048x2048-K80-eps0.35-12discs", 2048, 2048, 80, 0.35, 0.0,
                      0.99, 5.0, 1.0 / 60.0, 500, 16, 12)


# Lagrangian particles: 4,194,304 particles uniform in a 1024x1024 solver with
# the large workload's settings at 40 sweeps, 300 steps.
PARTICLES_1024 = Workload("particles-4M-1024x1024-K40-eps0.35-12discs", 1024, 1024, 40, 0.35,
                          0.0, 0.99, 5.0, 1.0 / 60.0, 300, 16, 12)
N_PARTICLES = 4_194_304


def uniform_particles(seed: int, n: int, width: int, height: int) -> np.ndarray:
    """n float32 positions (x, y) in cells, uniform over the grid, ordered by
    row-major cell (spatially coherent order: neighbouring threads deposit
    into neighbouring cells)."""
    rng = np.random.default_rng([seed, 3])
    pos = np.stack([rng.uniform(0, width - 1, n), rng.uniform(0, height - 1, n)], 1)
    pos = pos.astype(np.float32)
    key = np.floor(pos[:, 1] + 0.5).astype(np.int64) * width + np.floor(pos[:, 0] + 0.5)
    return np.ascontiguousarray(pos[np.argsort(key, kind="stable")])


@dataclass(frozen=True)
class BatchWorkload:
    """Many independent simulations: side lengths log-uniform in [64, 512]
    rounded to multiples of 16, Jacobi counts uniform in {20, 40, 80}, 0-6
    discs each, 8 Gaussian splats per simulation per step, eps 0, nu 0."""

    name: str
    n_sims: int
    steps: int
    splats_per_step: int = 8
    seed: int = 0

    def sides(self) -> np.ndarray:
        rng = np.random.default_rng([self.seed, 4])
        s = np.exp(rng.uniform(np.log(64), np.log(512), self.n_sims))
        return (16 * np.round(s / 16)).astype(np.int32)

    def iterations(self) -> np.ndarray:
        rng = np.random.default_rng([self.seed, 5])
        return rng.choice(np.array([20, 40, 80]), self.n_sims)

    def obstacles(self, sim: int, side: int) -> np.ndarray:
        rng = np.random.default_rng([self.seed, 6, sim])
        return circle_obstacles(rng, int(rng.integers(0, 7)), side, side)

    def forcing(self, sim: int, step: int, side: int) -> np.ndarray:
        rng = np.random.default_rng([self.seed, 7, sim, step])
        return gauss_splats(rng, self.splats_per_step, side, side, 5.0)


BATCH_512 = BatchWorkload("batch-512-sims-64to512-K20/40/80", 512, 100)


def gauss_splats(rng: np.random.Generator, n: int, width: int, height: int,
                 speed: float, radius_frac: float = 0.02,
                 amp_cells_per_s: float = 5.0) -> np.ndarray:
    """``n`` Gaussian splats as an (n, 6) float32 array.

    Centres uniform in the domain, radius ``radius_frac * min(W, H)`` cells,
    velocity amplitude uniform in [-amp, amp]^2 cells/s (stored as amp/speed),
    density amplitude uniform in [0, 1].
    """
    out = np.empty((n, SPLAT_FIELDS), np.float32)
    out[:, 0] = rng.random(n)
    out[:, 1] = rng.random(n)
    out[:, 2] = radius_frac * min(width, height)
    out[:, 3:5] = rng.uniform(-amp_cells_per_s, amp_cells_per_s, (n, 2)) / speed
    out[:, 5] = rng.random(n)
    return out


def circle_obstacles(rng: np.random.Generator, n: int, width: int, height: int,
                     rmin: float = 0.01, rmax: float = 0.05,
                     max_tries: int = 100000) -> np.ndarray:
    """``n`` non-overlapping discs as an (n, 3) float32 array (px, py, r_cells).

    Radius uniform in [rmin, rmax] * min(W, H); centres uniform over positions
    that keep the disc inside the grid; rejection sampling enforces no overlap.
    """
    side = min(width, height)
    discs: list[tuple[float, float, float]] = []
    tries = 0
    while len(discs) < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place non-overlapping obstacles")
        r = rng.uniform(rmin, rmax) * side
        cx = rng.uniform(r, width - r)
        cy = rng.uniform(r, height - r)
        if all(math.hypot(cx - x, cy - y) > r + rr for x, y, rr in discs):
            discs.append((cx, cy, r))
    out = np.array([(cx / width, cy / height, r) for cx, cy, r in discs], np.float32)
    return out.reshape(n, 3)


def step_forcing(seed: int, step: int, wl: Workload) -> np.ndarray:
    """The splats of step ``step`` of workload ``wl`` (independent stream per step)."""
    rng = np.random.default_rng([seed, 1, step])
    return gauss_splats(rng, wl.splats_per_step, wl.width, wl.height, wl.speed)


def workload_obstacles(seed: int, wl: Workload) -> np.ndarray:
    rng = np.random.default_rng([seed, 2])
    return circle_obstacles(rng, wl.n_obstacles, wl.width, wl.height)
