"""Lagrangian particles on the GPU against the oracle: positions and integer
particle->cell indices bit-exact, splatted density within the rounding of
unordered FP32 atomic sums (|gpu - oracle| <= 1e-5 x max density, the oracle
summing in double), mass conserved."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DENSITY_RTOL = 1e-5


def coupled_run(oracle, W, H, n, steps, seed, iterations=40, vorticity=0.35, n_obst=4,
                n_splats=8):
    from natrix_gb300 import FluidSimulator
    from natrix_gb300 import workloads as wl
    from natrix_gb300.core.particles import LagrangianParticles

    rng = np.random.default_rng(seed)
    pos0 = np.stack([rng.uniform(0, W - 1, n), rng.uniform(0, H - 1, n)], 1).astype(np.float32)
    sim = FluidSimulator(W, H)
    ref = oracle.OracleFluid(W, H, np.float32)
    for s in (sim, ref):
        s.iterations, s.vorticity, s.viscosity, s.speed, s.dissipation = (
            iterations, vorticity, 0.0, 5.0, 0.99)
    parts = LagrangianParticles(sim, pos0)
    rpos = pos0.copy()
    obst = wl.circle_obstacles(rng, n_obst, W, H, 0.02, 0.06)
    for _ in range(steps):
        splats = wl.gauss_splats(rng, n_splats, W, H, 5.0)
        for s in (sim, ref):
            for o in obst:
                s.add_circle_obstacle((float(o[0]), float(o[1])), float(o[2]))
            s.add_splats(splats)
            s.update(1 / 60)
        parts.step(1 / 60)
        oracle.particles_advect(rpos, ref.velocity, 1 / 60, 5.0)
    return sim, parts, rpos


def check(oracle, sim, parts, rpos):
    W, H = sim.width, sim.height
    got = parts.download()
    bad = np.argwhere(np.any(got != rpos, axis=1))
    assert bad.size == 0, f"{len(bad)} particles differ, first {bad[:3].ravel().tolist()}"
    np.testing.assert_array_equal(parts.cells(), oracle.particle_cells(rpos))
    rho = parts.density.cpu().numpy().astype(np.float64)
    want = oracle.particles_splat(rpos, W, H)
    assert np.max(np.abs(rho - want)) <= DENSITY_RTOL * max(want.max(), 1.0)
    assert abs(rho.sum() - rpos.shape[0]) <= 1e-4 * rpos.shape[0]


def test_particles_small_bit_exact(cuda, oracle):
    sim, parts, rpos = coupled_run(oracle, 200, 150, 50_000, steps=12, seed=3)
    check(oracle, sim, parts, rpos)
    parts.destroy()
    sim.destroy()


def test_particles_edges_and_clamp(cuda, oracle):
    """Particles on and beyond the walls: positions clamp to the grid, tent
    targets clamp onto the edge cells, mass is kept."""
    from natrix_gb300 import FluidSimulator
    from natrix_gb300.core.particles import LagrangianParticles

    W, H = 40, 30
    sim = FluidSimulator(W, H)
    ref = oracle.OracleFluid(W, H, np.float32)
    for s in (sim, ref):
        s.iterations, s.speed = 5, 200.0
        s.add_velocity((0.02, 0.5), (1.0, 0.0), 30.0)
        s.add_velocity((0.98, 0.03), (-1.0, -1.0), 30.0)
    pos = np.array([[0, 0], [W - 1, H - 1], [0.49, 0.51], [W - 1.5, 0], [17.5, 9.5],
                    [1e-7, H - 1 - 1e-6]], np.float32)
    parts = LagrangianParticles(sim, pos)
    rpos = pos.copy()
    for _ in range(5):
        for s in (sim, ref):
            s.update(1 / 60)
        parts.step(1 / 60)
        oracle.particles_advect(rpos, ref.velocity, 1 / 60, 200.0)
    check(oracle, sim, parts, rpos)
    parts.destroy()
    sim.destroy()


@pytest.mark.slow
def test_particles_full_workload(cuda, oracle):
    """4,194,304 particles in a 1024x1024 solver (40 sweeps, eps 0.35, discs,
    splat forcing) for 300 steps: positions and cells bit-exact, density
    within tolerance."""
    sim, parts, rpos = coupled_run(oracle, 1024, 1024, 4_194_304, steps=300, seed=11,
                                   n_obst=12, n_splats=16)
    check(oracle, sim, parts, rpos)
    parts.destroy()
    sim.destroy()
