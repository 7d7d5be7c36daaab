"""Batched simulations against independently stepped single simulators: every
simulation of a batch must equal, bit for bit, a FluidSimulator +
SmoothParticlesArea driven through the same calls, for every tile
configuration, sweeps-per-launch and with or without the CUDA graph."""
from __future__ import annotations

import numpy as np
import pytest

from tests.golden_replay import assert_equal_f32

pytestmark = pytest.mark.gpu

SIDES = [(64, 64), (80, 48), (96, 96), (128, 112), (144, 144), (208, 160), (256, 256),
         (272, 240), (384, 320)]


def build(iters, eps, nus, seed):
    from natrix_gb300 import FluidSimulator, SmoothParticlesArea
    from natrix_gb300.core.batch import FluidBatch

    batch = FluidBatch([w for w, _ in SIDES], [h for _, h in SIDES])
    singles = []
    for i, (w, h) in enumerate(SIDES):
        batch.set_params(i, speed=5.0, iterations=iters[i], dissipation=0.99,
                         vorticity=eps[i], viscosity=nus[i])
        batch.set_density_params(i, speed=5.0, dissipation=0.98)
        s = FluidSimulator(w, h)
        d = SmoothParticlesArea(w, h, s)
        s.speed, s.iterations, s.dissipation, s.vorticity, s.viscosity = (
            5.0, iters[i], 0.99, eps[i], nus[i])
        d.speed, d.dissipation = 5.0, 0.98
        singles.append((s, d))
    return batch, singles


def drive(batch, singles, steps, seed):
    from natrix_gb300 import workloads as wl

    rng = np.random.default_rng(seed)
    obst = [wl.circle_obstacles(rng, int(rng.integers(0, 4)), w, h, 0.03, 0.08)
            for (w, h) in SIDES]
    for _ in range(steps):
        for i, (w, h) in enumerate(SIDES):
            s, d = singles[i]
            for o in obst[i]:
                batch.add_circle_obstacle(i, (float(o[0]), float(o[1])), float(o[2]))
                s.add_circle_obstacle((float(o[0]), float(o[1])), float(o[2]))
            spl = wl.gauss_splats(rng, 4, w, h, 5.0)
            batch.add_splats(i, spl)
            s.add_splats(spl, d)
            if rng.random() < 0.5:
                pos, vel = (rng.random(), rng.random()), tuple(rng.uniform(-1, 1, 2))
                batch.add_velocity(i, pos, vel, 6.0)
                s.add_velocity(pos, vel, 6.0)
        batch.step(1 / 60)
        for s, d in singles:
            s.update(1 / 60)
            d.update(1 / 60)


def compare(batch, singles):
    from natrix_gb300 import _lib

    batch.sync()
    for i, (s, d) in enumerate(singles):
        for f in (_lib.FIELD_VELOCITY, _lib.FIELD_PRESSURE, _lib.FIELD_DIVERGENCE):
            assert_equal_f32(batch.download(i, f), s.download(f), f"sim {i} field {f}")
        assert_equal_f32(batch.download(i, _lib.FIELD_DENSITY), d.download(), f"sim {i} density")
        if s.vorticity > 0:
            assert_equal_f32(batch.download(i, _lib.FIELD_VORTICITY),
                             s.download(_lib.FIELD_VORTICITY), f"sim {i} vorticity")


@pytest.mark.parametrize("tuning,graph,persistent", [
    ({0: (0, 8), 1: (1, 8), 2: (2, 8)}, True, True),
    ({0: (0, 4), 1: (0, 8), 2: (1, 4)}, True, True),
    ({0: (1, 8), 1: (2, 3), 2: (0, 5)}, False, True),
    ({0: (0, 8), 1: (1, 8), 2: (2, 8)}, True, False),
    ({0: (1, 8), 1: (2, 3), 2: (0, 5)}, False, False),
])
def test_batch_equals_single_simulators(cuda, tuning, graph, persistent):
    """Persistent: the whole step in one launch (work items in dependency
    order); otherwise one launch per phase."""
    rng = np.random.default_rng(1)
    n = len(SIDES)
    iters = [int(x) for x in rng.choice([1, 9, 20, 40, 80], n)]
    eps = [0.0 if i % 3 else 0.35 for i in range(n)]
    nus = [0.1 if i % 4 == 1 else 0.0 for i in range(n)]
    batch, singles = build(iters, eps, nus, 2)
    batch.use_graph(graph)
    batch.use_persistent(persistent)
    for c, (cfg, spl) in tuning.items():
        batch.set_tuning(c, cfg, spl)
    drive(batch, singles, steps=5, seed=3)
    compare(batch, singles)
    total, per_step = batch.launches()
    assert per_step > 0 and total >= 5 * per_step
    if persistent:
        assert per_step == 1
    batch.destroy()
    for s, d in singles:
        d.destroy()
        s.destroy()


def test_batch_workload_sample_matches_oracle(cuda, oracle):
    """Three simulations of the 512-simulation workload's distribution against
    the float32 oracle, with the workload's own forcing and obstacles."""
    from natrix_gb300 import _lib
    from natrix_gb300 import workloads as wl
    from natrix_gb300.core.batch import FluidBatch

    spec = wl.BATCH_512
    sides = spec.sides()[:3]
    its = spec.iterations()[:3]
    batch = FluidBatch(list(sides), list(sides))
    refs = []
    for i, side in enumerate(sides):
        batch.set_params(i, speed=5.0, iterations=int(its[i]), dissipation=0.99, vorticity=0.0,
                         viscosity=0.0)
        batch.set_density_params(i, speed=5.0, dissipation=0.99)
        f = oracle.OracleFluid(int(side), int(side), np.float32)
        d = oracle.OracleDensity(int(side), int(side), f)
        f.speed, f.iterations, f.dissipation, f.vorticity, f.viscosity = 5.0, int(its[i]), 0.99, 0, 0
        d.speed, d.dissipation = 5.0, 0.99
        refs.append((f, d))
    for step in range(4):
        for i, side in enumerate(sides):
            f, d = refs[i]
            for o in spec.obstacles(i, int(side)):
                batch.add_circle_obstacle(i, (float(o[0]), float(o[1])), float(o[2]))
                f.add_circle_obstacle((float(o[0]), float(o[1])), float(o[2]))
            spl = spec.forcing(i, step, int(side))
            batch.add_splats(i, spl)
            f.add_splats(spl, d)
        batch.step(1 / 60)
        for f, d in refs:
            f.update(1 / 60)
            d.update(1 / 60)
    batch.sync()
    for i, (f, d) in enumerate(refs):
        assert_equal_f32(batch.download(i, _lib.FIELD_VELOCITY), f.velocity, f"sim {i} velocity")
        assert_equal_f32(batch.download(i, _lib.FIELD_PRESSURE), f.pressure, f"sim {i} pressure")
        assert_equal_f32(batch.download(i, _lib.FIELD_DENSITY), d.field, f"sim {i} density")
    batch.destroy()


def test_batch_512_workload_equals_single_simulators(cuda):
    """The whole 512-simulation workload (sides 64-512, 20/40/80 sweeps, 0-6
    discs, 8 splats each per step) stepped as one batch with its autotuned
    tiles and the captured graph, against 512 independently stepped
    FluidSimulator + SmoothParticlesArea pairs driven through the same calls:
    every simulation's velocity, pressure, divergence and density equal bit
    for bit after 3 steps."""
    from natrix_gb300 import FluidSimulator, SmoothParticlesArea
    from natrix_gb300 import workloads as wl
    from natrix_gb300.core.batch import FluidBatch

    spec = wl.BATCH_512
    sides, its = spec.sides(), spec.iterations()
    n = spec.n_sims
    assert n == 512

    def make_batch():
        b = FluidBatch(list(sides), list(sides))
        for i in range(n):
            b.set_params(i, speed=5.0, iterations=int(its[i]), dissipation=0.99,
                         vorticity=0.0, viscosity=0.0)
        b.set_density_params(-1, speed=5.0, dissipation=0.99)
        return b

    # tile shapes and sweeps per launch as the autotuner picks them (timed on
    # a batch of its own, so the compared batch starts from rest)
    tuner = make_batch()
    tuning = tuner.autotune(cache=False)
    tuner.destroy()
    batch = make_batch()
    for c, (cfg, spl) in tuning.items():
        batch.set_tuning(c, cfg, spl)
    singles = []
    for i in range(n):
        s = FluidSimulator(int(sides[i]), int(sides[i]))
        d = SmoothParticlesArea(int(sides[i]), int(sides[i]), s)
        s.speed, s.iterations, s.dissipation, s.vorticity, s.viscosity = (
            5.0, int(its[i]), 0.99, 0.0, 0.0)
        d.speed, d.dissipation = 5.0, 0.99
        singles.append((s, d))
    obst = [spec.obstacles(i, int(sides[i])) for i in range(n)]
    for step in range(3):
        for i in range(n):
            s, d = singles[i]
            for o in obst[i]:
                batch.add_circle_obstacle(i, (float(o[0]), float(o[1])), float(o[2]))
                s.add_circle_obstacle((float(o[0]), float(o[1])), float(o[2]))
            spl = spec.forcing(i, step, int(sides[i]))
            batch.add_splats(i, spl)
            s.add_splats(spl, d)
        batch.step(1 / 60)
        for s, d in singles:
            s.update(1 / 60)
            d.update(1 / 60)
    compare(batch, singles)
    batch.destroy()
    for s, d in singles:
        d.destroy()
        s.destroy()


def test_persistent_step_refuses_rows_wider_than_its_staging(cuda):
    """The persistent step stages rows of at most 3008 cells in shared
    memory: a wider simulation gets NATRIX_ERANGE with a clear message (and
    steps in the per-phase mode)."""
    from natrix_gb300 import _lib
    from natrix_gb300.core.batch import FluidBatch

    batch = FluidBatch([3040, 64], [8, 64])
    batch.set_params(-1, speed=5.0, iterations=3, dissipation=0.99, vorticity=0.0,
                     viscosity=0.0)
    with pytest.raises(_lib.NatrixError) as err:
        batch.step(1 / 60)
    assert err.value.code == _lib.NATRIX_ERANGE and "3008" in str(err.value)
    batch.use_persistent(False)
    batch.step(1 / 60)
    batch.sync()
    batch.destroy()


def test_persistent_step_many_tiny_simulations(cuda):
    """96 small grids with 1-3 sweeps each: nearly every item of the
    persistent step waits on a phase that finished a moment ago (the held
    completion signals are flushed before each such wait).  One launch per
    step must give the same fields, bit for bit, as one launch per phase."""
    from natrix_gb300 import _lib
    from natrix_gb300 import workloads as wl
    from natrix_gb300.core.batch import FluidBatch

    rng = np.random.default_rng(11)
    n = 96
    sides = [(int(w), int(h)) for w, h in zip(rng.choice([48, 64, 80, 96], n),
                                               rng.choice([32, 48, 64, 80], n))]
    iters = [int(k) for k in rng.choice([1, 2, 3], n)]
    splats = [[wl.gauss_splats(rng, 3, w, h, 5.0) for (w, h) in sides] for _ in range(4)]
    out = []
    for persistent in (True, False):
        b = FluidBatch([w for w, _ in sides], [h for _, h in sides])
        b.use_persistent(persistent)
        for i in range(n):
            b.set_params(i, speed=5.0, iterations=iters[i], dissipation=0.99, vorticity=0.0,
                         viscosity=0.0)
        b.set_density_params(-1, speed=5.0, dissipation=0.98)
        for step in range(4):
            for i, (w, h) in enumerate(sides):
                b.add_circle_obstacle(i, (0.5, 0.5), 0.1 * min(w, h))
                b.add_splats(i, splats[step][i])
            b.step(1 / 60)
        b.sync()
        out.append([(b.download(i, _lib.FIELD_VELOCITY), b.download(i, _lib.FIELD_PRESSURE),
                     b.download(i, _lib.FIELD_DENSITY)) for i in range(n)])
        b.destroy()
    for i in range(n):
        for a, c, what in zip(out[0][i], out[1][i], ("velocity", "pressure", "density")):
            assert_equal_f32(a, c, f"sim {i} {what}")
