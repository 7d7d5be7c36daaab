"""The seeded synthetic workloads against their stated shapes and
distributions (natrix_gb300/workloads.py): Gaussian splats, non-overlapping
discs inside the grid, the 512-simulation batch (sides 64-512 in multiples of
16, sweep counts in {20, 40, 80}, about 31.8 M cells), uniform particles, and
reproducibility from the seed."""
from __future__ import annotations

import math

import numpy as np

from natrix_gb300 import workloads as wl


def test_gauss_splats_ranges():
    rng = np.random.default_rng(0)
    W, H, speed = 2048, 1024, 5.0
    s = wl.gauss_splats(rng, 4000, W, H, speed)
    assert s.shape == (4000, wl.SPLAT_FIELDS) and s.dtype == np.float32
    assert np.all((s[:, :2] >= 0) & (s[:, :2] < 1))
    assert np.allclose(s[:, 2], 0.02 * min(W, H))
    # velocity amplitude uniform in [-5, 5] cells/s, stored divided by speed
    assert np.all(np.abs(s[:, 3:5]) <= 5.0 / speed + 1e-7)
    assert abs(float(s[:, 3:5].mean())) < 0.02 and float(np.abs(s[:, 3:5]).max()) > 0.9
    assert np.all((s[:, 5] >= 0) & (s[:, 5] <= 1))


def test_circle_obstacles_disjoint_inside_grid():
    for seed in range(5):
        rng = np.random.default_rng(seed)
        W = H = 2048
        d = wl.circle_obstacles(rng, 12, W, H)
        assert d.shape == (12, 3)
        r = d[:, 2].astype(np.float64)
        assert np.all((r >= 0.01 * W - 1e-3) & (r <= 0.05 * W + 1e-3))
        cx, cy = d[:, 0] * W, d[:, 1] * H
        assert np.all((cx - r >= -1e-2) & (cx + r <= W + 1e-2))
        assert np.all((cy - r >= -1e-2) & (cy + r <= H + 1e-2))
        for i in range(12):
            for j in range(i):
                assert math.hypot(cx[i] - cx[j], cy[i] - cy[j]) > r[i] + r[j] - 1e-2


def test_batch_workload_shapes():
    b = wl.BATCH_512
    sides = b.sides()
    assert len(sides) == 512
    assert np.all(sides % 16 == 0) and sides.min() >= 64 and sides.max() <= 512
    cells = int((sides.astype(np.int64) ** 2).sum())
    assert 28e6 < cells < 36e6  # E[N^2] of the log-uniform sides ~ 62k per simulation
    assert set(np.unique(b.iterations())) <= {20, 40, 80}
    counts = [len(b.obstacles(i, int(sides[i]))) for i in range(512)]
    assert min(counts) >= 0 and max(counts) <= 6
    f = b.forcing(3, 7, int(sides[3]))
    assert f.shape == (b.splats_per_step, wl.SPLAT_FIELDS)


def test_uniform_particles_in_grid_and_ordered():
    p = wl.uniform_particles(0, 100_000, 1024, 1024)
    assert p.shape == (100_000, 2) and p.dtype == np.float32
    assert np.all((p >= 0) & (p <= 1023))
    key = np.floor(p[:, 1] + 0.5).astype(np.int64) * 1024 + np.floor(p[:, 0] + 0.5)
    assert np.all(np.diff(key) >= 0)


def test_workloads_reproducible_from_seed():
    spec = wl.LARGE_2048
    a = wl.workload_obstacles(5, spec)
    b = wl.workload_obstacles(5, spec)
    assert np.array_equal(a, b)
    assert np.array_equal(wl.step_forcing(5, 9, spec), wl.step_forcing(5, 9, spec))
    assert not np.array_equal(wl.step_forcing(5, 9, spec), wl.step_forcing(5, 10, spec))
    assert np.array_equal(wl.uniform_particles(1, 1000, 64, 64),
                          wl.uniform_particles(1, 1000, 64, 64))
