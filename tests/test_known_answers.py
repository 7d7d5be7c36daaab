"""Known-answer tests of the oracle from the solver's mathematics (the
reference ships no tests, so these pin the restatement independently of the
shader sources)."""
from __future__ import annotations

import numpy as np


def test_uniform_velocity_advects_as_exact_shift(oracle):
    # v*dt*speed = 1 cell: every interior cell samples its left neighbour
    W, H = 16, 12
    v = np.zeros((H, W, 2), np.float32)
    v[..., 0] = 0.5
    out = np.zeros_like(v)
    mask = np.zeros((H, W), np.uint8)
    oracle.advect_velocity(v, out, mask, 0.5, 4.0, 1.0)
    assert np.all(out[:, 1:, 0] == 0.5) and np.all(out[..., 1] == 0.0)


def test_obstacle_cells_advect_to_zero(oracle):
    W, H = 12, 10
    v = np.full((H, W, 2), 0.3, np.float32)
    mask = np.zeros((H, W), np.uint8)
    mask[4:6, 3:7] = 1
    out = np.zeros_like(v)
    oracle.advect_velocity(v, out, mask, 0.1, 1.0, 1.0)
    assert np.all(out[4:6, 3:7] == 0)


def test_velocity_clamp_holds(oracle):
    W, H = 20, 20
    v = np.zeros((H, W, 2), np.float32)
    out = np.zeros_like(v)
    oracle.add_velocity(v, out, 0.5, 0.5, 50.0, -50.0, 8.0)
    assert out.max() <= 1.0 and out.min() >= -1.0 and out.max() == 1.0


def test_divergence_of_linear_field_is_constant(oracle):
    W, H = 16, 16
    y, x = np.mgrid[0:H, 0:W].astype(np.float64)
    v = np.stack([0.01 * x, -0.02 * y], -1)
    div = np.zeros((H, W))
    oracle.divergence(v, np.zeros((H, W), np.uint8), div)
    np.testing.assert_allclose(div[1:-1, 1:-1], 0.5 * (0.02 - 0.04), rtol=1e-12)


def test_vorticity_of_solid_rotation_is_constant(oracle):
    W, H = 16, 16
    y, x = np.mgrid[0:H, 0:W].astype(np.float64)
    v = np.stack([-(y - 8) * 0.01, (x - 8) * 0.01], -1)
    w = np.zeros((H, W))
    oracle.calc_vorticity(v, w)
    np.testing.assert_allclose(w[1:-1, 1:-1], 0.5 * (0.02 + 0.02), rtol=1e-12)


def test_zero_confinement_is_identity(oracle):
    rng = np.random.default_rng(0)
    v = rng.uniform(-1, 1, (9, 13, 2)).astype(np.float32)
    w = rng.normal(size=(9, 13)).astype(np.float32)
    out = np.zeros_like(v)
    oracle.apply_vorticity(v, out, w, 1 / 60, 0.0)
    assert np.array_equal(out, v)


def test_jacobi_fixed_point(oracle):
    """A pressure that satisfies the discrete operator is a fixed point."""
    rng = np.random.default_rng(1)
    W, H = 14, 11
    p = rng.normal(size=(H, W))
    mask = np.zeros((H, W), np.uint8)
    mask[5, 5] = 1
    # b = sum(p_nbr) - 4p with the sweep's neighbour rule
    b = np.zeros_like(p)
    for y in range(H):
        for x in range(W):
            def nb(xx, yy):
                xx, yy = min(max(xx, 0), W - 1), min(max(yy, 0), H - 1)
                return p[y, x] if mask[yy, xx] else p[yy, xx]
            b[y, x] = nb(x - 1, y) + nb(x + 1, y) + nb(x, y - 1) + nb(x, y + 1) - 4 * p[y, x]
    out = oracle.jacobi_n(p, b, mask, 1)
    np.testing.assert_allclose(out, p, atol=1e-12)
    assert oracle.relative_residual(p, b, mask) < 1e-12


def test_jacobi_reduces_residual(oracle):
    rng = np.random.default_rng(2)
    W, H = 24, 24
    b = rng.normal(size=(H, W))
    mask = np.zeros((H, W), np.uint8)
    p0 = np.zeros((H, W))
    r0 = oracle.relative_residual(p0, b, mask)
    r1 = oracle.relative_residual(oracle.jacobi_n(p0, b, mask, 200), b, mask)
    assert r0 == 1.0 or abs(r0 - 1.0) < 1e-12
    assert r1 < 0.5


def test_particles_rk2_uniform_flow(oracle):
    W, H = 32, 32
    v = np.zeros((H, W, 2), np.float32)
    v[..., 0] = 0.25
    pos = np.array([[10.0, 10.0], [30.5, 3.0]], np.float32)
    oracle.particles_advect(pos, v, 0.5, 8.0)  # displacement 1 cell in x
    np.testing.assert_array_equal(pos, np.array([[11.0, 10.0], [31.0, 3.0]], np.float32))
    cells = oracle.particle_cells(pos)
    np.testing.assert_array_equal(cells, [[11, 10], [31, 3]])
    rho = oracle.particles_splat(pos, W, H)
    assert abs(rho.sum() - 2.0) < 1e-6


def test_region_residual_ignores_per_region_constants(oracle):
    """A wall of obstacles splits the fluid into two regions; the residual
    with per-region means removed is blind to a constant added per region to
    the pressure or the divergence, while the global-mean residual is not
    (and no sweep can remove that part)."""
    rng = np.random.default_rng(4)
    W, H = 20, 16
    mask = np.zeros((H, W), np.uint8)
    mask[:, 9] = 1
    labels, n = oracle.fluid_labels(mask)
    assert n == 2 and labels[0, 0] != labels[0, 15] and labels[0, 9] == -1
    p = rng.normal(size=(H, W))
    b = rng.normal(size=(H, W))
    base = oracle.relative_residual_regions(p, b, mask)
    shift = np.where(labels == labels[0, 0], 3.0, -2.0) * (mask == 0)
    assert abs(oracle.relative_residual_regions(p + shift, b, mask) - base) < 1e-12
    b2 = b + shift
    p2 = oracle.jacobi_n(np.zeros((H, W)), b2, mask, 4000)
    assert oracle.relative_residual_regions(p2, b2, mask) < 1e-6
    assert oracle.relative_residual(p2, b2, mask) > 1e-2
    sums = oracle.residual_sums_regions(p, b, mask, labels, n)
    np.testing.assert_allclose(sums.sum(axis=0), oracle.residual_sums(p, b, mask), rtol=1e-12)
