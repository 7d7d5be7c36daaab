"""Headless visualisation kernels (natrix_render_density, natrix_quiver)
against the oracle's restatement of the demo's display shaders: every byte
and every arrow bit-exact, on odd sizes (scalar path), aligned sizes (16-byte
path), special values (NaN, negative, > 1, exact UNORM boundaries) and on a
live simulation's fields."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _density_cases(rng):
    odd = rng.uniform(-0.2, 1.2, (131, 257)).astype(np.float32)
    odd[0, :8] = [np.nan, -0.0, 0.0, 1.0, 2.0, 0.5 / 255, 254.5 / 255, np.inf]
    ramp = (np.arange(256, dtype=np.float32) / np.float32(255)).reshape(1, 256)
    ramp = np.repeat(ramp, 4, axis=0)
    wide = rng.uniform(0, 1, (256, 512)).astype(np.float32)
    return [odd, ramp, wide]


def test_render_density_bit_exact(cuda, oracle):
    import torch

    from natrix_gb300 import render

    rng = np.random.default_rng(3)
    for rho in _density_cases(rng):
        tex, col = render.render_density(torch.from_numpy(rho).cuda())
        torch.cuda.synchronize()
        wt, wc = oracle.render_density(rho)
        np.testing.assert_array_equal(tex.cpu().numpy(), wt)
        np.testing.assert_array_equal(col.cpu().numpy(), wc)
    # a pitched view (row stride > width) and one output only
    base = torch.from_numpy(rng.uniform(0, 1, (64, 100)).astype(np.float32)).cuda()
    view = base[:, 3:80]
    _, col = render.render_density(view, texture=False)
    np.testing.assert_array_equal(col.cpu().numpy(),
                                  oracle.render_density(view.cpu().numpy())[1])


def test_render_live_density_and_quiver(cuda, oracle):
    import torch

    from natrix_gb300 import FluidSimulator, SmoothParticlesArea, render
    from natrix_gb300 import workloads as wl

    W, H = 192, 128
    sim = FluidSimulator(W, H)
    den = SmoothParticlesArea(W, H, sim)
    sim.iterations, sim.vorticity, sim.viscosity, sim.speed, sim.dissipation = 20, 0.35, 0, 5.0, 0.99
    rng = np.random.default_rng(8)
    for _ in range(6):
        sim.add_circle_obstacle((0.4, 0.5), 10.0)
        sim.add_splats(wl.gauss_splats(rng, 6, W, H, 5.0), den)
        sim.update(1 / 60)
        den.update(1 / 60)
    tex, col = render.render_density(den)
    rho = den.density.cpu().numpy()
    wt, wc = oracle.render_density(rho)
    np.testing.assert_array_equal(tex.cpu().numpy(), wt)
    np.testing.assert_array_equal(col.cpu().numpy(), wc)
    v = sim.get_velocity_buffer().cpu().numpy()
    assert np.abs(v).max() > 0.01
    # integer tiles take the tile-per-block kernel, 12.5 the per-pixel one
    for window, tile in (((2 * W, 2 * H), 16.0), ((333, 217), 8.0), ((W, H), 64.0),
                         ((1000, 700), 32.0), ((301, 203), 12.5)):
        arrows, ov = render.quiver(sim, window, tile)
        torch.cuda.synchronize()
        wa, wo = oracle.quiver(v, window[0], window[1], tile)
        assert arrows.shape == wa.shape
        np.testing.assert_array_equal(arrows.cpu().numpy(), wa)
        np.testing.assert_array_equal(ov.cpu().numpy(), wo)
    # the composed frame is the overlay blended over the field colour
    arrows, ov = render.quiver(sim, (W, H), 16.0)
    frame = render.blend_over(ov, col)
    assert frame.shape == (H, W, 4)
    den.destroy()
    sim.destroy()


def test_render_rejects_bad_arguments(cuda):
    import torch

    from natrix_gb300 import render

    with pytest.raises(ValueError):
        render.render_density(torch.zeros(4, 4, dtype=torch.float64, device="cuda"))
    with pytest.raises(ValueError):
        render.quiver(torch.zeros(4, 4, 2, device="cuda"), (8, 8), 0.5)
