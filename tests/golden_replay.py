"""Replays of the golden vectors in tests/golden/ (written by make_golden.py
from the reference's own shaders) on any implementation with the
FluidSimulator / SmoothParticlesArea surface: the oracle (CPU tests) or the
GPU library (GPU tests)."""
from __future__ import annotations

import numpy as np


def replay_steps(data, fluid, density, on_keep):
    """Run the golden frame sequence (demo/simulation_demo.py:220-237 order)
    and call on_keep(step) at every step the fixture stores."""
    it, vort, visc, speed, diss, ddiss, dt = data["params"]
    fluid.iterations = int(it)
    fluid.vorticity = float(vort)
    fluid.viscosity = float(visc)
    fluid.speed = float(speed)
    fluid.dissipation = float(diss)
    density.speed = float(speed)
    density.dissipation = float(ddiss)
    forcing = data["forcing"]
    W = fluid.width
    keep = sorted(int(k.split("_")[1]) for k in data.files if k.startswith("vel_"))
    for s in range(forcing.shape[0]):
        fr = forcing[s]
        fluid.add_circle_obstacle((0.5, 0.5), W / 8)
        fluid.add_triangle_obstacle((0.1, 0.15), (0.3, 0.1), (0.2, 0.35), s % 2 == 0)
        fluid.update(1 / 60)
        density.update(1 / 60)
        fluid.add_velocity((float(fr[0]), float(fr[1])), (float(fr[2]), float(fr[3])),
                           float(fr[4]))
        density.add_particles((float(fr[5]), float(fr[6])), float(fr[7]), float(fr[8]))
        if s + 1 in keep:
            on_keep(s + 1)
    return keep


def assert_equal_f32(got, want, what):
    got = np.asarray(got)
    want = np.asarray(want)
    assert got.shape == want.shape, f"{what}: shape {got.shape} != {want.shape}"
    bad = np.argwhere(got != want)
    assert bad.size == 0, (f"{what}: {len(bad)} cells differ, first {bad[:3].tolist()}, "
                           f"max |d| {np.max(np.abs(got.astype(np.float64) - want))}")
