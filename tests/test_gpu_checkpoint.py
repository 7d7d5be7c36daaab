"""Checkpoint and resume on the GPU: a run interrupted by save -> fresh
objects -> load continues bit-identically to the uninterrupted run (fluid
fields, density, particles); the network's weights and Adam state resume
to the same next update."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _make(W, H, n_particles, seed):
    from natrix_gb300 import FluidSimulator, SmoothParticlesArea
    from natrix_gb300.core.particles import LagrangianParticles

    sim = FluidSimulator(W, H)
    sim.iterations, sim.vorticity, sim.viscosity, sim.speed, sim.dissipation = 30, 0.35, 0.1, 5.0, 0.99
    den = SmoothParticlesArea(W, H, sim)
    den.speed, den.dissipation = 5.0, 0.98
    rng = np.random.default_rng(seed)
    pos = np.stack([rng.uniform(0, W - 1, n_particles), rng.uniform(0, H - 1, n_particles)], 1)
    parts = LagrangianParticles(sim, pos.astype(np.float32))
    return sim, den, parts


def _steps(sim, den, parts, rng, n):
    from natrix_gb300 import workloads as wl

    W, H = sim.width, sim.height
    for _ in range(n):
        sim.add_circle_obstacle((0.3, 0.6), 7.0)
        sim.add_triangle_obstacle((0.6, 0.2), (0.8, 0.25), (0.7, 0.5), True)
        sim.add_splats(wl.gauss_splats(rng, 5, W, H, 5.0), den)
        sim.update(1 / 60)
        den.update(1 / 60)
        parts.step(1 / 60)


def _fields(sim, den, parts):
    from natrix_gb300 import _lib

    return [sim.download(f) for f in (_lib.FIELD_VELOCITY, _lib.FIELD_PRESSURE,
                                      _lib.FIELD_OBSTACLES)] + [den.download(), parts.download()]


def test_resume_is_bit_identical(cuda, tmp_path):
    from natrix_gb300 import checkpoint

    W, H = 160, 96
    sim, den, parts = _make(W, H, 5000, 1)
    rng = np.random.default_rng(2)
    _steps(sim, den, parts, rng, 4)
    path = checkpoint.save(tmp_path / "state.npz", sim=sim, density=den, particles=parts)
    state = rng.bit_generator.state
    _steps(sim, den, parts, rng, 5)
    want = _fields(sim, den, parts)
    for o in (parts, den, sim):
        o.destroy()

    sim2, den2, parts2 = _make(W, H, 5000, 99)  # different initial particles
    sim2.iterations, den2.dissipation = 3, 0.5  # overwritten by the checkpoint
    checkpoint.load(path, sim=sim2, density=den2, particles=parts2)
    assert sim2.iterations == 30 and den2.dissipation == 0.98
    rng2 = np.random.default_rng()
    rng2.bit_generator.state = state
    _steps(sim2, den2, parts2, rng2, 5)
    got = _fields(sim2, den2, parts2)
    for i, (a, b) in enumerate(zip(got[:4], want[:4])):
        np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8), err_msg=f"field {i}")
    np.testing.assert_array_equal(got[4], want[4])
    with pytest.raises(ValueError):
        from natrix_gb300 import FluidSimulator

        other = FluidSimulator(W + 16, H)
        try:
            checkpoint.load(path, sim=other)
        finally:
            other.destroy()
    for o in (parts2, den2, sim2):
        o.destroy()


def test_network_resume(cuda, tmp_path):
    """Weights, Adam moments and the step count restore exactly; training
    then continues like the uninterrupted run (the weight gradients sum with
    FP32 atomics, so the continuation agrees to rounding, not bit for bit)."""
    import torch

    from natrix_gb300 import checkpoint
    from natrix_gb300.core import warmstart as ws

    pairs = ws.make_pairs(64, 4, seed=3, rtol=1e-5, batch=4)
    net = ws.UNet(seed=0)
    ws.train(net, pairs, steps=3, batch=4)
    saved = {k: v.clone() for k, v in net.state_dict().items()}
    moments = [(m.clone(), v.clone()) for _, _, m, v in net.parameters()]
    path = checkpoint.save(tmp_path / "net.npz", net=net, pairs=pairs)
    ws.train(net, pairs, steps=2, batch=4, seed=5)
    want = {k: v.clone() for k, v in net.state_dict().items()}

    net2 = ws.UNet(seed=7)
    d = checkpoint.load(path, net=net2)
    assert net2.step_count == 3
    for k, v in net2.state_dict().items():
        assert torch.equal(v, saved[k]), k
    for (m0, v0), (_, _, m, v) in zip(moments, net2.parameters()):
        assert torch.equal(m, m0) and torch.equal(v, v0)
    pairs2 = checkpoint.restore_pairs(d)
    assert torch.equal(pairs2.target.cpu(), pairs.target.cpu())
    ws.train(net2, pairs2, steps=2, batch=4, seed=5)
    got = net2.state_dict()
    for k in want:
        if k == "head.b":
            # the loss is invariant to a constant shift of the prediction, so
            # this gradient is rounding noise that Adam scales to full steps
            continue
        step = (want[k] - saved[k]).abs().max().item()
        assert (got[k] - want[k]).abs().max().item() <= 2e-2 * max(step, 1e-6) + 1e-7, k
