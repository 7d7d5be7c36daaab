"""A step captured into a CUDA graph replays like stepping eagerly.

The sweep chain (one persistent launch for a step's sweeps on grids with a
tile for every SM) leaves its counters zeroed at the end of every launch, so
its launch parameters are the same each step and a captured step can be
replayed.  The queued splats are applied inside the captured step, so each
replay repeats them, as re-adding the same splats before each eager step
does."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H", [(1792, 1280), (200, 136)], ids=["chain", "launch-per-chunk"])
def test_captured_step_replays_like_eager_steps(cuda, W, H):
    import torch

    from natrix_gb300 import FluidSimulator, _lib
    from natrix_gb300 import workloads as wl

    rng = np.random.default_rng(5)
    splats = wl.gauss_splats(rng, 6, W, H, 5.0)

    def make():
        sim = FluidSimulator(W, H)
        sim.iterations, sim.vorticity, sim.viscosity = 40, 0.35, 0.0
        sim.speed, sim.dissipation = 5.0, 0.99
        return sim

    eager, graphed = make(), make()
    for sim in (eager, graphed):  # one eager step each: kernel attributes set, obstacles reset
        sim.add_splats(splats)
        sim.update(1 / 60)
    torch.cuda.synchronize()

    for _ in range(3):
        eager.add_splats(splats)
        eager.update(1 / 60)

    capture = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    graphed.add_splats(splats)
    with torch.cuda.graph(graph, stream=capture):
        graphed.update(1 / 60)
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()

    for field in (_lib.FIELD_VELOCITY, _lib.FIELD_PRESSURE, _lib.FIELD_DIVERGENCE,
                  _lib.FIELD_VORTICITY):
        a, b = eager.download(field), graphed.download(field)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"field {field} differs"
    eager.sync()
    graphed.sync()
    eager.destroy()
    graphed.destroy()
