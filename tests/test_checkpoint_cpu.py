"""Checkpoint format on the CPU: training pairs round-trip exactly, foreign
or newer archives are refused."""
from __future__ import annotations

import numpy as np
import pytest


def test_pairs_round_trip(tmp_path):
    import torch

    from natrix_gb300 import checkpoint
    from natrix_gb300.core.warmstart import PairSet

    g = torch.Generator().manual_seed(0)
    pairs = PairSet(torch.randn(3, 8, 32, generator=g), (torch.rand(3, 8, 32, generator=g) > 0.8)
                    .to(torch.uint8), torch.rand(3, generator=g), torch.randn(3, 8, 8, generator=g),
                    torch.rand(3, dtype=torch.float64, generator=g), 17)
    path = checkpoint.save(tmp_path / "pairs.npz", pairs=pairs, compress=True)
    back = checkpoint.restore_pairs(checkpoint.read(path), device="cpu")
    for name in ("div", "mask", "inv_scale", "target", "rel_residual"):
        a, b = getattr(pairs, name), getattr(back, name)
        assert a.dtype == b.dtype and torch.equal(a, b), name
    assert back.cg_iterations == 17 and back.n == 3


def test_foreign_and_newer_archives_refused(tmp_path):
    from natrix_gb300 import checkpoint

    np.savez(tmp_path / "x.npz", a=np.zeros(2))
    with pytest.raises(ValueError, match="not a"):
        checkpoint.read(tmp_path / "x.npz")
    np.savez(tmp_path / "y.npz", format=np.array(checkpoint.FORMAT),
             version=np.array(checkpoint.VERSION + 1))
    with pytest.raises(ValueError, match="newer"):
        checkpoint.read(tmp_path / "y.npz")
