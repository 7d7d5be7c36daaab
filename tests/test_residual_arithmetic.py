"""The residual kernels' float-float arithmetic (ResidSums in
natrix_gb300/csrc/common.cuh), restated in NumPy float32 and checked against
extended precision on the CPU: the compensated six-term sum of the stencil
(Sum2), exact squares (TwoProd) and Dekker add2 running sums over a thread's
eight cells must give r within 1e-13 of the terms' magnitudes and the sums
of squares within 1e-13 over all threads, even where the stencil cancels
(pressures 4e5 times the divergence, as near convergence on a 2048x2048
grid).  The GPU tests then hold the kernels to 1e-9 of the oracle's FP64
sums."""
from __future__ import annotations

import numpy as np
import pytest

F32 = np.float32


def two_sum(a, b):
    s = (a + b).astype(F32)
    bb = (s - a).astype(F32)
    return s, ((a - (s - bb)).astype(F32) + (b - bb).astype(F32)).astype(F32)


def two_prod(a, b):
    # the low part of a float product is exact in double (the kernel uses an FMA)
    p = (a * b).astype(F32)
    e = (a.astype(np.float64) * b.astype(np.float64) - p.astype(np.float64)).astype(F32)
    return p, e


def ff_add(ah, al, bh, bl):
    sh, sl = two_sum(ah, bh)
    e = (sl + (al + bl).astype(F32)).astype(F32)
    h = (sh + e).astype(F32)
    return h, (e - (h - sh).astype(F32)).astype(F32)


def resid_sums(b, pc, x1, x2, y1, y2):
    """Per-thread sums over axis 1 (cells), as ResidSums::add does cell by cell."""
    z = np.zeros(b.shape[0], F32)
    acc = {k: (z.copy(), z.copy()) for k in ("r", "rr", "b", "bb")}
    for k in range(b.shape[1]):
        th, c = two_sum(b[:, k], -x1[:, k])
        for t in (-x2[:, k], -y1[:, k], -y2[:, k], (F32(4) * pc[:, k]).astype(F32)):
            th, e = two_sum(th, t)
            c = (c + e).astype(F32)
        rh, rl = two_sum(th, c)
        acc["r"] = ff_add(*acc["r"], rh, rl)
        sh, sl = two_prod(rh, rh)
        sl = (sl + (F32(2) * rh * rl).astype(F32)).astype(F32)
        acc["rr"] = ff_add(*acc["rr"], sh, sl)
        acc["b"] = ff_add(*acc["b"], b[:, k], z)
        acc["bb"] = ff_add(*acc["bb"], *two_prod(b[:, k], b[:, k]))
    return {k: h.astype(np.float64) + l for k, (h, l) in acc.items()}


@pytest.mark.parametrize("scale", [1.0, 1e5, 4e5])
def test_float_float_residual_sums(scale):
    rng = np.random.default_rng(int(scale))
    T, N = 20000, 8
    pc = (rng.normal(size=(T, N)) * scale).astype(F32)
    # neighbours close to the centre: the stencil cancels to a small residual
    nb = [(pc + rng.normal(size=(T, N)).astype(F32) * F32(scale * 1e-3)).astype(F32)
          for _ in range(4)]
    b = rng.normal(size=(T, N)).astype(F32)
    L = np.longdouble
    r = b.astype(L) - ((nb[0].astype(L) + nb[1] + nb[2] + nb[3]) - 4 * pc.astype(L))
    want = {"r": r.sum(1), "rr": (r * r).sum(1), "b": b.astype(L).sum(1),
            "bb": (b.astype(L) ** 2).sum(1)}
    got = resid_sums(b, pc, *nb)
    w = {k: v.astype(np.float64) for k, v in want.items()}
    # r: within 1e-13 of the sum of the six terms' magnitudes (the Sum2 bound)
    terms = (np.abs(b).astype(L) + sum(np.abs(x).astype(L) for x in nb) +
             4 * np.abs(pc).astype(L)).sum(1).astype(np.float64)
    assert (np.abs(got["r"] - w["r"]) / terms).max() < 1e-13
    # r^2 per thread follows from that bound (r is small next to the terms);
    # b and b^2 carry no cancellation
    assert (np.abs(got["rr"] - w["rr"]) / w["rr"]).max() < 1e-9
    assert (np.abs(got["b"] - w["b"]) / np.abs(b).astype(np.float64).sum(1)).max() < 1e-13
    assert (np.abs(got["bb"] - w["bb"]) / w["bb"]).max() < 1e-13
    # over all threads, as the kernel's block and grid sums add them
    for k in ("rr", "bb"):
        assert abs(got[k].sum() - float(want[k].sum())) / float(want[k].sum()) < 1e-13
    # plain FP32 would not do: its stencil loses r entirely at these scales
    if scale >= 1e5:
        r32 = (b - ((nb[0] + nb[1] + nb[2] + nb[3]) - F32(4) * pc)).astype(F32)
        rel32 = np.abs((r32.astype(np.float64) ** 2).sum(1) - want["rr"].astype(np.float64)) / \
            want["rr"].astype(np.float64)
        assert rel32.max() > 1e-6
