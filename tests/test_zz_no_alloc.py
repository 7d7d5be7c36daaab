"""natrix_residual_noalloc: the residual reduction for callers that cannot
allocate device memory (its scratch is a fixed array inside the library).

Checked through the C ABI against natrix_residual, the handle-based entry
point whose scratch natrix_create allocates, on two calls in a row with
different pressure systems; the tolerance is the one the residual's oracle
check uses (relative 1e-9: double sums).  This file is collected last so a
run that stops at the first failure has run every other test before it."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_residual_matches_handle_residual(cuda):
    import torch

    from natrix_gb300 import FluidSimulator, _lib

    lib = _lib.load()
    W, H = 150, 97
    sim = FluidSimulator(W, H)
    sim.iterations = 25
    rng = np.random.default_rng(31)
    mask = np.zeros((H, W), np.uint8)
    yy, xx = np.mgrid[0:H, 0:W]
    mask[(xx - 40) ** 2 + (yy - 50) ** 2 <= 12 ** 2] = 1
    mask[(xx - 110) ** 2 + (yy - 30) ** 2 <= 8 ** 2] = 2
    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)
    out = torch.zeros(5, dtype=torch.float64, device="cuda")

    for call in range(2):
        # a fresh pressure system each call: forcing, the step's own sweeps
        sim.upload(_lib.FIELD_OBSTACLES, mask)
        sim.add_velocity((rng.random(), rng.random()), tuple(rng.uniform(-1, 1, 2)), 20.0)
        sim.update(1 / 60)
        want = sim.residual_sums()

        p = sim.pressure
        div = sim.divergence
        pitch = p.stride(0)
        assert div.stride(0) == pitch
        # the caller's own mask buffer, laid out with the same row pitch
        dmask = torch.zeros((H, pitch), dtype=torch.uint8, device="cuda")
        dmask[:, :W] = torch.from_numpy(mask).cuda()
        rc = lib.natrix_residual_noalloc(_ptr(p), _ptr(div), _ptr(dmask), W, H, pitch,
                                         _ptr(out), sptr)
        _lib.check(rc)
        stream.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9,
                                   err_msg=f"call {call + 1}")
        assert got[0] == np.count_nonzero(mask == 0)

    # sizes beyond the static scratch are rejected with a clear error
    big = 4096 * 4096 + 1
    rc = lib.natrix_residual_noalloc(_ptr(p), _ptr(div), None, big, 1, big, _ptr(out), sptr)
    assert rc == _lib.NATRIX_ERANGE
    assert b"maximum" in lib.natrix_last_error()
    # so is a row pitch beyond the kernel's 32-bit row indexing (2^31 itself
    # included); nothing is launched
    rc = lib.natrix_residual_noalloc(_ptr(p), _ptr(div), None, W, H, 1 << 31, _ptr(out), sptr)
    assert rc == _lib.NATRIX_ERANGE
    assert b"pitch" in lib.natrix_last_error()
    sim.destroy()
