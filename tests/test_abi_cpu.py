"""Host-side checks that need no GPU: the library loads and exports every
entry point include/natrix.h declares, the Python surface matches the
reference's, and parameter validation raises like the reference."""
from __future__ import annotations

import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(natrix_\w+)\s*\(", text, re.M))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("natrix_create", "natrix_step", "natrix_destroy", "natrix_density_step",
                 "natrix_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from natrix_gb300 import _lib
    from natrix_gb300 import build as nb

    nb.build()
    lib = _lib.load()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"
    # every declared symbol has a ctypes signature in a binding
    from natrix_gb300.core import warmstart

    bound = set(_lib.SIGNATURES) | set(warmstart._SIGS)
    unbound = [n for n in declared_symbols() if n not in bound]
    assert not unbound, f"no ctypes signature: {unbound}"
    assert lib.natrix_version().startswith(b"natrix_gb300")


def test_last_error_is_empty_string_initially():
    from natrix_gb300 import _lib

    assert isinstance(_lib.load().natrix_last_error(), bytes)


def test_create_rejects_bad_sizes_without_gpu():
    import ctypes

    from natrix_gb300 import _lib

    h = ctypes.c_void_p()
    rc = _lib.load().natrix_create(0, 5, ctypes.byref(h))
    assert rc == _lib.NATRIX_EINVAL and not h
    rc = _lib.load().natrix_create(40000, 5, ctypes.byref(h))
    assert rc == _lib.NATRIX_ERANGE


def _bare(cls):
    return object.__new__(cls)


@pytest.mark.parametrize("prop,bad,msg", [
    ("speed", 0, "'Speed' should be greater than zero"),
    ("iterations", 0, "'Iterations' should be grater than zero"),
    ("dissipation", -1.0, "'Dissipation' should be grater than zero"),
    ("vorticity", -0.1, "'Vorticity' should be grater or equal than zero"),
    ("viscosity", -0.1, "'Viscosity' should be greater or equal than zero"),
])
def test_property_validation_matches_reference(prop, bad, msg):
    from natrix_gb300 import FluidSimulator

    sim = _bare(FluidSimulator)
    with pytest.raises(ValueError, match=re.escape(msg)):
        setattr(sim, prop, bad)
    setattr(sim, prop, {"speed": 3.0, "iterations": 7, "dissipation": 0.5,
                        "vorticity": 0.0, "viscosity": 0.0}[prop])


def test_defaults_match_reference():
    from natrix_gb300 import FluidSimulator, SmoothParticlesArea

    sim = _bare(FluidSimulator)
    assert (sim.speed, sim.iterations, sim.dissipation, sim.vorticity, sim.viscosity) == (
        500.0, 50, 1.0, 0.0, 0.1)
    assert FluidSimulator.has_borders is True and FluidSimulator.simulate is True
    d = _bare(SmoothParticlesArea)
    assert (d.speed, d.dissipation) == (500.0, 1.0)
    with pytest.raises(ValueError, match="'Dissipation' should be grater than zero"):
        d.dissipation = 0


def test_reference_import_path():
    from natrix.core.fluid_simulator import FluidSimulator as A

    from natrix_gb300 import FluidSimulator as B

    assert A is B
    # the demo's density class keeps its own import path
    # (demo/simulation_demo.py:29 of the reference)
    from demo.smooth_particles_area import SmoothParticlesArea as C

    from natrix_gb300 import SmoothParticlesArea as D

    assert C is D


def test_add_density_without_a_grid_raises():
    from natrix_gb300 import FluidSimulator

    sim = _bare(FluidSimulator)
    sim._density_grids = []
    with pytest.raises(RuntimeError, match="no density grid"):
        sim.add_density((0.5, 0.5), 1.0, 2.0)
    sim.simulate = False  # mutating calls are no-ops when simulate is False
    sim.add_density((0.5, 0.5), 1.0, 2.0)


def test_entry_points_validate_before_touching_the_device():
    """Arguments the C ABI refuses come back as error codes without any
    device call (so these run on a machine without a GPU): the no-allocation
    residual, the weight gradient's channel rule and the CG grid limits."""
    import ctypes

    from natrix_gb300 import _lib
    from natrix_gb300.core import warmstart as ws

    lib = _lib.load()
    nn = ws._lib_nn()
    P = ctypes.c_void_p
    fake = P(256)  # never dereferenced: validation fails first
    # natrix_residual_noalloc: NULL inputs, bad sizes, grids over the static scratch
    assert lib.natrix_residual_noalloc(None, fake, None, 8, 8, 8, fake, None) == _lib.NATRIX_EINVAL
    assert lib.natrix_residual_noalloc(fake, fake, None, 8, 8, 4, fake, None) == _lib.NATRIX_EINVAL
    assert lib.natrix_residual_noalloc(fake, fake, None, 8192, 8192, 8192, fake,
                                       None) == _lib.NATRIX_ERANGE
    assert b"static" in lib.natrix_last_error()
    # a row pitch the kernel's 32-bit indexing cannot hold has its own error
    assert lib.natrix_residual_noalloc(fake, fake, None, 8, 8, 1 << 31, fake,
                                       None) == _lib.NATRIX_ERANGE
    assert b"pitch" in lib.natrix_last_error()
    # weight gradient: channel counts must be multiples of 8
    assert nn.natrix_nn_wgrad(fake, 12, fake, 16, None, 0, 1, 8, 8, fake, fake,
                              None) == _lib.NATRIX_EINVAL
    assert b"multiples of 8" in lib.natrix_last_error()
    # CG: at most 65535 images and 2^31 cells per image
    assert nn.natrix_nn_cg_apply(fake, None, 70000, 8, 8, 32, fake, None) == _lib.NATRIX_ERANGE
    assert nn.natrix_nn_cg_axpy(fake, fake, fake, fake, 1.0, 2, 1 << 31, None) == _lib.NATRIX_ERANGE
    assert nn.natrix_nn_cg_update(fake, fake, fake, fake, fake, fake, fake, 70000, 64,
                                  None) == _lib.NATRIX_ERANGE
    # empty batches are a no-op
    assert nn.natrix_nn_cg_dir(fake, fake, fake, fake, 0, 64, None) == _lib.NATRIX_OK
