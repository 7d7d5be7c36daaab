"""The launch modes chosen once per process give bit-identical fields.

NATRIX_PDL=0 launches the step's kernels in plain stream order instead of
with programmatic dependent launch; NATRIX_JACOBI_VARIANT=0 runs the sweeps
with the shared-memory tile kernel on every grid (no register tiles, no tile
deal, gradient subtraction in its own launch), 1 / 2 / 3 / 4 with one
register tile shape (128x128, 128x144, 128x32, or 128x72 regions on 8-warp
CTAs two per SM) whatever the grid size;
NATRIX_SPARSE_FORCING=0 applies a step's velocity ops over the whole grid
instead of the blocks they reach (with the first op's clamp then done by the
advection's reads); NATRIX_JACOBI_CHAIN=0 runs a step's sweeps as one launch
per 8-sweep chunk instead of one persistent launch whose tiles wait on their
neighbours' previous chunk (used where the grid has a tile for every SM:
here with the 128x32 tiles, 640 of them).  Each mode runs in a child
process on the same seeded workload and must reproduce the default run's
velocity, pressure, divergence, vorticity and density bytes exactly."""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

SCRIPT = r"""
import hashlib, json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from natrix_gb300 import FluidSimulator, SmoothParticlesArea, _lib
from natrix_gb300 import workloads as wl

case = json.loads(sys.argv[2])
W, H = case["W"], case["H"]
sim = FluidSimulator(W, H)
den = SmoothParticlesArea(W, H, sim)
sim.iterations, sim.vorticity, sim.viscosity = case["K"], case["vort"], case["visc"]
sim.speed, sim.dissipation = 5.0, 0.99
den.speed, den.dissipation = 5.0, 0.99
rng = np.random.default_rng(7)
discs = wl.circle_obstacles(rng, 6, W, H, 0.03, 0.08)
out = {}
for step in range(6):
    for o in discs:
        sim.add_circle_obstacle((float(o[0]), float(o[1])), float(o[2]))
    sim.add_splats(wl.gauss_splats(rng, 5, W, H, 5.0), den)
    sim.update(1 / 60)
    den.update(1 / 60)
for name, field in (("velocity", _lib.FIELD_VELOCITY), ("pressure", _lib.FIELD_PRESSURE),
                    ("divergence", _lib.FIELD_DIVERGENCE), ("vorticity", _lib.FIELD_VORTICITY)):
    out[name] = hashlib.sha256(sim.download(field).tobytes()).hexdigest()
out["density"] = hashlib.sha256(den.download().tobytes()).hexdigest()
sim.sync()
print(json.dumps(out))
"""


# over 1024 forcing blocks: the step lists the blocks its splats reach
DEFAULT = {"W": 1056, "H": 1024, "K": 40, "vort": 0.35, "visc": 0.0}


def run_mode(env_extra, case=DEFAULT):
    env = dict(os.environ)
    for k in ("NATRIX_PDL", "NATRIX_JACOBI_VARIANT", "NATRIX_SPARSE_FORCING",
              "NATRIX_JACOBI_CHAIN"):
        env.pop(k, None)
    env.update(env_extra)
    res = subprocess.run([sys.executable, "-c", SCRIPT, str(ROOT), json.dumps(case)], env=env,
                         capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    return json.loads(res.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("env", [{"NATRIX_PDL": "0"}, {"NATRIX_JACOBI_VARIANT": "0"},
                                 {"NATRIX_JACOBI_VARIANT": "1"}, {"NATRIX_JACOBI_VARIANT": "2"},
                                 {"NATRIX_JACOBI_VARIANT": "3"}, {"NATRIX_SPARSE_FORCING": "0"},
                                 {"NATRIX_JACOBI_CHAIN": "0"},
                                 {"NATRIX_JACOBI_CHAIN": "0", "NATRIX_JACOBI_VARIANT": "3"}],
                         ids=["plain-stream-order", "shared-memory-sweeps", "register-tiles-a",
                              "register-tiles-b", "register-tiles-c", "full-grid-forcing",
                              "launch-per-chunk", "launch-per-chunk-c"])
def test_launch_mode_bit_identical(cuda, env):
    base = run_mode({})
    alt = run_mode(env)
    for k in base:
        assert alt[k] == base[k], f"{k} differs under {env}"


# 1792x1280: 192 tiles of 112x112 (the chain, tiles ordered by the marks) or,
# forced, 1280 tiles of 112x16 (the chain over more tiles than the marks
# cover: claimed in index order) or 368 tiles of 112x56 (8-warp CTAs, two
# per SM)
CHAIN = {"W": 1792, "H": 1280, "K": 40, "vort": 0.35, "visc": 0.0}


@pytest.mark.parametrize("env", [{"NATRIX_JACOBI_CHAIN": "0"}, {"NATRIX_JACOBI_VARIANT": "3"},
                                 {"NATRIX_JACOBI_VARIANT": "4"},
                                 {"NATRIX_JACOBI_VARIANT": "4", "NATRIX_JACOBI_CHAIN": "0"}],
                         ids=["launch-per-chunk", "short-tiles-unordered", "two-ctas-per-sm",
                              "two-ctas-per-sm-per-chunk"])
def test_sweep_chain_bit_identical(cuda, env):
    base = run_mode({}, CHAIN)
    alt = run_mode(env, CHAIN)
    for k in base:
        assert alt[k] == base[k], f"{k} differs under {env}"
