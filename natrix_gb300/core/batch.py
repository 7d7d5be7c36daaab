"""Many independent simulations of uneven sizes advanced together.

``FluidBatch`` drives the batched C ABI (natrix_batch_*): every simulation is
a FluidSimulator with a density grid of its own size; one launch per phase
covers all of them and the step is replayed from a captured CUDA graph.  The
Jacobi tile configuration and sweeps per launch are chosen per size class by
``autotune`` (timed on the batch itself, cached per GPU model).
"""
from __future__ import annotations

import ctypes
import json
from pathlib import Path

import numpy as np
import torch

from .. import _lib
from .._lib import Params, call
from .fluid_simulator import _stream

SIZE_CLASSES = ("side<=128", "side<=256", "side>256")
# (config, sweeps per launch) candidates: 0 = 64x32 shared-memory tiles,
# 1 = 112x112 register tiles, 2 = 112x128 register tiles
CANDIDATES = [(0, 8), (0, 4), (1, 8), (2, 8), (1, 4)]
CACHE = Path(__file__).resolve().parents[1] / "_lib" / "autotune.json"


def size_class(w: int, h: int) -> int:
    side = max(w, h)
    return 0 if side <= 128 else (1 if side <= 256 else 2)


class FluidBatch:
    def __init__(self, widths, heights):
        torch.cuda.init()
        self.widths = [int(w) for w in widths]
        self.heights = [int(h) for h in heights]
        self.n = len(self.widths)
        w = (ctypes.c_int32 * self.n)(*self.widths)
        h = (ctypes.c_int32 * self.n)(*self.heights)
        self._handle = ctypes.c_void_p()
        call("natrix_batch_create", self.n, w, h, ctypes.byref(self._handle))
        self.tuning = {}
        self.persistent = True

    @property
    def handle(self):
        if not self._handle:
            raise RuntimeError("batch has been destroyed")
        return self._handle

    def set_params(self, sim: int = -1, speed=500.0, iterations=50, dissipation=1.0,
                   vorticity=0.0, viscosity=0.1, has_borders=True):
        p = Params(float(speed), int(iterations), float(dissipation), float(vorticity),
                   float(viscosity), int(bool(has_borders)), 1, 0)
        call("natrix_batch_set_params", self.handle, int(sim), ctypes.byref(p))

    def set_density_params(self, sim: int = -1, speed=500.0, dissipation=1.0):
        call("natrix_batch_set_density_params", self.handle, int(sim), float(speed),
             float(dissipation))

    def set_tuning(self, size_cls: int, config: int, sweeps_per_launch: int):
        call("natrix_batch_set_tuning", self.handle, int(size_cls), int(config),
             int(sweeps_per_launch))
        self.tuning[int(size_cls)] = (int(config), int(sweeps_per_launch))

    def use_graph(self, enable: bool):
        call("natrix_batch_set_graph", self.handle, 1 if enable else 0)

    def use_persistent(self, enable: bool):
        """One persistent launch per step (default), or one launch per phase."""
        call("natrix_batch_set_persistent", self.handle, 1 if enable else 0)
        self.persistent = bool(enable)

    def add_velocity(self, sim, position, velocity, radius):
        call("natrix_batch_add_velocity", self.handle, int(sim), position[0], position[1],
             velocity[0], velocity[1], radius)

    def add_splats(self, sim, splats):
        arr = np.ascontiguousarray(splats, np.float32).reshape(-1, _lib.SPLAT_FLOATS)
        call("natrix_batch_add_splats", self.handle, int(sim),
             arr.ctypes.data, arr.shape[0])

    def add_circle_obstacle(self, sim, position, radius, static=False):
        call("natrix_batch_add_circle_obstacle", self.handle, int(sim), position[0], position[1],
             radius, 1 if static else 0)

    def add_splats_bulk(self, counts: np.ndarray, splats: np.ndarray):
        """All simulations' splats at once: counts[n], splats (sum(counts), 6)."""
        c = np.ascontiguousarray(counts, np.int32)
        arr = np.ascontiguousarray(splats, np.float32)
        call("natrix_batch_add_splats_bulk", self.handle, c.ctypes.data, arr.ctypes.data)

    def add_circles_bulk(self, counts: np.ndarray, circles: np.ndarray):
        """All simulations' discs at once: counts[n], circles (sum(counts), 3)."""
        c = np.ascontiguousarray(counts, np.int32)
        arr = np.ascontiguousarray(circles, np.float32)
        call("natrix_batch_add_circles_bulk", self.handle, c.ctypes.data, arr.ctypes.data)

    def step(self, dt: float):
        call("natrix_batch_step", self.handle, float(dt), _stream())

    def download(self, sim: int, field: int) -> np.ndarray:
        shape = (self.heights[sim], self.widths[sim])
        if field == _lib.FIELD_VELOCITY:
            shape = shape + (2,)
        out = np.empty(shape, np.float32)
        call("natrix_batch_download", self.handle, int(sim), int(field),
             out.ctypes.data_as(ctypes.c_void_p), _stream())
        torch.cuda.current_stream().synchronize()
        return out

    def launches(self):
        total = ctypes.c_int64()
        per = ctypes.c_int32()
        call("natrix_batch_launches", self.handle, ctypes.byref(total), ctypes.byref(per))
        return total.value, per.value

    def sync(self):
        call("natrix_batch_sync", self.handle, _stream())

    def classes(self):
        return sorted({size_class(w, h) for w, h in zip(self.widths, self.heights)})

    def autotune(self, steps: int = 3, dt: float = 1 / 60, cache: bool = True,
                 candidates=CANDIDATES) -> dict:
        """Pick (tile config, sweeps per launch) per size class by timing whole
        batch steps with CUDA events (queued forcing is not needed: the sweeps
        dominate).  Results are cached per GPU model and class signature."""
        key = self._cache_key()
        if cache and CACHE.exists():
            data = json.loads(CACHE.read_text())
            if key in data:
                for c, (cfg, spl) in data[key].items():
                    self.set_tuning(int(c), cfg, spl)
                return dict(self.tuning)
        best = {}
        for c in self.classes():
            timings = []
            for cfg, spl in candidates:
                self.set_tuning(c, cfg, spl)
                timings.append((self._time_steps(steps, dt), cfg, spl))
            _, cfg, spl = min(timings)
            self.set_tuning(c, cfg, spl)
            best[c] = (cfg, spl)
        self.sync()
        if cache:
            data = json.loads(CACHE.read_text()) if CACHE.exists() else {}
            data[key] = {str(c): list(v) for c, v in best.items()}
            CACHE.parent.mkdir(exist_ok=True)
            CACHE.write_text(json.dumps(data, indent=1))
        return best

    def _time_steps(self, steps: int, dt: float) -> float:
        """Milliseconds per batch step with the current tuning: two untimed
        steps, then `steps` steps between CUDA events on the current stream."""
        for _ in range(2):
            self.step(dt)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(steps):
            self.step(dt)
        ev1.record()
        ev1.synchronize()
        return ev0.elapsed_time(ev1) / steps

    def _cache_key(self) -> str:
        name = torch.cuda.get_device_name()
        hist = np.bincount([size_class(w, h) for w, h in zip(self.widths, self.heights)],
                           minlength=3)
        mode = "persistent" if getattr(self, "persistent", True) else "per-phase"
        return (f"{name}|{mode}|classes={hist.tolist()}"
                f"|cells={sum(w * h for w, h in zip(self.widths, self.heights))}")

    def destroy(self):
        if self._handle:
            call("natrix_batch_destroy", self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
