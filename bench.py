"""Benchmark of the per-step fluid solver (cell-updates/s, % of HBM roofline).

Default workload: 2048x2048 FP32, vorticity confinement 0.35, viscosity 0, 80
Jacobi sweeps, 12 circular obstacles re-added every step, 16 Gaussian splats
per step on velocity and density, density advection, dt = 1/60.  A "step" is
one frame: obstacles, forcing, FluidSimulator.update, SmoothParticlesArea.update.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl natrix|reference]
                  [--workload large|small|particles|batch|warmstart|unet-forward|
                              unet-train|render|aux]

The other workloads print their own line: particles (4M Lagrangian particles
coupled to a 1024x1024 solver), batch (512 simulations of uneven size in one
graph-captured launch per phase), warmstart (network training on solver pairs
and the time to a residual target with and without the network's guess),
unet-forward / unet-train (network throughput), render (display buffers) and
aux (the kernels outside the default step, each timed at full size).

One JSON line on rank 0.  `value` is timed with CUDA events on the launching
stream with the fields resident on the device (the per-step forcing records,
~1.5 KB, travel host->device inside the kernel launches' parameter blocks, as
they do for any caller).
`e2e` adds, every step, a device->host read of the density frame into pinned
host memory through the C ABI (on a copy stream, overlapping the next step).  `roofline` is the Jacobi
phase (the dominant kernel), timed live with CUDA events around its launches.
`cpu_baseline` times the CPU oracle (float32, all host threads) on a bounded
sample of the same workload.  `--impl reference` times that CPU
implementation alone, as the reference arm.

Multi-GPU: the path does not shard (one simulation per GPU); with N ranks each
rank advances its own replica ("replicas only", weak scaling) and `value` is
the total over ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import csv
import ctypes
import json
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from natrix_gb300 import replicas  # noqa: E402
from natrix_gb300 import workloads as wl  # noqa: E402

# Algorithmic bytes per cell (float2 velocity 8 B, float scalars 4 B, uint8
# obstacle mask and neighbour flags 1 B; each kernel reads its inputs once and
# writes its outputs once).
BYTES = {
    "forcing": 24,           # velocity r/w 16 + density r/w 8
    "advect": 17,            # velocity in 8, mask 1, velocity out 8
    "density_advect": 17,    # density in 4, velocity 8, mask 1, density out 4
    "vorticity_calc": 12,    # velocity 8, vorticity out 4
    "vorticity_apply": 20,   # velocity 8, vorticity 4, velocity out 8
    "divergence": 13,        # velocity 8, mask 1, divergence out 4
    "jacobi_sweep": 13,      # pressure 4, divergence 4, flags 1, pressure out 4
    "subtract_gradient": 21, # velocity 8, pressure 4, flags 1, velocity out 8
}


def step_bytes_per_cell(spec: wl.Workload) -> int:
    """Per-sweep-equivalent model: every kernel of the reference's dispatch
    list (one per Jacobi sweep) reads its inputs and writes its outputs once.
    Temporal blocking never moves most of these bytes, so this is a work
    measure, not a bandwidth bound."""
    b = BYTES["forcing"] + BYTES["advect"] + BYTES["density_advect"] + BYTES["divergence"]
    b += BYTES["subtract_gradient"] + BYTES["jacobi_sweep"] * spec.iterations
    if spec.vorticity > 0:
        b += BYTES["vorticity_calc"] + BYTES["vorticity_apply"]
    return b


# Algorithmic bytes per cell of the launches this build runs (each launch
# reads its inputs once and writes its outputs once):
LAUNCH_BYTES = {
    "forcing": 24,          # velocity r/w 16 + density r/w 8
    "advect": 17,
    "density_advect": 17,
    "vorticity": 20,        # curl and confinement in one pass: velocity in 8 + out 8, vorticity 4
    "divergence": 18,       # velocity 8, mask 1, divergence 4, flags 1, first sweep's pressure 4
    "sweep_launch": 13,     # pressure 4, divergence 4, flags 1 read; pressure 4 written
    "fused_gradient": 16,   # velocity in 8 + out 8 on the last sweep launch
    "subtract_gradient": 21,
}


def step_floor_bytes_per_cell(spec: wl.Workload, sweep_chunks: float, fused: float) -> float:
    """Attainable floor of one step with the launch structure run here:
    sweep_chunks chunks of up to 8 sweeps per step (each reads its inputs and
    writes the pressure once), `fused` of which (0 or 1) also subtract the
    gradient."""
    b = (LAUNCH_BYTES["forcing"] + LAUNCH_BYTES["advect"] + LAUNCH_BYTES["density_advect"]
         + LAUNCH_BYTES["divergence"] + LAUNCH_BYTES["sweep_launch"] * sweep_chunks
         + LAUNCH_BYTES["fused_gradient"] * fused
         + LAUNCH_BYTES["subtract_gradient"] * (1.0 - fused))
    if spec.vorticity > 0:
        b += LAUNCH_BYTES["vorticity"]
    return b


def issue_roof(instructions, launch_ms, clocks):
    """Warp instructions issued per second by the sweep launch against the
    SMs' issue limit (4 per SM per clock at the sampled SM clock)."""
    import torch

    if not instructions or not launch_ms:
        return None
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz")
    if not mhz:
        return None
    achieved = instructions / (launch_ms / 1e3)
    peak = 4.0 * sms * mhz * 1e6
    return {"warp_instructions_per_launch": instructions, "achieved_per_s": achieved,
            "peak_per_s": peak, "frac": achieved / peak, "sm_mhz": mhz}


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """SM clock, its maximum and the clock-event reasons during the timed
    region: back to back (every 0.2 ms) through NVML (ctypes on the driver's
    libnvidia-ml, read-only queries) from a thread, or every 200 ms from nvidia-smi when
    NVML cannot be loaded."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason* bits (nvml.h)
    REASON_BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20,
                   "hw_thermal_slowdown": 0x40}

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None
        self.rows = []  # NVML samples: (sm_mhz, max_mhz, reasons bitmask)
        self.thread = None
        self.stop = None
        self.nvml = None

    def _nvml_open(self):
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            return None
        h = ctypes.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.gpu), ctypes.byref(h)) != 0:
            lib.nvmlShutdown()
            return None
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        return lib, h, reasons

    def _poll(self):
        lib, h, reasons = self.nvml
        sm, mx, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        # the maximum clock is a constant of the board: read it once, then
        # poll the current clock and the event reasons back to back
        if lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) != 0:
            return
        while not self.stop.is_set():
            if (lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(sm)) == 0 and
                    reasons(h, ctypes.byref(rs)) == 0):
                self.rows.append((sm.value, mx.value, rs.value))
            self.stop.wait(0.0002)

    def __enter__(self):
        import threading
        try:
            self.nvml = self._nvml_open()
        except (OSError, AttributeError):
            self.nvml = None
        if self.nvml is not None:
            self.stop = threading.Event()
            self.thread = threading.Thread(target=self._poll, daemon=True)
            self.thread.start()
            return self
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.thread is not None:
            self.stop.set()
            self.thread.join(timeout=5)
            self.nvml[0].nvmlShutdown()
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.thread is not None:
            if not self.rows:
                return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
            names = sorted(n for n, bit in self.REASON_BITS.items()
                           if any(r[2] & bit for r in self.rows))
            return {"sm_mhz": float(np.median([r[0] for r in self.rows])),
                    "sm_max_mhz": float(max(r[1] for r in self.rows)), "reasons": names,
                    "samples": len(self.rows), "source": "nvml"}
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = []
        with open(self.path) as f:
            for r in csv.reader(f):
                if len(r) >= 9:
                    rows.append([c.strip() for c in r])
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows), "source": "nvidia-smi"}


def make_spec(name: str) -> wl.Workload:
    return {"large": wl.LARGE_2048, "small": wl.SMALL_256,
            "particles": wl.PARTICLES_1024}[name]


def workload_config(spec: wl.Workload, extra=None):
    cfg = {"workload": spec.name, "grid": [spec.width, spec.height],
           "jacobi_sweeps": spec.iterations, "vorticity": spec.vorticity,
           "viscosity": spec.viscosity, "dissipation": spec.dissipation, "speed": spec.speed,
           "dt": spec.dt, "splats_per_step": spec.splats_per_step,
           "obstacles": spec.n_obstacles, "density_grid": [spec.width, spec.height],
           "dtype": "fp32", "l2": "working set per step > L2 (no explicit flush)"}
    if extra:
        cfg.update(extra)
    return cfg


# ------------------------------------------------------------------ CPU legs
def cpu_run(spec: wl.Workload, steps: int, warmup: int, seed: int = 0):
    """Time the float32 CPU oracle (OpenMP, all host threads) on `steps`
    frames after `warmup` frames; returns (seconds per step, threads)."""
    from oracle import oracle as O

    f = O.OracleFluid(spec.width, spec.height, np.float32)
    d = O.OracleDensity(spec.width, spec.height, f)
    f.iterations, f.vorticity, f.viscosity = spec.iterations, spec.vorticity, spec.viscosity
    f.speed, f.dissipation = spec.speed, spec.dissipation
    d.speed, d.dissipation = spec.speed, spec.dissipation
    obst = wl.workload_obstacles(seed, spec)
    times = []
    for i in range(warmup + steps):
        splats = wl.step_forcing(seed, i, spec)
        t0 = time.perf_counter()
        for o in obst:
            f.add_circle_obstacle((float(o[0]), float(o[1])), float(o[2]))
        f.add_splats(splats, d)
        f.update(spec.dt)
        d.update(spec.dt)
        if i >= warmup:
            times.append(time.perf_counter() - t0)
    return float(np.mean(times)), O.num_threads()


def cpu_sample_steps(spec: wl.Workload) -> int:
    """Frames of the cpu_baseline sample: about 10 s of CPU work."""
    return 160 if spec.width >= 1024 else 2000


# most frames the reference arm times (2000 x ~60 ms at 2048x2048)
REFERENCE_MAX_STEPS = 2000


def run_reference(args, spec):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    cells = spec.width * spec.height
    # the same K timed frames after W warm-up frames as the GPU arm (about
    # 60 ms per 2048x2048 frame on 16 host threads), capped so that the run
    # stays within a few minutes
    steps = max(1, min(args.steps, REFERENCE_MAX_STEPS))
    warm = max(0, min(args.warmup, REFERENCE_MAX_STEPS))
    sec, threads = cpu_run(spec, steps, warm)
    value = cells / sec
    sample = f"{steps} timed frames after {warm} warm-up of the {spec.width}x{spec.height} workload"
    line = {
        "impl": "reference", "metric": "cell-updates/s", "value": value,
        "unit": "cell-updates/s", "n_gpus": args.gpus, "steps": steps, "warmup": warm,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded splats and discs)",
        "config": workload_config(spec, {"parallelism": f"replicas{world}"}),
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": ("the reference's own path is bgfx compute shaders that need a graphics "
                 "stack (unavailable on this box); its CPU stand-in is the C oracle, a "
                 "float32 restatement of those shaders pinned bit-for-bit to them"),
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU leg
def measure_grid(spec: wl.Workload, steps: int, warmup: int, seed: int, barrier=None,
                 local: int = 0, sample_clocks: bool = True) -> dict:
    """One single-grid workload through the public API: `warmup` untimed
    frames, `steps` frames between CUDA events on the launching stream, the
    next `steps` frames again with the Jacobi phases also bracketed by the
    library's own events (events between launches stop programmatic
    dependent launch from overlapping them, so the step time is taken
    without them), then `steps` more frames end to end, each with its
    density frame read back into pinned host memory.  Returns the times and
    the library's launch statistics of the second pass."""
    import torch

    from natrix_gb300 import FluidSimulator, SmoothParticlesArea, _lib

    barrier = barrier or (lambda: None)
    W, H = spec.width, spec.height
    sim = FluidSimulator(W, H)
    den = SmoothParticlesArea(W, H, sim)
    sim.iterations, sim.vorticity, sim.viscosity = spec.iterations, spec.vorticity, spec.viscosity
    sim.speed, sim.dissipation = spec.speed, spec.dissipation
    den.speed, den.dissipation = spec.speed, spec.dissipation
    obst = wl.workload_obstacles(seed, spec)
    total = warmup + 3 * steps
    forcing = [wl.step_forcing(seed, i, spec) for i in range(total)]
    stream = torch.cuda.current_stream()

    def frame(i):
        for o in obst:
            sim.add_circle_obstacle((float(o[0]), float(o[1])), float(o[2]))
        sim.add_splats(forcing[i], den)
        sim.update(spec.dt)
        den.update(spec.dt)

    for i in range(warmup):
        frame(i)
    sim.sync()
    torch.cuda.synchronize()

    lib = _lib.load()
    stats = _lib.Stats()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) if sample_clocks else _NoClocks() as clocks:
        ev0.record(stream)
        for i in range(warmup, warmup + steps):
            frame(i)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    sim.sync()

    # the same number of frames with the Jacobi phases timed by the library
    lib.natrix_get_stats(sim.handle, stats, 1)
    lib.natrix_set_timing(sim.handle, 1)
    ev2, ev3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    ev2.record(stream)
    for i in range(warmup + steps, warmup + 2 * steps):
        frame(i)
    ev3.record(stream)
    torch.cuda.synchronize()
    barrier()
    lib.natrix_set_timing(sim.handle, 0)
    ms_phase_events = ev2.elapsed_time(ev3)
    _lib.check(lib.natrix_get_stats(sim.handle, stats, 1))
    sim.sync()

    # e2e: the same frames through the C ABI, each frame's density read back
    # into pinned host memory.  The read of frame k runs on a copy stream
    # while frame k+1 computes (frame k+1 only reads that buffer); frame k+2,
    # which overwrites it, waits for the copy.  The clock stops after the
    # last copy has landed.
    hosts = [torch.empty((H, W), dtype=torch.float32).pin_memory() for _ in range(2)]
    hptrs = [ctypes.c_void_p(h.data_ptr()) for h in hosts]
    copy_stream = torch.cuda.Stream()
    cptr = ctypes.c_void_p(copy_stream.cuda_stream)
    copied = [None, None]
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for k, i in enumerate(range(warmup + 2 * steps, total)):
        if copied[k % 2] is not None:
            stream.wait_event(copied[k % 2])
        frame(i)
        ready = torch.cuda.Event()
        ready.record(stream)
        copy_stream.wait_event(ready)
        _lib.check(lib.natrix_density_download(den.handle, hptrs[k % 2], cptr))
        copied[k % 2] = torch.cuda.Event()
        copied[k % 2].record(copy_stream)
    copy_stream.synchronize()
    stream.synchronize()
    t_e2e = time.perf_counter() - t0
    barrier()
    sim.sync()
    den.destroy()
    sim.destroy()
    return {"ms": ms, "ms_phase_events": ms_phase_events, "ms_e2e": t_e2e * 1e3, "stats": stats,
            "clocks": clocks.summary()}


class _NoClocks:
    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def summary(self):
        return None


def run_natrix(args, spec):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            dist.barrier()

    W, H = spec.width, spec.height
    cells = W * H
    seed = replicas.replica_seed(rank)
    m = measure_grid(spec, args.steps, args.warmup, seed, barrier, local)
    ms, t_e2e, stats = m["ms"], m["ms_e2e"] / 1e3, m["stats"]
    launches = int(stats.kernel_launches)

    ms, ms_e2e, ms_ev = replicas.max_over_ranks([ms, t_e2e * 1e3, m["ms_phase_events"]],
                                                device="cuda")
    value = replicas.whole_job_rate(cells * args.steps, world, ms / 1e3)
    e2e_value = replicas.whole_job_rate(cells * args.steps, world, ms_e2e / 1e3)

    peak, peak_kind = load_peaks()
    step_b = step_bytes_per_cell(spec)
    jl = max(int(stats.timed_launches), 1)
    launch_ms = stats.jacobi_ms / jl
    sweeps_per_launch = stats.timed_sweeps / jl
    # Algorithmic bytes of one sweep launch: pressure, divergence and flags
    # read once, pressure written once, whatever the number of sweeps it
    # fuses; a launch that also subtracts the pressure gradient (the last of
    # a step when fused) reads and writes the velocity as well.
    fused_per_launch = int(stats.timed_fused) / jl
    # a chunk is the up to 8 sweeps a tile keeps on chip; on grids with a
    # tile for every SM one persistent launch runs all chunks of a step
    chunks_per_launch = max(1, math.ceil(sweeps_per_launch / 8 - 1e-9))
    chain = chunks_per_launch > 1
    alg_bytes = (LAUNCH_BYTES["sweep_launch"] * chunks_per_launch +
                 LAUNCH_BYTES["fused_gradient"] * fused_per_launch) * cells
    achieved = alg_bytes / (launch_ms / 1e3) / 1e9
    profile = ("jacobi_chain_%dx%d.txt" if chain else "jacobi_rt_%dx%d.txt") % (W, H)
    traffic = load_traffic(profile)
    instructions = load_instructions(profile)
    sweep_launches_per_step = jl / max(int(stats.timed_phases), 1)
    chunks_per_step = sweep_launches_per_step * chunks_per_launch
    fused_per_step = int(stats.timed_fused) / max(int(stats.timed_phases), 1)
    floor_b = step_floor_bytes_per_cell(spec, chunks_per_step, fused_per_step)
    if chain:
        kernel_desc = ("jacobi sweep chain: every 8-sweep chunk of the step in one persistent "
                       "launch (TMA tiles; a tile waits for its 3x3 neighbours' previous chunk)")
        bytes_model = ("13 B per cell per chunk (pressure, divergence, flags read once; "
                       "pressure written once), plus 16 B per cell (velocity in and out) on "
                       "the last chunk, which also subtracts the gradient")
    else:
        kernel_desc = "jacobi sweep launch (temporally blocked, TMA tiles)"
        bytes_model = ("13 B per cell per launch (pressure, divergence, flags read once; "
                       "pressure written once), plus 16 B per cell (velocity in and out) on "
                       "the launch that also subtracts the gradient")

    if rank == 0:
        # per-frame host->device bytes (carried in the launches' parameter
        # blocks): splat records for velocity and density, obstacle shapes,
        # two step-parameter blocks (sizes of the C structs)
        h2d = 32 * spec.splats_per_step * 2 + 32 * spec.n_obstacles + 48 * 2
        cpu = None
        if not args.no_cpu:
            csec, threads = cpu_run(spec, cpu_sample_steps(spec), 1)
            cpu = {"value": cells / csec, "unit": "cell-updates/s", "cores": threads,
                   "kind": "port",
                   "sample": f"{cpu_sample_steps(spec)} frames after 1 warm-up, "
                             f"{W}x{H}, float32 C oracle (OpenMP)"}
        line = {
            "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Gaussian splats and non-overlapping discs)",
            "config": workload_config(spec, {"parallelism": f"replicas{world}"}),
            # the whole step against the attainable floor of the launches it
            # runs (each launch reads its inputs and writes its outputs once)
            "hbm_roofline_step": {
                "bytes_per_cell_step": floor_b,
                "sweep_launches_per_step": sweep_launches_per_step,
                "sweep_chunks_per_step": chunks_per_step,
                "achieved_gbs": value * floor_b / 1e9,
                "frac": value * floor_b / 1e9 / peak,
                "peak_gbs": peak, "peak_kind": peak_kind,
                "frac_of_nominal_8000": value * floor_b / 1e9 / 8000.0},
            # work measure, not a bandwidth: the reference's dispatch list
            # moves these bytes (one Jacobi dispatch per sweep)
            "per_sweep_equivalent": {
                "bytes_per_cell_step": step_b,
                "gbs": value * step_b / 1e9},
            # Jacobi cell-sweeps per second: inside the step (all K sweeps of
            # every timed step over the whole step time) and inside the
            # Jacobi phase alone (sweeps over the phase's own launch time)
            "jacobi_cell_sweeps_per_s": {
                "per_step_time": value * spec.iterations,
                "per_jacobi_time": cells * sweeps_per_launch / (launch_ms / 1e3) * world},
            "roofline": {"kernel": kernel_desc,
                         "bound": "hbm",
                         # what the kernel's time is spent on (its profile):
                         # the HBM fraction below is of its algorithmic bytes
                         "limiter": "FP32 issue and the per-sweep CTA barrier (8 sweeps "
                                    "on chip per chunk), not DRAM",
                         "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "dram_gbs": (traffic / (launch_ms / 1e3) / 1e9) if traffic else None,
                         "dram_frac": (traffic / (launch_ms / 1e3) / 1e9 / peak)
                         if traffic else None,
                         "peak_kind": peak_kind,
                         "launch_ms": launch_ms, "sweeps_per_launch": sweeps_per_launch,
                         "chunks_per_launch": chunks_per_launch,
                         # CUDA events around each step's Jacobi phase, in a
                         # second timed pass of as many frames (the events
                         # keep the phase's first and last launch from
                         # overlapping their neighbours)
                         "launch_ms_pass": {"steps": args.steps,
                                            "ms_per_step": ms_ev / args.steps},
                         "bytes_per_launch": alg_bytes,
                         "bytes_model": bytes_model,
                         "traffic_source": "profiles/" + profile,
                         # the issue roof the kernel is held under: warp
                         # instructions per launch (same profile) over the
                         # launch time, against 4 per SM and clock
                         "issue": issue_roof(instructions, launch_ms, m["clocks"])},
            "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": cells * 4},
            "gpu_launches": launches,
            "gpu_launches_per_step": launches / args.steps,
            "clocks": m["clocks"],
            "cpu_baseline": cpu,
        }
        if not args.no_extras and world == 1:
            line["other_configs"] = other_configs(args)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def other_configs(args) -> dict:
    """Short measurements of the other workloads, attached to the default
    line: the 256x256 solver over its full 200 steps (with its CPU oracle
    rate), the 4M-particle step and the 512-simulation batch (20 steps each).
    Each is timed with CUDA events like its own bench line."""
    out = {}
    small = wl.SMALL_256
    m = measure_grid(small, small.steps, 5, 0, sample_clocks=False)
    cells = small.width * small.height
    value = cells * small.steps / (m["ms"] / 1e3)
    entry = {"workload": small.name, "steps": small.steps, "ms_per_step": m["ms"] / small.steps,
             "value": value, "unit": "cell-updates/s",
             "e2e": cells * small.steps / (m["ms_e2e"] / 1e3),
             "gpu_launches_per_step": int(m["stats"].kernel_launches) / small.steps}
    if not args.no_cpu:
        csec, threads = cpu_run(small, small.steps, 1)
        entry["cpu_baseline"] = {"value": cells / csec, "cores": threads, "kind": "port",
                                 "sample": f"{small.steps} frames after 1 warm-up"}
        entry["vs_cpu"] = value / (cells / csec)
    out["small_256"] = entry
    ns = argparse.Namespace(steps=20, warmup=5, no_cpu=True)
    p = particles_line(ns, wl.PARTICLES_1024)
    out["particles_4m"] = {"workload": p["config"]["workload"], "steps": 20,
                           "ms_per_step": p["ms_per_step"], "value": p["value"],
                           "unit": p["unit"], "coupled_frame": p["coupled_frame"]}
    b = batch_line(ns)
    out["batch_512"] = {k: b[k] for k in ("ms_per_step", "value", "unit",
                                          "hbm_roofline_step", "gpu_launches_per_step",
                                          "launch_per_phase")
                        if k in b}
    out["batch_512"]["workload"] = b["config"]["workload"]
    out["batch_512"]["steps"] = 20
    if "e2e" in b:
        out["batch_512"]["e2e"] = b["e2e"]
    return out


def load_traffic(profile):
    """DRAM bytes (read + write) per Jacobi launch from the committed ncu
    summary `profiles/<profile>` (jacobi_rt_<W>x<H>.txt for the launch per
    chunk, jacobi_chain_<W>x<H>.txt for the one-launch chain), if any."""
    p = ROOT / "profiles" / profile
    if not p.exists():
        return None
    vals = [float(line.split()[-1]) for line in p.read_text().splitlines()
            if "traffic (dram read + write) MB" in line]
    return sum(vals) / len(vals) * 1e6 if vals else None


def load_instructions(profile):
    """Warp instructions per Jacobi launch (smsp__inst_executed.sum) from the
    same committed ncu summary, if any."""
    p = ROOT / "profiles" / profile
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        parts = line.split()
        if parts[:1] == ["smsp__inst_executed.sum"] and len(parts) >= 3 and parts[2] == "M":
            return float(parts[1]) * 1e6
    return None


def run_particles(args, spec):
    print(json.dumps(particles_line(args, spec)), flush=True)


def particles_line(args, spec):
    """Lagrangian particles coupled to the solver: particle-steps/s of the
    particle kernel (RK2 + 3x3 splat) and of the whole coupled frame."""
    import torch

    from natrix_gb300 import FluidSimulator
    from natrix_gb300.core.particles import LagrangianParticles

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    W, H, n = spec.width, spec.height, wl.N_PARTICLES
    sim = FluidSimulator(W, H)
    sim.iterations, sim.vorticity, sim.viscosity = spec.iterations, spec.vorticity, spec.viscosity
    sim.speed, sim.dissipation = spec.speed, spec.dissipation
    parts = LagrangianParticles(sim, wl.uniform_particles(0, n, W, H))
    obst = wl.workload_obstacles(0, spec)
    forcing = [wl.step_forcing(0, i, spec) for i in range(args.warmup + args.steps)]
    stream = torch.cuda.current_stream()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]

    def frame(i, ev=None):
        for o in obst:
            sim.add_circle_obstacle((float(o[0]), float(o[1])), float(o[2]))
        sim.add_splats(forcing[i])
        sim.update(spec.dt)
        if ev:
            ev[0].record(stream)
        parts.step(spec.dt)
        if ev:
            ev[1].record(stream)

    for i in range(args.warmup):
        frame(i)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clocks:
        e0.record(stream)
        for k in range(args.steps):
            frame(args.warmup + k, evs[k])
        e1.record(stream)
        torch.cuda.synchronize()
    sim.sync()
    frame_ms = e0.elapsed_time(e1) / args.steps
    part_ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
    peak, peak_kind = load_peaks()
    alg = 16.0 * n + 4.0 * W * H  # positions read + write, density clear
    line = {
        "metric": "particle-steps/s", "value": n / (part_ms / 1e3), "unit": "particle-steps/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": part_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (uniform particles, seeded splats and discs)",
        "config": workload_config(spec, {"particles": n}),
        "coupled_frame": {"ms_per_step": frame_ms,
                          "particle_steps_per_s": n / (frame_ms / 1e3),
                          "cell_updates_per_s": W * H / (frame_ms / 1e3)},
        "roofline": {"kernel": "particles (RK2 + 3x3 splat, red.add.f32)", "bound": "hbm",
                     "achieved": alg / (part_ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": alg / (part_ms / 1e3) / 1e9 / peak, "traffic": None,
                     "peak_kind": peak_kind,
                     "bytes_model": "16 B per particle + 4 B per density cell",
                     "limiter": "the splat's float atomics in L2, not DRAM",
                     "atomics_per_s": 9.0 * n / (part_ms / 1e3)},
        "clocks": clocks.summary(),
    }
    parts.destroy()
    sim.destroy()
    return line


def run_batch(args):
    print(json.dumps(batch_line(args)), flush=True)


def batch_line(args):
    """512 independent simulations (sides 64-512, 20/40/80 sweeps, 0-6 discs,
    8 splats each per step): one persistent launch per step (the default),
    the same step as one graph-replayed launch per phase, and looping the
    single-grid simulator over the same simulations."""
    import torch

    from natrix_gb300 import FluidSimulator, SmoothParticlesArea
    from natrix_gb300.core.batch import FluidBatch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    spec = wl.BATCH_512
    sides, its = spec.sides(), spec.iterations()
    n = spec.n_sims
    total_steps = args.warmup + args.steps
    obst = [spec.obstacles(i, int(sides[i])) for i in range(n)]
    ocounts = np.array([len(o) for o in obst], np.int32)
    ocat = np.concatenate([o for o in obst if len(o)] or [np.zeros((0, 3), np.float32)])
    forcing = [np.concatenate([spec.forcing(i, k, int(sides[i])) for i in range(n)])
               for k in range(total_steps)]
    fcounts = np.full(n, spec.splats_per_step, np.int32)
    batch = FluidBatch(list(sides), list(sides))
    for i in range(n):
        batch.set_params(i, speed=5.0, iterations=int(its[i]), dissipation=0.99, vorticity=0.0,
                         viscosity=0.0)
    batch.set_density_params(-1, speed=5.0, dissipation=0.99)
    stream = torch.cuda.current_stream()

    def frame(k):
        batch.add_circles_bulk(ocounts, ocat)
        batch.add_splats_bulk(fcounts, forcing[k])
        batch.step(1 / 60)

    def timed(sample_clocks):
        for k in range(args.warmup):
            frame(k)
        batch.sync()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) if sample_clocks \
                else _NoClocks() as clocks:
            e0.record(stream)
            for k in range(args.warmup, total_steps):
                frame(k)
            e1.record(stream)
            torch.cuda.synchronize()
        batch.sync()
        return e0.elapsed_time(e1) / args.steps, clocks.summary()

    # the default (one persistent launch per step), then the same work as
    # one graph-replayed launch per phase
    batch.use_persistent(True)
    tuning = batch.autotune()
    ms, clock_summary = timed(True)
    launches_total, per_step = batch.launches()
    batch.use_persistent(False)
    tuning_phased = batch.autotune()
    ms_phased, _ = timed(False)
    _, per_step_phased = batch.launches()
    cells = float((sides.astype(np.float64) ** 2).sum())
    # per-sweep model (every sweep an HBM pass) and the floor of the launch
    # structure run: forcing 24, advection 17, divergence with the first
    # sweep 18, 13 per sweep item chain of 8 sweeps, gradient subtraction
    # 21, density advection 17 B per cell
    cells_each = sides.astype(np.float64) ** 2
    model_bytes = float((cells_each * (92 + 13 * its)).sum())
    sweep_launches = np.ceil((its - 1) / 8.0)
    floor_bytes = float((cells_each * (24 + 17 + 18 + 13 * sweep_launches + 21 + 17)).sum())
    batch.destroy()

    # looping the single-grid simulator over the same simulations
    loop_ms = None
    if not args.no_cpu:
        sims = []
        for i in range(n):
            s = FluidSimulator(int(sides[i]), int(sides[i]))
            d = SmoothParticlesArea(int(sides[i]), int(sides[i]), s)
            s.speed, s.iterations, s.dissipation, s.vorticity, s.viscosity = (
                5.0, int(its[i]), 0.99, 0.0, 0.0)
            d.speed, d.dissipation = 5.0, 0.99
            sims.append((s, d))
        loop_steps = 3
        off = np.concatenate([[0], np.cumsum(fcounts)])

        def loop_frame(k):
            f = forcing[k]
            for i, (s, d) in enumerate(sims):
                for o in obst[i]:
                    s.add_circle_obstacle((float(o[0]), float(o[1])), float(o[2]))
                s.add_splats(f[off[i]:off[i + 1]], d)
                s.update(1 / 60)
                d.update(1 / 60)

        loop_frame(0)
        torch.cuda.synchronize()
        l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0.record(stream)
        for k in range(1, 1 + loop_steps):
            loop_frame(k)
        l1.record(stream)
        torch.cuda.synchronize()
        loop_ms = l0.elapsed_time(l1) / loop_steps
        for s, d in sims:
            d.destroy()
            s.destroy()
    peak, peak_kind = load_peaks()
    line = {
        "metric": "cell-updates/s", "value": cells / (ms / 1e3), "unit": "cell-updates/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded sides, sweeps, discs and splats)",
        "config": {"workload": spec.name, "simulations": n, "cells": cells,
                   "sides": [int(sides.min()), int(sides.max())],
                   "jacobi_sweeps": {str(k): int((its == k).sum()) for k in (20, 40, 80)},
                   "tuning": {wl_name: list(v) for wl_name, v in
                              zip(("side<=128", "side<=256", "side>256"),
                                  [tuning.get(c, (None, None)) for c in range(3)])}},
        "hbm_roofline_step": {"bytes_per_step": floor_bytes,
                              "achieved_gbs": floor_bytes / (ms / 1e3) / 1e9,
                              "frac": floor_bytes / (ms / 1e3) / 1e9 / peak, "peak_gbs": peak,
                              "peak_kind": peak_kind,
                              "limiter": "the Jacobi items' sweeps (FP32 issue), not DRAM"},
        # work measure, not a bandwidth: one HBM pass per sweep
        "per_sweep_equivalent": {"bytes_per_step": model_bytes,
                                 "gbs": model_bytes / (ms / 1e3) / 1e9},
        "gpu_launches_per_step": per_step,
        "launch_per_phase": {"ms_per_step": ms_phased, "value": cells / (ms_phased / 1e3),
                             "gpu_launches_per_step": per_step_phased,
                             "tuning": {str(c): list(v) for c, v in tuning_phased.items()},
                             "time_vs_persistent": ms_phased / ms},
        "looped_single_grid": None if loop_ms is None else {
            "ms_per_step": loop_ms, "value": cells / (loop_ms / 1e3),
            "speedup_of_batch": loop_ms / ms},
        "clocks": clock_summary,
    }
    return line


def run_warmstart(args):
    """Learned warm start: train on solver-generated 512x512 pairs, then time
    the solve to relative residual 1e-4 at 512x512, 1024x1024 and 2048x2048
    from zero and from the network's guess (with the fallback rule)."""
    import torch

    from natrix_gb300.core import warmstart as ws

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    t0 = time.perf_counter()
    pairs = ws.make_pairs(512, args.pairs, seed=0, rtol=1e-6, batch=64)
    t_data = time.perf_counter() - t0
    net = ws.UNet(seed=0)
    t0 = time.perf_counter()
    losses = ws.train(net, pairs, steps=args.train_steps, batch=64, lr=1e-3, lam=1.0)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    # tensor-core convolution throughput: one forward of a 64 x 512 x 512 batch
    div, mask, inv = pairs.div[:64].contiguous(), pairs.mask[:64].contiguous(), pairs.inv_scale[:64].contiguous()
    P = div.shape[2]
    for _ in range(2):
        net.forward(div, mask, inv, 512, 512, P)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        net.forward(div, mask, inv, 512, 512, P)
    e1.record()
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1) / 5
    flops, _ = ws.forward_cost(64, 512, 512)
    results = {}
    for size in (512, 1024, 2048):
        sim, m = ws.evaluation_system(size, seed=7)
        regions = ws.Regions(m.view(1, size, -1), 1, size, size)
        removed = ws.project_divergence(sim, regions)
        exact = ws.exact_pressure(sim, regions)
        floor = ws.fp32_floor(sim, regions, exact)
        # 1e-4 where FP32 storage of the pressure can reach it with margin,
        # else the first of these tolerances at least 3x above the floor
        rtol = next(t for t in (1e-4, 2e-4, 5e-4, 1e-3, 2e-3, 5e-3, 1e-2) if t >= 3 * floor)
        diag = ws.guess_diagnostics(sim, net, m, regions, exact)
        zero = ws.warm_start_solve(sim, None, m, rtol=rtol, time_limit_s=args.solve_limit,
                                   regions=regions)
        cnn = ws.warm_start_solve(sim, net, m, rtol=rtol, time_limit_s=args.solve_limit,
                                  regions=regions)
        forced = ws.warm_start_solve(sim, net, m, rtol=rtol, time_limit_s=args.solve_limit,
                                     regions=regions, force=True)
        sim.destroy()
        results[str(size)] = {"rtol": rtol, "fp32_floor": floor, "mean_removed": removed,
                              "zero": zero, "network": cnn, "network_forced": forced,
                              "guess": diag,
                              "speedup": zero["seconds"] / max(cnn["seconds"], 1e-9),
                              "speedup_forced": zero["seconds"] / max(forced["seconds"], 1e-9)}
    peak = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["bf16_tflops"] \
        if (ROOT / "MEASURED_PEAKS.json").exists() else 1900.0
    line = {
        "metric": "seconds to the relative-residual target at 2048x2048 (network warm start)",
        "value": results["2048"]["network"]["seconds"], "unit": "s", "n_gpus": 1,
        "steps": args.train_steps, "warmup": 0, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 (f32 accumulate), f32 sweeps",
        "data": "synthetic (solver-generated pairs)",
        "config": {"workload": "unet-warm-start", "train_grid": 512, "pairs": pairs.n,
                   "train_steps": args.train_steps, "batch": 64, "lr": 1e-3,
                   "cg_rel_residual_max": float(pairs.rel_residual.max()),
                   "cg_iterations": pairs.cg_iterations},
        "loss": {"first10": float(np.mean(losses[:10])), "last10": float(np.mean(losses[-10:]))},
        "time": {"data_s": t_data, "train_s": t_train,
                 "train_images_per_s": args.train_steps * 64 / t_train},
        "conv_forward": {"batch": 64, "grid": 512, "ms": fwd_ms, "tflops": flops / fwd_ms / 1e9,
                         "peak_tflops": peak, "frac": flops / fwd_ms / 1e9 / peak},
        "solve": results,
    }
    print(json.dumps(line), flush=True)


def run_render(args):
    """Headless display of a 2048x2048 density frame: texture + plasma colour
    (12 bytes per pixel: 4 read, 8 written) and a 4096x4096 quiver overlay of
    the velocity (16-pixel tiles), timed with CUDA events per frame."""
    import torch

    from natrix_gb300 import FluidSimulator, SmoothParticlesArea, render

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    spec = make_spec("large")
    W, H = spec.width, spec.height
    sim = FluidSimulator(W, H)
    den = SmoothParticlesArea(W, H, sim)
    sim.iterations, sim.vorticity, sim.viscosity, sim.speed, sim.dissipation = (
        spec.iterations, spec.vorticity, spec.viscosity, spec.speed, spec.dissipation)
    den.speed, den.dissipation = spec.speed, spec.dissipation
    rng = np.random.default_rng(3)
    for _ in range(5):
        sim.add_splats(wl.gauss_splats(rng, spec.splats_per_step, W, H, spec.speed), den)
        sim.update(spec.dt)
        den.update(spec.dt)
    rho = den.density
    vel = sim.get_velocity_buffer()
    tex = torch.empty(H, W, 4, dtype=torch.uint8, device="cuda")
    col = torch.empty_like(tex)
    win = (2 * W, 2 * H)
    nx, ny = render.quiver_tiles(win, 16.0)
    arrows = torch.empty(ny, nx, 2, device="cuda")
    ov = torch.empty(win[1], win[0], 4, dtype=torch.uint8, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    from natrix_gb300._lib import load as natrix_lib

    lib = natrix_lib()

    def density_frame():
        return lib.natrix_render_density(ctypes.c_void_p(rho.data_ptr()), W, H, rho.stride(0),
                                  ctypes.c_void_p(tex.data_ptr()), ctypes.c_void_p(col.data_ptr()),
                                  W, st)

    def quiver_frame():
        return lib.natrix_quiver(ctypes.c_void_p(vel.data_ptr()), W, H, vel.stride(0) // 2, win[0],
                          win[1], ctypes.c_float(16.0), ctypes.c_void_p(arrows.data_ptr()),
                          ctypes.c_void_p(ov.data_ptr()), win[0], st)

    def timed(fn):
        for _ in range(args.warmup):
            if fn() != 0:
                raise RuntimeError(lib.natrix_last_error().decode())
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    d_ms, q_ms = timed(density_frame), timed(quiver_frame)
    hbm, kind = load_peaks()
    d_bytes = 12.0 * W * H
    q_bytes = 4.0 * win[0] * win[1]
    line = {
        "metric": "density frames/s (2048x2048 texture + colour)", "value": 1e3 / d_ms,
        "unit": "frames/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": d_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u8 (f32 in)", "data": "synthetic (solver frames)",
        "config": {"workload": "render-2048x2048+quiver-4096x4096-tile16",
                   "l2": "density 16.8 MB read, 33.6 MB written per frame (< L2)"},
        "roofline": {"bound": "hbm", "achieved": d_bytes / d_ms / 1e6, "peak": hbm,
                     "unit": "GB/s", "frac": d_bytes / d_ms / 1e6 / hbm, "traffic": None,
                     "peak_kind": kind},
        "quiver": {"ms": q_ms, "gbs": q_bytes / q_ms / 1e6, "frac": q_bytes / q_ms / 1e6 / hbm,
                   "window": list(win), "tiles": [nx, ny]},
    }
    print(json.dumps(line), flush=True)
    den.destroy()
    sim.destroy()


def run_unet_train(args):
    """Warm-start network training throughput: Adam steps (forward, loss,
    backward, update) on --batch x 512 x 512 synthetic inputs against a fixed
    synthetic target, timed with CUDA events; the training images/s the
    warm-start leg reports, without its data generation."""
    import torch

    from natrix_gb300.core import warmstart as ws

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    B, H, W = args.batch, 512, 512
    P = (W + 31) // 32 * 32
    g = torch.Generator(device="cuda").manual_seed(0)
    div = torch.randn(B, H, P, device="cuda", generator=g)
    mask = (torch.rand(B, H, P, device="cuda", generator=g) < 0.05).to(torch.uint8)
    inv = ws.inv_scale_of(div[:, :, :W], mask[:, :, :W])
    target = torch.randn(B, H, W, device="cuda", generator=g)
    net = ws.UNet(seed=0)
    for _ in range(args.warmup):
        net.train_step(div, mask, inv, target, H, W, P)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        net.train_step(div, mask, inv, target, H, W, P)
    e1.record()
    torch.cuda.synchronize()
    net.check_status()
    ms = e0.elapsed_time(e1) / args.steps
    print(json.dumps({
        "metric": "U-Net training images/s (512x512)", "value": B / ms * 1e3, "unit": "images/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 (f32 accumulate, f32 master weights)", "data": "synthetic",
        "config": {"workload": f"unet-train-{B}x512x512", "batch": B, "optimizer": "adam"},
    }), flush=True)


def run_aux(args):
    """The kernels outside the default step, each at a full working size and
    timed with CUDA events over --steps calls after --warmup, so that every
    kernel of the library has a measured bandwidth (ncu launch lists of this
    workload give the per-kernel split):

    * on a 2048x2048 system after 5 steps of the large workload's settings:
      the FP64 residual (natrix_residual: two launches and a 40-byte read-back
      with a host wait per call), the per-region residual
      (natrix_residual_regions), the allocation-free residual
      (natrix_residual_noalloc), 80 Jacobi sweeps (natrix_jacobi, 10 launches
      of 8; NATRIX_JACOBI_VARIANT=0 selects the shared-memory sweep kernel)
      and a step with viscosity 0.1 (its extra launch, against one without);
    * the FP64 conjugate-gradient kernels on 16 x 512 x 512;
    * Adam over the warm-start network's parameters, with the bf16 repack;
    * the integer cells of 4M particles (natrix_particles_cells, with the
      32 MB read-back into pinned host memory).

    Algorithmic bytes per cell or element (each input read once, each output
    written once): residual 10 (pressure, divergence, mask, flags), per-region
    residual 13 (pressure, divergence, flags, label), allocation-free 9
    (pressure, divergence, mask), sweep launch 13, CG apply 17 (direction 8,
    mask 1, product 8), dot 17, axpy 24, direction update 24, fused apply+dot
    17, fused update 48 (x, r, d, q read; x, r written), Adam 28 per
    parameter (weight, gradient, two moments read; weight and moments
    written)."""
    import torch

    from natrix_gb300 import _lib
    from natrix_gb300.core import warmstart as ws
    from natrix_gb300.core.particles import LagrangianParticles

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    hbm, kind = load_peaks()
    lib = _lib.load()

    def timed(fn, n=None):
        n = n or args.steps
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    kernels = {}

    def report(name, ms, nbytes, launches, note=None):
        gbs = nbytes / ms / 1e6
        kernels[name] = {"us_per_call": ms * 1e3, "bytes": nbytes, "launches_per_call": launches,
                         "gbs": gbs, "frac": gbs / hbm}
        if note:
            kernels[name]["note"] = note

    # 2048x2048 solver system
    N = 2048
    sim, mask = ws.evaluation_system(N, seed=7)
    cells = N * N
    regions = ws.Regions(mask.view(1, N, -1), 1, N, N)
    labels, n_labels = regions.image_labels(0)
    sums = torch.empty(n_labels, 5, dtype=torch.float64, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p, div = sim.pressure, sim.divergence
    pitch = p.stride(0)
    dmask = torch.zeros(N, pitch, dtype=torch.uint8, device="cuda")
    dmask[:, :N] = mask.view(N, -1)[:, :N]
    out5 = torch.empty(5, dtype=torch.float64, device="cuda")

    report("residual", timed(sim.residual_sums), 10.0 * cells, 2,
           "per call: k_residual, k_residual_final, 40-byte read-back, host wait")

    def regions_call():
        _lib.check(lib.natrix_residual_regions(sim.handle, ctypes.c_void_p(labels.data_ptr()),
                                               n_labels, ctypes.c_void_p(sums.data_ptr()), st))

    report("residual_regions", timed(regions_call), 13.0 * cells, 1,
           f"k_residual_labels over {n_labels} regions (plus a memset of the sums)")

    def noalloc_call():
        _lib.check(lib.natrix_residual_noalloc(ctypes.c_void_p(p.data_ptr()),
                                               ctypes.c_void_p(div.data_ptr()),
                                               ctypes.c_void_p(dmask.data_ptr()), N, N, pitch,
                                               ctypes.c_void_p(out5.data_ptr()), st))

    report("residual_noalloc", timed(noalloc_call), 9.0 * cells, 2,
           "k_residual_noalloc, k_residual_noalloc_final")
    variant = "shared-memory (k_jacobi_tb)" if os.environ.get("NATRIX_JACOBI_VARIANT") == "0" \
        else "register-tiled (k_jacobi_rt)"
    report("jacobi_80_sweeps", timed(lambda: sim.jacobi(80)), 10 * 13.0 * cells, 10,
           f"{variant}, 10 launches of 8 sweeps")

    rng = np.random.default_rng(11)

    def step():
        sim.add_splats(wl.gauss_splats(rng, 16, N, N, 5.0))
        sim.update(1 / 60)

    plain_ms = timed(step)
    sim.viscosity = 0.1
    viscous_ms = timed(step)
    sim.viscosity = 0.0
    report("viscosity", max(viscous_ms - plain_ms, 1e-6), 16.0 * cells, 1,
           f"step with viscosity 0.1 ({viscous_ms:.4f} ms) minus without ({plain_ms:.4f} ms); "
           "k_viscosity reads and writes the velocity")
    sim.sync()

    # FP64 conjugate-gradient kernels, 16 x 512 x 512
    B, H, W = 16, 512, 512
    P = (W + 31) // 32 * 32
    g = torch.Generator(device="cuda").manual_seed(0)
    m = (torch.rand(B, H, P, device="cuda", generator=g) < 0.05).to(torch.uint8)
    d = torch.randn(B, H, W, dtype=torch.float64, device="cuda", generator=g)
    r = torch.randn_like(d)
    x = torch.zeros_like(d)
    q = torch.empty_like(d)
    rr = torch.ones(B, dtype=torch.float64, device="cuda")
    rr2, dq = torch.ones_like(rr), torch.ones_like(rr)
    per, n_el = H * W, B * H * W
    P_ = ws._p
    S = ws._s
    report("cg_apply", timed(lambda: ws._call("natrix_nn_cg_apply", P_(d), P_(m), B, H, W, P,
                                              P_(q), S())), 17.0 * n_el, 1)
    report("cg_dot", timed(lambda: ws._call("natrix_nn_cg_dot", P_(d), P_(q), P_(m), B, H, W, P,
                                            P_(dq), S())), 17.0 * n_el, 1,
           "FP64 sums per image")
    # axpy adds +-rr/dq times the direction: alternate the sign so x stays bounded
    report("cg_axpy", timed(lambda: (ws._call("natrix_nn_cg_axpy", P_(x), P_(d), P_(rr), P_(dq),
                                              1.0, B, per, S()),
                                     ws._call("natrix_nn_cg_axpy", P_(x), P_(d), P_(rr), P_(dq),
                                              -1.0, B, per, S()))) / 2, 24.0 * n_el, 1)
    report("cg_dir", timed(lambda: ws._call("natrix_nn_cg_dir", P_(d), P_(r), P_(rr2), P_(rr), B,
                                            per, S())), 24.0 * n_el, 1,
           "direction = r + (rr_new / rr) direction, with rr_new = rr")
    report("cg_apply_dot", timed(lambda: ws._call("natrix_nn_cg_apply_dot", P_(d), P_(m), B, H, W,
                                                  P, P_(q), P_(dq), S())), 17.0 * n_el, 1,
           "fused apply and d.q (q = 0 on obstacles)")
    # update with rr = 0: x and r are rewritten unchanged, rr_new recomputed
    zero = torch.zeros_like(rr)
    report("cg_update", timed(lambda: ws._call("natrix_nn_cg_update", P_(x), P_(r), P_(d), P_(q),
                                               P_(zero), P_(dq), P_(rr2), B, per, S())),
           48.0 * n_el, 1, "fused x += a d, r -= a q and r.r")

    # Adam over the network's parameters, then the bf16 repack of the weights
    net = ws.UNet(seed=0)
    n_params = sum(w.numel() for w, _, _, _ in net.parameters())
    n_tensors = len(net.parameters())
    report("adam", timed(lambda: net.adam(lr=1e-6)), 28.0 * n_params,
           n_tensors + 2 * len(net.layers),
           f"{n_params} parameters in {n_tensors} tensors, plus {2 * len(net.layers)} "
           "k_pack launches (launch-bound)")

    # integer cells of 4M particles in a 1024x1024 fluid
    spec = wl.PARTICLES_1024
    from natrix_gb300 import FluidSimulator

    fluid = FluidSimulator(spec.width, spec.height)
    n = wl.N_PARTICLES
    parts = LagrangianParticles(fluid, wl.uniform_particles(0, n, spec.width, spec.height))
    host = torch.empty(n, 2, dtype=torch.int32, pin_memory=True)

    def cells_call():
        _lib.check(lib.natrix_particles_cells(parts.handle, ctypes.c_void_p(host.data_ptr()), st))

    report("particle_cells", timed(cells_call), 16.0 * n, 1,
           "k_particle_cells (positions 8 B in, cells 8 B out) plus the 32 MB read-back "
           "to pinned host memory, which dominates")
    parts.destroy()
    fluid.destroy()
    sim.destroy()
    worst = min(v["frac"] for k, v in kernels.items() if k not in ("adam", "particle_cells"))
    print(json.dumps({
        "metric": "auxiliary kernels: per-region residual HBM GB/s (2048x2048)",
        "value": kernels["residual_regions"]["gbs"], "unit": "GB/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": kernels["residual_regions"]["us_per_call"] / 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 fields, f64 sums", "data": "synthetic (solver state, seeded fields)",
        "config": {"workload": "aux-kernels-2048x2048+cg-16x512x512+4M-particles",
                   "l2": "2048x2048 fields re-read back to back (within L2 between calls)",
                   "jacobi_variant": variant},
        "peak": hbm, "peak_kind": kind, "lowest_frac_bandwidth_bound": worst,
        "kernels": kernels,
    }), flush=True)


def run_unet_forward(args):
    """Warm-start network inference throughput: one forward pass of
    --batch x 512 x 512 (synthetic divergence and obstacle fields) per step,
    timed with CUDA events; roofline against the forward's algorithmic HBM
    bytes (warmstart.forward_cost), tensor FLOP/s reported beside it."""
    import torch

    from natrix_gb300.core import warmstart as ws

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    B, H, W = args.batch, 512, 512
    P = (W + 31) // 32 * 32
    g = torch.Generator(device="cuda").manual_seed(0)
    div = torch.randn(B, H, P, device="cuda", generator=g)
    mask = (torch.rand(B, H, P, device="cuda", generator=g) < 0.05).to(torch.uint8)
    inv = ws.inv_scale_of(div[:, :, :W], mask[:, :, :W])
    net = ws.UNet(seed=0)
    for _ in range(args.warmup):
        net.forward(div, mask, inv, H, W, P)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        net.forward(div, mask, inv, H, W, P)
    e1.record()
    torch.cuda.synchronize()
    net.check_status()
    ms = e0.elapsed_time(e1) / args.steps
    flops, nbytes = ws.forward_cost(B, H, W)
    hbm, kind = load_peaks()
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    tc_peak = float(peaks.get("bf16_tflops", 1900.0))
    gbs = nbytes / ms / 1e6
    print(json.dumps({
        "metric": "U-Net forward images/s (512x512)", "value": B / ms * 1e3, "unit": "images/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 (f32 accumulate)", "data": "synthetic",
        "config": {"workload": f"unet-forward-{B}x512x512", "batch": B,
                   "l2": "activations of a 64-image batch exceed L2"},
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                     "frac": gbs / hbm, "traffic": None, "peak_kind": kind,
                     "algorithmic_bytes": nbytes},
        "tensor": {"tflops": flops / ms / 1e9, "peak": tc_peak, "frac": flops / ms / 1e9 / tc_peak},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 500 for the 2048x2048 workload, else 50)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["natrix", "reference"], default="natrix")
    ap.add_argument("--workload", choices=["large", "small", "particles", "batch", "warmstart",
                                           "unet-forward", "unet-train", "render", "aux"],
                    default="large")
    ap.add_argument("--batch", type=int, default=64, help="unet-forward: images per pass")
    ap.add_argument("--pairs", type=int, default=512, help="warmstart: training pairs")
    ap.add_argument("--train-steps", type=int, default=400, help="warmstart: Adam steps")
    ap.add_argument("--solve-limit", type=float, default=120.0,
                    help="warmstart: seconds allowed per solve")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload: skip the short runs of the other workloads")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 500 if args.workload == "large" else 50
    if args.warmup < 3 and args.impl == "natrix":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "warmstart":
        run_warmstart(args)
        return
    if args.workload == "unet-forward":
        run_unet_forward(args)
        return
    if args.workload == "unet-train":
        run_unet_train(args)
        return
    if args.workload == "aux":
        return run_aux(args)
    if args.workload == "render":
        run_render(args)
        return
    spec = make_spec(args.workload)
    if args.impl == "reference":
        run_reference(args, spec)
    elif args.workload == "particles":
        run_particles(args, spec)
    else:
        run_natrix(args, spec)


if __name__ == "__main__":
    main()
