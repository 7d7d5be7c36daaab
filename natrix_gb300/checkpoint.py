"""State checkpoints: solver fields, density, particles, the warm-start
network (weights and Adam moments) and generated training pairs, in one
on-disk format.

No reference counterpart (natrix keeps its state in bgfx buffers only).  A
checkpoint is a NumPy ``.npz`` archive (uncompressed by default) whose keys
are ``<part>/<name>``; ``format`` and ``version`` identify it.  Restoring
into a simulator of the same size and then stepping reproduces the
uninterrupted run bit for bit: the fields are copied through the C ABI
(natrix_download / natrix_upload) after the queued add_* calls are applied,
and the obstacle mask is stored as the next step will see it.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from . import _lib

FORMAT = "natrix-gb300-checkpoint"
VERSION = 1

_FLUID_FIELDS = {
    "velocity": _lib.FIELD_VELOCITY,
    "pressure": _lib.FIELD_PRESSURE,
    "divergence": _lib.FIELD_DIVERGENCE,
    "vorticity": _lib.FIELD_VORTICITY,
    "obstacles": _lib.FIELD_OBSTACLES,
}
_FLUID_PARAMS = ("speed", "iterations", "dissipation", "vorticity", "viscosity", "has_borders",
                 "simulate", "sweeps_per_launch")


def fluid_state(sim) -> dict:
    d = {f"fluid/{k}": sim.download(f) for k, f in _FLUID_FIELDS.items()}
    d["fluid/size"] = np.array([sim.width, sim.height], np.int64)
    d["fluid/params"] = np.array([float(getattr(sim, k)) for k in _FLUID_PARAMS], np.float64)
    return d


def restore_fluid(sim, d: dict) -> None:
    w, h = (int(x) for x in d["fluid/size"])
    if (w, h) != (sim.width, sim.height):
        raise ValueError(f"checkpoint holds a {w}x{h} simulator, not {sim.width}x{sim.height}")
    prm = d["fluid/params"]
    sim.speed, sim.iterations, sim.dissipation = float(prm[0]), int(prm[1]), float(prm[2])
    sim.vorticity, sim.viscosity = float(prm[3]), float(prm[4])
    sim.has_borders, sim.simulate, sim.sweeps_per_launch = bool(prm[5]), bool(prm[6]), int(prm[7])
    for k, f in _FLUID_FIELDS.items():
        sim.upload(f, d[f"fluid/{k}"])


def density_state(area) -> dict:
    return {"density/rho": area.download(),
            "density/size": np.array([area.width, area.height], np.int64),
            "density/params": np.array([float(area.speed), float(area.dissipation),
                                        float(area.simulate)], np.float64)}


def restore_density(area, d: dict) -> None:
    w, h = (int(x) for x in d["density/size"])
    if (w, h) != (area.width, area.height):
        raise ValueError(f"checkpoint holds a {w}x{h} density, not {area.width}x{area.height}")
    prm = d["density/params"]
    area.speed, area.dissipation, area.simulate = float(prm[0]), float(prm[1]), bool(prm[2])
    area.upload(d["density/rho"])


def network_state(net) -> dict:
    d = {f"unet/{k}": v.numpy() for k, v in net.state_dict().items()}
    for i, (_, _, m, v) in enumerate(net.parameters()):
        d[f"unet/adam/{i}/m"] = m.cpu().numpy()
        d[f"unet/adam/{i}/v"] = v.cpu().numpy()
    d["unet/adam/step"] = np.array(net.step_count, np.int64)
    return d


def restore_network(net, d: dict) -> None:
    import torch

    net.load_state_dict({k[5:]: torch.from_numpy(np.asarray(v)) for k, v in d.items()
                         if k.startswith("unet/") and not k.startswith("unet/adam/")})
    for i, (_, _, m, v) in enumerate(net.parameters()):
        if f"unet/adam/{i}/m" in d:
            m.copy_(torch.from_numpy(d[f"unet/adam/{i}/m"]))
            v.copy_(torch.from_numpy(d[f"unet/adam/{i}/v"]))
    if "unet/adam/step" in d:
        net.step_count = int(d["unet/adam/step"])


def pairs_state(pairs) -> dict:
    return {"pairs/div": pairs.div.cpu().numpy(), "pairs/mask": pairs.mask.cpu().numpy(),
            "pairs/inv_scale": pairs.inv_scale.cpu().numpy(),
            "pairs/target": pairs.target.cpu().numpy(),
            "pairs/rel_residual": pairs.rel_residual.cpu().numpy(),
            "pairs/cg_iterations": np.array(pairs.cg_iterations, np.int64)}


def restore_pairs(d: dict, device: str = "cuda"):
    import torch

    from .core.warmstart import PairSet

    t = {k: torch.from_numpy(np.asarray(d[f"pairs/{k}"]))
         for k in ("div", "mask", "inv_scale", "target", "rel_residual")}
    return PairSet(t["div"].to(device), t["mask"].to(device), t["inv_scale"].to(device),
                   t["target"].to(device), t["rel_residual"], int(d["pairs/cg_iterations"]))


def save(path, sim=None, density=None, particles=None, net=None, pairs=None,
         compress: bool = False) -> Path:
    """Write the given parts to ``path`` (a ``.npz`` archive)."""
    d = {"format": np.array(FORMAT), "version": np.array(VERSION, np.int64)}
    if sim is not None:
        d.update(fluid_state(sim))
    if density is not None:
        d.update(density_state(density))
    if particles is not None:
        d["particles/positions"] = particles.download()
    if net is not None:
        d.update(network_state(net))
    if pairs is not None:
        d.update(pairs_state(pairs))
    path = Path(path)
    with open(path, "wb") as f:
        (np.savez_compressed if compress else np.savez)(f, **d)
    return path


def read(path) -> dict:
    """All arrays of a checkpoint, after checking its format and version."""
    with np.load(path, allow_pickle=False) as z:
        d = {k: z[k] for k in z.files}
    if str(d.get("format", "")) != FORMAT:
        raise ValueError(f"{path}: not a {FORMAT} archive")
    if int(d["version"]) > VERSION:
        raise ValueError(f"{path}: version {int(d['version'])} is newer than {VERSION}")
    return d


def load(path, sim=None, density=None, particles=None, net=None) -> dict:
    """Restore the parts present in ``path`` into the given objects (of the
    same sizes); returns the raw arrays (training pairs: ``restore_pairs``)."""
    d = read(path)
    if sim is not None:
        restore_fluid(sim, d)
    if density is not None:
        restore_density(density, d)
    if particles is not None:
        particles.upload(d["particles/positions"])
    if net is not None:
        restore_network(net, d)
    return d


__all__ = ["save", "load", "read", "restore_pairs", "FORMAT", "VERSION"]
