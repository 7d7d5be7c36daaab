"""Write the golden vectors in tests/golden/ from the reference's own compute
shaders, compiled on the CPU through the GLSL shim (oracle/build_ref.sh).

Run in a checkout that has the reference sources:
    python tests/golden/make_golden.py [REFERENCE_ROOT]

Outputs (small .npz files, committed):
  kernels_<W>x<H>.npz  seeded inputs and the output of every shader, one
                       dispatch each, in the oracle's layouts
  steps_<W>x<H>.npz    a coupled FluidSimulator + SmoothParticlesArea run
                       (obstacles, add_velocity, add_particles, update) with
                       the state after selected steps
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import ref as R  # noqa: E402

OUT = Path(__file__).resolve().parent
F = R.F


def kernels_case(W: int, H: int, seed: int) -> dict:
    rng = np.random.default_rng(seed)
    L = R.lib()
    d: dict[str, np.ndarray] = {}
    v = rng.uniform(-1, 1, (H, W, 2)).astype(np.float32)
    # a few exact integer backtraces and far-outside ones
    v[0, :4] = [[0.0, 0.0], [1.0, -1.0], [-1.0, 1.0], [0.5, 0.25]]
    mask = (rng.random((H, W)) < 0.12).astype(np.uint8)
    mask[rng.random((H, W)) < 0.04] = 2
    obs = R.obs_to_vec2(mask)
    params = dict(dt=np.float32(1 / 60), speed=np.float32(500.0), diss=np.float32(0.99),
                  scale=np.float32(0.35))
    d.update({k: np.asarray(x) for k, x in params.items()})
    d["vel"], d["mask"] = v, mask

    out = np.zeros_like(v)
    L.ref_advect_velocity(R._p(v), R._p(out), R._p(obs), W, H, F(params["dt"]),
                          F(params["speed"]), F(params["diss"]))
    d["advect"] = out.copy()
    # a slower speed keeps most backtraces inside the grid
    L.ref_advect_velocity(R._p(v), R._p(out), R._p(obs), W, H, F(params["dt"]), F(60.0),
                          F(1.0))
    d["advect_speed60"] = out.copy()

    vb = v.copy()
    L.ref_init_boundaries(R._p(vb), W, H)
    d["init_boundaries"] = vb

    w = np.zeros((H, W), np.float32)
    L.ref_calc_vorticity(R._p(v), R._p(w), W, H)
    d["vorticity"] = w.copy()
    L.ref_apply_vorticity(R._p(v), R._p(out), R._p(w), W, H, F(params["dt"]),
                          F(params["scale"]))
    d["apply_vorticity"] = out.copy()

    nu = 0.1
    alpha = 1.0 / nu
    rbeta = 1.0 / (4.0 + alpha)
    d["nu"] = np.asarray(nu)
    L.ref_viscosity(R._p(v), R._p(out), W, H, F(alpha), F(rbeta))
    d["viscosity"] = out.copy()

    div = np.zeros((H, W), np.float32)
    L.ref_divergence(R._p(v), R._p(obs), R._p(div), W, H)
    d["divergence"] = div.copy()

    p = rng.normal(size=(H, W)).astype(np.float32)
    d["p"] = p
    pa, pb = R.scalar_to_vec2(p), np.zeros((H, W, 2), np.float32)
    for s in range(7):
        L.ref_poisson(R._p(pa), R._p(pb), R._p(div), R._p(obs), W, H)
        pa, pb = pb, pa
        if s == 0:
            d["jacobi1"] = pa[..., 0].copy()
    d["jacobi7"] = pa[..., 0].copy()
    # zero start, the way update() runs it
    pa, pb = np.zeros((H, W, 2), np.float32), np.zeros((H, W, 2), np.float32)
    for s in range(13):
        L.ref_poisson(R._p(pa), R._p(pb), R._p(div), R._p(obs), W, H)
        pa, pb = pb, pa
    d["jacobi13_zero"] = pa[..., 0].copy()

    L.ref_subtract_gradient(R._p(v), R._p(out), R._p(R.scalar_to_vec2(p)), R._p(obs), W, H)
    d["subtract_gradient"] = out.copy()

    av = dict(px=0.31, py=0.62, vx=0.8, vy=-0.45, r=6.5)
    d["add_velocity_args"] = np.array([av["px"], av["py"], av["vx"], av["vy"], av["r"]],
                                      np.float32)
    L.ref_add_velocity(R._p(v), R._p(out), W, H, F(av["px"]), F(av["py"]), F(av["vx"]),
                       F(av["vy"]), F(av["r"]))
    d["add_velocity"] = out.copy()

    m2 = np.zeros((H, W, 2), np.float32)
    L.ref_add_circle_obstacle(R._p(m2), W, H, F(0.45), F(0.55), F(5.5), 0)
    L.ref_add_triangle_obstacle(R._p(m2), W, H, F(0.1), F(0.1), F(0.9), F(0.25), F(0.4),
                                F(0.85), 1)
    L.ref_add_circle_obstacle(R._p(m2), W, H, F(0.8), F(0.8), F(3.0), 1)
    d["obstacles_raster"] = R.vec2_to_obs(m2)

    rho = rng.uniform(0, 3, (H, W)).astype(np.float32)
    d["rho"] = rho
    ro = rho.copy()
    L.ref_add_particle(R._p(rho), R._p(ro), W, H, F(0.5), F(0.45), F(7.0), F(40.0),
                       (W + 15) // 16)
    d["add_particle"] = ro.copy()
    Wv, Hv = W // 2 + 1, H // 2 + 1
    vv = rng.uniform(-1, 1, (Hv, Wv, 2)).astype(np.float32)
    mv = (rng.random((Hv, Wv)) < 0.1).astype(np.uint8)
    d["vel_half"], d["mask_half"] = vv, mv
    L.ref_advect_particle(R._p(rho), R._p(ro), R._p(v), R._p(obs), W, H, W, H, F(params["dt"]),
                          F(200.0), F(0.98))
    d["advect_particle"] = ro.copy()
    L.ref_advect_particle(R._p(rho), R._p(ro), R._p(vv), R._p(R.obs_to_vec2(mv)), W, H, Wv,
                          Hv, F(params["dt"]), F(200.0), F(0.98))
    d["advect_particle_half"] = ro.copy()
    return d


def steps_case(W: int, H: int, seed: int, steps: int, keep: tuple[int, ...],
               iterations: int, vorticity: float, viscosity: float, speed: float) -> dict:
    rng = np.random.default_rng(seed)
    f = R.RefFluid(W, H)
    dn = R.RefDensity(W, H, f)
    f.iterations, f.vorticity, f.viscosity, f.speed, f.dissipation = (
        iterations, vorticity, viscosity, speed, 0.99)
    dn.speed, dn.dissipation = speed, 0.98
    d: dict[str, np.ndarray] = {
        "params": np.array([iterations, vorticity, viscosity, speed, 0.99, 0.98, 1 / 60],
                           np.float64)}
    forcing = np.zeros((steps, 9), np.float32)  # px py vx vy r | dpx dpy dr ds
    for s in range(steps):
        forcing[s] = [rng.random(), rng.random(), rng.uniform(-1, 1), rng.uniform(-1, 1),
                      rng.uniform(3, 9), rng.random(), rng.random(), rng.uniform(4, 10),
                      rng.uniform(10, 80)]
    d["forcing"] = forcing
    for s in range(steps):
        fr = forcing[s]
        # demo frame order (demo/simulation_demo.py:220-237)
        f.add_circle_obstacle((0.5, 0.5), W / 8)
        f.add_triangle_obstacle((0.1, 0.15), (0.3, 0.1), (0.2, 0.35), s % 2 == 0)
        f.update(1 / 60)
        dn.update(1 / 60)
        f.add_velocity((fr[0], fr[1]), (fr[2], fr[3]), fr[4])
        dn.add_particles((fr[5], fr[6]), fr[7], fr[8])
        if s + 1 in keep:
            d[f"vel_{s + 1}"] = f.velocity.copy()
            d[f"pressure_{s + 1}"] = f.pressure.copy()
            d[f"div_{s + 1}"] = f.divergence.copy()
            d[f"vort_{s + 1}"] = f.vorticity_field.copy()
            d[f"density_{s + 1}"] = dn.field.copy()
    return d


def main(argv):
    # reference checkout: argv[1], else what oracle/build_ref.sh finds
    ref_root = argv[1] if len(argv) > 1 else None
    if not R.build(ref_root):
        raise SystemExit("reference sources not found; cannot make golden vectors")
    for (W, H, seed) in [(17, 23, 11), (64, 48, 12)]:
        np.savez_compressed(OUT / f"kernels_{W}x{H}.npz", **kernels_case(W, H, seed))
    np.savez_compressed(OUT / "steps_48x40.npz",
                        **steps_case(48, 40, 21, 30, (1, 10, 30), 20, 0.35, 0.1, 200.0))
    np.savez_compressed(OUT / "steps_33x29_defaults.npz",
                        **steps_case(33, 29, 22, 10, (1, 10), 50, 0.0, 0.1, 500.0))
    for p in sorted(OUT.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main(sys.argv)
