"""The CPU oracle against the golden vectors written from the reference's own
shaders (tests/golden/make_golden.py), against the reference shaders compiled
here when their sources are present, and against float64 (CPU only)."""
from __future__ import annotations

import numpy as np
import pytest

from tests.golden_replay import assert_equal_f32, replay_steps

KERNEL_FILES = ["kernels_17x23.npz", "kernels_64x48.npz"]


@pytest.fixture(scope="module", params=KERNEL_FILES)
def kern(request, golden_dir):
    return np.load(golden_dir / request.param)


def test_golden_kernels_bit_exact(oracle, kern):
    O = oracle
    d = kern
    v, mask = d["vel"], d["mask"]
    H, W = mask.shape
    dt, speed, diss, scale = (float(d[k]) for k in ("dt", "speed", "diss", "scale"))
    out = np.zeros_like(v)
    O.advect_velocity(v, out, mask, dt, speed, diss)
    assert_equal_f32(out, d["advect"], "advect")
    O.advect_velocity(v, out, mask, dt, 60.0, 1.0)
    assert_equal_f32(out, d["advect_speed60"], "advect speed 60")
    vb = v.copy()
    O.init_boundaries(vb)
    assert_equal_f32(vb, d["init_boundaries"], "init boundaries")
    w = np.zeros((H, W), np.float32)
    O.calc_vorticity(v, w)
    assert_equal_f32(w, d["vorticity"], "calc vorticity")
    O.apply_vorticity(v, out, w, dt, scale)
    assert_equal_f32(out, d["apply_vorticity"], "apply vorticity")
    O.viscosity(v, out, float(d["nu"]))
    assert_equal_f32(out, d["viscosity"], "viscosity")
    div = np.zeros((H, W), np.float32)
    O.divergence(v, mask, div)
    assert_equal_f32(div, d["divergence"], "divergence")
    p = d["p"]
    assert_equal_f32(O.jacobi_n(p, div, mask, 1), d["jacobi1"], "1 jacobi sweep")
    assert_equal_f32(O.jacobi_n(p, div, mask, 7), d["jacobi7"], "7 jacobi sweeps")
    assert_equal_f32(O.jacobi_n(np.zeros_like(p), div, mask, 13), d["jacobi13_zero"],
                     "13 sweeps from zero")
    O.subtract_gradient(v, out, p, mask)
    assert_equal_f32(out, d["subtract_gradient"], "subtract gradient")
    a = d["add_velocity_args"]
    O.add_velocity(v, out, *[float(x) for x in a])
    assert_equal_f32(out, d["add_velocity"], "add velocity")
    m = np.zeros((H, W), np.uint8)
    O.add_circle_obstacle(m, 0.45, 0.55, 5.5)
    O.add_triangle_obstacle(m, (0.1, 0.1), (0.9, 0.25), (0.4, 0.85), True)
    O.add_circle_obstacle(m, 0.8, 0.8, 3.0)
    np.testing.assert_array_equal(m, d["obstacles_raster"])
    rho = d["rho"]
    ro = np.zeros_like(rho)
    O.add_particle(rho, ro, 0.5, 0.45, 7.0, 40.0)
    assert_equal_f32(ro, d["add_particle"], "add particle")
    O.advect_particle(rho, ro, v, mask, dt, 200.0, 0.98)
    assert_equal_f32(ro, d["advect_particle"], "advect particle")
    O.advect_particle(rho, ro, d["vel_half"], d["mask_half"], dt, 200.0, 0.98)
    assert_equal_f32(ro, d["advect_particle_half"], "advect particle, half-size velocity")


@pytest.mark.parametrize("name", ["steps_48x40.npz", "steps_33x29_defaults.npz"])
def test_golden_steps_bit_exact(oracle, golden_dir, name):
    d = np.load(golden_dir / name)
    W, H = d["vel_1"].shape[1], d["vel_1"].shape[0]
    f = oracle.OracleFluid(W, H, np.float32)
    dn = oracle.OracleDensity(W, H, f)

    def check(step):
        assert_equal_f32(f.velocity, d[f"vel_{step}"], f"velocity after step {step}")
        assert_equal_f32(f.pressure, d[f"pressure_{step}"], f"pressure after step {step}")
        assert_equal_f32(f.divergence, d[f"div_{step}"], f"divergence after step {step}")
        assert_equal_f32(f.vorticity_field, d[f"vort_{step}"], f"vorticity after step {step}")
        assert_equal_f32(dn.field, d[f"density_{step}"], f"density after step {step}")

    keep = replay_steps(d, f, dn, check)
    assert keep


def test_reference_shaders_pin(oracle):
    """Oracle float32 == the reference's own shader sources compiled on the
    CPU, on fresh random inputs (only where the reference is present)."""
    from oracle import ref as R

    if not R.available() and not R.build():
        pytest.skip("reference shader sources not present on this machine")
    O = oracle
    rng = np.random.default_rng(123)
    for W, H in [(31, 17), (16, 64)]:
        v = rng.uniform(-1, 1, (H, W, 2)).astype(np.float32)
        mask = (rng.random((H, W)) < 0.2).astype(np.uint8)
        obs = R.obs_to_vec2(mask)
        a, b = np.zeros_like(v), np.zeros_like(v)
        O.advect_velocity(v, a, mask, 0.02, 300.0, 0.97)
        R.lib().ref_advect_velocity(R._p(v), R._p(b), R._p(obs), W, H, R.F(0.02), R.F(300.0),
                                    R.F(0.97))
        assert_equal_f32(a, b, "advect vs reference shader")
        p = rng.normal(size=(H, W)).astype(np.float32)
        div = rng.normal(size=(H, W)).astype(np.float32)
        pa = O.jacobi_n(p, div, mask, 1)
        pb = np.zeros((H, W, 2), np.float32)
        R.lib().ref_poisson(R._p(R.scalar_to_vec2(p)), R._p(pb), R._p(div), R._p(obs), W, H)
        assert_equal_f32(pa, pb[..., 0], "jacobi vs reference shader")
    # a coupled multi-step run with every optional stage enabled
    W, H = 40, 36
    f = O.OracleFluid(W, H, np.float32)
    rf = R.RefFluid(W, H)
    for s in (f, rf):
        s.iterations, s.vorticity, s.viscosity, s.speed, s.dissipation = 15, 0.5, 0.2, 300.0, 0.98
    for step in range(12):
        pos = (rng.random(), rng.random())
        vel = tuple(float(x) for x in rng.uniform(-1, 1, 2))
        for s in (f, rf):
            s.add_circle_obstacle((0.3, 0.6), 5.0)
            s.add_velocity(pos, vel, 7.0)
            s.update(1 / 60)
    assert_equal_f32(f.velocity, rf.velocity, "12 steps vs reference shaders")
    assert_equal_f32(f.pressure, rf.pressure, "12 steps pressure vs reference shaders")


def test_float64_tracks_float32(oracle):
    """The float64 instantiation is the same algorithm: after a few steps it
    stays within float32 rounding of the float32 run."""
    W, H = 48, 40
    runs = {}
    for dt in (np.float32, np.float64):
        f = oracle.OracleFluid(W, H, dt)
        f.iterations, f.vorticity, f.viscosity, f.speed, f.dissipation = 30, 0.35, 0.0, 5.0, 0.99
        rng = np.random.default_rng(3)
        from natrix_gb300 import workloads as wl

        for _ in range(5):
            f.add_splats(wl.gauss_splats(rng, 4, W, H, 5.0))
            f.update(1 / 60)
        runs[dt] = f
    a, b = runs[np.float32], runs[np.float64]
    scale = np.max(np.abs(b.velocity))
    assert np.max(np.abs(a.velocity - b.velocity)) <= 1e-5 * max(scale, 1.0)
    assert np.max(np.abs(a.pressure - b.pressure)) <= 1e-4 * max(np.max(np.abs(b.pressure)), 1)


def test_expf_accuracy(oracle):
    """The splat weight's exp (Cody-Waite + degree-7 Taylor) against libm's
    correctly rounded expf on the argument range the splats use."""
    xs = np.linspace(-9.5, 0.0, 20001, dtype=np.float32)
    ours = np.array([oracle.expf(float(x)) for x in xs], np.float32)
    want = np.exp(xs.astype(np.float64))
    rel = np.abs(ours.astype(np.float64) - want) / want
    assert np.max(rel) < 4 * np.finfo(np.float32).eps


def test_add_particle_rows_quirk(oracle):
    """AddParticle reaches only rows < 16*ceil(W/16) (the reference launches
    the x group count in y too); taller grids keep the other rows."""
    W, H = 20, 70
    rho = np.zeros((H, W), np.float32)
    out = np.zeros_like(rho)
    oracle.add_particle(rho, out, 0.5, 0.5, 30.0, 10.0)  # centre at row 35
    rows = oracle.add_particle_rows(W, H)
    assert rows == 32
    assert np.all(out[rows:] == 0) and np.any(out[:rows] > 0)
