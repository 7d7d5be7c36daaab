"""Headless visualisation oracle (oracle/render.c): known answers and an
independent numpy float32 restatement of the field shader's colour map."""
from __future__ import annotations

import zlib

import numpy as np

F = np.float32


def _hash(n):
    s = F(np.sin(np.float64(n)))
    y = F(s * F(43758.5453123))
    return F(y - np.floor(y))


def _fbm(x):
    v, a = F(0), F(0.5)
    for _ in range(5):
        fl = F(np.floor(x))
        fc = F(x - fl)
        r0, r1 = _hash(fl), _hash(F(fl + F(1)))
        v = F(v + F(a * F(r0 + F(fc * F(r1 - r0)))))
        x = F(F(x * F(2)) + F(100))
        a = F(a * F(0.5))
    return v


PLASMA = np.array([
    [0.05873234392399702, 0.02333670892565664, 0.5433401826748754],
    [2.176514634195958, 0.2383834171260182, 0.7539604599784036],
    [-2.689460476458034, -7.455851135738909, 3.110799939717086],
    [6.130348345893603, 42.3461881477227, -28.51885465332158],
    [-11.10743619062271, -82.66631109428045, 60.13984767418263],
    [10.02306557647065, 71.41361770095349, -54.07218655560067],
    [-3.658713842777788, -22.93153465461149, 18.19190778539828]], np.float32)


def _unorm8(v):
    v = F(v)
    if not v > 0:
        return 0
    if v >= 1:
        return 255
    return int(np.rint(F(v * F(255))))


def test_palette_matches_numpy_restatement(oracle):
    pal = oracle.plasma_palette()
    for k in range(256):
        c = F(F(k) / F(255))
        t = _fbm(c)
        want = []
        for ch in range(3):
            r = PLASMA[6, ch]
            for i in range(5, -1, -1):
                r = F(PLASMA[i, ch] + F(t * r))
            want.append(_unorm8(r))
        want.append(_unorm8(c))
        assert list(pal[k]) == want, k
    assert list(pal[:, 3]) == list(range(256))


def test_render_density_unorm_rules(oracle):
    rho = np.array([[np.nan, -1.0, 0.0, 2.0, 1.0, 0.5 / 255, 1.5 / 255, 0.5]], np.float32)
    tex, col = oracle.render_density(rho)
    assert list(tex[0, :, 0]) == [0, 0, 0, 255, 255, _unorm8(rho[0, 5]), 2, 128]
    assert (tex == tex[..., :1]).all()
    pal = oracle.plasma_palette()
    np.testing.assert_array_equal(col[0], pal[tex[0, :, 0]])


def test_quiver_uniform_flow(oracle):
    VW, VH, T = 16, 8, 16.0
    v = np.zeros((VH, VW, 2), np.float32)
    v[..., 0], v[..., 1] = 0.25, -0.5
    arrows, ov = oracle.quiver(v, 2 * VW, 2 * VH, T)
    assert arrows.shape == (1, 2, 2)
    # -v * (window / grid) * T * 0.4
    np.testing.assert_allclose(arrows[..., 0], -0.25 * 2 * T * 0.4, rtol=1e-6)
    np.testing.assert_allclose(arrows[..., 1], 0.5 * 2 * T * 0.4, rtol=1e-6)
    # the arrow runs through its tile centre; the tile corners are far from it
    assert ov[:16, :16, 3].max() >= 200 and ov[0, 0, 3] == 0
    assert 0 < ov[8, 8, 3] < 255  # (0.5, 0.5) from the centre: 0.67 px off the shaft
    assert (ov[..., :3] == 255).all()
    _, ov0 = oracle.quiver(np.zeros_like(v), 2 * VW, 2 * VH, T)
    assert (ov0[..., 3] == 0).all()


def test_quiver_samples_only_x_bilinearly(oracle):
    """The shader mixes with vec2(delta, 0): x is interpolated, y is the
    lower-left corner's value."""
    VW, VH = 4, 4
    v = np.zeros((VH, VW, 2), np.float32)
    v[..., 0] = np.arange(VW, dtype=np.float32)[None, :] * 0.1
    v[..., 1] = np.arange(VW, dtype=np.float32)[None, :] * 0.1
    # one tile of 1 pixel at window 8x8: centre (0.5, 0.5) -> fPos = 3.5
    arrows, _ = oracle.quiver(v, 8, 8, 8.0, overlay=False)
    f = (1 - F(4.0) / F(8.0)) * F(4)  # tile centre 4.0 -> fPos 2.0: exact corner
    assert f == 2.0
    arrows, _ = oracle.quiver(v, 7, 7, 7.0, overlay=False)
    fx = F(F(1) - F(3.5) / F(7)) * F(4)  # 2.0
    assert fx == 2.0
    arrows, _ = oracle.quiver(v, 6, 6, 5.0, overlay=False)
    # tile 0 centre 2.5 of 6 -> fPos = (1 - 2.5/6) * 4 = 2.333: lo 2, hi 3
    vx = F(0.2) + F(F(F(1 - F(2.5) / F(6)) * F(4)) - F(2)) * F(F(0.3) - F(0.2))
    ax = F(F(F(-1.0 * vx) * F(F(6) / F(4))) * F(5)) * F(0.4)
    ay = F(F(F(-1.0 * F(0.2)) * F(F(6) / F(4))) * F(5)) * F(0.4)
    assert arrows[0, 0, 0] == ax and arrows[0, 0, 1] == ay


def test_png_writer_round_trip(tmp_path):
    from natrix_gb300.render import write_png

    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (5, 7, 4), dtype=np.uint8)
    path = tmp_path / "f.png"
    write_png(path, img)
    data = path.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    i = data.index(b"IDAT")
    n = int.from_bytes(data[i - 4:i], "big")
    raw = zlib.decompress(data[i + 4:i + 4 + n])
    rows = np.frombuffer(raw, np.uint8).reshape(5, 1 + 7 * 4)
    assert (rows[:, 0] == 0).all()
    np.testing.assert_array_equal(rows[:, 1:].reshape(5, 7, 4), img)
