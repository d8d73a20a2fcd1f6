"""Gradient sky (no env map): the oracle's sun NEE + skylight ambient against
a closed form, and its transcendentals against numpy."""
import math

import numpy as np

import oracle as orc_mod
from conftest import load_pkg


def test_sun_and_skylight_on_a_lambert_plane_closed_form(orc):
    pt = load_pkg()
    s = pt.Scene()
    a = (0.6, 0.4, 0.2)
    s.plane(1, (0.0, 1.0, 0.0), 0.0, 0, a)      # y = 0, facing up
    s.env(None)
    elev = 30.0
    s.set_cvar("r_sun_elevation", elev)
    s.set_cvar("r_max_bounces", 1)
    s.set_cvar("r_spp", 1)
    s.camera((0.0, 5.0, 0.0), 0.0, -1.4, 30.0)
    W = H = 8
    head, prm = s.push(W, H)
    assert head.env_map_present == 0 and prm.sun_and_mode[3] == 0.0
    img, _ = orc_mod.render(s.packed(), head, prm, W, H, 1, fp64=True)
    se = math.sin(math.radians(elev))
    am = 1.0 / max(se, 0.04)
    warmth = min(max((am - 1.0) * 0.18, 0.0), 1.0)
    sun_col = np.array([1.00, 0.97, 0.92]) + warmth * (np.array([1.55, 0.55, 0.20]) - np.array([1.00, 0.97, 0.92]))
    direct = sun_col * 80.0 * math.exp(-0.3 * am) * np.array(a) / 3.14159265358979 * se
    expect = direct + np.array(a) * 1.0          # gradient dome at the up normal is white
    np.testing.assert_allclose(img[..., :3].reshape(-1, 3), np.broadcast_to(expect, (W * H, 3)), rtol=2e-5)


def test_fp32_and_fp64_gradient_sky_renders_agree(orc):
    pt = load_pkg()
    s = pt.Scene().synth(0, seed=3)
    s.env(None)
    s.set_cvar("r_sun_elevation", 4.0)           # low sun: oval disc, warm colour
    s.set_cvar("r_spp", 4)
    W, H = 48, 32
    head, prm = s.push(W, H)
    assert prm.sun_extra[2] < 0.999
    a32, _ = orc_mod.render(s.packed(), head, prm, W, H, 1)
    a64, _ = orc_mod.render(s.packed(), head, prm, W, H, 1, fp64=True)
    assert a32[..., :3].mean() > 0.05
    # same paths except where fp32 rounding flips a discrete decision
    close = np.isclose(a32[..., :3], a64[..., :3], rtol=1e-3, atol=1e-4).all(axis=2)
    assert close.mean() > 0.9


def test_transcendentals_against_numpy(orc):
    lib = orc.load()
    import ctypes
    for n in ("oracle_expf", "oracle_logf", "oracle_asinf"):
        getattr(lib, n).restype = ctypes.c_float
        getattr(lib, n).argtypes = [ctypes.c_float]
    lib.oracle_powf.restype = ctypes.c_float
    lib.oracle_powf.argtypes = [ctypes.c_float, ctypes.c_float]
    rng = np.random.default_rng(0)
    for x in rng.uniform(-30, 30, 500).astype(np.float32):
        assert abs(lib.oracle_expf(float(x)) - math.exp(float(x))) <= 3e-7 * math.exp(float(x))
    for x in (10 ** rng.uniform(-20, 20, 500)).astype(np.float32):
        assert abs(lib.oracle_logf(float(x)) - math.log(float(x))) <= 3e-7 * max(1.0, abs(math.log(float(x))))
    for x in rng.uniform(-1, 1, 500).astype(np.float32):
        assert abs(lib.oracle_asinf(float(x)) - math.asin(float(x))) <= 5e-7
    for t, y in zip(rng.uniform(1e-3, 1, 500).astype(np.float32), rng.uniform(3, 8, 500).astype(np.float32)):
        r = float(t) ** float(y)
        assert abs(lib.oracle_powf(float(t), float(y)) - r) <= 1e-5 * r
    assert lib.oracle_expf(0.0) == 1.0 and lib.oracle_powf(0.5, 0.0) == 1.0
