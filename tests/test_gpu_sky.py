"""Gradient sky (no env map: sky dome + sun and moon discs, sun/moon NEE and
skylight ambient) on the GPU against the fp32 oracle, bit for bit."""
import math

import numpy as np
import pytest

import oracle as orc_mod

pytestmark = pytest.mark.gpu

MODES = [pytest.param(0, id="wide_sah"), pytest.param(1, id="reference_bvh")]


def _render_both(pt, orc, dev, s, W, H, frames, prm_edit=None, mode=0):
    dev.set_traversal(mode)
    dev.upload(s)
    dev.set_target(W, H)
    head, prm = s.push(W, H, frame_index=5, reset=1)
    if prm_edit:
        prm_edit(prm)
    dev.render(head, prm, frames)
    g = dev.read_accum()
    o, _ = orc.render(s.packed(), head, prm, W, H, frames)
    return g, o


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("elev", [30.0, 4.0])
def test_gradient_sky_scene_bit_exact(pt, orc, dev, mode, elev):
    s = pt.Scene().synth(0, seed=1)
    s.env(None)
    s.set_cvar("r_sun_elevation", elev)
    s.set_cvar("r_spp", 2)
    g, o = _render_both(pt, orc, dev, s, 64, 48, 2, mode=mode)
    assert g[..., :3].mean() > 0.01
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


def _sun_dir(elev_deg, azim_deg):
    e, a = math.radians(elev_deg), math.radians(azim_deg)
    return np.array([math.cos(e) * math.sin(a), math.sin(e), -math.cos(e) * math.cos(a)])


def test_sun_and_moon_discs_bit_exact(pt, orc, dev):
    """Camera aimed at a low sun (4 deg: oval disc, warm halo) with a textured
    moon 1.2 deg beside it; primary misses evaluate sunDisc and moonDisc."""
    s = pt.Scene()
    s.sphere(1, 0.0, -1000.0, 0.0, 10.0, 0, (0.5, 0.5, 0.5))   # far below: rays miss it
    s.env(None)
    elev, az = 4.0, 120.0
    s.set_cvar("r_sun_elevation", elev)
    s.set_cvar("r_sun_azimuth", az)
    s.set_cvar("r_sun_size", 1.5)
    s.camera((0.0, 0.0, 0.0), math.radians(az + 0.6), math.radians(elev + 0.5), 4.0)
    rng = np.random.default_rng(9)
    moon = np.concatenate([rng.uniform(0.2, 1.0, (16, 32, 3)), np.ones((16, 32, 1))], axis=2).astype(np.float32)
    s.moon(moon)
    md = _sun_dir(elev + 1.2, az + 1.0)

    def edit(prm):
        prm.moon_dir_phase[0], prm.moon_dir_phase[1], prm.moon_dir_phase[2] = map(float, md)
        prm.moon_dir_phase[3] = 1.9
        prm.moon_extra[0], prm.moon_extra[1], prm.moon_extra[2] = 1.2, 1.0, 0.7

    W, H = 96, 64
    g, o = _render_both(pt, orc, dev, s, W, H, 1, prm_edit=edit)
    lum = g[..., :3].max(axis=2)
    assert lum.max() > 2.0                  # the sun disc is in view
    assert (lum > np.median(lum) + 0.02).sum() > 40   # disc + halo pixels above the dome
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


def test_moon_above_horizon_needs_a_texture(pt, dev):
    s = pt.Scene().synth(0, seed=1)
    s.env(None)
    dev.upload(s)
    dev.set_target(16, 16)
    head, prm = s.push(16, 16)
    prm.moon_dir_phase[1] = 0.5
    with pytest.raises(pt.PtError):
        dev.render(head, prm, 1)
    prm.moon_dir_phase[1] = -1.0
    prm.sun_and_mode[3] = 3.0                  # Hosek-Wilkie dome: not built
    with pytest.raises(pt.PtError):
        dev.render(head, prm, 1)


def test_adjoint_under_the_gradient_sky_matches_fp64_oracle(pt, orc, dev):
    s = pt.Scene().synth(3, seed=0, scale=0.3)
    s.env(None)
    s.set_cvar("r_spp", 2)
    W, H = 48, 40
    head, prm = s.push(W, H, 0, 1)
    pk = s.packed()
    nm = pk.material_count
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    dev.diff_forward(head, prm, 1)
    img = dev.read_accum()
    o, _ = orc.render(pk, head, prm, W, H, 1)
    assert np.array_equal(img.view(np.uint32), o.view(np.uint32))
    w = np.random.default_rng(4).standard_normal((H, W, 3)).astype(np.float32)
    ga, ge = dev.diff_backward(w, nm)
    oa, oe = orc_mod.adjoint(pk, head, prm, W, H, 1, w)
    for g, og in ((ga, oa), (ge, oe)):
        tol = 1e-5 * np.abs(og).max() + 1e-4 * np.abs(og)
        assert np.all(np.abs(g - og) <= tol)


PROC = """
cam_pos 0 2 7
cam_yaw {yaw}
cam_pitch {pitch}
cam_fov 60
r_sky_mode procedural
r_show_stars 0
r_sun_elevation {elev}
r_sun_azimuth 30
r_spp 2
r_max_bounces 3
prim_plane 1 0 1 0 0 lambert 0.6 0.6 0.6
prim_sphere 10 0 1 0 1 lambert 0.85 0.85 0.85
prim_sphere 11 -2.2 0.8 0.5 0.8 dielectric 1 1 1 0 1.5
light_point 1 -3 2.5 -1 20 8 8
light_spot 2 -1 2.5 -1 0 -1 0 25 15 10 30 10
"""


@pytest.mark.parametrize("elev,yaw,pitch", [(55.0, 0, -12), (1.5, 30, 1), (-30.0, 0, -10)],
                         ids=["noon", "sunset_facing_sun", "night"])
def test_procedural_sky_bit_exact(pt, orc, dev, elev, yaw, pitch):
    s = pt.Scene()
    rep, n = s.exec_cfg(PROC.format(elev=elev, yaw=yaw, pitch=pitch))
    assert n == 0, rep
    W, H = 72, 48
    head, prm = s.push(W, H, frame_index=11, reset=1)
    assert prm.sun_and_mode[3] == 2.0 and prm.stars == 0 and prm.sun_extra[3] > 6e6
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, 2)
    g = dev.read_accum()
    o, _ = orc.render(s.packed(), head, prm, W, H, 2)
    assert g[..., :3].mean() > 0.003
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


def test_procedural_stars_are_refused(pt, dev):
    s = pt.Scene()
    s.exec_cfg(PROC.format(elev=-20, yaw=0, pitch=0) + "r_show_stars 1\n")
    dev.upload(s)
    dev.set_target(16, 16)
    head, prm = s.push(16, 16)
    assert prm.stars == 1
    with pytest.raises(pt.PtError):
        dev.render(head, prm, 1)
