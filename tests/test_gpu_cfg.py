"""Scenes from console (.cfg) text on the GPU: bit-exact with the oracle, and
a white furnace (albedo-1 Lambert sphere under a uniform env of radiance 1)
converges to radiance 1 everywhere."""
import numpy as np
import pytest

from test_cfg import write_hdr

pytestmark = pytest.mark.gpu

FURNACE = """
cam_pos 0 0 4
cam_yaw 0
cam_pitch 0
cam_fov 40
r_sky_mode hdri
r_env_map furnace.hdr
r_env_intensity 2
r_mis 1
r_spp 4
r_max_bounces 4
r_firefly_clamp 0
prim_sphere 1 0 0 0 1 lambert 1 1 1
"""


def test_furnace_from_cfg_is_bit_exact_and_conserves_energy(pt, orc, dev, tmp_path):
    q = np.full((16, 32, 4), 128, np.uint8)              # RGBE 128,128,128,e=128 -> 0.5
    write_hdr(str(tmp_path / "furnace.hdr"), q)
    s = pt.Scene()
    rep, n = s.exec_cfg(FURNACE, str(tmp_path))
    assert n == 0, rep
    W = H = 48
    head, prm = s.push(W, H, frame_index=0, reset=1)
    assert head.env_map_present == 1
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, 2)
    g = dev.read_accum().copy()
    o, _ = orc.render(s.packed(), head, prm, W, H, 2)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
    dev.render(head, prm, 256)                           # 1,024 samples per pixel
    img = dev.read_accum()[..., :3]
    assert abs(img.mean() - 1.0) < 0.005
    assert np.abs(img - 1.0).max() < 0.15


GRADIENT = """
cam_pos 0 2.5 6
cam_pitch -18
cam_fov 55
r_sky_mode gradient
r_sun_elevation 25
r_sun_azimuth 200
r_spp 2
r_max_bounces 4
prim_plane 1 0 1 0 0 lambert 0.6 0.6 0.6
prim_sphere 10 0 1 0 1 lambert 0.85 0.85 0.85
prim_sphere 11 2 0.7 0.5 0.7 dielectric 1 1 1 0 1.5
prim_sphere 12 -2 0.7 0.5 0.7 metal 0.9 0.6 0.3 0.2
light_point 1 -3 2.5 -1 20 8 8
light_quad 4 3 2.5 -1 0 -1 0 1 0 0 0.4 0.4 30 30 10
"""


@pytest.mark.parametrize("mode", [0, 1])
def test_gradient_sky_scene_from_cfg_bit_exact(pt, orc, dev, mode):
    s = pt.Scene()
    rep, n = s.exec_cfg(GRADIENT)
    assert n == 0, rep
    W, H = 64, 40
    head, prm = s.push(W, H, frame_index=3, reset=1)
    assert head.env_map_present == 0 and prm.sun_and_mode[3] == 0.0
    dev.set_traversal(mode)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, 2)
    g = dev.read_accum()
    o, _ = orc.render(s.packed(), head, prm, W, H, 2)
    assert g[..., :3].mean() > 0.05
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


@pytest.mark.parametrize("srgb", [False, True])
def test_tonemap_kernel_equals_oracle_for_every_operator(pt, orc, dev, srgb, tmp_path):
    s = pt.Scene()
    s.exec_cfg(GRADIENT)
    W, H = 64, 40
    head, prm = s.push(W, H, frame_index=3, reset=1)
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, 4)
    acc = dev.read_accum()
    for op in range(5):
        g = dev.tonemap(exposure=1.3, op=op, srgb=srgb)
        o = orc.tonemap(acc, 1.3, op, srgb)
        st, _ = pt.imgdiff(g, o)
        assert st.max_delta == 0.0, (op, st.max_delta)
    pt.write_png(str(tmp_path / "frame.png"), g)
