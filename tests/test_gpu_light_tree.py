"""Light-tree NEE (r_light_tree 1, the reference default) on the GPU against
the fp32 oracle, bit for bit: one light (a one-leaf tree draws no random
number), four mixed lights, and 200 coloured point lights."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(pt, n_lights, seed=0):
    s = pt.Scene()
    s.exec_cfg("""
cam_pos 0 6 14
cam_pitch -22
cam_fov 55
r_sky_mode procedural
r_sun_elevation -30
r_spp 2
r_max_bounces 3
r_light_tree 1
prim_plane 1 0 1 0 0 lambert 0.70 0.70 0.70
prim_sphere 10 0 1 0 1 lambert 0.85 0.85 0.85
prim_sphere 11 2.5 0.8 1 0.8 dielectric 1 1 1 0 1.5
prim_sphere 12 -2.5 0.8 1 0.8 metal 0.9 0.9 0.9 0.1
""")
    rng = np.random.default_rng(seed)
    if n_lights == 4:
        s.light_point(1, (-3, 2.5, -1), (20, 8, 8))
        s.light_spot(2, (-1, 2.5, -1), (0, -1, 0), 25, 15, (10, 30, 10))
        s.light_sphere(3, (1, 2.5, -1), 0.3, (10, 10, 30))
        s.light_quad(4, (3, 2.5, -1), (0, -1, 0), (1, 0, 0), 0.4, 0.4, (30, 30, 10))
    else:
        for i in range(n_lights):
            p = (rng.uniform(-12, 12), 2.5, rng.uniform(-12, 6))
            s.light_point(i + 1, p, tuple(rng.uniform(0.4, 3.0, 3)))
    return s


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("n_lights", [1, 4, 200])
def test_light_tree_render_bit_exact(pt, orc, dev, n_lights, mode):
    s = _scene(pt, n_lights)
    W, H = 72, 48
    head, prm = s.push(W, H, frame_index=1, reset=1)
    assert prm.light_tree_enabled == 1 and prm.light_tree_node_count == 2 * n_lights - 1
    dev.set_traversal(mode)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, 2)
    g = dev.read_accum()
    o, _ = orc.render(s.packed(), head, prm, W, H, 2)
    assert g[..., :3].mean() > 0.01
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


def test_light_tree_changes_the_estimator_not_its_mean(pt, dev):
    """Tree and uniform picks are two unbiased estimators of the same image."""
    s = _scene(pt, 200)
    W, H = 48, 32
    dev.upload(s)
    dev.set_target(W, H)
    head, prm = s.push(W, H, frame_index=0, reset=1)
    dev.render(head, prm, 256)
    a = dev.read_accum()[..., :3].astype(np.float64)
    s.set_cvar("r_light_tree", 0)
    head, prm = s.push(W, H, frame_index=0, reset=1)
    assert prm.light_tree_enabled == 0
    dev.render(head, prm, 256)
    b = dev.read_accum()[..., :3].astype(np.float64)
    assert abs(a.mean() - b.mean()) < 0.02 * b.mean()


def test_light_tree_count_mismatch_is_rejected(pt, dev):
    s = _scene(pt, 4)
    dev.upload(s)
    dev.set_target(16, 16)
    head, prm = s.push(16, 16)
    prm.light_tree_node_count = 5
    with pytest.raises(pt.PtError):
        dev.render(head, prm, 1)
