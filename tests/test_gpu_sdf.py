"""SDF clusters on the GPU against the oracle: closest-hit ids and distances
bit for bit (analytic prims + SDF clusters + mesh together), and renders bit
for bit in both traversal modes, with a dielectric SDF in the shadow rays.
Fractal leaves (Mandelbulb, Mandelbox, Apollonian) the same way, their hit ids
carrying the accepted march step."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCENE = """
cam_pos 0 2.2 7
cam_pitch -12
cam_fov 55
r_sky_mode procedural
r_sun_elevation 40
r_spp 2
r_max_bounces 4
prim_plane 1 0 1 0 0 lambert 0.6 0.6 0.6
prim_sphere 10 2.6 0.8 0.4 0.8 metal 0.9 0.8 0.7 0.1
sdf_sphere 1 0.8 0 1 0 lambert 0.9 0.3 0.2
sdf_box 2 0.5 0.6 0.5 0.6 1.1 0 lambert 0.2 0.4 0.9
sdf_smin 3 1 2 0.35 lambert 0.6 0.5 0.4
sdf_torus 4 0.9 0.25 -2.2 0.6 0.3 dielectric 1 1 1
sdf_capsule 5 0.6 0.3 1.2 0.9 -1.5 metal 0.9 0.9 0.9
sdf_round_box 6 0.5 0.3 0.5 0.1 -0.8 0.45 1.6 lambert 0.8 0.8 0.2
sdf_sdiff 7 6 5 0.05 lambert 0.4 0.7 0.4
light_point 1 -2 3 2 15 15 15
"""


def _scene(pt, with_mesh=True):
    s = pt.Scene()
    rep, n = s.exec_cfg(SCENE)
    assert n == 0, rep
    if with_mesh:   # a small box mesh that the SDFs and analytic prims overlap
        pos = np.array([[x, y, z] for x in (-3.2, -2.0) for y in (0.0, 1.4) for z in (-2.0, -0.8)], np.float32)
        idx = np.array([[0, 2, 1], [1, 2, 3], [4, 5, 6], [5, 7, 6], [0, 1, 4], [1, 5, 4],
                        [2, 6, 3], [3, 6, 7], [0, 4, 2], [2, 4, 6], [1, 3, 5], [3, 7, 5]], np.uint32)
        s.mesh(pos, idx)
    return s


@pytest.mark.parametrize("mode", [0, 1])
def test_sdf_trace_probe_bit_exact(pt, orc, dev, mode):
    s = _scene(pt)
    dev.set_traversal(mode)
    dev.upload(s)
    head, prm = s.push(8, 8)
    rng = np.random.default_rng(5)
    n = 20000
    ro = np.zeros((n, 4), np.float32)
    ro[:, :3] = rng.uniform(-4, 4, (n, 3)) + np.array([0, 1.5, 5])
    d = rng.uniform(-4, 4, (n, 3)) + np.array([0, 0.5, 0]) - ro[:, :3]
    rd = np.zeros((n, 4), np.float32)
    rd[:, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    g_hit, g_t = dev.trace(ro, rd)
    o_hit, o_t, _ = orc.trace(s.packed(), head, prm, ro, rd)
    assert ((o_hit & 0x80000000) != 0).sum() - (o_hit == 0xFFFFFFFF).sum() > 500   # SDF hits present
    mism = np.flatnonzero((g_hit != o_hit) | (g_t != o_t))
    assert mism.size == 0, (mism.size, mism[:5])


@pytest.mark.parametrize("mode", [0, 1])
def test_sdf_render_bit_exact(pt, orc, dev, mode):
    s = _scene(pt)
    W, H = 72, 48
    head, prm = s.push(W, H, frame_index=2, reset=1)
    dev.set_traversal(mode)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, 2)
    g = dev.read_accum()
    o, _ = orc.render(s.packed(), head, prm, W, H, 2)
    assert g[..., :3].mean() > 0.02
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


def test_sdf_batch_equals_plain(pt, dev):
    s = _scene(pt, with_mesh=False)
    scene = pt.Device(0)
    scene.upload(s)
    W, H = 40, 32
    head, prm = s.push(W, H, frame_index=4, reset=1)
    batch = pt.Device(0)
    batch.batch_render([scene], [(0, W, H, head, prm)], 1)
    b = batch.batch_read(0, W, H)
    scene.set_target(W, H)
    scene.render(head, prm, 1)
    assert np.array_equal(b.view(np.uint32), scene.read_accum().view(np.uint32))
    batch.close()
    scene.close()


FRACTAL_SCENE = """
cam_pos 0 3 9
cam_pitch -14
cam_fov 60
r_sky_mode procedural
r_sun_elevation 35
r_spp 1
r_max_bounces 3
prim_plane 1 0 1 0 0 lambert 0.6 0.6 0.6
sdf_mandelbulb 1 8 1.3 0 1.3 0 lambert 0.9 0.5 0.2
sdf_mandelbox 2 2.5 4.2 -5 4.2 -7 metal 0.8 0.8 0.9
sdf_apollonian 3 1.3 1.8 3.5 1.8 -1 lambert 0.4 0.7 0.9
sdf_sphere 4 0.6 -2.5 0.6 2 dielectric 1 1 1
light_point 1 2 5 4 25 25 25
"""


def _fractal_scene(pt):
    s = pt.Scene()
    rep, n = s.exec_cfg(FRACTAL_SCENE)
    assert n == 0, rep
    return s


@pytest.mark.parametrize("mode", [0, 1])
def test_sdf_fractal_probe_bit_exact(pt, orc, dev, mode):
    s = _fractal_scene(pt)
    dev.set_traversal(mode)
    dev.upload(s)
    head, prm = s.push(8, 8)
    rng = np.random.default_rng(8)
    n = 6000
    ro = np.zeros((n, 4), np.float32)
    ro[:, :3] = rng.uniform(-3, 3, (n, 3)) + np.array([0, 3, 9])
    d = rng.uniform(-5, 5, (n, 3)) + np.array([-0.5, 2.0, -3]) - ro[:, :3]
    rd = np.zeros((n, 4), np.float32)
    rd[:, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    g_hit, g_t = dev.trace(ro, rd)
    o_hit, o_t, _ = orc.trace(s.packed(), head, prm, ro, rd)
    frac = ((o_hit & 0xC0000000) == 0x80000000) & ((o_hit & 0xFFFFF) < 3)
    assert frac.sum() > 300 and ((o_hit >> 20) & 0x1FF)[frac].max() > 4   # fractal hits with step bits
    mism = np.flatnonzero((g_hit != o_hit) | (g_t != o_t))
    assert mism.size == 0, (mism.size, mism[:5])


@pytest.mark.parametrize("mode", [0, 1])
def test_sdf_fractal_render_bit_exact(pt, orc, dev, mode):
    s = _fractal_scene(pt)
    W, H = 48, 32
    head, prm = s.push(W, H, frame_index=1, reset=1)
    dev.set_traversal(mode)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, 1)
    g = dev.read_accum()
    o, _ = orc.render(s.packed(), head, prm, W, H, 1)
    assert g[..., :3].mean() > 0.02
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


def test_sdf_count_mismatch_and_bad_ops_are_rejected(pt, dev):
    s = _scene(pt, with_mesh=False)
    dev.upload(s)
    dev.set_target(16, 16)
    head, prm = s.push(16, 16)
    prm.sdf_params[0] = 1
    with pytest.raises(pt.PtError):
        dev.render(head, prm, 1)
    bad = np.zeros(112, np.float32)
    bad[3:4].view(np.uint32)[0] = 1
    bad[16:20].view(np.uint32)[:] = [10, 0, 0, 0]          # an op past the last one
    with pytest.raises(pt.PtError):
        dev._check(dev.lib.pt_gpu_upload_sdf(dev.h, bad.ctypes.data_as(pt.P(pt.f32)), 1))


PROC_SCENE = """
cam_pos 0 2.5 9
cam_pitch -12
cam_fov 55
r_sky_mode procedural
r_sun_elevation 40
r_spp 1
r_max_bounces 3
r_sdf_max_iters 192
r_sdf_procedural_ops 1
prim_plane 1 0 1 0 0.8 lambert 0.6 0.6 0.6
sdf_box 1 4 0.25 4 0 -0.5 0 lambert 0.45 0.55 0.40
sdf_displace_noise 2 1 0.25 0.5 5 lambert 0.45 0.55 0.40
sdf_box 10 0.3 1.0 0.3 -2 1 0 metal 0.85 0.55 0.20
sdf_twist 11 10 1.8 metal 0.85 0.55 0.20
sdf_capsule 20 1.0 0.3 2 1.2 0 dielectric 1 1 1
sdf_bend 21 20 0.5 dielectric 1 1 1
sdf_sphere 30 0.18 0 1.8 -2.5 lambert 0.85 0.30 0.45
sdf_repeat_limited 31 30 0.6 0 0 3 0 0 lambert 0.85 0.30 0.45
sdf_sphere 40 0.2 3.5 0.4 0 lambert 0.5 0.5 0.5
sdf_repeat 41 40 0 0 0.9 lambert 0.5 0.5 0.5
light_point 1 -2 4 3 20 20 20
"""


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("on", [1, 0, 2])
def test_sdf_procedural_render_bit_exact(pt, orc, dev, mode, on):
    """Procedural ops 5-9 (fBm displace, twist, bend, limited and unbounded
    repetition; a dielectric bent capsule in the shadow rays) render bit for bit
    as the oracle does: on with central-difference normals (1), off, where they
    read as empty (0), and on with forward-mode AD normals (2)."""
    s = pt.Scene()
    rep, n = s.exec_cfg(PROC_SCENE + "r_sdf_procedural_ops %d\n" % on)
    assert n == 0, rep
    W, H = 64, 48
    head, prm = s.push(W, H, frame_index=3, reset=1)
    assert prm.sdf_procedural_ops == on
    dev.set_traversal(mode)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, 2)
    g = dev.read_accum()
    o, _ = orc.render(s.packed(), head, prm, W, H, 2)
    assert g[..., :3].mean() > 0.02
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


def test_sdf_procedural_batch_equals_plain(pt, dev):
    s = pt.Scene()
    rep, n = s.exec_cfg(PROC_SCENE)
    assert n == 0, rep
    scene = pt.Device(0)
    scene.upload(s)
    W, H = 40, 32
    head, prm = s.push(W, H, frame_index=4, reset=1)
    batch = pt.Device(0)
    batch.batch_render([scene], [(0, W, H, head, prm)], 1)
    b = batch.batch_read(0, W, H)
    scene.set_target(W, H)
    scene.render(head, prm, 1)
    assert np.array_equal(b.view(np.uint32), scene.read_accum().view(np.uint32))
    batch.close()
    scene.close()
