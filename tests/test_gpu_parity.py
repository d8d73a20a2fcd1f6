"""GPU path vs the fp32 oracle, through the C-ABI.  The kernels evaluate the
shader's expressions in the same order with no FMA contraction, IEEE div/sqrt
and the same polynomial transcendentals, so the bar is bit-exact: identical
hit ids and t, identical accumulation buffers."""
import numpy as np
import pytest

from conftest import first_tested_wins, xorshift_rays, xorshift_spheres

pytestmark = pytest.mark.gpu

MODES = [pytest.param(0, id="wide_sah"), pytest.param(1, id="reference_bvh")]


def random_rays(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    ro = np.zeros((n, 4), np.float32)
    ro[:, :3] = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    rd = np.zeros((n, 4), np.float32)
    rd[:, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    return ro, rd


def check_trace(pt, orc, dev, s, ro, rd, mode=0):
    dev.set_traversal(mode)
    dev.upload(s)
    head, prm = s.push(8, 8)
    g_hit, g_t = dev.trace(ro, rd)
    o_hit, o_t, _ = orc.trace(s.packed(), head, prm, ro, rd)
    mism = np.flatnonzero((g_hit != o_hit) | (g_t != o_t))
    assert mism.size == 0, f"{mism.size} of {ro.shape[0]} rays differ, first {mism[:5]}"
    return o_hit


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("n,seed", [(50, 0xABCDEF01), (2000, 0x12345678)])
def test_trace_xorshift_spheres(pt, orc, dev, n, seed, mode):
    s = pt.Scene()
    for i, c in enumerate(xorshift_spheres(n, seed)):
        s.sphere(i, *map(float, c[:3]), float(c[3]), 0, (0.5, 0.5, 0.5))
    s.env(np.zeros((2, 4, 3), np.float32))
    ro, rd = xorshift_rays(1000, 0x12345678)
    hit = check_trace(pt, orc, dev, s, ro, rd, mode)
    assert (hit != 0xFFFFFFFF).sum() > 50


@pytest.mark.parametrize("mode", MODES)
def test_trace_c0_scene(pt, orc, dev, mode):
    s = pt.Scene().synth(0, seed=0)
    ro, rd = random_rays(20000, -12, 12, 1)
    hit = check_trace(pt, orc, dev, s, ro, rd, mode)
    assert ((hit & (1 << 30)) != 0).sum() > 100 and (hit < (1 << 30)).sum() > 100


@pytest.mark.parametrize("mode", MODES)
def test_trace_c1_scene_small(pt, orc, dev, mode):
    s = pt.Scene().synth(1, seed=0, scale=0.02)
    ro, rd = random_rays(20000, -60, 60, 2)
    ro[:, 1] = np.abs(ro[:, 1]) + 0.5
    check_trace(pt, orc, dev, s, ro, rd, mode)
    if mode == 0:
        info = dev.accel_info()
        assert info.mesh_wide == 1 and info.prims_wide == 1 and info.mesh_wide_nodes > 0


def grid_mesh_scene(pt, n=24):
    xs = np.linspace(-6, 6, n + 1, dtype=np.float32)
    pos = np.array([[x, 0.0, z] for z in xs for x in xs], np.float32)
    idx = []
    for j in range(n):
        for i in range(n):
            a = j * (n + 1) + i
            idx += [[a, a + n + 1, a + 1], [a + 1, a + n + 1, a + n + 2]]
    s = pt.Scene()
    s.mesh(pos, np.array(idx, np.uint32))
    s.env(np.zeros((2, 4, 3), np.float32))
    return s, xs


def vertex_rays(xs, m, seed):
    """Tilted rays aimed exactly at shared vertices of the grid: several triangles
    report (nearly) the same distance, so the tie rule decides the winner."""
    rng = np.random.default_rng(seed)
    n = xs.size - 1
    tgt = np.stack([xs[rng.integers(0, n + 1, m)], np.zeros(m, np.float32), xs[rng.integers(0, n + 1, m)]], 1)
    ro = np.zeros((m, 4), np.float32)
    ro[:, :3] = tgt + np.stack([rng.uniform(-2, 2, m), np.full(m, 5.0), rng.uniform(-2, 2, m)], 1)
    d = tgt.astype(np.float64) - ro[:, :3]
    rd = np.zeros((m, 4), np.float32)
    rd[:, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    return ro, rd


def test_trace_shared_vertex_ties_reference_walk_is_bit_exact(pt, orc, dev):
    s, xs = grid_mesh_scene(pt)
    ro, rd = vertex_rays(xs, 4000, 9)
    check_trace(pt, orc, dev, s, ro, rd, mode=1)


def test_trace_shared_vertex_ties_wide_tree(pt, orc, dev):
    """Equal distances on several triangles are resolved by the reference rank,
    and a triangle whose reference leaf box the ray only touches at a corner
    (these rays aim at grid vertices, so about one in five does),
    where the reference's unpadded slab test rounds tmax below tmin and the
    reference walk never tests it, is dropped as the reference drops it: the
    wide tree returns the reference walk's (the oracle's) hits exactly.  Against
    the brute-force first-tested-wins rule over every triangle the intersector
    accepts, the rays that differ are exactly those corner cases, where the
    brute force keeps a hit the reference walk does not."""
    s, xs = grid_mesh_scene(pt)
    ro, rd = vertex_rays(xs, 1500, 9)
    o_hit = check_trace(pt, orc, dev, s, ro, rd, mode=0)
    want_hit, _ = first_tested_wins(s.arrays(), ro, rd)
    corner = np.flatnonzero(o_hit != want_hit)
    print(f"{corner.size} of {len(ro)} rays lose a corner-touched triangle in the reference walk")
    assert (want_hit[corner] != 0xFFFFFFFF).all()


def test_trace_full_c1_rays_agreement(pt, orc, dev):
    """2^17 camera + 2^17 random rays of the full 2.46 M-triangle scene: both
    the reference walk and the wide tree return the oracle's hits bit for bit."""
    s = pt.Scene().synth(1, seed=0)
    W, H = 1920, 1080
    head, prm = s.push(W, H)
    rng = np.random.default_rng(11)
    m = 1 << 17
    px, py = rng.uniform(0, W, m), rng.uniform(0, H, m)
    u = (px / W) * 2 - 1
    v = -((py / H) * 2 - 1)
    fwd, right, up = (np.array(x[:3], np.float64) for x in (head.fwd_aspect, head.right_xyz, head.up_xyz))
    d = fwd + np.outer(u * head.fwd_aspect[3] * head.pos_fovtan[3], right) + np.outer(v * head.pos_fovtan[3], up)
    ro = np.zeros((2 * m, 4), np.float32)
    rd = np.zeros((2 * m, 4), np.float32)
    ro[:m, :3] = head.pos_fovtan[:3]
    rd[:m, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    ro2, rd2 = random_rays(m, -100, 100, 12)
    ro2[:, 1] = np.abs(ro2[:, 1]) * 0.1 + 0.05
    ro[m:], rd[m:] = ro2, rd2
    o_hit, o_t, _ = orc.trace(s.packed(), head, prm, ro, rd)
    check_trace(pt, orc, dev, s, ro, rd, mode=1)
    dev.set_traversal(0)
    dev.upload(s)
    g_hit, g_t = dev.trace(ro, rd)
    np.testing.assert_array_equal(g_hit, o_hit)
    np.testing.assert_array_equal(g_t, o_t)


def render_both(pt, orc, dev, s, W, H, frames, mode=0):
    dev.set_traversal(mode)
    dev.upload(s)
    dev.set_target(W, H)
    head, prm = s.push(W, H, frame_index=11, reset=1)
    dev.render(head, prm, frames)
    g = dev.read_accum()
    o, c = orc.render(s.packed(), head, prm, W, H, frames)
    return g, o, c


@pytest.mark.parametrize("mode", MODES)
def test_render_c0_bit_exact(pt, orc, dev, mode):
    s = pt.Scene().synth(0, seed=3)
    g, o, c = render_both(pt, orc, dev, s, 48, 40, 2, mode)
    st = dev.stats()
    assert st.extension_rays == c.ext_rays
    assert st.shadow_rays == c.shadow_rays
    np.testing.assert_array_equal(g, o)
    assert (g[..., 3] == 2).all() and g[..., :3].max() > 0


@pytest.mark.parametrize("mode", MODES)
def test_render_c1_small_bit_exact(pt, orc, dev, mode):
    s = pt.Scene().synth(1, seed=4, scale=0.02)
    g, o, c = render_both(pt, orc, dev, s, 64, 36, 3, mode)
    assert dev.stats().shadow_rays == c.shadow_rays
    np.testing.assert_array_equal(g, o)
    assert g[..., :3].max() > 0


def test_render_mis_off_and_no_clamp_bit_exact(pt, orc, dev):
    s = pt.Scene().synth(1, seed=5, scale=0.02)
    s.set_cvar("r_mis", 0)
    s.set_cvar("r_firefly_clamp", 0)
    s.set_cvar("r_caustics", 0)
    g, o, _ = render_both(pt, orc, dev, s, 40, 30, 2)
    np.testing.assert_array_equal(g, o)


def test_render_lights_of_every_type_bit_exact(pt, orc, dev):
    s = pt.Scene()
    s.plane(1, (0, 1, 0), 0.0, 0, (0.7, 0.7, 0.7))
    s.sphere(2, 0, 1, 0, 1, 0, (0.8, 0.3, 0.2))
    s.sphere(3, 2.5, 0.7, 0.5, 0.7, 2, (1, 1, 1), 0, 1.5)
    s.sphere(4, -2.5, 0.8, 0, 0.8, 1, (0.9, 0.9, 0.9), 0.1)
    s.emission(4, (0.5, 0.2, 0.1))
    s.light_point(1, (0, 5, 2), (20, 20, 20))
    s.light_spot(2, (3, 4, 3), (-0.5, -1, -0.5), 40, 20, (30, 25, 20))
    s.light_sphere(3, (-3, 4, 2), 0.5, (8, 8, 8))
    s.light_quad(4, (0, 6, -2), (0, -1, 0), (1, 0, 0), 1.0, 0.5, (10, 10, 10))
    s.env(np.full((8, 16, 3), 0.05, np.float32))
    s.camera((0, 2, 8), 0.0, -0.15, 50)
    s.set_cvar("r_spp", 4)
    g, o, _ = render_both(pt, orc, dev, s, 40, 32, 2)
    np.testing.assert_array_equal(g, o)


def test_wave_batching_does_not_change_the_result(pt, dev):
    s = pt.Scene().synth(1, seed=6, scale=0.02)
    dev.upload(s)
    W, H = 32, 24
    dev.set_target(W, H)
    head, prm = s.push(W, H, 0, 1)
    outs = []
    for fpw in (1, 3, 0):
        dev.set_wave_frames(fpw)
        dev.render(head, prm, 5)
        outs.append(dev.read_accum())
    dev.set_wave_frames(0)
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[0], outs[2])


def test_resume_from_saved_accumulation(pt, dev):
    """frames 0..3 in one call == frames 0..1, save, restore, frames 2..3."""
    s = pt.Scene().synth(0, seed=7)
    dev.upload(s)
    W, H = 24, 24
    dev.set_target(W, H)
    head, prm = s.push(W, H, 0, 1)
    dev.render(head, prm, 4)
    ref = dev.read_accum()
    dev.render(head, prm, 2)
    saved = dev.read_accum()
    dev.set_target(W, H)
    dev.write_accum(saved)
    head2, prm2 = s.push(W, H, 2, 0)
    dev.render(head2, prm2, 2)
    np.testing.assert_array_equal(dev.read_accum(), ref)


def test_invalid_inputs_are_rejected(pt, dev):
    import ctypes
    lib = pt.load()
    recs = np.zeros((4, 28), np.float32)
    bad = (pt.PtBvhNode * 3)()
    bad[0].count = 0
    bad[0].left_first = 0          # child index not after its parent: would loop
    rc = lib.pt_gpu_upload_prims(dev.h, pt.fptr(recs), 4, 0, bad, 3)
    assert rc == -1
    bad[0].left_first = 1
    bad[1].count = 9               # leaf range past the records
    bad[2].count = 1
    assert lib.pt_gpu_upload_prims(dev.h, pt.fptr(recs), 4, 0, bad, 3) == -1
    s = pt.Scene().synth(0)
    dev.upload(s)
    dev.set_target(8, 8)
    head, prm = s.push(8, 8)
    head.prim_count += 1
    assert lib.pt_gpu_render(dev.h, ctypes.byref(head), ctypes.byref(prm), 1) == -1
    head.prim_count -= 1
    head.tlas_present = 1
    assert lib.pt_gpu_render(dev.h, ctypes.byref(head), ctypes.byref(prm), 1) == -6


def test_full_size_c1_frame_matches_oracle_on_crops(pt, orc, dev):
    """1920x1080 C1 frame: finite, count 1, and three 16x16 crops identical to the oracle."""
    s = pt.Scene().synth(1, seed=0)
    W, H = 1920, 1080
    dev.set_traversal(0)
    dev.upload(s)
    info = dev.accel_info()
    assert info.mesh_wide == 1 and info.prims_wide == 1
    dev.set_target(W, H)
    head, prm = s.push(W, H, 0, 1)
    dev.render(head, prm, 1)
    g = dev.read_accum()
    assert np.isfinite(g).all() and (g[..., 3] == 1).all()
    assert dev.stats().extension_rays >= W * H
    acc = np.zeros((H, W, 4), np.float32)
    for (x0, y0) in ((952, 532), (100, 900), (1700, 200)):
        orc.render(s.packed(), head, prm, W, H, 1, accum=acc, crop=(x0, y0, x0 + 16, y0 + 16))
        np.testing.assert_array_equal(g[y0:y0 + 16, x0:x0 + 16], acc[y0:y0 + 16, x0:x0 + 16])


def _batch_setup(pt):
    scenes = [pt.Scene().synth(1, seed=k, scale=0.02) for k in range(3)] + [pt.Scene().synth(0, seed=9)]
    devs = []
    for s in scenes:
        d = pt.Device(0)
        d.upload(s)
        devs.append(d)
    sizes = [(32, 24), (48, 40), (16, 16), (40, 32), (30, 18), (64, 36), (8, 4)]
    views = []
    for i, (w, h) in enumerate(sizes):
        k = i % len(scenes)
        head, prm = scenes[k].push(w, h, frame_index=10 + 3 * i, reset=1)
        head.spp = 1 + (i % 3)
        head.max_bounces = 3 + (i % 6)
        views.append((k, w, h, head, prm))
    return scenes, devs, views


def test_batch_render_equals_plain_render_per_view(pt, dev):
    scenes, devs, views = _batch_setup(pt)
    for use_graph in (1, 0):
        batch = pt.Device(0)
        batch.batch_set_tuning(4, 8, use_graph)
        batch.batch_render(devs, views, frames=2)
        st = batch.stats()
        assert st.extension_rays > 0 and st.shadow_rays > 0
        for i, (k, w, h, head, prm) in enumerate(views):
            d = devs[k]
            d.set_target(w, h)
            d.render(head, prm, 2)
            np.testing.assert_array_equal(batch.batch_read(i, w, h), d.read_accum(), err_msg=f"view {i}")
        batch.close()


def test_batch_autotune_keeps_results(pt, dev):
    scenes, devs, views = _batch_setup(pt)
    batch = pt.Device(0)
    t = batch.batch_autotune(devs, views)
    assert 1 <= t.persistent_blocks_per_sm <= 4 and t.shade_threads in (256, 512)
    assert t.camera_tile_w in (4, 8, 16, 32) and t.octant_grouping in (0, 1) and t.use_graph in (0, 1)
    d_ms, t_ms = batch.batch_tuning_gain()
    assert 0 < t_ms <= d_ms
    batch.batch_render(devs, views, frames=1)
    k, w, h, head, prm = views[1]
    devs[k].set_target(w, h)
    devs[k].render(head, prm, 1)
    np.testing.assert_array_equal(batch.batch_read(1, w, h), devs[k].read_accum())


@pytest.mark.parametrize("tile,octants,shade", [(4, 1, 512), (16, 0, 256), (32, 1, 256)])
def test_batch_launch_shapes_keep_results(pt, dev, tile, octants, shade):
    """Every launch-shape knob the autotuner searches (camera tile, octant
    grouping of the queue, shading block) leaves each view bit-identical to its
    plain render."""
    scenes, devs, views = _batch_setup(pt)
    batch = pt.Device(0)
    batch.batch_set_tuning(3, 4, 1, shade, tile, octants)
    batch.batch_render(devs, views, frames=1)
    for i, (k, w, h, head, prm) in enumerate(views):
        devs[k].set_target(w, h)
        devs[k].render(head, prm, 1)
        np.testing.assert_array_equal(batch.batch_read(i, w, h), devs[k].read_accum(), err_msg=f"view {i}")
    with pytest.raises(pt.PtError):
        batch.batch_set_tuning(4, 8, 1, 384, 8, 1)
    batch.close()


@pytest.mark.parametrize("mode", MODES)
def test_records_without_a_bvh_are_scanned_linearly_far_away(pt, orc, dev, mode):
    """With fewer finite records than r_analytic_bvh_threshold there is no
    analytic BVH and the reference tests every record linearly, in record order,
    with no bounding box in front of it (shaders/PathTrace.slang:2402-2434).
    From ~10^4 units away a sphere's float intersection cancels badly
    (b^2 - (|oc|^2 - r^2) with |oc|^2 ~ 10^8) and reports hits for rays that
    pass a few units outside it; a box test would cull those rays.  Both
    traversal modes must return the oracle's hits bit for bit, these far hits
    included (shadow rays from far ground points toward lights beside a sphere
    meet exactly this case)."""
    s = pt.Scene()
    s.env(np.full((4, 8, 3), 0.1, np.float32))
    s.plane(1, (0.0, 1.0, 0.0), 0.0, 0, (0.7, 0.7, 0.7))
    s.sphere(10, 0.0, 1.0, 0.0, 1.0, 0, (0.85, 0.85, 0.85))
    s.sphere(11, 3.0, 1.5, -2.0, 0.5, 1, (0.9, 0.9, 0.9))
    head, prm = s.push(8, 8)
    assert prm.bvh_params[1] == 0
    rng = np.random.default_rng(17)
    n = 1 << 14
    ang = rng.uniform(0, 2 * np.pi, n)
    dist = 10 ** rng.uniform(3, 4.3, n)
    o = np.stack([dist * np.cos(ang), rng.uniform(1e-3, 0.05, n), dist * np.sin(ang)], 1)
    tgt = np.array([0.0, 1.0, 0.0]) + rng.uniform(-6, 6, (n, 3)) * [1, 0.3, 1]
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    ro = np.zeros((n, 4), np.float32)
    rd = np.zeros((n, 4), np.float32)
    ro[:, :3], rd[:, :3] = o, d
    o_hit, o_t, _ = orc.trace(s.packed(), head, prm, ro, rd)
    dev.set_traversal(mode)
    dev.upload(s)
    g_hit, g_t = dev.trace(ro, rd)
    np.testing.assert_array_equal(g_hit, o_hit)
    np.testing.assert_array_equal(g_t, o_t)
    # some of these hits are the far-field artefact: the ray's true distance
    # from the sphere centre exceeds the radius
    c = np.array([0.0, 1.0, 0.0])
    oc = c - ro[:, :3].astype(np.float64)
    miss_dist = np.linalg.norm(oc - (oc * rd[:, :3]).sum(1, keepdims=True) * rd[:, :3], axis=1)
    assert ((o_hit == 1) & (miss_dist > 1.05)).any()


def _mixed_scene(pt, n=400, seed=31, with_sdf=False):
    """Small spheres and small triangles interleaved in the same places, so that
    the merged tree's SAH build makes leaves holding both kinds, which it splits
    into a triangle leaf and a record leaf.  A plane is tested linearly."""
    rng = np.random.default_rng(seed)
    s = pt.Scene()
    s.env(np.full((4, 8, 3), 0.3, np.float32))
    s.plane(1, (0.0, 1.0, 0.0), 9.0, 0, (0.6, 0.6, 0.6))
    c = rng.uniform(-8.0, 8.0, (n, 3))
    for i in range(n):
        s.sphere(100 + i, *c[i], float(rng.uniform(0.05, 0.3)), i % 3, (0.7, 0.5, 0.3))
    pos = (c[:, None, :] + rng.uniform(-0.4, 0.4, (n, 1, 3)) + rng.uniform(-0.9, 0.9, (n, 3, 3))).reshape(-1, 3)
    idx = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    s.mesh(pos.astype(np.float32), idx)
    if with_sdf:
        s.sdf_leaf(500, 0, (0.8,), (0.0, 0.0, 0.0), 0, (0.8, 0.8, 0.8))
    s.camera((0.0, 2.0, 24.0), 0.0, 0.0, 50.0)
    return s


@pytest.mark.parametrize("with_sdf", [False, True])
def test_merged_tree_matches_the_reference(pt, orc, dev, with_sdf):
    """Spheres in a BVH plus a mesh, no SDF cluster: the wide-tree kernels walk
    one merged tree over both.  Its hits are the reference walk's (each item
    keeps its reference tie rank), on rays and in renders; with an SDF cluster
    the dispatch keeps the two trees (the cluster sits between them in the
    reference's order) and is bit-exact as well."""
    s = _mixed_scene(pt, with_sdf=with_sdf)
    dev.set_traversal(0)
    dev.upload(s)
    info = dev.accel_info()
    assert info.mesh_wide and info.prims_wide and info.merged_wide_nodes > 0
    ro, rd = random_rays(1 << 14, -12.0, 12.0, 41)
    head, prm = s.push(8, 8)
    o_hit, o_t, _ = orc.trace(s.packed(), head, prm, ro, rd)
    g_hit, g_t = dev.trace(ro, rd)
    agree = g_hit == o_hit
    assert agree.mean() >= 0.9999, agree.mean()
    assert np.array_equal(g_t[agree], o_t[agree])
    hit = o_hit != 0xFFFFFFFF
    assert (hit & ((o_hit & (1 << 30)) != 0)).sum() > 100 and (hit & ((o_hit & (1 << 30)) == 0)).sum() > 100
    W, H = 64, 48
    dev.set_target(W, H)
    head, prm = s.push(W, H, frame_index=3, reset=1)
    dev.render(head, prm, 2)
    o, _ = orc.render(s.packed(), head, prm, W, H, 2)
    assert np.array_equal(dev.read_accum().view(np.uint32), o.view(np.uint32))
