"""Host builders against the reference's own builders: golden fixtures made by
the reference's AnalyticBvh / TriangleBvh / BuildEnvCdf compiled from source
(tests/golden/make_golden.py), the reference CDF test's 4x4 known answer
(tests/hdrimage_cdf_test.cpp:233-294), and the Engine packing rules."""
import ctypes
import os

import numpy as np
import pytest

from conftest import ROOT, xorshift_spheres

G = np.load(os.path.join(ROOT, "tests", "golden", "reference_builders.npz"))


def product_analytic_bvh(pt, cr):
    n = cr.shape[0]
    nodes = (pt.PtBvhNode * max(2 * n, 1))()
    perm = np.zeros(max(n, 1), np.uint32)
    m = ctypes.c_uint32()
    assert pt.load().pt_build_analytic_bvh(pt.fptr(cr), n, nodes, ctypes.byref(m), pt.uptr(perm)) == 0
    return np.frombuffer(nodes, np.uint32).reshape(-1, 8)[: m.value].copy(), perm[:n]


def product_tri_bvh(pt, pos, idx):
    nt = max(idx.size // 3, 1)
    nodes = (pt.PtBvhNode * (2 * nt))()
    perm = np.zeros(nt, np.uint32)
    m, k = ctypes.c_uint32(), ctypes.c_uint32()
    assert pt.load().pt_build_triangle_bvh(pt.fptr(pos), pos.size // 3, pt.uptr(idx), idx.size, nodes,
                                           ctypes.byref(m), pt.uptr(perm), ctypes.byref(k)) == 0
    return np.frombuffer(nodes, np.uint32).reshape(-1, 8)[: m.value].copy(), perm[: k.value]


def product_env_cdf(pt, img, mask=None):
    H, W = img.shape[:2]
    marg = np.zeros(H, np.float32)
    cond = np.zeros(H * W, np.float32)
    tot = ctypes.c_double()
    mk = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    assert pt.load().pt_build_env_cdf(pt.fptr(np.ascontiguousarray(img, np.float32)), W, H,
                                      None if mk is None else mk.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                      pt.fptr(marg), pt.fptr(cond), ctypes.byref(tot)) == 0
    return marg, cond.reshape(H, W), tot.value


@pytest.mark.parametrize("name", ["s50", "s2000"])
def test_analytic_bvh_matches_reference_golden(pt, name):
    nodes, perm = product_analytic_bvh(pt, G[f"{name}_cr"])
    np.testing.assert_array_equal(nodes, G[f"{name}_nodes"])
    np.testing.assert_array_equal(perm, G[f"{name}_perm"])


def test_analytic_bvh_golden_inputs_are_the_reference_scene():
    np.testing.assert_array_equal(G["s50_cr"], xorshift_spheres(50, 0xABCDEF01))


def test_analytic_bvh_edge_cases(pt):
    nodes, perm = product_analytic_bvh(pt, np.zeros((0, 4), np.float32))
    assert nodes.shape[0] == 0
    nodes, perm = product_analytic_bvh(pt, np.array([[0, 0, 5, 1]], np.float32))
    assert nodes.shape[0] == 1 and nodes[0, 7] == 1 and perm[0] == 0
    # many prims on one splitting plane / identical centroids: every prim reachable once
    cr = np.zeros((37, 4), np.float32)
    cr[:, 3] = 0.5
    nodes, perm = product_analytic_bvh(pt, cr)
    assert sorted(perm.tolist()) == list(range(37))
    leaves = nodes[nodes[:, 7] > 0]
    assert leaves[:, 7].max() <= 4


def test_triangle_bvh_matches_reference_golden(pt):
    nodes, perm = product_tri_bvh(pt, G["tri_pos"], G["tri_idx"])
    np.testing.assert_array_equal(nodes, G["tri_nodes"])
    np.testing.assert_array_equal(perm, G["tri_perm"])
    assert (G["tri_idx"].shape[0] - 1) not in perm.tolist()   # out-of-range triangle skipped


def test_triangle_bvh_bad_index_count_is_empty(pt):
    nodes, perm = product_tri_bvh(pt, G["tri_pos"], G["tri_idx"].reshape(-1)[:10])
    assert nodes.shape[0] == 0 and perm.size == 0


@pytest.mark.parametrize("masked", [False, True])
def test_env_cdf_matches_reference_golden(pt, masked):
    sfx = "_m" if masked else ""
    marg, cond, tot = product_env_cdf(pt, G["env_img"], G["env_mask"] if masked else None)
    np.testing.assert_array_equal(marg, G["env_marg" + sfx])
    np.testing.assert_array_equal(cond, G["env_cond" + sfx])
    assert tot == float(G["env_total" + sfx])


def test_env_cdf_4x4_known_answer(pt):
    W = H = 4
    img = np.zeros((H, W, 3), np.float32)
    for v in range(H):
        img[v] = (v + 1) / H
    marg, cond, tot = product_env_cdf(pt, img)
    st = np.sin(np.pi * (np.arange(H) + 0.5) / H)
    rows = W * (np.arange(H) + 1) / H * st
    assert tot == pytest.approx(rows.sum(), rel=1e-6)
    ref_m = (np.cumsum(rows) / rows.sum()).astype(np.float32)
    ref_m[-1] = 1.0
    np.testing.assert_allclose(marg, ref_m, rtol=1e-5)
    np.testing.assert_allclose(cond, np.tile((np.arange(W) + 1) / W, (H, 1)), rtol=1e-5)


def test_env_cdf_zero_image(pt):
    marg, cond, tot = product_env_cdf(pt, np.zeros((8, 16, 3), np.float32))
    assert tot == 0.0 and not marg.any() and not cond.any()


def test_live_reference_builders_when_available(pt, orc):
    """Random inputs through the reference's builders compiled from source
    (present only where the reference tree is)."""
    if orc.load_ref() is None:
        pytest.skip("reference builders not built here")
    rng = np.random.default_rng(7)
    for n in (5, 17, 300, 4096):
        cr = np.concatenate([rng.uniform(-50, 50, (n, 3)), rng.uniform(0.01, 3, (n, 1))], 1).astype(np.float32)
        a, b = product_analytic_bvh(pt, cr), orc.ref_analytic_bvh(cr)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
    pos = rng.uniform(-5, 5, (999, 3)).astype(np.float32)
    idx = rng.integers(0, 999, (1500, 3)).astype(np.uint32)
    a, b = product_tri_bvh(pt, pos, idx), orc.ref_triangle_bvh(pos, idx)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    img = rng.lognormal(0, 1.5, (64, 128, 3)).astype(np.float32)
    a, b = product_env_cdf(pt, img), orc.ref_env_cdf(img)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[2] == b[2]


def test_scene_packing_rules(pt):
    """Planes first, finite prims in BVH leaf order, user id in v2.w, lights in id order
    (src/engine/Engine.cpp:4743-5003, 5235-5330)."""
    s = pt.Scene()
    s.set_cvar("r_analytic_bvh_threshold", 4)
    for i, c in enumerate(xorshift_spheres(20, 99)):
        s.sphere(100 - i, *c[:3], c[3], i % 3, (0.5, 0.5, 0.5))
    s.plane(7, (0, 2, 0), 1.0, 0, (0.8, 0.8, 0.8))
    s.light_quad(5, (0, 5, 0), (0, -1, 0), (1, 0, 0), 0.5, 0.25, (15, 15, 15))
    s.light_point(2, (1, 2, 3), (4, 5, 6))
    a = s.arrays()
    assert a["linear"] == 1 and a["prims"][0, 8] == 1.0 and a["prims"][0, 1] == 1.0
    assert a["prims"][0, 11].view(np.uint32) == 7
    fin = a["prims"][1:]
    ids = fin[:, 11].view(np.uint32)
    assert sorted(ids.tolist()) == list(range(81, 101))
    # leaf order = reference builder over the finite prims in id order
    cr = np.stack([fin[:, 0], fin[:, 1], fin[:, 2], fin[:, 3]], 1)
    order = np.argsort(ids)
    nodes, perm = product_analytic_bvh(pt, np.ascontiguousarray(cr[order]))
    np.testing.assert_array_equal(a["bvh"], nodes)
    np.testing.assert_array_equal(ids[np.argsort(ids)][perm], ids)
    assert a["lights"][0, 7] == 0.0 and a["lights"][1, 7] == 3.0   # id 2 point, id 5 quad
    np.testing.assert_allclose(a["lights"][1, 12:15], [0.5, 0, 0])
    assert a["lights"][1, 15] == 0.25


def test_hdri_extraction_keeps_the_sun(pt):
    s = pt.Scene()
    img = np.full((64, 128, 3), 0.2, np.float32)
    img[20:23, 40:43] = 1e4          # 9-pixel bright cluster
    img[50, 100] = 1e4               # single pixel: dropped (< 3 pixels) and unmasked
    s.env(img)
    a = s.arrays()
    assert a["hdri_count"] == 1
    assert a["hdri_dir_pmf"][0, 3] == pytest.approx(1.0)
    c = a["env_conditional"]
    assert (c[21, 41] <= c[21, 40])   # masked pixel adds no CDF mass
    assert c[50, 100] > c[50, 99]     # the dropped cluster stays in the CDF


def _halton_jitter(frame_index):
    """The engine's sub-pixel jitter with the denoiser on, in float32 as it
    computes it (src/engine/Engine.cpp:8241-8252)."""
    f32 = np.float32

    def ri(i, base):
        f, r = f32(1.0), f32(0.0)
        while i > 0:
            f = f32(f / f32(base))
            r = f32(r + f32(f * f32(i % base)))
            i //= base
        return r

    hi = frame_index % 16 + 1
    return f32(ri(hi, 2) - f32(0.5)), f32(ri(hi, 3) - f32(0.5))


def test_push_fills_the_engine_jitter_when_the_denoiser_is_on(pt):
    s = pt.Scene().synth(0, seed=1)
    head, _ = s.push(32, 32, frame_index=7)
    assert head.denoiser_enabled == 0 and tuple(head.halton_jitter) == (0.0, 0.0)
    s.set_cvar("r_denoiser", 1)
    for fi in (0, 5, 15, 16, 1000):
        head, _ = s.push(32, 32, frame_index=fi)
        assert head.denoiser_enabled == 1
        jx, jy = _halton_jitter(fi)
        assert np.float32(head.halton_jitter[0]) == jx and np.float32(head.halton_jitter[1]) == jy
    head, _ = s.push(32, 32, frame_index=0)
    # frame 0 -> Halton index 1: 1/2 - 1/2 = 0 and float(1/3) - 1/2
    assert np.float32(head.halton_jitter[0]) == np.float32(0.0)
    assert np.float32(head.halton_jitter[1]) == np.float32(np.float32(1.0 / 3.0) - np.float32(0.5))
