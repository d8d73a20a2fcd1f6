"""The reference's own unit cases for the builders and samplers on this path
that the golden and live comparisons do not already spell out, restated on
this library's builders and the oracle (names give the reference test they
follow):

* tests/pt_renderer_triangle_bvh_test.cpp: empty BVH (:304), single triangle hit
  and miss (:333), collinear triangle (:381), many triangles on one splitting
  plane (:441), node boxes contain their triangles (:563);
* tests/hdrimage_cdf_test.cpp: monotone CDFs ending at 1 (:154, :192), a single
  bright pixel (:302), dark rows (:381), the sin(theta) marginal of a uniform image
  (:425), pdf guards (:646);
* tests/pt_renderer_light_tree_test.cpp: empty input (:156), coincident lights
  (:230), every leaf reachable at 500 and 1000 lights (:212)."""
import ctypes

import numpy as np

from conftest import load_pkg, xorshift_rays
from test_builders import product_env_cdf, product_tri_bvh
from test_light_tree import _lights, _pmf
from test_oracle import naive_mt


def product_tri_bvh_nodes(pt, pos, idx):
    return product_tri_bvh(pt, np.ascontiguousarray(pos, np.float32), np.ascontiguousarray(idx, np.uint32))


def _mesh_trace(pt, orc, pos, idx, ro, rd):
    s = pt.Scene()
    s.mesh(np.asarray(pos, np.float32), np.asarray(idx, np.uint32))
    s.env(np.zeros((2, 4, 3), np.float32))
    head, prm = s.push(8, 8)
    hit, t, _ = orc.trace(s.packed(), head, prm, np.asarray(ro, np.float32), np.asarray(rd, np.float32))
    return np.where(hit == 0xFFFFFFFF, -1, (hit & ~np.uint32(1 << 30)).astype(np.int64)), t


# ---- triangle BVH ----------------------------------------------------------

def test_triangle_bvh_empty_and_single_triangle(orc):
    pt = load_pkg()
    nodes, perm = product_tri_bvh_nodes(pt, np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
    assert nodes.shape[0] == 0
    s = pt.Scene()
    s.env(np.zeros((2, 4, 3), np.float32))
    head, prm = s.push(8, 8)
    ro, rd = xorshift_rays(50, 0xE111)
    hit, _, _ = orc.trace(s.packed(), head, prm, ro, rd)
    assert (hit == 0xFFFFFFFF).all()
    pos = [[-1, -1, 5], [1, -1, 5], [0, 1, 5]]
    ro = np.zeros((2, 4), np.float32)
    rd = np.array([[0, 0, 1, 0], [1, 0, 0, 0]], np.float32)
    ids, t = _mesh_trace(pt, orc, pos, [[0, 1, 2]], ro, rd)
    assert ids[0] == 0 and abs(t[0] - 5.0) < 1e-5 and ids[1] == -1


def test_triangle_bvh_collinear_triangle_and_shared_plane(orc):
    pt = load_pkg()
    rng = np.random.default_rng(8)
    c = rng.uniform(-5, 5, (40, 1, 3))
    pos = (c + rng.uniform(-1, 1, (40, 3, 3))).reshape(-1, 3).astype(np.float32)
    pos[0:3] = [[0, 0, 4], [1, 1, 4], [2, 2, 4]]              # collinear: zero area
    idx = np.arange(120, dtype=np.uint32).reshape(-1, 3)
    nodes, perm = product_tri_bvh_nodes(pt, pos, idx)
    assert sorted(perm.tolist()) == list(range(40))
    n = 400
    ro = np.zeros((n, 4), np.float32)
    d = rng.normal(size=(n, 3))
    ro[:, :3] = 20 * d / np.linalg.norm(d, axis=1, keepdims=True)
    tgt = c[rng.integers(0, 40, n), 0] + rng.uniform(-0.5, 0.5, (n, 3))   # aimed at the triangles
    rd = np.zeros((n, 4), np.float32)
    rd[:, :3] = (tgt - ro[:, :3]) / np.linalg.norm(tgt - ro[:, :3], axis=1, keepdims=True)
    ids, t = _mesh_trace(pt, orc, pos, idx, ro, rd)
    nid, nt = naive_mt(pos, idx, ro, rd)
    assert (ids == nid).mean() >= 0.995 and (nid >= 0).sum() > 100
    # 33 triangles with one centroid: every one in the tree once
    tri = np.array([[-1, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    pos2 = np.concatenate([tri + np.float32(0.001) * k for k in range(33)])
    pos2 -= pos2.reshape(33, 3, 3).mean(axis=1).repeat(3, 0) - np.array([0, 0.333, 0], np.float32)
    nodes2, perm2 = product_tri_bvh_nodes(pt, pos2, np.arange(99, dtype=np.uint32).reshape(-1, 3))
    assert sorted(perm2.tolist()) == list(range(33))


def test_triangle_bvh_node_boxes_contain_their_triangles():
    pt = load_pkg()
    rng = np.random.default_rng(9)
    c = rng.uniform(-8, 8, (300, 1, 3))
    pos = (c + rng.uniform(-1.5, 1.5, (300, 3, 3))).reshape(-1, 3).astype(np.float32)
    idx = np.arange(900, dtype=np.uint32).reshape(-1, 3)
    nodes, perm = product_tri_bvh_nodes(pt, pos, idx)
    lo, hi = nodes[:, 0:3].view(np.float32), nodes[:, 4:7].view(np.float32)
    lf, cnt = nodes[:, 3], nodes[:, 7]

    def below(i):
        return list(perm[lf[i]:lf[i] + cnt[i]]) if cnt[i] > 0 else below(lf[i]) + below(lf[i] + 1)

    for i in range(nodes.shape[0]):
        for tr in below(i):
            v = pos[idx[tr]]
            assert np.all(lo[i] <= v.min(0)) and np.all(hi[i] >= v.max(0)), (i, tr)


# ---- env CDF ---------------------------------------------------------------

def test_env_cdf_monotone_bright_pixel_dark_rows_and_sin_theta():
    pt = load_pkg()
    rng = np.random.default_rng(2)
    H, W = 16, 24
    img = rng.uniform(0, 3, (H, W, 3)).astype(np.float32)
    img[4:7] = 0.0                                              # dark rows
    marg, cond, tot = product_env_cdf(pt, img)
    assert np.all(np.diff(marg) >= 0) and marg[-1] == 1.0
    assert np.all(np.diff(cond, axis=1) >= 0) and np.all(cond[~np.isin(np.arange(H), [4, 5, 6]), -1] == 1.0)
    assert marg[4] == marg[3] and marg[5] == marg[3] and marg[6] == marg[3]   # no mass in dark rows
    # one bright pixel: the CDFs step from 0 to 1 exactly there
    one = np.zeros((H, W, 3), np.float32)
    one[9, 13] = 5.0
    m1, c1, t1 = product_env_cdf(pt, one)
    assert np.all(m1[:9] == 0) and np.all(m1[9:] == 1.0)
    assert np.all(c1[9, :13] == 0) and np.all(c1[9, 13:] == 1.0)
    # uniform white: marginal increments follow sin(theta) of the row centres
    m2, _, _ = product_env_cdf(pt, np.ones((H, W, 3), np.float32))
    inc = np.diff(np.concatenate([[0.0], m2.astype(np.float64)]))
    want = np.sin(np.pi * (np.arange(H) + 0.5) / H)
    np.testing.assert_allclose(inc, want / want.sum(), rtol=1e-5, atol=1e-7)


def test_env_pdf_guards(orc):
    """Zero total luminance -> pdf 0 for any draw; directions at the poles
    (sin(theta) below the guard) -> pdfEnvMapDir 0."""
    pt = load_pkg()
    s = pt.Scene()
    s.env(np.zeros((8, 16, 3), np.float32))
    head, prm = s.push(8, 8)
    u = np.linspace(0, 0.999, 64, dtype=np.float32)
    _, pdf, pdf_eval = orc.env_sample(s.packed(), head, prm, u, u[::-1].copy())
    assert (pdf == 0).all() and (pdf_eval == 0).all()
    s2 = pt.Scene()
    s2.set_cvar("r_hdri_extract_percentile", 0.0)
    s2.env(np.random.default_rng(1).uniform(0.1, 1.0, (8, 16, 3)).astype(np.float32))
    head2, prm2 = s2.push(8, 8)
    _, pdf2, _ = orc.env_sample(s2.packed(), head2, prm2, np.array([0.3], np.float32), np.array([0.5], np.float32))
    assert pdf2[0] > 0                                          # a normal draw away from the poles


# ---- light tree --------------------------------------------------------------

def test_light_tree_empty_coincident_and_large():
    pt = load_pkg()
    assert len(pt.build_light_tree(np.zeros(0, pt.LIGHT_INPUT_DTYPE))) == 0
    hp = np.array([0.5, 2.0, -1.0])
    nf = np.array([0.0, 1.0, 0.0])
    a = _lights(pt, 9, 4)
    a["pos"] = (1.0, 1.0, 1.0)                                   # all coincident
    pmf = _pmf(pt.build_light_tree(a), hp, nf)
    assert len(pmf) == 9 and abs(sum(pmf.values()) - 1.0) < 1e-9
    for n in (500, 1000):
        nodes = pt.build_light_tree(_lights(pt, n, n))
        assert len(nodes) == 2 * n - 1
        assert sorted(nodes[nodes["count"] == 1]["left_first"].tolist()) == list(range(n))
