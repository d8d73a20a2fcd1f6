"""Light-tree builder (pt_build_light_tree): bit-identical to the reference's
BuildLightTree (golden trees from the reference builder compiled from its
sources), plus the structural and selection-PMF properties the reference's own
tests check (tests/pt_renderer_light_tree_test.cpp:156-423)."""
import os

import numpy as np
import pytest

from conftest import load_pkg

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_builders.npz")


@pytest.mark.parametrize("name", ["lt1", "lt7", "lt200", "lt16c"])
def test_light_tree_equals_reference_golden(name):
    pt = load_pkg()
    g = np.load(GOLD)
    inp = g[f"{name}_in"].reshape(-1).view(pt.LIGHT_INPUT_DTYPE)
    nodes = pt.build_light_tree(inp)
    assert np.array_equal(nodes.view(np.uint8).reshape(len(nodes), 64), g[f"{name}_nodes"])


def test_light_tree_equals_reference_builder_live():
    import oracle
    if oracle.load_ref() is None:
        pytest.skip("reference builders not built here")
    pt = load_pkg()
    rng = np.random.default_rng(3)
    for n in (2, 3, 5, 33, 257):
        a = np.zeros(n, pt.LIGHT_INPUT_DTYPE)
        a["type"] = rng.integers(0, 4, n)
        a["pos"] = rng.uniform(-20, 20, (n, 3))
        a["pos"][: n // 3] = a["pos"][0]                 # coincident groups
        a["radius"] = rng.uniform(0.0, 2.0, n)
        a["intensity"] = rng.uniform(0, 30, (n, 3))
        d = rng.normal(size=(n, 3))
        a["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
        a["cos_outer"] = rng.uniform(-0.5, 0.99, n)
        a["u_vec"] = rng.uniform(-2, 2, (n, 3))
        a["v_half"] = rng.uniform(-1, 1, n)
        mine = pt.build_light_tree(a).view(np.uint8).reshape(-1, 64)
        assert np.array_equal(mine, oracle.ref_light_tree(a))


def _lights(pt, n, seed):
    rng = np.random.default_rng(seed)
    a = np.zeros(n, pt.LIGHT_INPUT_DTYPE)
    a["type"] = np.arange(n) % 4
    a["pos"] = rng.uniform(-10, 10, (n, 3))
    a["radius"] = 0.5
    a["intensity"] = 1.0
    a["dir"] = (0, 1, 0)
    a["cos_outer"] = 0.5
    a["u_vec"] = (1, 0, 0)
    a["v_half"] = 1.0
    return a


def _importance(nd, hp, nf):   # the traversal's importance, in double
    c = 0.5 * (nd["aabb_min"].astype(np.float64) + nd["aabb_max"])
    to = c - hp
    d2 = max(float(to @ to), 1e-12)
    dir_to = to / np.sqrt(d2)
    ext = 0.5 * (nd["aabb_max"].astype(np.float64) - nd["aabb_min"])
    fall = 1.0 / max(d2, max(float(ext @ ext), 1e-12))
    orient = 1.0
    ch = float(nd["cone_cos_half"])
    if ch > -0.999:
        ce = -float(nd["cone_axis"].astype(np.float64) @ dir_to)
        orient = min(max((ce - (ch - 0.2)) / 0.2, 0.0), 1.0)
    return max(float(nd["intensity"]) * fall * orient * max(0.0, float(nf @ dir_to)), 1e-8)


def _pmf(nodes, hp, nf):
    out, stack = {}, [(0, 1.0)]
    while stack:
        i, p = stack.pop()
        nd = nodes[i]
        if nd["count"] == 1:
            out[int(nd["left_first"])] = out.get(int(nd["left_first"]), 0.0) + p
            continue
        l, r = int(nd["left_first"]), int(nd["left_first"]) + 1
        il, ir = _importance(nodes[l], hp, nf), _importance(nodes[r], hp, nf)
        pl = float(il) / (float(il) + float(ir))
        stack += [(l, p * pl), (r, p * (1 - pl))]
    return out


@pytest.mark.parametrize("n", [1, 2, 3, 4, 7, 16, 64, 200])
def test_light_tree_structure_and_selection_pmf(n):
    pt = load_pkg()
    nodes = pt.build_light_tree(_lights(pt, n, 7 * n + 1))
    assert len(nodes) == 2 * n - 1
    leaves = nodes[nodes["count"] == 1]
    assert sorted(leaves["left_first"].tolist()) == list(range(n))
    for i, nd in enumerate(nodes):
        if nd["count"] == 0:
            l, r = nodes[nd["left_first"]], nodes[nd["left_first"] + 1]
            assert nd["left_first"] > i
            assert np.all(nd["aabb_min"] <= np.minimum(l["aabb_min"], r["aabb_min"]) + 1e-5)
            assert np.all(nd["aabb_max"] >= np.maximum(l["aabb_max"], r["aabb_max"]) - 1e-5)
            assert np.isclose(nd["intensity"], l["intensity"] + r["intensity"], rtol=1e-6)
    hp = np.array([2.5, 1.0, -3.0])
    nf = np.array([0.3, 0.9, 0.2])
    nf /= np.linalg.norm(nf)
    pmf = _pmf(nodes, hp, nf)
    assert len(pmf) == n and min(pmf.values()) > 0
    assert abs(sum(pmf.values()) - 1.0) < 1e-9


def test_brighter_light_is_picked_more_often():
    pt = load_pkg()
    a = np.zeros(2, pt.LIGHT_INPUT_DTYPE)
    a["pos"] = [(-4, 3, 0), (4, 3, 0)]
    a["intensity"] = [(1, 1, 1), (100, 100, 100)]
    a["dir"] = (0, 1, 0)
    a["u_vec"] = (1, 0, 0)
    pmf = _pmf(pt.build_light_tree(a), np.zeros(3), np.array([0.0, 1.0, 0.0]))
    assert pmf[1] > pmf[0] and pmf[1] / (pmf[0] + pmf[1]) > 0.9
