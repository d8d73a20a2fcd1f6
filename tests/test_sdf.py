"""SDF clusters on the host and in the oracle: bounding boxes equal the
reference's ComputeSdfAabb (golden + live), the console commands build the
same clusters as the API, and a sphere-traced SDF sphere lands on the analytic
sphere's surface within the trace epsilon."""
import ctypes
import os

import numpy as np
import pytest

import oracle as orc_mod
from conftest import load_pkg

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_builders.npz")


def _box(pt, nodes, count):
    lo = np.zeros(3, np.float32)
    hi = np.zeros(3, np.float32)
    P = ctypes.POINTER(ctypes.c_float)
    a = np.ascontiguousarray(nodes, np.float32)
    rc = pt.load().pt_sdf_cluster_box(a.ctypes.data_as(P), count, lo.ctypes.data_as(P), hi.ctypes.data_as(P))
    return (lo, hi) if rc == 0 else None


def test_sdf_boxes_equal_reference_golden():
    pt = load_pkg()
    g = np.load(GOLD)
    for nodes, n, box in zip(g["sdf_nodes"], g["sdf_counts"], g["sdf_boxes"]):
        r = _box(pt, nodes, int(n))
        assert (r is not None) == (box[6] == 1.0)
        if r:
            assert np.array_equal(np.concatenate(r), box[:6])


def test_sdf_procedural_op_boxes_equal_reference_golden():
    """Ops 5-9 (fBm displace, twist, bend, repeat, limited repeat): the
    reference bounds them on the host in every build."""
    pt = load_pkg()
    g = np.load(GOLD)
    for nodes, n, box in zip(g["sdf_proc_nodes"], g["sdf_proc_counts"], g["sdf_proc_boxes"]):
        r = _box(pt, nodes, int(n))
        assert (r is not None) == (box[6] == 1.0)
        if r:
            assert np.array_equal(np.concatenate(r), box[:6])


def test_sdf_boxes_equal_reference_live():
    if orc_mod.load_ref() is None:
        pytest.skip("reference builders not built here")
    pt = load_pkg()
    rng = np.random.default_rng(9)
    for _ in range(200):
        n = 3
        nodes = np.zeros((8, 12), np.float32)
        for i in range(2):
            nodes[i, :4].view(np.uint32)[:] = [0, rng.integers(0, 5), 0, 0]
            nodes[i, 4:8] = rng.uniform(-0.5, 2, 4)
            nodes[i, 8:11] = rng.uniform(-4, 4, 3)
        nodes[2, :4].view(np.uint32)[:] = [rng.integers(1, 5), 0, 0, 1]
        nodes[2, 4] = rng.uniform(-0.5, 1)
        want = orc_mod.ref_sdf_aabb(nodes, n)
        got = _box(pt, nodes, n)
        assert (want is None) == (got is None)
        if want:
            assert np.array_equal(np.concatenate(got), np.concatenate(want))
    for _ in range(300):   # a procedural op (5..9) over a leaf
        nodes = np.zeros((8, 12), np.float32)
        nodes[0, :4].view(np.uint32)[:] = [0, rng.integers(0, 5), 0, 0]
        nodes[0, 4:8] = rng.uniform(0.1, 2, 4)
        nodes[0, 8:11] = rng.uniform(-4, 4, 3)
        op = int(rng.integers(5, 10))
        nodes[1, :4].view(np.uint32)[:] = [op, 0, 0, 0]
        nodes[1, 4:8] = rng.uniform(-0.5, 3, 4)
        if op == 5:
            nodes[1, 6:7].view(np.uint32)[0] = rng.integers(0, 9)
        if op == 9:
            nodes[1, 7:8].view(np.uint32)[0] = (int(rng.integers(0, 1024)) | (int(rng.integers(0, 1024)) << 10)
                                                | (int(rng.integers(0, 1024)) << 20))
        want = orc_mod.ref_sdf_aabb(nodes, 2)
        got = _box(pt, nodes, 2)
        assert (want is None) == (got is None)
        if want:
            assert np.array_equal(np.concatenate(got), np.concatenate(want))


def test_sdf_commands_build_the_same_clusters_as_the_api():
    pt = load_pkg()
    a = pt.Scene()
    rep, n = a.exec_cfg("""
sdf_sphere 1 0.8 0 1 0 lambert 0.9 0.2 0.2
sdf_box 2 0.5 0.6 0.7 1 1 0 metal 0.8 0.8 0.8
sdf_smin 3 1 2 0.3 lambert 0.5 0.6 0.7
sdf_torus 4 1.2 0.3 -2 1 0 dielectric 1 1 1
sdf_capsule 5 0.7 0.25 2 1 -1 lambert 0.3 0.9 0.3
sdf_round_box 6 0.4 0.4 0.4 0.1 0 3 0 metal 0.9 0.9 0.2
sdf_sdiff 7 6 5 0.05 lambert 0.4 0.4 0.4
sdf_twist 8 4 0.5
""")
    assert n == 1 and "sdf_twist" in rep
    b = pt.Scene()
    b.sdf_leaf(1, 0, [0.8], (0, 1, 0), 0, (0.9, 0.2, 0.2))
    b.sdf_leaf(2, 1, [0.5, 0.6, 0.7], (1, 1, 0), 1, (0.8, 0.8, 0.8))
    b.sdf_combine(3, 1, 2, 1, 0.3, 0, (0.5, 0.6, 0.7))
    b.sdf_leaf(4, 3, [1.2, 0.3], (-2, 1, 0), 2, (1, 1, 1))
    b.sdf_leaf(5, 4, [0.7, 0.25], (2, 1, -1), 0, (0.3, 0.9, 0.3))
    b.sdf_leaf(6, 2, [0.4, 0.4, 0.4, 0.1], (0, 3, 0), 1, (0.9, 0.9, 0.2))
    b.sdf_combine(7, 6, 5, 2, 0.05, 0, (0.4, 0.4, 0.4))
    pa, pb = a.packed(), b.packed()
    assert pa.sdf_count == pb.sdf_count == 3
    xa = np.ctypeslib.as_array(pa.sdf_clusters, (pa.sdf_count * 112,)).view(np.uint32)
    xb = np.ctypeslib.as_array(pb.sdf_clusters, (pb.sdf_count * 112,)).view(np.uint32)
    assert np.array_equal(xa, xb)
    ha, qa = a.push(32, 32)
    assert qa.sdf_params[0] == 3 and qa.sdf_params[1] == 128 and abs(qa.sdf_params_f[0] - 1e-4) < 1e-9


def test_sdf_sphere_trace_lands_on_the_sphere(orc):
    pt = load_pkg()
    s = pt.Scene()
    s.sdf_leaf(1, 0, [1.5], (0.5, -0.25, 0.0), 0, (0.7, 0.7, 0.7))
    s.env(np.zeros((2, 4, 3), np.float32))
    head, prm = s.push(8, 8)
    rng = np.random.default_rng(2)
    n = 2000
    ro = np.zeros((n, 4), np.float32)
    ro[:, 2] = 8.0
    tgt = rng.uniform(-1.2, 1.2, (n, 3)) + np.array([0.5, -0.25, 0.0])
    d = tgt - ro[:, :3]
    rd = np.zeros((n, 4), np.float32)
    rd[:, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    hit, t, _ = orc.trace(s.packed(), head, prm, ro, rd)
    hits = hit != 0xFFFFFFFF
    assert hits.sum() > 500 and np.all(hit[hits] == 0x80000000)
    p = ro[hits, :3] + rd[hits, :3] * t[hits, None]
    r = np.linalg.norm(p - np.array([0.5, -0.25, 0.0]), axis=1)
    assert np.abs(r - 1.5).max() < 2e-4                    # |d| < eps at the accepted point


def test_sdf_fractal_boxes_equal_reference_golden():
    pt = load_pkg()
    g = np.load(GOLD)
    refused = 0
    for nodes, n, box in zip(g["sdf_frac_nodes"], g["sdf_frac_counts"], g["sdf_frac_boxes"]):
        r = _box(pt, nodes, int(n))
        assert (r is not None) == (box[6] == 1.0)
        refused += r is None
        if r:
            assert np.array_equal(np.concatenate(r), box[:6])
    assert refused >= 1                                  # a non-positive bound radius is refused


FRACTALS = """
sdf_mandelbulb 1 8 1.3 0 1.2 0 lambert 0.9 0.5 0.2
sdf_mandelbox 2 2.5 4.2 -6 4 -8 metal 0.8 0.8 0.9
sdf_apollonian 3 1.3 1.8 5 1.8 -3 lambert 0.4 0.7 0.9
"""


def test_sdf_fractal_commands_build_the_same_clusters_as_the_api():
    pt = load_pkg()
    a = pt.Scene()
    rep, n = a.exec_cfg(FRACTALS + "r_sdf_fractal_iters 10\nr_sdf_fractal_power 6\nr_sdf_de_eps_scale 0.5\n")
    assert n == 0, rep
    b = pt.Scene()
    b.sdf_leaf(1, 6, [8, 1.3], (0, 1.2, 0), 0, (0.9, 0.5, 0.2))
    b.sdf_leaf(2, 7, [2.5, 4.2], (-6, 4, -8), 1, (0.8, 0.8, 0.9))
    b.sdf_leaf(3, 8, [1.3, 1.8], (5, 1.8, -3), 0, (0.4, 0.7, 0.9))
    pa, pb = a.packed(), b.packed()
    assert pa.sdf_count == pb.sdf_count == 3
    xa = np.ctypeslib.as_array(pa.sdf_clusters, (pa.sdf_count * 112,))
    xb = np.ctypeslib.as_array(pb.sdf_clusters, (pb.sdf_count * 112,))
    assert np.array_equal(xa.view(np.uint32), xb.view(np.uint32))
    assert np.allclose(xa[[0, 1, 2, 4, 5, 6]], [-1.3, -0.1, -1.3, 1.3, 2.5, 1.3], atol=1e-6)   # side 2*bound
    _, q = a.push(16, 16)
    assert (q.sdf_params[3], q.sdf_params_f[1], q.sdf_params_f[2]) == (10, 6.0, 0.5)
    _, q = b.push(16, 16)
    assert (q.sdf_params[3], q.sdf_params_f[1], q.sdf_params_f[2]) == (12, 8.0, 1.0)


def test_sdf_fractal_leaves_are_not_combined():
    pt = load_pkg()
    s = pt.Scene()
    with pytest.raises(pt.PtError, match="fractal leaves cannot take part") as e:
        s.exec_cfg("sdf_mandelbulb 1 8 1.3 0 1 0 lambert 1 1 1\n"
                   "sdf_sphere 2 0.5 2 1 0 lambert 1 1 1\n"
                   "sdf_smin 3 1 2 0.2 lambert 1 1 1\n"
                   "sdf_mandelbox 4 2.5 0 0 0 0 lambert 1 1 1\n")
    assert "+1 more" in str(e.value)                     # the zero bound radius is refused too


def test_sdf_fractal_trace_accepts_within_the_step_epsilon(orc):
    """A fractal hit is accepted where |DE| falls below eps*(1 + scale*step);
    the id carries the step, and the normal is a unit vector facing the ray."""
    pt = load_pkg()
    s = pt.Scene()
    rep, n = s.exec_cfg(FRACTALS)
    assert n == 0, rep
    s.env(np.zeros((2, 4, 3), np.float32))
    head, prm = s.push(8, 8)
    rng = np.random.default_rng(4)
    centres = np.array([[0, 1.2, 0], [-6, 4, -8], [5, 1.8, -3]], np.float32)
    n = 1500
    which = rng.integers(0, 3, n)
    ro = np.zeros((n, 4), np.float32)
    ro[:, :3] = centres[which] + np.array([0.3, 2.0, 9.0], np.float32)
    tgt = centres[which] + rng.uniform(-1.0, 1.0, (n, 3))
    d = tgt - ro[:, :3]
    rd = np.zeros((n, 4), np.float32)
    rd[:, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    hit, t, _ = orc.trace(s.packed(), head, prm, ro, rd)
    sdf = (hit & 0xC0000000) == 0x80000000
    clusters = hit[sdf] & 0xFFFFF
    assert sdf.sum() > 300 and set(np.unique(clusters)) == {0, 1, 2}
    steps = (hit[sdf] >> 20) & 0x1FF
    assert steps.max() > 4 and steps.max() < 128
    p = ro[sdf, :3] + rd[sdf, :3] * t[sdf, None]
    bound = np.array([1.3, 4.2, 1.8], np.float32)[clusters]
    assert np.all(np.abs(p - centres[clusters]).max(axis=1) <= bound * (1 + 1e-5))
    h64, t64, _ = orc.trace(s.packed(), head, prm, ro, rd, fp64=True)
    assert (h64 & 0xC00FFFFF == hit & 0xC00FFFFF).mean() > 0.95   # the float64 march sees the same clusters
