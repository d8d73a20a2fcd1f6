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
sdf_twist 8 4 0.5 dielectric 1 1 1
sdf_displace_noise 9 3 0.05 2 lambert 0.5 0.6 0.7
""")
    assert n == 0, rep
    b = pt.Scene()
    b.sdf_leaf(1, 0, [0.8], (0, 1, 0), 0, (0.9, 0.2, 0.2))
    b.sdf_leaf(2, 1, [0.5, 0.6, 0.7], (1, 1, 0), 1, (0.8, 0.8, 0.8))
    b.sdf_combine(3, 1, 2, 1, 0.3, 0, (0.5, 0.6, 0.7))
    b.sdf_leaf(4, 3, [1.2, 0.3], (-2, 1, 0), 2, (1, 1, 1))
    b.sdf_leaf(5, 4, [0.7, 0.25], (2, 1, -1), 0, (0.3, 0.9, 0.3))
    b.sdf_leaf(6, 2, [0.4, 0.4, 0.4, 0.1], (0, 3, 0), 1, (0.9, 0.9, 0.2))
    b.sdf_combine(7, 6, 5, 2, 0.05, 0, (0.4, 0.4, 0.4))
    b.sdf_wrap(8, 4, 6, [0.5], 2, (1, 1, 1))
    b.sdf_wrap(9, 3, 5, [0.05, 2, 4], 0, (0.5, 0.6, 0.7))     # octaves: r_sdf_displace_octaves
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


# ---- procedural ops 5-9 (shaders/SdfPrimitives.slang:504-1245) ----

PROC = """
sdf_box 1 1.5 0.25 1.5 0 -0.5 0 lambert 0.45 0.55 0.40
sdf_displace_noise 2 1 0.25 0.5 5 lambert 0.45 0.55 0.40
sdf_box 10 0.3 1.0 0.3 -2 1 0 metal 0.85 0.55 0.20
sdf_twist 11 10 1.8 metal 0.85 0.55 0.20
sdf_capsule 20 1.0 0.3 2 1.2 0 lambert 0.30 0.55 0.85
sdf_bend 21 20 0.5 lambert 0.30 0.55 0.85
sdf_sphere 30 0.18 0 1.8 -2.5 lambert 0.85 0.30 0.45
sdf_repeat_limited 31 30 0.6 0 0 3 0 0 lambert 0.85 0.30 0.45
sdf_sphere 40 0.2 3 0.5 0 lambert 0.5 0.5 0.5
sdf_sphere 41 0.15 3.1 0.6 0.05 lambert 0.5 0.5 0.5
sdf_smin 42 40 41 0.1 lambert 0.5 0.5 0.5
sdf_repeat 43 42 0 0 0.9 lambert 0.5 0.5 0.5
"""
# cluster centres (id order: 2, 11, 21, 31, 43) and a span to aim across
PROC_AIM = np.array([[0, -0.3, 0, 1.4], [-2, 1, 0, 0.6], [2, 1.2, 0, 1.2], [0, 1.8, -2.5, 1.9],
                     [3, 0.5, 0, 3.0]], np.float32)


def _proc_scene(pt, on=True):
    s = pt.Scene()
    rep, n = s.exec_cfg(("r_sdf_procedural_ops 1\n" if on else "") + PROC)
    assert n == 0, rep
    s.env(np.zeros((2, 4, 3), np.float32))
    return s


def _clusters(s):
    ps = s.packed()
    a = np.ctypeslib.as_array(ps.sdf_clusters, shape=(ps.sdf_count * 112,)).copy()
    return a.reshape(ps.sdf_count, 112)


# An independent float64 restatement of the reference's procedural field, over
# the packed cluster layout: hash, value noise, fBm, the phase-1 walker with the
# noise band, and the root warps.
def _hash32(x):
    x = x.astype(np.uint64) & np.uint64(0xFFFFFFFF)
    x ^= x >> 16
    x = (x * 0x7feb352d) & 0xFFFFFFFF
    x ^= x >> 15
    x = (x * 0x846ca68b) & 0xFFFFFFFF
    x ^= x >> 16
    return x


def _hash3(i, j, k):
    h = _hash32(i)
    h = _hash32(h ^ j)
    h = _hash32(h ^ k)
    return h.astype(np.float32).astype(np.float64) * 2.0 ** -32


def _noise(p):
    ip = np.floor(p)
    f = p - ip
    c = (ip.astype(np.int64) & 0xFFFFFFFF).astype(np.uint64)
    u = f * f * f * (f * (f * 6 - 15) + 10)
    n = {}
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                n[dx, dy, dz] = _hash3((c[:, 0] + dx) & 0xFFFFFFFF, (c[:, 1] + dy) & 0xFFFFFFFF,
                                       (c[:, 2] + dz) & 0xFFFFFFFF)
    # trilinear mix of the eight lattice values with the quintic weights
    x0 = n[0, 0, 0] + (n[1, 0, 0] - n[0, 0, 0]) * u[:, 0]
    x1 = n[0, 1, 0] + (n[1, 1, 0] - n[0, 1, 0]) * u[:, 0]
    x2 = n[0, 0, 1] + (n[1, 0, 1] - n[0, 0, 1]) * u[:, 0]
    x3 = n[0, 1, 1] + (n[1, 1, 1] - n[0, 1, 1]) * u[:, 0]
    y0 = x0 + (x1 - x0) * u[:, 1]
    y1 = x2 + (x3 - x2) * u[:, 1]
    return y0 + (y1 - y0) * u[:, 2]


def _fbm(p, octaves):
    v, amp, frq = 0.0, 1.0, 1.0
    for _ in range(min(octaves, 6)):
        v = v + amp * (2 * _noise(p * frq) - 1)
        amp, frq = amp * 0.5, frq * 2
    return v


def _leaf(p, shape, q):
    if shape == 0:
        return np.linalg.norm(p, axis=1) - q[0]
    if shape in (1, 2):
        d = np.abs(p) - q[:3]
        o = np.linalg.norm(np.maximum(d, 0), axis=1) + np.minimum(d.max(axis=1), 0)
        return o if shape == 1 else o - q[3]
    if shape == 4:
        y = np.clip(p[:, 1], -q[0], q[0])
        return np.linalg.norm(np.stack([p[:, 0], p[:, 1] - y, p[:, 2]], 1), axis=1) - q[1]
    raise AssertionError(shape)


def _walk(C, nc, p):
    d = []
    for i in range(nc):
        node = C[16 + 12 * i:28 + 12 * i]
        op, shape, a, b = node[:4].view(np.uint32)
        q, c = node[4:8].astype(np.float64), node[8:11].astype(np.float64)
        if op == 0:
            v = _leaf(p - c, shape, q)
        elif op == 1:   # smooth union
            h = np.clip(0.5 + 0.5 * (d[b] - d[a]) / q[0], 0, 1)
            v = d[b] + h * (d[a] - d[b]) - q[0] * h * (1 - h)
        elif op == 5:   # fBm band
            v = d[a] + q[0] * _fbm(p * q[1], int(node[6:7].view(np.uint32)[0]))
        else:
            raise AssertionError(op)
        d.append(v)
    return d[-1]


def _field(C, p):
    count = int(C[3:4].view(np.uint32)[0])
    root = C[16 + 12 * (count - 1):28 + 12 * (count - 1)]
    op, child = int(root[:1].view(np.uint32)[0]), int(root[2:3].view(np.uint32)[0])
    r = root[4:8].astype(np.float64)
    if op == 6:
        th = r[0] * p[:, 1]
        c, s = np.cos(th), np.sin(th)
        return 0.5 * _walk(C, child + 1, np.stack([c * p[:, 0] - s * p[:, 2], p[:, 1], s * p[:, 0] + c * p[:, 2]], 1))
    if op == 7:
        th = r[0] * p[:, 0]
        c, s = np.cos(th), np.sin(th)
        return 0.5 * _walk(C, child + 1, np.stack([p[:, 0], c * p[:, 1] - s * p[:, 2], s * p[:, 1] + c * p[:, 2]], 1))
    if op in (8, 9):
        pk = int(root[7:8].view(np.uint32)[0])
        lim = np.array([pk & 0x3FF, (pk >> 10) & 0x3FF, (pk >> 20) & 0x3FF], np.float64)
        q = p.copy()
        for j in range(3):
            if r[j] > 1e-6:
                k = np.sign(p[:, j] / r[j]) * np.floor(np.abs(p[:, j] / r[j]) + 0.5)   # half away from zero
                if op == 9:
                    k = np.clip(k, -lim[j], lim[j])
                q[:, j] = p[:, j] - r[j] * k
        return _walk(C, child + 1, q)
    return _walk(C, count, p)


def _proc_rays(n, seed):
    rng = np.random.default_rng(seed)
    which = rng.integers(0, len(PROC_AIM), n)
    ro = np.zeros((n, 4), np.float32)
    ro[:, :3] = np.array([0.5, 4.0, 9.0], np.float32) + rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    tgt = PROC_AIM[which, :3] + rng.uniform(-1, 1, (n, 3)) * PROC_AIM[which, 3:]
    d = tgt - ro[:, :3]
    rd = np.zeros((n, 4), np.float32)
    rd[:, :3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    return ro, rd


def test_sdf_wrap_commands_build_the_reference_nodes():
    """sdf_displace_noise/twist/bend/repeat/repeat_limited append one op node over
    the child's nodes (Engine.cpp wrap_proc): child_a = the child's root, octaves and
    limits packed into float bits, the child consumed."""
    pt = load_pkg()
    s = _proc_scene(pt)
    C = _clusters(s)
    assert C.shape[0] == 5
    expect = [(5, 2, [0.25, 0.5]), (6, 2, [1.8]), (7, 2, [0.5]), (9, 2, [0.6, 0, 0]), (8, 4, [0, 0, 0.9])]
    for c, (op, count, prm) in zip(C, expect):
        assert int(c[3:4].view(np.uint32)[0]) == count
        root = c[16 + 12 * (count - 1):28 + 12 * (count - 1)]
        assert list(root[:4].view(np.uint32)) == [op, 0, count - 2, 0]
        assert np.allclose(root[4:4 + len(prm)], prm)
    assert int(C[0, 16 + 12 + 6:16 + 12 + 7].view(np.uint32)[0]) == 5                 # octaves
    assert int(C[3, 16 + 12 + 7:16 + 12 + 8].view(np.uint32)[0]) == 3                 # lx | ly<<10 | lz<<20
    assert C[4, 2] == -1000.0 and C[4, 6] == 1000.0                                 # z repeats: +-1000 m


def test_sdf_wrap_commands_refuse_what_the_reference_refuses():
    pt = load_pkg()
    for bad in ("sdf_twist 2 1 1.0 lambert 1 1 1",                                  # no child 1
                "sdf_box 1 1 1 1 0 0 0 lambert 1 1 1\nsdf_displace_noise 2 1 0 0.5 lambert 1 1 1",   # amp 0
                "sdf_box 1 1 1 1 0 0 0 lambert 1 1 1\nsdf_repeat_limited 2 1 1 1 1 1 1 1024 lambert 1 1 1",
                "sdf_box 1 1 1 1 0 0 0 lambert 1 1 1\nsdf_bend 2 1 0.5 lambert 1 1 1\nsdf_twist 3 2 1 lambert 1 1 1"):
        with pytest.raises(pt.PtError):
            pt.Scene().exec_cfg(bad)
    s = pt.Scene()   # displacement over a warp nests (a point-displacement op)
    rep, n = s.exec_cfg("sdf_box 1 1 1 1 0 0 0 lambert 1 1 1\nsdf_bend 2 1 0.5 lambert 1 1 1\n"
                        "sdf_displace_noise 3 2 0.1 1 3 lambert 1 1 1")
    assert n == 0, rep


def test_sdf_procedural_field_matches_a_float64_restatement(orc):
    """Every fp64-oracle hit on a procedural cluster lies on the reference's field
    (|d| below the trace epsilon) as an independent float64 restatement computes it."""
    pt = load_pkg()
    s = _proc_scene(pt)
    head, prm = s.push(8, 8)
    C = _clusters(s)
    ro, rd = _proc_rays(3000, 11)
    hit, t, _ = orc.trace(s.packed(), head, prm, ro, rd, fp64=True)
    sdf = (hit & 0xC0000000) == 0x80000000
    ids = hit & 0xFFFFF
    assert sdf.sum() > 500 and set(np.unique(ids[sdf])) == {0, 1, 2, 3, 4}
    for k in range(5):
        m = sdf & (ids == k)
        p = ro[m, :3].astype(np.float64) + rd[m, :3].astype(np.float64) * t[m, None].astype(np.float64)
        d = _field(C[k], p)
        # the march accepted |d| < 1e-4; t is returned as float32 (|dt| <= 6e-7 t)
        assert np.abs(d).max() < 1e-4 + 2e-6 * np.abs(t[m]).max() * 2, (k, np.abs(d).max())


def test_sdf_procedural_ops_off_reads_as_empty_and_fp32_tracks_fp64(orc):
    """Flag off (the reference's default build): the wrapped clusters are never hit.
    Flag on: the fp32 oracle sees the clusters the fp64 oracle sees, at nearly the same t."""
    pt = load_pkg()
    ro, rd = _proc_rays(2000, 12)
    s0 = _proc_scene(pt, on=False)
    head, prm = s0.push(8, 8)
    assert prm.sdf_procedural_ops == 0
    h0, _, _ = orc.trace(s0.packed(), head, prm, ro, rd)
    assert np.all(h0 == 0xFFFFFFFF)
    s1 = _proc_scene(pt)
    head, prm = s1.push(8, 8)
    assert prm.sdf_procedural_ops == 1
    h32, t32, _ = orc.trace(s1.packed(), head, prm, ro, rd)
    h64, t64, _ = orc.trace(s1.packed(), head, prm, ro, rd, fp64=True)
    same = h32 == h64
    assert same.mean() > 0.98
    hit = same & (h32 != 0xFFFFFFFF)
    assert np.median(np.abs(t32[hit] - t64[hit]) / t64[hit]) < 1e-4


def test_sdf_forward_ad_normals_agree_with_central_differences(orc):
    """r_sdf_procedural_ops 2 (the reference built with PT_SDF_AUTODIFF too) shades
    procedural clusters with forward-mode AD normals under r_sdf_normal_mode 0 and
    with central differences under 1; the two renders agree closely (the reference's
    acceptance bar: the two normals within 1e-3), and mode 1 equals the
    central-difference build."""
    pt = load_pkg()
    cfg = ("cam_pos 0 2.5 9\ncam_pitch -12\ncam_fov 55\nr_sky_mode procedural\nr_sun_elevation 40\n"
           "r_max_bounces 2\nlight_point 1 -2 4 3 20 20 20\n" + PROC)
    imgs = {}
    for mode, nm in ((1, 0), (2, 1), (2, 0)):
        s = pt.Scene()
        rep, n = s.exec_cfg(cfg + "r_sdf_procedural_ops %d\nr_sdf_normal_mode %d\n" % (mode, nm))
        assert n == 0, rep
        head, prm = s.push(48, 36, frame_index=2, reset=1)
        assert prm.sdf_procedural_ops == mode and prm.sdf_params_f[3] == nm
        imgs[mode, nm], _ = orc.render(s.packed(), head, prm, 48, 36, 2)
    assert np.array_equal(imgs[1, 0].view(np.uint32), imgs[2, 1].view(np.uint32))
    a, c = imgs[2, 0][..., :3], imgs[1, 0][..., :3]
    assert not np.array_equal(a, c)
    assert np.abs(a - c).mean() / c.mean() < 2e-3, np.abs(a - c).mean() / c.mean()
