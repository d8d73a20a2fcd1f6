"""Shared fixtures.  `-m gpu` tests need a CUDA device and call the product
through its C-ABI; everything else runs on CPU (oracle, host builders, ABI
symbol checks)."""
import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
PKG_DIR = os.path.join(ROOT, "demont-engine_gb300")


def load_pkg():
    if "demont_gb300" in sys.modules:
        return sys.modules["demont_gb300"]
    spec = importlib.util.spec_from_file_location(
        "demont_gb300", os.path.join(PKG_DIR, "__init__.py"), submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["demont_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the product through its C-ABI")


@pytest.fixture(scope="session")
def pt():
    mod = load_pkg()
    if not os.path.exists(mod.LIB_PATH):
        spec = importlib.util.spec_from_file_location("pt_build", os.path.join(PKG_DIR, "build.py"))
        b = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(b)
        b.build()
    mod.load()
    return mod


@pytest.fixture(scope="session")
def orc():
    import oracle
    if not os.path.exists(oracle.LIB):
        oracle.build(ref=False)
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def dev(pt):
    d = pt.Device(0)
    yield d
    d.close()


class XorShift32:
    """The reference tests' platform-independent PRNG
    (tests/pt_core_analytic_bvh_test.cpp:61-80)."""

    def __init__(self, seed):
        self.state = seed if seed else 0xDEADBEEF

    def next(self):
        x = self.state
        x ^= (x << 13) & 0xFFFFFFFF
        x ^= x >> 17
        x ^= (x << 5) & 0xFFFFFFFF
        self.state = x
        return x

    def unitf(self):
        return np.float32(self.next() >> 8) * np.float32(1.0 / (1 << 24))

    def rangef(self, lo, hi):
        lo, hi = np.float32(lo), np.float32(hi)
        return np.float32(lo + (hi - lo) * self.unitf())


def xorshift_spheres(n, seed):
    """MakeRandomSphereScene (tests/pt_core_analytic_bvh_test.cpp:241-256)."""
    rng = XorShift32(seed)
    out = np.zeros((n, 4), np.float32)
    for i in range(n):
        out[i, 0] = rng.rangef(-10, 10)
        out[i, 1] = rng.rangef(-10, 10)
        out[i, 2] = rng.rangef(-10, 10)
        out[i, 3] = rng.rangef(0.2, 1.0)
    return out


def xorshift_rays(n, seed):
    """MakeRay (tests/pt_core_analytic_bvh_test.cpp:289-311): origins on a
    >= 15 m shell, aimed at targets in [-14, 14]^3."""
    rng = XorShift32(seed)
    ro = np.zeros((n, 4), np.float32)
    rd = np.zeros((n, 4), np.float32)
    for i in range(n):
        while True:
            o = [rng.rangef(-25, 25) for _ in range(3)]
            if o[0] * o[0] + o[1] * o[1] + o[2] * o[2] >= np.float32(225.0):
                break
        t = [rng.rangef(-14, 14) for _ in range(3)]
        d = np.array([t[k] - o[k] for k in range(3)], np.float32)
        n2 = np.float32(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
        inv = np.float32(1.0) / np.sqrt(n2)
        ro[i, :3] = o
        rd[i, :3] = d * inv
    return ro, rd


def reference_ranks(nodes, n_slots):
    """Visit ordinal of every leaf slot in the reference traversal: depth first,
    right child popped first (shaders/PathTrace.slang:2592-2636)."""
    rank = np.full(n_slots, -1, np.int64)
    st, o = [0], 0
    while st:
        i = st.pop()
        lf, cnt = int(nodes[i][3]), int(nodes[i][7])
        if cnt > 0:
            rank[lf:lf + cnt] = np.arange(o, o + cnt)
            o += cnt
        else:
            st += [lf, lf + 1]
    return rank


def mt_all(e1, e2, v0, o, d):
    """Two-sided Moller-Trumbore of one ray against every triangle, float32,
    the shader's operation order (shaders/PathTrace.slang:2610-2627)."""
    f = np.float32
    pv = np.stack([d[1] * e2[:, 2] - d[2] * e2[:, 1], d[2] * e2[:, 0] - d[0] * e2[:, 2],
                   d[0] * e2[:, 1] - d[1] * e2[:, 0]], 1).astype(f)
    det = ((e1[:, 0] * pv[:, 0] + e1[:, 1] * pv[:, 1]) + e1[:, 2] * pv[:, 2]).astype(f)
    ok = np.abs(det) >= f(1e-8)
    inv = (f(1) / np.where(ok, det, f(1))).astype(f)
    tv = (o - v0).astype(f)
    u = (((tv[:, 0] * pv[:, 0] + tv[:, 1] * pv[:, 1]) + tv[:, 2] * pv[:, 2]) * inv).astype(f)
    qv = np.stack([tv[:, 1] * e1[:, 2] - tv[:, 2] * e1[:, 1], tv[:, 2] * e1[:, 0] - tv[:, 0] * e1[:, 2],
                   tv[:, 0] * e1[:, 1] - tv[:, 1] * e1[:, 0]], 1).astype(f)
    v = (((d[0] * qv[:, 0] + d[1] * qv[:, 1]) + d[2] * qv[:, 2]) * inv).astype(f)
    t = (((e2[:, 0] * qv[:, 0] + e2[:, 1] * qv[:, 1]) + e2[:, 2] * qv[:, 2]) * inv).astype(f)
    ok &= (u >= 0) & (u <= 1) & (v >= 0) & (u + v <= 1) & (t > f(1e-3))
    return ok, t


def first_tested_wins(arrays, ro, rd):
    """The reference's closest-hit rule over EVERY triangle its intersector
    accepts: smallest t, ties to the earliest in the reference traversal order.
    Returns hit ids in the pt_gpu_trace_closest encoding, and t."""
    pos, idx = arrays["positions"], arrays["indices"]
    perm = arrays["tri_perm"]
    rank_slot = reference_ranks(arrays["tri_bvh"], perm.size)
    rank = np.full(idx.shape[0], np.iinfo(np.int64).max)
    rank[perm] = rank_slot
    v0 = pos[idx[:, 0]]
    e1 = (pos[idx[:, 1]] - v0).astype(np.float32)
    e2 = (pos[idx[:, 2]] - v0).astype(np.float32)
    hit = np.full(ro.shape[0], 0xFFFFFFFF, np.uint32)
    tout = np.zeros(ro.shape[0], np.float32)
    for i in range(ro.shape[0]):
        ok, t = mt_all(e1, e2, v0, ro[i, :3], rd[i, :3])
        if ok.any():
            tm = t[ok].min()
            cand = np.flatnonzero(ok & (t == tm))
            hit[i] = (1 << 30) | int(cand[np.argmin(rank[cand])])
            tout[i] = tm
    return hit, tout
