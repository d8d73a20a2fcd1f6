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
