"""TEST INFRASTRUCTURE ONLY -- ctypes binding of the CPU oracle.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this package, to verify the GPU results and as the CPU baseline; the product
never imports it.

  liboracle.so        CPU restatement of the reference path tracer (fp32 + fp64),
                      built from oracle/pt_oracle.cpp by oracle/Makefile
  _ref/libref_builders.so
                      the reference's own AnalyticBvh / TriangleBvh / BuildEnvCdf
                      compiled from the reference sources (only where the
                      reference tree is present; never shipped)
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_builders.so")


def _reference_tree():
    """The reference source tree: PT_REFERENCE_TREE when set, else the REF
    default of oracle/Makefile (the recipe that compiles the reference's
    builders from their sources).  None when no such tree exists here: the
    tests that read it skip, and the GPU host never has it."""
    env = os.environ.get("PT_REFERENCE_TREE")
    if env:
        return env
    try:
        r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref"],
                           capture_output=True, text=True, timeout=30)
        path = r.stdout.strip()
    except Exception:
        return None
    return path if path and os.path.isdir(os.path.join(path, "src", "renderer")) else None


REF_TREE = _reference_tree()

u32 = ctypes.c_uint32
f32 = ctypes.c_float
P = ctypes.POINTER


class OracleCounters(ctypes.Structure):
    _fields_ = [("rays", ctypes.c_uint64), ("nodes", ctypes.c_uint64), ("tris", ctypes.c_uint64),
                ("prims", ctypes.c_uint64), ("ext_rays", ctypes.c_uint64),
                ("shadow_rays", ctypes.c_uint64), ("ext_nodes", ctypes.c_uint64),
                ("ext_tris", ctypes.c_uint64), ("ext_prims", ctypes.c_uint64)]


def build(ref: bool | None = None):
    """make -C oracle (and the reference builders when the reference tree exists)."""
    targets = ["all"]
    if ref is None:
        ref = REF_TREE is not None
    if ref and REF_TREE:
        targets.append("ref")
    extra = [f"REF={REF_TREE}"] if REF_TREE else []
    subprocess.run(["make", "-s", "-C", HERE, *extra, *targets], check=True)


_lib = None
_ref = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(ref=False)
        _lib = ctypes.CDLL(LIB)
        _lib.oracle_trace.restype = ctypes.c_int
        _lib.oracle_render.restype = ctypes.c_int
        _lib.oracle_adjoint.restype = ctypes.c_int
        for n in ("oracle_sinf", "oracle_cosf", "oracle_acosf"):
            getattr(_lib, n).restype = f32
            getattr(_lib, n).argtypes = [f32]
        _lib.oracle_atan2f.restype = f32
        _lib.oracle_atan2f.argtypes = [f32, f32]
        _lib.oracle_pcg_hash.restype = u32
        _lib.oracle_pcg_hash.argtypes = [u32]
    return _lib


def load_ref():
    """The reference's builders compiled from source, or None where unavailable."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB):
        _ref = ctypes.CDLL(REF_LIB)
    return _ref


def render(packed, head, prm, W, H, frames=1, accum=None, crop=None, fp64=False, threads=0):
    """Render `frames` frames; returns (accum (H, W, 4) float32, OracleCounters)."""
    lib = load()
    if accum is None:
        accum = np.zeros((H, W, 4), np.float32)
    x0, y0, x1, y1 = crop if crop is not None else (0, 0, W, H)
    c = OracleCounters()
    rc = lib.oracle_render(ctypes.byref(packed), ctypes.byref(head), ctypes.byref(prm), u32(W), u32(H),
                           u32(frames), accum.ctypes.data_as(P(f32)), u32(x0), u32(y0), u32(x1), u32(y1),
                           ctypes.c_int(1 if fp64 else 0), ctypes.c_int(threads), ctypes.byref(c))
    if rc != 0:
        raise RuntimeError(f"oracle_render failed: {rc}")
    return accum, c


def capture_rays(packed, head, prm, W, H, bounce, crop=None, threads=0):
    """The extension rays bounce `bounce` of frame head.frame_index traces, for
    every sample of the pixels in crop = (x0, y0, x1, y1): (ro4, rd4) float32
    arrays of shape (n, 4), only the samples whose path reached that bounce."""
    lib = load()
    x0, y0, x1, y1 = crop if crop is not None else (0, 0, W, H)
    spp = max(int(head.spp), 1)
    n = (x1 - x0) * (y1 - y0) * spp
    ro = np.zeros((n, 4), np.float32)
    rd = np.zeros((n, 4), np.float32)
    rc = lib.oracle_capture_rays(ctypes.byref(packed), ctypes.byref(head), ctypes.byref(prm), u32(W), u32(H),
                                 u32(bounce), u32(x0), u32(y0), u32(x1), u32(y1), ro.ctypes.data_as(P(f32)),
                                 rd.ctypes.data_as(P(f32)), ctypes.c_int(threads))
    if rc != 0:
        raise RuntimeError(f"oracle_capture_rays failed: {rc}")
    live = np.any(rd[:, :3] != 0.0, axis=1)
    return ro[live], rd[live]


def software_preview(packed, head, prm, W, H, accum=None, threads=0):
    """The reference's Software-backend preview estimator, one frame into
    `accum` (H, W, 4); returns (accum, OracleCounters).  A timed CPU baseline."""
    lib = load()
    if accum is None:
        accum = np.zeros((H, W, 4), np.float32)
    c = OracleCounters()
    rc = lib.oracle_software_preview(ctypes.byref(packed), ctypes.byref(head), ctypes.byref(prm), u32(W), u32(H),
                                     accum.ctypes.data_as(P(f32)), ctypes.c_int(threads), ctypes.byref(c))
    if rc != 0:
        raise RuntimeError(f"oracle_software_preview failed: {rc}")
    return accum, c


def env_sample(packed, head, prm, xu, xv):
    """sampleEnvMap for uniform pairs -> (dirs (n, 3), pdf (n,), pdfEnvMapDir(dirs) (n,))."""
    lib = load()
    xu = np.ascontiguousarray(xu, np.float32)
    xv = np.ascontiguousarray(xv, np.float32)
    n = xu.shape[0]
    d = np.zeros((n, 4), np.float32)
    p = np.zeros(n, np.float32)
    q = np.zeros(n, np.float32)
    rc = lib.oracle_env_sample(ctypes.byref(packed), ctypes.byref(head), ctypes.byref(prm), u32(n),
                               xu.ctypes.data_as(P(f32)), xv.ctypes.data_as(P(f32)), d.ctypes.data_as(P(f32)),
                               p.ctypes.data_as(P(f32)), q.ctypes.data_as(P(f32)))
    if rc != 0:
        raise RuntimeError(f"oracle_env_sample failed: {rc}")
    return d[:, :3], p, q


def adjoint(packed, head, prm, W, H, frames, dl_di, threads=0):
    """FP64 adjoint: (grad_albedo, grad_emission), each (material_count, 3) float64,
    of a `frames`-frame render from reset for dLoss/dImage = dl_di (H, W, 3|4)."""
    lib = load()
    d = np.zeros((H, W, 4), np.float32)
    d[..., :3] = np.asarray(dl_di, np.float32)[..., :3]
    n = packed.material_count
    ga = np.zeros((max(n, 1), 3), np.float64)
    ge = np.zeros((max(n, 1), 3), np.float64)
    dp = P(ctypes.c_double)
    rc = lib.oracle_adjoint(ctypes.byref(packed), ctypes.byref(head), ctypes.byref(prm), u32(W), u32(H),
                            u32(frames), d.ctypes.data_as(P(f32)), ctypes.c_int(threads),
                            ga.ctypes.data_as(dp), ge.ctypes.data_as(dp))
    if rc != 0:
        raise RuntimeError(f"oracle_adjoint failed: {rc}")
    return ga[:n], ge[:n]


def tonemap(accum, exposure, op=0, srgb=False):
    """(H, W, 4) accumulation -> (H, W, 4) uint8 (oracle_tonemap)."""
    lib = load()
    a = np.ascontiguousarray(accum, np.float32)
    out = np.zeros(a.shape[:2] + (4,), np.uint8)
    lib.oracle_tonemap.argtypes = [P(f32), u32, f32, u32, ctypes.c_int, ctypes.c_void_p]
    rc = lib.oracle_tonemap(a.ctypes.data_as(P(f32)), u32(a.shape[0] * a.shape[1]), f32(exposure), u32(op),
                            ctypes.c_int(1 if srgb else 0), out.ctypes.data)
    if rc != 0:
        raise RuntimeError("oracle_tonemap failed")
    return out


def trace(packed, head, prm, ro4, rd4, fp64=False):
    lib = load()
    ro4 = np.ascontiguousarray(ro4, np.float32)
    rd4 = np.ascontiguousarray(rd4, np.float32)
    n = ro4.shape[0]
    hit = np.empty(n, np.uint32)
    t = np.empty(n, np.float32)
    c = OracleCounters()
    rc = lib.oracle_trace(ctypes.byref(packed), ctypes.byref(head), ctypes.byref(prm),
                          ro4.ctypes.data_as(P(f32)), rd4.ctypes.data_as(P(f32)), u32(n),
                          hit.ctypes.data_as(P(u32)), t.ctypes.data_as(P(f32)),
                          ctypes.c_int(1 if fp64 else 0), ctypes.byref(c))
    if rc != 0:
        raise RuntimeError(f"oracle_trace failed: {rc}")
    return hit, t, c


def ref_light_tree(inputs):
    """The reference's BuildLightTree over a structured array of the
    LightInput layout (demont_gb300.LIGHT_INPUT_DTYPE); returns the node bytes
    as a uint8 array of n x 64."""
    lib = load_ref()
    inputs = np.ascontiguousarray(inputs)
    out = np.zeros(max(2 * len(inputs) - 1, 1) * 64, np.uint8)
    n = u32(0)
    lib.ref_build_light_tree.argtypes = [ctypes.c_void_p, u32, ctypes.c_void_p, P(u32)]
    lib.ref_build_light_tree(inputs.ctypes.data, u32(len(inputs)), out.ctypes.data, ctypes.byref(n))
    return out[: n.value * 64].reshape(n.value, 64)


def ref_sdf_aabb(nodes12, count):
    """The reference's ComputeSdfAabb over `count` SdfNode records (12 words
    each); returns (lo, hi) or None when it rejects the cluster."""
    lib = load_ref()
    lo = np.zeros(3, np.float32)
    hi = np.zeros(3, np.float32)
    a = np.ascontiguousarray(nodes12, np.float32)
    lib.ref_sdf_aabb.argtypes = [ctypes.c_void_p, u32, P(f32), P(f32)]
    rc = lib.ref_sdf_aabb(a.ctypes.data, u32(count), lo.ctypes.data_as(P(f32)), hi.ctypes.data_as(P(f32)))
    return (lo, hi) if rc == 0 else None


def ref_analytic_bvh(centers_radii):
    """AnalyticBvh::Build of the reference itself: (nodes (m, 8) uint32, perm)."""
    lib = load_ref()
    cr = np.ascontiguousarray(centers_radii, np.float32)
    n = cr.shape[0]
    nodes = np.zeros((max(2 * n, 1), 8), np.uint32)
    perm = np.zeros(max(n, 1), np.uint32)
    m = u32()
    lib.ref_build_analytic_bvh(cr.ctypes.data_as(P(f32)), u32(n), nodes.ctypes.data_as(ctypes.c_void_p),
                               ctypes.byref(m), perm.ctypes.data_as(P(u32)))
    return nodes[: m.value].copy(), perm[:n].copy()


def ref_triangle_bvh(positions, indices):
    lib = load_ref()
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
    idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
    nt = max(idx.size // 3, 1)
    nodes = np.zeros((2 * nt, 8), np.uint32)
    perm = np.zeros(nt, np.uint32)
    m, k = u32(), u32()
    lib.ref_build_triangle_bvh(pos.ctypes.data_as(P(f32)), u32(pos.size // 3), idx.ctypes.data_as(P(u32)),
                               u32(idx.size), nodes.ctypes.data_as(ctypes.c_void_p), ctypes.byref(m),
                               perm.ctypes.data_as(P(u32)), ctypes.byref(k))
    return nodes[: m.value].copy(), perm[: k.value].copy()


def ref_env_cdf(rgb, mask=None):
    lib = load_ref()
    a = np.ascontiguousarray(rgb, np.float32)
    H, W = a.shape[:2]
    marg = np.zeros(H, np.float32)
    cond = np.zeros(H * W, np.float32)
    tot = ctypes.c_double()
    mk = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    lib.ref_build_env_cdf(a.ctypes.data_as(P(f32)), u32(W), u32(H),
                          None if mk is None else mk.ctypes.data_as(P(ctypes.c_uint8)),
                          marg.ctypes.data_as(P(f32)), cond.ctypes.data_as(P(f32)), ctypes.byref(tot))
    return marg, cond.reshape(H, W), tot.value
