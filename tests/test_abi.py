"""The C-ABI library loads on a machine without a GPU and exports every entry
point that include/*.h declares (no compute calls here)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_functions():
    names = []
    for h in ("pt_gpu.h", "pt_scene.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(pt_[a-z0-9_]+)\s*\(", src, re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(pt):
    lib = pt.load()
    names = declared_functions()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_every_declared_symbol_has_a_binding(pt):
    assert set(declared_functions()) <= set(pt.SIGNATURES), set(declared_functions()) - set(pt.SIGNATURES)


def test_struct_layouts_match_the_reference_sizes(pt):
    # the 112-byte push head (src/rhi_software/SoftwareTracer.cpp:56) and the
    # 32-byte BVH node (src/renderer/AnalyticBvh.h:202)
    assert ctypes.sizeof(pt.PtPushHead) == 112
    assert ctypes.sizeof(pt.PtBvhNode) == 32


def test_version_string(pt):
    assert b"sm_103a" in pt.load().pt_gpu_version()


def test_no_gpu_create_fails_cleanly(pt):
    """Without a usable device pt_gpu_create must return an error, not crash."""
    import torch
    if torch.cuda.is_available():
        return
    try:
        pt.Device(0)
    except pt.PtError as e:
        assert e.code == -2
    else:  # pragma: no cover
        raise AssertionError("pt_gpu_create succeeded without a GPU")
