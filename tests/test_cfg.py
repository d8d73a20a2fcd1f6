"""Scene-fixture front end (.cfg console syntax) and the Radiance .hdr reader."""
import glob
import os
import struct

import numpy as np
import pytest

import oracle
from conftest import load_pkg

REF = oracle.REF_TREE   # the reference source tree, when present (fixtures are read from it)


def write_hdr(path, quads, rle=True):
    """quads: (H, W, 4) uint8 RGBE.  rle: adaptive run-length scanlines (runs for
    repeated bytes, literals otherwise), else flat quadruples."""
    H, W, _ = quads.shape
    out = bytearray(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n" + f"-Y {H} +X {W}\n".encode())
    for y in range(H):
        if not rle:
            out += quads[y].tobytes()
            continue
        out += bytes([2, 2, W >> 8, W & 255])
        for c in range(4):
            ch = quads[y, :, c].tolist()
            x = 0
            while x < W:
                run = 1
                while x + run < W and ch[x + run] == ch[x] and run < 127:
                    run += 1
                if run >= 3:
                    out += bytes([128 + run, ch[x]])
                    x += run
                else:
                    n = 1
                    while x + n < W and n < 128 and not (x + n + 2 < W and ch[x + n] == ch[x + n + 1] == ch[x + n + 2]):
                        n += 1
                    out += bytes([n]) + bytes(ch[x:x + n])
                    x += n
    with open(path, "wb") as f:
        f.write(out)


def decode(quads):
    e = quads[..., 3].astype(np.int32)
    sc = np.where(e > 0, np.ldexp(np.float32(1.0), e - 136), 0.0).astype(np.float32)
    return (quads[..., :3].astype(np.float32) * sc[..., None]).astype(np.float32)


@pytest.mark.parametrize("W,rle", [(37, True), (5, False), (64, True)])
def test_hdr_reader_decodes_rle_and_flat_scanlines(tmp_path, W, rle):
    pt = load_pkg()
    pt.load()
    rng = np.random.default_rng(W)
    q = rng.integers(0, 256, (6, W, 4), dtype=np.uint8)
    q[:, : W // 2, 0] = 77          # runs
    q[2, :, 3] = 0                  # zero exponent row -> black
    p = str(tmp_path / "t.hdr")
    write_hdr(p, q, rle=rle and W >= 8)
    img = pt.load_hdr(p)
    assert np.array_equal(img, decode(q))


def test_hdr_reader_matches_the_reference_loader():
    import ctypes

    import oracle
    ref = oracle.load_ref()
    if ref is None or not os.path.isdir(os.path.join(REF, "assets", "hdri")):
        pytest.skip("reference loader not built here")
    pt = load_pkg()
    pt.load()
    fn = ref.ref_load_radiance_hdr
    fn.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32),
                   ctypes.POINTER(ctypes.c_uint32)]
    for name in ("uniform_gray.hdr", "sunset.hdr"):
        path = os.path.join(REF, "assets", "hdri", name)
        w, h = ctypes.c_uint32(), ctypes.c_uint32()
        assert fn(path.encode(), None, 0, ctypes.byref(w), ctypes.byref(h)) == 0
        want = np.empty((h.value, w.value, 3), np.float32)
        assert fn(path.encode(), want.ctypes.data, want.size, ctypes.byref(w), ctypes.byref(h)) == 0
        assert np.array_equal(pt.load_hdr(path), want)


CFG = """
// a scene in the console syntax
cam_pos 0 4.5 6
cam_yaw 10
cam_pitch -30
cam_fov 50
r_spp 3
r_max_bounces 5
r_sky_mode gradient
r_sun_elevation 35
prim_plane 1 0 1 0 0 lambert 0.7 0.7 0.7
prim_sphere 10 -1 1 0 1 metal 0.9 0.8 0.6 0.2
prim_sphere 11  1.5 0.6 0.5 0.6 dielectric 1 1 1 0 1.45
prim_sphere 12  3 1 -2 1 lambert 0.2 0.3 0.9
prim_set_emission 12 0.5 0.2 0.1
prim_set_roughness 10 0.35
prim_set_ior 11 1.6
prim_sphere 13 9 9 9 1 lambert 1 1 1
prim_remove 13
light_point 1 -3 3 1 20 18 15
light_spot 2 2 4 2 0 -1 0 40 20 10 12 14
light_sphere 3 0 5 -3 0.5 8 8 9
light_quad 4 0 6 0 0 -1 0 1 0 0 0.5 0.25 12 12 12
r_bloom 1
editor_gizmo translate
"""


def test_cfg_builds_the_same_scene_as_the_api():
    pt = load_pkg()
    a = pt.Scene()
    rep, n = a.exec_cfg(CFG)
    assert n == 2 and "r_bloom" in rep and "editor_gizmo" in rep
    b = pt.Scene()
    b.camera((0, 4.5, 6), np.radians(10), np.radians(-30), 50)
    for k, v in (("r_spp", 3), ("r_max_bounces", 5), ("r_sky_mode", 0), ("r_sun_elevation", 35)):
        b.set_cvar(k, v)
    b.plane(1, (0, 1, 0), 0, 0, (0.7, 0.7, 0.7))
    b.sphere(10, -1, 1, 0, 1, 1, (0.9, 0.8, 0.6), rough=0.35)
    b.sphere(11, 1.5, 0.6, 0.5, 0.6, 2, (1, 1, 1), rough=0.0, ior=1.6)
    b.sphere(12, 3, 1, -2, 1, 0, (0.2, 0.3, 0.9))
    b.emission(12, (0.5, 0.2, 0.1))
    b.light_point(1, (-3, 3, 1), (20, 18, 15))
    b.light_spot(2, (2, 4, 2), (0, -1, 0), 40, 20, (10, 12, 14))
    b.light_sphere(3, (0, 5, -3), 0.5, (8, 8, 9))
    b.light_quad(4, (0, 6, 0), (0, -1, 0), (1, 0, 0), 0.5, 0.25, (12, 12, 12))
    ha, pa = a.push(64, 48)
    hb, pb = b.push(64, 48)
    assert bytes(ha) == bytes(hb) and bytes(pa) == bytes(pb)
    xa, xb = a.arrays(), b.arrays()
    for k in xa:
        va, vb = np.asarray(xa[k]), np.asarray(xb[k])
        if va.dtype == np.float32:                  # prim records hold bit-cast u32 fields (NaN patterns)
            va, vb = va.view(np.uint32), vb.view(np.uint32)
        assert np.array_equal(va, vb), k


def test_cfg_reports_malformed_lines_and_keeps_going():
    pt = load_pkg()
    s = pt.Scene()
    with pytest.raises(pt.PtError) as e:
        s.exec_cfg("prim_sphere 1 0 0 0 1 lambert 1 1 1\nprim_sphere 2 0 0 zero 1 lambert 1 1 1\n"
                   "light_point 5 0 3 0 1 1 1\nprim_set_albedo 99 1 1 1\n")
    assert "line 2" in str(e.value)
    assert s.packed().prim_count == 1 and s.packed().light_count == 1


def test_every_reference_fixture_loads():
    if not os.path.isdir(os.path.join(REF, "tests", "goldens", "scenes")):
        pytest.skip("reference fixtures not present")
    pt = load_pkg()
    files = sorted(glob.glob(os.path.join(REF, "tests", "goldens", "scenes", "*.cfg")))
    assert len(files) > 40
    for f in files:
        s = pt.Scene()
        rep, n = s.load_cfg(f, REF)
        assert "ERROR" not in rep, (f, rep)
        s.push(32, 32)
