"""The reference's own image goldens, for the scenes whose estimator is this
path's: its golden cells render a fixture for 64 frames with the denoiser off,
tone-map it to 8 bits and compare it with `tests/goldens/Darwin/<scene>__metal__off.png`
by `tools/imgdiff` (per-pixel RGBA L2 distance; a cell passes when the mean
distance is at most MEAN_DELTA and at most FAIL_PERCENT of the pixels are
farther than MAX_DELTA; thresholds per cell from `tests/CMakeLists.txt:499-1000`).

Here the fp32 oracle renders each fixture on the engine's startup state (its
default `r_env_map assets/hdri/sunset.hdr`, then the fixture's commands), the
oracle's tone map makes the 8-bit image, and the reference's thresholds are
applied.  The GPU path is bit-identical to the oracle (the `-m gpu` parity
tests), so passing these cells pins the GPU path to the reference's goldens
too.  The fixtures and PNGs are read in place from the reference tree; the
test is skipped where that tree is absent."""
import os
import struct
import zlib

import numpy as np
import pytest

import oracle
from conftest import load_pkg

REF = oracle.REF_TREE
SCENES = os.path.join(REF, "tests", "goldens", "scenes")
GOLDENS = os.path.join(REF, "tests", "goldens", "Darwin")

# scene: (MAX_DELTA, MEAN_DELTA, FAIL_PERCENT) of its metal/off golden cell
CELLS = {
    "env_glass_furnace": (16.0, 2.0, 1.0),
    "light_tree_200_pts": (32.0, 4.0, 2.0),
    "sdf_smin_row": (32.0, 4.0, 2.0),
    "sdf_fractals": (32.0, 4.0, 2.0),
}


def read_png(path):
    """8-bit RGB/RGBA PNG -> (H, W, 4) uint8 (the format's five row filters)."""
    b = open(path, "rb").read()
    assert b[:8] == b"\x89PNG\r\n\x1a\n"
    i, idat = 8, b""
    w = h = ct = 0
    while i < len(b):
        n = struct.unpack(">I", b[i:i + 4])[0]
        kind, data = b[i + 4:i + 8], b[i + 8:i + 8 + n]
        i += 12 + n
        if kind == b"IHDR":
            w, h, depth, ct = struct.unpack(">IIBB", data[:10])
            assert depth == 8 and data[12] == 0, "8-bit, non-interlaced only"
        elif kind == b"IDAT":
            idat += data
    ch = {2: 3, 6: 4}[ct]
    stride = w * ch
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, stride + 1)
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f, line = raw[y, 0], raw[y, 1:].astype(np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            cur = np.zeros(stride, np.int32)
            for x in range(stride):
                a = cur[x - ch] if x >= ch else 0
                if f == 1:
                    p = a
                elif f == 3:
                    p = (a + prev[x]) >> 1
                else:
                    c = prev[x - ch] if x >= ch else 0
                    pa, pb, pc = abs(prev[x] - c), abs(a - c), abs(a + prev[x] - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (prev[x] if pb <= pc else c)
                cur[x] = (line[x] + p) & 255
        out[y] = cur
        prev = cur.astype(np.int32)
    img = out.reshape(h, w, ch)
    if ch == 3:
        img = np.concatenate([img, np.full((h, w, 1), 255, np.uint8)], -1)
    return img


@pytest.mark.parametrize("scene", sorted(CELLS))
def test_oracle_passes_the_reference_golden_cell(orc, scene):
    cfg = os.path.join(SCENES, scene + ".cfg")
    png = os.path.join(GOLDENS, scene + "__metal__off.png")
    if not (os.path.isfile(cfg) and os.path.isfile(png)):
        pytest.skip("reference goldens not present")
    pt = load_pkg()
    s = pt.Scene()
    rep, n = s.exec_cfg("r_env_map assets/hdri/sunset.hdr\n", base_dir=REF)   # engine startup default
    assert n == 0, rep
    rep, n = s.load_cfg(cfg, base_dir=REF)
    assert "command outside this path" not in rep, rep           # every scene command is in scope
    W, H = int(s.get_cvar("app_window_width")), int(s.get_cvar("app_window_height"))
    head, prm = s.push(W, H, 0, 1)
    acc, _ = orc.render(s.packed(), head, prm, W, H, 64)
    img = orc.tonemap(acc, s.get_cvar("r_exposure"), int(s.get_cvar("r_tonemap_op")), True)
    gold = read_png(png)
    assert gold.shape == img.shape
    max_delta, mean_delta, fail_percent = CELLS[scene]
    st, _ = pt.imgdiff(img, gold, max_delta)
    assert st.mean_delta <= mean_delta and st.bad_percent <= fail_percent, \
        (st.mean_delta, st.bad_percent, st.max_delta)
