"""The reference's golden-image cells whose estimator is this library's path,
from the committed fixture tests/golden/reference_cells.npz (written by
tests/golden/make_reference_cells.py from the reference tree): the scene
fixtures, the Darwin metal/off golden PNGs, the cells' imgdiff thresholds and
the environment maps they load.

A golden cell of the reference renders its fixture for 64 frames with the
denoiser off, tone-maps it to 8 bits and compares it with the golden PNG by
`tools/imgdiff`: per-pixel RGBA L2 distance; the cell passes when the mean
distance is at most MEAN_DELTA and at most FAIL_PERCENT of the pixels are
farther than MAX_DELTA (thresholds per cell from tests/CMakeLists.txt:499-1000).
The scene is built on the engine's startup state: its default
`r_env_map assets/hdri/sunset.hdr`, then the fixture's commands."""
import os
import struct
import zlib

import numpy as np

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_cells.npz")
FRAMES = 64


def cells():
    z = np.load(FIXTURE)
    return sorted(k[4:] for k in z.files if k.startswith("cfg_"))


def read_png(data):
    """8-bit RGB/RGBA PNG bytes -> (H, W, 4) uint8 (the format's five row filters)."""
    b = bytes(data)
    assert b[:8] == b"\x89PNG\r\n\x1a\n"
    i, idat = 8, b""
    w = h = ct = 0
    while i < len(b):
        n = struct.unpack(">I", b[i:i + 4])[0]
        kind, chunk = b[i + 4:i + 8], b[i + 8:i + 8 + n]
        i += 12 + n
        if kind == b"IHDR":
            w, h, depth, ct = struct.unpack(">IIBB", chunk[:10])
            assert depth == 8 and chunk[12] == 0, "8-bit, non-interlaced only"
        elif kind == b"IDAT":
            idat += chunk
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


def load_cell(pt, scene, workdir):
    """(Scene, golden RGBA8, (MAX_DELTA, MEAN_DELTA, FAIL_PERCENT)) of one cell.
    The fixture's files are laid out under `workdir` as in the reference tree
    (assets/hdri/*.hdr, the .cfg) so the cfg front end reads them unchanged."""
    z = np.load(FIXTURE)
    hdri = os.path.join(workdir, "assets", "hdri")
    os.makedirs(hdri, exist_ok=True)
    for k in z.files:
        if k.startswith("hdr_"):
            with open(os.path.join(hdri, k[4:] + ".hdr"), "wb") as f:
                f.write(z[k].tobytes())
    cfg = os.path.join(workdir, scene + ".cfg")
    with open(cfg, "wb") as f:
        f.write(z["cfg_" + scene].tobytes())
    s = pt.Scene()
    rep, n = s.exec_cfg("r_env_map assets/hdri/sunset.hdr\n", base_dir=workdir)   # engine startup default
    assert n == 0, rep
    rep, n = s.load_cfg(cfg, base_dir=workdir)
    assert "command outside this path" not in rep, rep           # every scene command is in scope
    return s, read_png(z["png_" + scene]), tuple(float(x) for x in z["thr_" + scene])


def passes(pt, img, gold, thr):
    """imgdiff of the cell: (passed, stats)."""
    max_delta, mean_delta, fail_percent = thr
    st, _ = pt.imgdiff(img, gold, max_delta)
    return (st.mean_delta <= mean_delta and st.bad_percent <= fail_percent), st
