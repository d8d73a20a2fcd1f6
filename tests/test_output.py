"""Output step: PNG/PPM capture, imgdiff metrics, and the oracle's tone map
against a float64 restatement of each operator."""
import struct
import zlib

import numpy as np
import pytest

import oracle as orc_mod
from conftest import load_pkg


def read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF
        if typ == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 6
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 4 * w)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].reshape(h, w, 4)


@pytest.mark.parametrize("w,h", [(3, 2), (200, 170)])   # 200x170x4 spans several stored blocks
def test_png_and_ppm_round_trip(tmp_path, w, h):
    pt = load_pkg()
    img = np.random.default_rng(w).integers(0, 256, (h, w, 4), dtype=np.uint8)
    pt.write_png(str(tmp_path / "a.png"), img)
    assert np.array_equal(read_png(str(tmp_path / "a.png")), img)
    pt.write_ppm(str(tmp_path / "a.ppm"), img)
    data = open(tmp_path / "a.ppm", "rb").read()
    head = f"P6\n{w} {h}\n255\n".encode()
    assert data[:len(head)] == head
    assert np.array_equal(np.frombuffer(data[len(head):], np.uint8).reshape(h, w, 3), img[..., :3])


def test_imgdiff_metrics():
    pt = load_pkg()
    rng = np.random.default_rng(1)
    a = rng.integers(0, 256, (40, 30, 4), dtype=np.uint8)
    b = a.copy()
    b[5:10, 3:8, 1] = np.clip(b[5:10, 3:8, 1].astype(int) + 40, 0, 255)
    b[0, 0] = 255 - a[0, 0]
    st, hm = pt.imgdiff(a, b, bad_threshold=10.0, heatmap=True)
    d = np.sqrt(((a.astype(np.int64) - b.astype(np.int64)) ** 2).sum(axis=2))
    assert st.total_pixels == 1200 and st.max_delta == pytest.approx(d.max())
    assert st.mean_delta == pytest.approx(d.mean()) and st.rms_delta == pytest.approx(np.sqrt((d ** 2).mean()))
    assert st.bad_pixels == int((d > 10).sum()) and st.bad_percent == pytest.approx(100 * (d > 10).mean())
    assert tuple(hm[0, 0]) == (255, 255, 100, 255) and tuple(hm[20, 20]) == (0, 0, 0, 255)
    st0, _ = pt.imgdiff(a, a)
    assert st0.max_delta == 0 and st0.bad_pixels == 0


def _reference_ops(c):
    """float64 restatements of the five operators + the sRGB OETF."""
    aces = np.clip((c * (2.51 * c + 0.03)) / (c * (2.43 * c + 0.59) + 0.14), 0, 1)
    rein = np.clip(c / (1 + c), 0, 1)
    lin = np.clip(c, 0, 1)
    ir = np.array([[0.842479062253094, 0.0784335999999992, 0.0792237451477643],
                   [0.0423282422610123, 0.878468636469772, 0.0791661274605434],
                   [0.0423756549057051, 0.0784336, 0.879142973793104]])
    v = c @ ir.T
    v = (np.clip(np.log2(np.maximum(v, 1e-10)), -12.47393, 4.026069) + 12.47393) / (4.026069 + 12.47393)
    v = 15.5 * v ** 6 - 40.14 * v ** 5 + 31.96 * v ** 4 - 6.868 * v ** 3 + 0.4298 * v ** 2 + 0.1191 * v - 0.00232
    orm = np.array([[1.19687900512017, -0.0980208811401368, -0.0990297440797205],
                    [-0.0528968517574562, 1.15190312990417, -0.0989611768448433],
                    [-0.0529716355144438, -0.0980434501171241, 1.15107367264116]])
    agx = np.clip(np.maximum(np.maximum(v, 0) @ orm.T, 0) ** 2.2, 0, 1)
    x = c.min(axis=-1, keepdims=True)
    cc = c - np.where(x < 0.08, x - 6.25 * x * x, 0.04)
    peak = cc.max(axis=-1, keepdims=True)
    d = 1 - 0.76
    npk = 1 - d * d / (peak + d - 0.76)
    g = 1 - 1 / (0.15 * (peak - npk) + 1)
    with np.errstate(invalid="ignore", divide="ignore"):     # the black pixel takes the other branch
        comp = cc * (npk / peak)
    khr = np.where(peak < 0.76, cc, comp + g * (npk - comp))
    return [aces, agx, khr, rein, lin]


@pytest.mark.parametrize("srgb", [False, True])
def test_oracle_tonemap_operators(srgb):
    rng = np.random.default_rng(4)
    acc = np.zeros((32, 48, 4), np.float32)
    acc[..., :3] = np.exp(rng.normal(-1.0, 1.8, (32, 48, 3))).astype(np.float32)
    acc[0, 0, :3] = 0.0
    exposure = 0.7
    refs = _reference_ops(acc[..., :3].astype(np.float64) * exposure)
    for op, ref in enumerate(refs):
        got = orc_mod.tonemap(acc, exposure, op, srgb).astype(np.int64)
        r = np.clip(ref, 0, 1)
        if srgb:
            r = np.where(r < 0.0031308, r * 12.92, 1.055 * np.power(r, 1 / 2.4) - 0.055)
        want = np.floor(np.clip(r, 0, 1) * 255 + 0.5).astype(np.int64)
        assert np.abs(got[..., :3] - want).max() <= 1, op
        assert np.all(got[..., 3] == 255)
