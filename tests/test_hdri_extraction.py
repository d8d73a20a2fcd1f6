"""The HDRI cluster extraction (the env-map light extraction of
ReloadEnvMap, src/engine/Engine.cpp:4370-4535) against an independent float64
numpy restatement.

The reference's Engine.cpp does not build on its own here (it needs the whole
engine), so this extraction has no reference binary to run against; its parity
with the reference rests on this restatement of the cited lines.  The
restatement uses another algorithm for the same definition: connected
components by scipy.ndimage.label (4-connected) with the labels on columns 0
and W-1 merged (the lat-long map wraps in u, not in v), per-cluster sums by
np.bincount, the selection by a stable sort.  The product follows the
reference's own scheme (a depth-first flood fill with an explicit stack), so the
double sums run in another order: directions, fluxes and pmfs are compared at
float32 precision, the light count, the kept set and its order, and the CDF
mask exactly.

The definition (Engine.cpp line ranges):
  * luminance 0.2126 r + 0.7152 g + 0.0722 b in float; no extraction unless the
    peak exceeds 0.5 (:4382-4397);
  * threshold = the (N - max(1, floor(N * f)))-th smallest luminance, f =
    r_hdri_extract_percentile clamped to [1e-6, 0.5], raised to 5% of the peak
    and to 0.5; mask = luminance >= threshold (:4398-4426);
  * 4-connected clusters with horizontal wrap; per pixel dOmega =
    2 pi^2 / N * sin(theta), theta = pi (v + 0.5) / H, phi = 2 pi (u + 0.5) / W - pi,
    direction (sin theta cos phi, cos theta, sin theta sin phi) weighted by the
    double luminance times dOmega, flux = rgb dOmega, lum = luminance dOmega
    (:4430-4488);
  * clusters sorted by lum descending (ties: discovery order, i.e. the raster
    position of a cluster's first pixel; std::sort is an insertion sort below 17
    elements, so ties stay in that order for the cluster counts used here),
    at most 8 kept, clusters of fewer than 3 pixels skipped; pmf =
    float(lum) * float(1 / sum of kept lum); pixels of clusters not kept leave
    the mask (:4490-4525).
The mask is checked through the environment CDF it produces: the product's
scene CDF must equal pt_build_env_cdf (BuildEnvCdf, pinned bit for bit to the
reference elsewhere) over the restatement's mask."""

import numpy as np
import pytest
from scipy import ndimage

from test_builders import product_env_cdf

F32 = np.float32


def extract_reference(rgb, top_frac=0.005):
    """(lights [(dir float32[3], flux float32[3], pmf float32)], mask (H, W) bool)."""
    rgb = np.asarray(rgb, F32)
    H, W, _ = rgb.shape
    N = W * H
    r, g, b = rgb[..., 0], rgb[..., 1], rgb[..., 2]
    lum = (F32(0.2126) * r + F32(0.7152) * g) + F32(0.0722) * b
    peak = max(F32(0.0), lum.max())
    mask = np.zeros((H, W), bool)
    if peak > F32(0.5):
        f = min(max(top_frac, 1e-6), 0.5)
        k = N - max(1, int(float(N) * f))
        thresh = np.partition(lum.ravel(), k)[k]
        if thresh < F32(0.05) * peak:
            thresh = F32(0.05) * peak
        if thresh < F32(0.5):
            thresh = F32(0.5)
        mask = lum >= thresh
    lab, n = ndimage.label(mask, structure=[[0, 1, 0], [1, 1, 1], [0, 1, 0]])
    # merge labels across the u seam (union-find)
    parent = list(range(n + 1))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for v in range(H):
        a, c = lab[v, 0], lab[v, W - 1]
        if a and c:
            ra, rc = find(a), find(c)
            if ra != rc:
                parent[max(ra, rc)] = min(ra, rc)
    root = np.array([find(i) for i in range(n + 1)])
    lab = root[lab]
    # discovery order: raster position of each cluster's first pixel
    flat = lab.ravel()
    ids, first = np.unique(flat[flat > 0], return_index=True)
    first = np.flatnonzero(flat > 0)[first]
    order_ids = ids[np.argsort(first, kind="stable")]
    dense = np.zeros(n + 1, np.int64)
    dense[order_ids] = np.arange(len(order_ids))
    nc = len(order_ids)
    vv, uu = np.nonzero(lab)
    cid = dense[lab[vv, uu]]
    theta = np.pi * (vv + 0.5) / H
    phi = 2.0 * np.pi * (uu + 0.5) / W - np.pi
    d_omega = (2.0 * np.pi * np.pi / N) * np.sin(theta)
    r64, g64, b64 = (rgb[vv, uu, c].astype(np.float64) for c in range(3))
    lum64 = (0.2126 * r64 + 0.7152 * g64) + 0.0722 * b64
    wdir = lum64 * d_omega
    dirs = np.stack([np.sin(theta) * np.cos(phi), np.cos(theta), np.sin(theta) * np.sin(phi)], 1)
    cdir = np.stack([np.bincount(cid, dirs[:, a] * wdir, nc) for a in range(3)], 1)
    cw = np.bincount(cid, wdir, nc)
    flux = np.stack([np.bincount(cid, x * d_omega, nc) for x in (r64, g64, b64)], 1)
    clum = np.bincount(cid, lum64 * d_omega, nc)
    pixels = np.bincount(cid, minlength=nc)
    kept, total = [], 0.0
    for i in np.argsort(-clum, kind="stable"):
        if len(kept) >= 8:
            break
        if pixels[i] < 3 or cw[i] <= 0.0:
            continue
        kept.append(i)
        total += clum[i]
    lights = []
    inv_total = F32(1.0 / total) if total > 0 else F32(0)
    for i in kept:
        d = cdir[i] / np.sqrt(cdir[i] @ cdir[i])
        lights.append((d.astype(F32), flux[i].astype(F32), F32(clum[i]) * inv_total))
    keep = np.zeros(nc, bool)
    keep[kept] = True
    out_mask = mask.copy()
    out_mask[vv[~keep[cid]], uu[~keep[cid]]] = False
    return lights, out_mask


def product_extract(pt, rgb, top_frac=None):
    s = pt.Scene()
    if top_frac is not None:
        s.set_cvar("r_hdri_extract_percentile", top_frac)
    s.env(rgb)
    return s.arrays()


def check(pt, rgb, top_frac=None, expect_count=None):
    a = product_extract(pt, rgb, top_frac)
    lights, mask = extract_reference(rgb, 0.005 if top_frac is None else top_frac)
    if expect_count is not None:
        assert len(lights) == expect_count
    assert a["hdri_count"] == len(lights)
    for i, (d, flux, pmf) in enumerate(lights):
        np.testing.assert_allclose(a["hdri_dir_pmf"][i, :3], d, rtol=1e-6, atol=1e-6)
        np.testing.assert_allclose(a["hdri_col"][i, :3], flux, rtol=1e-6)
        np.testing.assert_allclose(a["hdri_dir_pmf"][i, 3], pmf, rtol=1e-6)
    assert not a["hdri_dir_pmf"][len(lights):].any()
    marg, cond, total = product_env_cdf(pt, rgb, mask.astype(np.uint8))
    np.testing.assert_array_equal(a["env_conditional"], cond)
    np.testing.assert_array_equal(a["env_marginal"], marg)
    assert a["env_total"] == total
    return a, lights, mask


def base_map(H=64, W=128, seed=0):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.1, 0.3, (H, W, 3)).astype(F32)


def test_several_clusters_one_across_the_seam(pt):
    img = base_map()
    img[10:13, 20:24] = (9e3, 8e3, 7e3)          # 12 px
    img[30:33, 126:128] = 6e3                    # seam cluster, left part
    img[30:33, 0:3] = 6e3                        # ... and its right part: one cluster of 15 px
    img[45:47, 60:63] = (2e3, 3e3, 1e3)          # 6 px
    img[55, 90:92] = 1e4                         # 2 px: below the 3-pixel minimum
    a, lights, mask = check(pt, img, expect_count=3)
    assert mask[30, 127] and mask[30, 0] and not mask[55, 90]
    # the seam cluster's direction points at the seam (phi = +-pi: x < 0, z ~ 0)
    seam = [d for d, _, _ in lights if d[0] < -0.5]
    assert len(seam) == 1 and abs(seam[0][2]) < 0.05


def test_tied_clusters_keep_discovery_order(pt):
    img = base_map(seed=1)
    img[20:22, 30:33] = 5e3                      # two identical clusters in the same rows
    img[20:22, 90:93] = 5e3
    img[40:42, 50:52] = 4e3                      # dimmer than the tied pair
    a, lights, _ = check(pt, img, expect_count=3)
    assert lights[0][2] == lights[1][2]
    assert a["hdri_dir_pmf"][0, 0] != a["hdri_dir_pmf"][1, 0]


def test_more_than_eight_candidates_keep_the_eight_brightest(pt):
    img = base_map(H=96, W=192, seed=2)
    for i in range(12):
        v, u = 8 + 7 * i, 10 + 15 * i
        img[v:v + 2, u:u + 2] = 1e3 * (i + 1)   # distinct fluxes
    a, lights, mask = check(pt, img, expect_count=8)
    # the four dimmest candidates are back in the CDF
    for i in range(4):
        v, u = 8 + 7 * i, 10 + 15 * i
        assert not mask[v, u]


def test_percentile_threshold_above_the_floors(pt):
    # a broad bright band: the 99.5th percentile lies above 5% of the peak and 0.5
    img = base_map(seed=3)
    img[5:9, :] = np.linspace(50, 90, 128, dtype=F32)[None, :, None]
    img[60, 5:9] = 100.0
    a, lights, mask = check(pt, img)
    assert 0 < len(lights) <= 8
    assert mask.sum() == max(1, int(64 * 128 * 0.005))


@pytest.mark.parametrize("top_frac", [0.05, 1e-7, 0.9])
def test_percentile_cvar_and_its_clamp(pt, top_frac):
    img = base_map(seed=4)
    img[5:9, 10:40] = np.linspace(10, 40, 30, dtype=F32)[None, :, None]
    img[50:52, 70:73] = 200.0
    check(pt, img, top_frac)


def test_dim_map_extracts_nothing(pt):
    img = base_map(seed=5) * F32(0.5)           # peak <= 0.5: no extraction
    a, lights, mask = check(pt, img, expect_count=0)
    assert not mask.any()


def test_synthetic_sun_env_of_the_triangle_scene(pt):
    """The 2048 x 1024 log-normal environment with the 0.5 deg sun disc of the
    triangle+analytic configuration: its extracted light list as the restatement
    computes it."""
    s = pt.Scene().synth(1, seed=0)
    p = s.packed()
    W, H = p.env_w, p.env_h
    rgba = np.ctypeslib.as_array(p.env_rgba, (H * W * 4,)).reshape(H, W, 4)
    rgb = np.ascontiguousarray(rgba[..., :3])
    a, lights, mask = check(pt, rgb)
    assert len(lights) >= 1 and lights[0][2] > 0.5    # the sun dominates
    print(f"triangle-scene env: {len(lights)} HDRI light(s); sun dir {lights[0][0]}, pmf {lights[0][2]:.4f}; "
          f"{int(mask.sum())} masked texels")
