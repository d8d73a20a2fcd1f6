"""Environment-map importance sampling, checked the way the reference checks
its own (`tests/hdrimage_cdf_test.cpp`): sampled texels follow the CDF's
distribution (chi-square round trip, :487), the pdf a sample is drawn with
equals the pdf evaluated at its direction (pdf inversion, :580), a texel of zero
luminance is never drawn, and the sampler is deterministic.  The sampler is
the oracle's fp32 instance, which the GPU matches bit for bit in the renders."""
import numpy as np
import pytest

from conftest import load_pkg


def _scene(img, mask_hdri=False):
    pt = load_pkg()
    s = pt.Scene()
    if not mask_hdri:
        s.set_cvar("r_hdri_extract_percentile", 0.0)    # no cluster extraction: the plain CDF
    s.env(img)
    head, prm = s.push(8, 8)
    return s, head, prm


def _texel_of(d, W, H):
    th = np.arccos(np.clip(d[:, 1], -1, 1))
    ph = np.arctan2(d[:, 2], d[:, 0])
    u = np.minimum(((ph + np.pi) / (2 * np.pi) * W).astype(np.int64), W - 1)
    v = np.minimum((th / np.pi * H).astype(np.int64), H - 1)
    return v * W + u


def _cdf_probabilities(a, W, H):
    marg = a["env_marginal"].astype(np.float64)
    cond = a["env_conditional"].astype(np.float64).reshape(H, W)
    prow = np.diff(np.concatenate([[0.0], marg]))
    pcol = np.diff(np.concatenate([np.zeros((H, 1)), cond], axis=1), axis=1)
    return (prow[:, None] * pcol).ravel()


def test_env_sampling_chi_square_round_trip(orc):
    rng = np.random.default_rng(3)
    H, W = 16, 32
    img = rng.uniform(0.05, 1.0, (H, W, 3)).astype(np.float32)
    img[5, 7] = 40.0                                         # a bright spot, as in the reference test
    s, head, prm = _scene(img)
    n = 400_000
    xu = rng.random(n, dtype=np.float32)
    xv = rng.random(n, dtype=np.float32)
    d, pdf, _ = orc.env_sample(s.packed(), head, prm, xu, xv)
    got = np.bincount(_texel_of(d.astype(np.float64), W, H), minlength=W * H)
    p = _cdf_probabilities(s.arrays(), W, H)
    exp = p * n
    keep = exp >= 5
    chi2 = (((got[keep] - exp[keep]) ** 2) / exp[keep]).sum()
    dof = int(keep.sum()) - 1
    # chi-square with dof degrees of freedom: mean dof, sd sqrt(2 dof); 5 sd is far out
    assert chi2 < dof + 5 * np.sqrt(2 * dof), (chi2, dof)
    assert got[~keep].sum() <= 5 * max(1, int((~keep).sum()))


def test_env_pdf_inversion_and_zero_texels(orc):
    rng = np.random.default_rng(4)
    H, W = 16, 32
    img = rng.uniform(0.0, 2.0, (H, W, 3)).astype(np.float32)
    img[3:6, 10:14] = 0.0                                     # dark texels must never be drawn
    s, head, prm = _scene(img)
    n = 100_000
    xu = rng.random(n, dtype=np.float32)
    xv = rng.random(n, dtype=np.float32)
    d, pdf, pdf_eval = orc.env_sample(s.packed(), head, prm, xu, xv)
    ok = pdf > 0
    assert ok.mean() > 0.999
    np.testing.assert_allclose(pdf_eval[ok], pdf[ok], rtol=1e-6)   # the texel centre maps back to its texel
    tex = _texel_of(d.astype(np.float64), W, H)
    dark = np.zeros((H, W), bool)
    dark[3:6, 10:14] = True
    assert not dark.ravel()[tex].any()
    # pdf = lum * W * H / (2 pi^2 * total) (pdfEnvMapDir) at each drawn texel
    lum = (0.2126 * img[..., 0] + 0.7152 * img[..., 1] + 0.0722 * img[..., 2]).ravel()[tex]
    total = float(s.arrays()["env_total"])
    np.testing.assert_allclose(pdf[ok], (lum * W * H / (2 * np.pi ** 2 * total))[ok], rtol=2e-5)


def test_env_sampling_is_deterministic(orc):
    rng = np.random.default_rng(5)
    img = rng.uniform(0.0, 1.0, (8, 16, 3)).astype(np.float32)
    s, head, prm = _scene(img)
    xu = rng.random(1000, dtype=np.float32)
    xv = rng.random(1000, dtype=np.float32)
    a = orc.env_sample(s.packed(), head, prm, xu, xv)
    b = orc.env_sample(s.packed(), head, prm, xu, xv)
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
