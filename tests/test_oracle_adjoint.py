"""The FP64 adjoint oracle against central finite differences of the fp32
oracle render with common random numbers (same pixel seeds).  With Russian
roulette off and no firefly clamp the per-sample estimator is a polynomial in
the material albedos and linear in the emissions, so the adjoint and the
central difference agree per sample, up to fp32 rounding of the images."""
import numpy as np

import oracle as orc_mod
from conftest import load_pkg


def _setup(rr_start):
    pt = load_pkg()
    s = pt.Scene().synth(3, seed=0, scale=0.3)
    s.set_cvar("r_spp", 2)
    s.set_cvar("r_rr_start", rr_start)
    W = H = 32
    head, prm = s.push(W, H, 0, 1)
    pk = s.packed()
    n = pk.material_count
    mats = np.ctypeslib.as_array(pk.materials, (n * 12,)).reshape(n, 12).copy()
    return s, W, H, head, prm, pk, mats


def _loss(orc, s, W, H, w, m):
    s.materials(m)
    head, prm = s.push(W, H, 0, 1)
    a, _ = orc.render(s.packed(), head, prm, W, H, 1)
    return float((a[..., :3].astype(np.float64) * w).sum())


def test_oracle_adjoint_matches_central_differences(orc):
    s, W, H, head, prm, pk, mats = _setup(rr_start=6)   # depth 6: no roulette
    w = np.random.default_rng(7).standard_normal((H, W, 3)).astype(np.float32)
    ga, ge = orc_mod.adjoint(pk, head, prm, W, H, 1, w)
    assert np.abs(ga).max() > 0 and np.abs(ge).max() > 0
    eps = 1e-3
    checked = 0
    for which, g, col0 in (("albedo", ga, 0), ("emission", ge, 4)):
        for k in np.argsort(-np.abs(g).ravel())[:6]:
            r, c = divmod(int(k), 3)
            mp, mm = mats.copy(), mats.copy()
            mp[r, col0 + c] += eps
            mm[r, col0 + c] -= eps
            fd = (_loss(orc, s, W, H, w, mp) - _loss(orc, s, W, H, w, mm)) / (2 * eps)
            assert abs(g[r, c] - fd) <= 2e-3 * abs(fd) + 1e-4, (which, r, c, g[r, c], fd)
            checked += 1
    assert checked == 12


def test_oracle_adjoint_rejects_the_firefly_clamp(orc):
    s, W, H, head, prm, pk, mats = _setup(rr_start=3)
    prm.firefly_clamp = 10.0
    w = np.ones((H, W, 3), np.float32)
    try:
        orc_mod.adjoint(pk, head, prm, W, H, 1, w)
    except RuntimeError as e:
        assert "-7" in str(e)
    else:
        raise AssertionError("firefly clamp accepted")
