"""Differentiable render through the C-ABI (pt_gpu_diff_forward/backward):
the recorded forward equals the plain render bit for bit, the path-replay
gradients equal the FP64 adjoint oracle's (same fp32 paths, derivatives
summed in double), and they match central finite differences of GPU renders
with common random numbers (eps 1e-3)."""
import numpy as np
import pytest

import oracle as orc_mod

pytestmark = pytest.mark.gpu


def _scene(pt, scale, spp, rr_start, W, H):
    s = pt.Scene().synth(3, seed=0, scale=scale)
    s.set_cvar("r_spp", spp)
    s.set_cvar("r_rr_start", rr_start)
    head, prm = s.push(W, H, 0, 1)
    pk = s.packed()
    n = pk.material_count
    mats = np.ctypeslib.as_array(pk.materials, (n * 12,)).reshape(n, 12).copy()
    return s, head, prm, pk, mats


@pytest.mark.parametrize("rr_start", [3, 6])
def test_adjoint_matches_fp64_oracle(pt, orc, dev, rr_start):
    W, H, F = 64, 48, 2
    s, head, prm, pk, mats = _scene(pt, 0.3, 4, rr_start, W, H)
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, F)
    plain = dev.read_accum().copy()
    dev.diff_forward(head, prm, F)
    img = dev.read_accum()
    assert np.array_equal(img.view(np.uint32), plain.view(np.uint32))
    o, _ = orc.render(pk, head, prm, W, H, F)
    assert np.array_equal(img.view(np.uint32), o.view(np.uint32))
    w = np.random.default_rng(3).standard_normal((H, W, 3)).astype(np.float32)
    ga, ge = dev.diff_backward(w, mats.shape[0])
    oa, oe = orc_mod.adjoint(pk, head, prm, W, H, F, w)
    for g, og in ((ga, oa), (ge, oe)):
        assert np.abs(og).max() > 0
        tol = 1e-5 * np.abs(og).max() + 1e-4 * np.abs(og)
        bad = np.argwhere(np.abs(g - og) > tol)
        assert bad.size == 0, (bad[:5], g[tuple(bad[0])], og[tuple(bad[0])])


def test_adjoint_matches_central_differences(pt, dev):
    W, H, F = 128, 96, 1
    s, head, prm, pk, mats = _scene(pt, 0.5, 8, 6, W, H)   # depth 6, no roulette
    dev.upload(s)
    dev.set_target(W, H)
    rng = np.random.default_rng(11)
    target = rng.uniform(0.0, 0.3, (H, W, 3)).astype(np.float32)
    dev.diff_forward(head, prm, F)
    img = dev.read_accum()[..., :3].astype(np.float64)
    dl = (2.0 * (img - target)).astype(np.float32)          # L2 loss
    ga, ge = dev.diff_backward(dl, mats.shape[0])

    def loss(m):
        dev.materials(m)
        dev.render(head, prm, F)
        return float(((dev.read_accum()[..., :3].astype(np.float64) - target) ** 2).sum())

    eps = 1e-3
    # 32 parameters: the 24 albedo channels and 8 emission channels with the
    # largest gradients (the rest of the 256 rows are barely visible at this size)
    picks = [("a", int(k)) for k in np.argsort(-np.abs(ga).ravel())[:24]]
    picks += [("e", int(k)) for k in np.argsort(-np.abs(ge).ravel())[:8]]
    errs = []
    for kind, k in picks:
        r, c = divmod(k, 3)
        col = c if kind == "a" else 4 + c
        mp, mm = mats.copy(), mats.copy()
        mp[r, col] += eps
        mm[r, col] -= eps
        fd = (loss(mp) - loss(mm)) / (2 * eps)
        g = ga[r, c] if kind == "a" else ge[r, c]
        errs.append(abs(g - fd) / max(abs(fd), 1e-12))
        assert abs(g - fd) <= 0.02 * abs(fd), (kind, r, c, g, fd)
    dev.materials(mats)
    assert np.median(errs) < 2e-3


def test_adjoint_matches_central_differences_under_roulette(pt, dev):
    """Roulette from bounce 3, the differentiable configuration's estimator.
    With common random numbers alone its per-sample finite differences are
    flip noise (a decision u > p(theta) changes for a few samples).  The
    nominal render records every survival probability and the renders at
    theta +- eps reuse them (pt_gpu_set_roulette_freeze): the paths are then the
    same and each sample is a smooth function of the parameters, whose gradient
    is what the replay computes (it holds the probabilities fixed too)."""
    W, H, F = 128, 96, 1
    s, head, prm, pk, mats = _scene(pt, 0.5, 8, 3, W, H)
    assert prm.rr_start == 3 and head.max_bounces > 3
    dev.upload(s)
    dev.set_target(W, H)
    rng = np.random.default_rng(12)
    target = rng.uniform(0.0, 0.3, (H, W, 3)).astype(np.float32)
    dev.diff_forward(head, prm, F)
    img = dev.read_accum()[..., :3].astype(np.float64)
    ga, ge = dev.diff_backward((2.0 * (img - target)).astype(np.float32), mats.shape[0])
    dev.render(head, prm, F)
    plain = dev.read_accum().copy()
    dev.set_roulette_freeze(1)
    try:
        dev.render(head, prm, F)                                 # records; the image is unchanged
        assert np.array_equal(dev.read_accum().view(np.uint32), plain.view(np.uint32))
        dev.set_roulette_freeze(2)
        dev.render(head, prm, F)                                 # replays the same probabilities
        assert np.array_equal(dev.read_accum().view(np.uint32), plain.view(np.uint32))

        def loss(m):
            dev.materials(m)
            dev.render(head, prm, F)
            return float(((dev.read_accum()[..., :3].astype(np.float64) - target) ** 2).sum())

        eps = 1e-3
        picks = [("a", int(k)) for k in np.argsort(-np.abs(ga).ravel())[:24]]
        picks += [("e", int(k)) for k in np.argsort(-np.abs(ge).ravel())[:8]]
        errs = []
        for kind, k in picks:
            r, c = divmod(k, 3)
            col = c if kind == "a" else 4 + c
            mp, mm = mats.copy(), mats.copy()
            mp[r, col] += eps
            mm[r, col] -= eps
            fd = (loss(mp) - loss(mm)) / (2 * eps)
            g = ga[r, c] if kind == "a" else ge[r, c]
            errs.append(abs(g - fd) / max(abs(fd), 1e-12))
            assert abs(g - fd) <= 0.02 * abs(fd), (kind, r, c, g, fd)
        assert np.median(errs) < 2e-3
    finally:
        dev.set_roulette_freeze(0)
        dev.materials(mats)


def test_roulette_freeze_state_errors(pt, dev):
    W, H = 32, 24
    s, head, prm, pk, mats = _scene(pt, 0.1, 2, 3, W, H)
    dev.upload(s)
    dev.set_target(W, H)
    dev.set_roulette_freeze(0)
    with pytest.raises(pt.PtError):               # nothing recorded
        dev.set_roulette_freeze(2)
    with pytest.raises(pt.PtError):
        dev.set_roulette_freeze(3)
    try:
        dev.set_roulette_freeze(1)
        dev.render(head, prm, 1)
        dev.set_roulette_freeze(2)
        with pytest.raises(pt.PtError):           # another frame count than recorded
            dev.render(head, prm, 2)
        dev.render(head, prm, 1)
    finally:
        dev.set_roulette_freeze(0)


def test_adjoint_state_and_argument_errors(pt, dev):
    W, H = 32, 32
    s, head, prm, pk, mats = _scene(pt, 0.1, 1, 3, W, H)
    dev.upload(s)
    dev.set_target(W, H)
    dl = np.ones((H, W, 3), np.float32)
    with pytest.raises(pt.PtError):               # no recorded forward after the upload
        dev.diff_backward(dl, mats.shape[0])
    bad = type(prm).from_buffer_copy(prm)
    bad.firefly_clamp = 10.0
    with pytest.raises(pt.PtError):
        dev.diff_forward(head, bad, 1)
    h2 = type(head).from_buffer_copy(head)
    h2.reset_accum = 0
    with pytest.raises(pt.PtError):
        dev.diff_forward(h2, prm, 1)
    dev.diff_forward(head, prm, 1)
    dev.diff_backward(dl, mats.shape[0])
    dev.materials(mats)                            # an upload invalidates the record
    with pytest.raises(pt.PtError):
        dev.diff_backward(dl, mats.shape[0])


def test_batched_adjoint_equals_per_view_adjoints(pt, dev):
    import math
    s = pt.Scene().synth(4, seed=0, scale=0.02)
    s.set_cvar("r_spp", 2)
    pk = s.packed()
    nm = pk.material_count
    scene = pt.Device(0)
    scene.upload(s)
    views = []
    for i, side in enumerate((64, 40, 96)):
        yaw = 2 * math.pi * i / 3
        pos = (60 * math.sin(yaw), 40.0, -60 * math.cos(yaw))
        s.camera(pos, math.atan2(-pos[0], pos[2]), -math.atan2(40.0, 60.0), 50.0)
        head, prm = s.push(side, side, frame_index=100 * i, reset=1)
        views.append((side, side, head, prm))
    rng = np.random.default_rng(5)
    dls = [rng.standard_normal((h, w, 3)).astype(np.float32) for (w, h, _, _) in views]
    batch = pt.Device(0)
    batch.batch_diff_forward(scene, views)
    imgs = [batch.batch_read(i, w, h).copy() for i, (w, h, _, _) in enumerate(views)]
    ga, ge = batch.batch_diff_backward(dls, nm)
    sa, se = np.zeros_like(ga), np.zeros_like(ge)
    for i, (w, h, head, prm) in enumerate(views):
        scene.set_target(w, h)
        scene.diff_forward(head, prm, 1)
        assert np.array_equal(scene.read_accum().view(np.uint32), imgs[i].view(np.uint32))
        a, e = scene.diff_backward(dls[i], nm)
        sa += a
        se += e
    assert np.abs(sa).max() > 0
    np.testing.assert_allclose(ga, sa, rtol=1e-9, atol=1e-12 * np.abs(sa).max())
    np.testing.assert_allclose(ge, se, rtol=1e-9, atol=1e-12 * max(np.abs(se).max(), 1e-30))
    batch.close()
    scene.close()


def test_batch_frames_per_wave_equals_plain_frames(pt, dev):
    """A batched view with frames_per_wave = n accumulates the same n frames as
    a plain n-frame render, bit for bit (and the adjoint of one such view equals
    the plain adjoint of the n frames)."""
    s = pt.Scene().synth(4, seed=0, scale=0.02)
    s.set_cvar("r_spp", 1)
    nm = s.packed().material_count
    scene = pt.Device(0)
    scene.upload(s)
    W, H, n = 72, 40, 4
    head, prm = s.push(W, H, frame_index=77, reset=1)
    batch = pt.Device(0)
    batch.batch_render([scene], [(0, W, H, head, prm, n)], 2)    # 2 waves x 4 frames
    b = batch.batch_read(0, W, H)
    scene.set_target(W, H)
    scene.render(head, prm, 2 * n)
    assert np.array_equal(b.view(np.uint32), scene.read_accum().view(np.uint32))
    dl = np.random.default_rng(2).standard_normal((H, W, 3)).astype(np.float32)
    batch.batch_diff_forward(scene, [(W, H, head, prm, n)])
    ga, ge = batch.batch_diff_backward([dl], nm)
    scene.diff_forward(head, prm, n)
    pa, pe = scene.diff_backward(dl, nm)
    assert np.abs(pa).max() > 0
    np.testing.assert_allclose(ga, pa, rtol=1e-9, atol=1e-12 * np.abs(pa).max())
    batch.close()
    scene.close()


def test_torch_autograd_function_wraps_forward_backward(pt, dev):
    torch = pytest.importorskip("torch")
    W, H = 48, 32
    s, head, prm, pk, mats = _scene(pt, 0.2, 2, 3, W, H)
    dev.upload(s)
    fn = pt.material_render_fn(dev, s, W, H, frames=1)
    albedo = torch.tensor(mats[:, 0:3], dtype=torch.float64, requires_grad=True)
    emission = torch.tensor(mats[:, 4:7], dtype=torch.float64, requires_grad=True)
    img = fn(albedo, emission)
    target = torch.zeros_like(img)
    loss = ((img - target) ** 2).sum()
    loss.backward()
    # the same gradient straight through the C-ABI
    dev.diff_forward(head, prm, 1)
    ref = dev.read_accum()[..., :3]
    assert np.array_equal(ref, img.detach().numpy())
    ga, ge = dev.diff_backward(2.0 * ref, mats.shape[0])
    np.testing.assert_allclose(albedo.grad.numpy(), ga, rtol=1e-12, atol=0)
    np.testing.assert_allclose(emission.grad.numpy(), ge, rtol=1e-12, atol=0)
