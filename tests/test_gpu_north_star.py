"""The two correctness criteria of the path as a whole, on the GPU through the
C-ABI.

1. Converged images against the FP64 oracle.  The GPU renders >= 1024 samples
   per pixel; the FP64 instance of the oracle renders the same pixels with the
   same RNG streams (the same frame indices).  The reference's own RMSE is the
   noise floor of its estimator at that sample count: the RMSE between two FP64
   renders of the scene with disjoint RNG streams (frame indices offset by
   2^24), eps_ref.  The GPU image must lie within eps_ref + 1e-3 (RMSE over the
   HDR RGB channels) of the FP64 image.  The GPU's fp32 paths equal the fp32
   oracle's bit for bit; against FP64 they part only where rounding moves a
   decision (a roulette draw, a Fresnel pick), so the GPU-vs-FP64 RMSE sits well
   below eps_ref.

2. Closest-hit ids on the rays a render really traces.  The fp32 oracle
   records the extension rays of bounce 0 and bounce 1 of every sample of
   whole frames (oracle_capture_rays; these are the GPU render's own rays, bit
   for bit), 2^20 rays per case.  Both the reference-order walk of the reference
   BVHs (traversal mode 1) and the 4-wide SAH trees (mode 0, the default) must
   return the oracle's hit ids and distances exactly (the bar is 99.99%).  The
   wide trees' boxes are padded, so they reach hits that the reference's
   unpadded slab test rounds away where a ray grazes a box's edge; the wide
   kernels re-trace such a segment with the reference walk.

3. The whole 256 x 256 analytic workload: 64 frames of 16 spp in one call
   (4.2 M paths, 116 M segments), in the default mode, against the fp32 oracle
   over the same frames: the same segment counts and the same image bit for
   bit.  Two of its primary rays graze box 2's outer edge and are pinned on
   their own."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_RAYS = 1 << 20
SEED_OFFSET = 1 << 24


def rmse(a, b):
    d = a[..., :3].astype(np.float64) - b[..., :3].astype(np.float64)
    return float(np.sqrt((d * d).mean()))


# (configuration, seed, width, height, frames): the plain analytic scene at
# 16 spp x 64 frames, and the triangle+analytic scene (2.46 M triangles, 1,024
# spheres, env map with an extracted sun) at 1 spp x 1024 frames
CONVERGED = [(0, 1, 64, 64, 64), (1, 0, 128, 72, 1024)]


@pytest.mark.parametrize("config,seed,W,H,frames", CONVERGED)
def test_converged_image_matches_the_fp64_oracle(pt, orc, dev, config, seed, W, H, frames):
    s = pt.Scene().synth(config, seed=seed)
    head, prm = s.push(W, H, frame_index=0, reset=1)
    assert max(head.spp, 1) * frames >= 1024
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, frames)
    gpu = dev.read_accum()
    f64, _ = orc.render(s.packed(), head, prm, W, H, frames, fp64=True)
    head_b, _ = s.push(W, H, frame_index=SEED_OFFSET, reset=1)
    f64_b, _ = orc.render(s.packed(), head_b, prm, W, H, frames, fp64=True)
    eps_ref = rmse(f64, f64_b)
    err = rmse(gpu, f64)
    mean = float(f64[..., :3].astype(np.float64).mean())
    print(f"config {config} {W}x{H} {max(head.spp, 1) * frames} spp: GPU vs FP64 RMSE {err:.6g}, "
          f"eps_ref {eps_ref:.6g} (image mean {mean:.6g})")
    assert np.isfinite(gpu).all() and (gpu[..., 3] == frames).all()
    assert err <= eps_ref + 1e-3, (err, eps_ref)


def render_rays(orc, s, W, H, bounce, n, crop=None):
    """n of the rays bounce `bounce` traces over consecutive frames (as many
    frames as it takes to reach n), evenly spaced over them so that they cover
    the whole image."""
    ros, rds, got, f = [], [], 0, 0
    while got < n:
        head, prm = s.push(W, H, frame_index=f, reset=1)
        ro, rd = orc.capture_rays(s.packed(), head, prm, W, H, bounce, crop=crop)
        ros.append(ro)
        rds.append(rd)
        got += len(ro)
        f += 1
    pick = np.linspace(0, got - 1, n).round().astype(np.int64)
    return np.concatenate(ros)[pick], np.concatenate(rds)[pick], head, prm


@pytest.fixture(scope="module")
def scenes(pt):
    return {0: pt.Scene().synth(0, seed=5), 1: pt.Scene().synth(1, seed=0)}


# (configuration, width, height, crop): the plain analytic scene at its
# 256 x 256 x 16 spp, and the full 1920 x 1080 triangle+analytic frame
RAY_CASES = [(0, 256, 256, None), (1, 1920, 1080, None)]


@pytest.mark.parametrize("bounce", [0, 1])
@pytest.mark.parametrize("config,W,H,crop", RAY_CASES)
def test_hit_ids_on_the_rays_a_render_traces(pt, orc, dev, scenes, config, W, H, crop, bounce):
    s = scenes[config]
    ro, rd, head, prm = render_rays(orc, s, W, H, bounce, N_RAYS, crop)
    assert len(ro) == N_RAYS
    o_hit, o_t, _ = orc.trace(s.packed(), head, prm, ro, rd)
    dev.set_traversal(1)
    dev.upload(s)
    r_hit, r_t = dev.trace(ro, rd)
    np.testing.assert_array_equal(r_hit, o_hit)
    np.testing.assert_array_equal(r_t, o_t)
    dev.set_traversal(0)
    dev.upload(s)
    w_hit, w_t = dev.trace(ro, rd)
    agree = w_hit == o_hit
    print(f"config {config} bounce {bounce}: {N_RAYS} rays, {int((o_hit != 0xFFFFFFFF).sum())} hits, "
          f"wide-tree hit-id agreement {agree.mean():.7f} ({int((~agree).sum())} differ)")
    np.testing.assert_array_equal(w_hit, o_hit)
    np.testing.assert_array_equal(w_t, o_t)


# Primary rays of the 256 x 256 analytic scene (seed 0; frames 1 and 58, from
# the camera at (0, 0, 28)) that pass within rounding of box 2's outer edge
# y = -7.6174984: triangle 25 reports a hit (u + v = 1 - 6e-8 and 1 - 2.4e-7),
# but the reference's slab test of the leaf holding it rounds the ray out, so
# the reference walk, and the oracle, report a miss
EDGE_RAYS = np.array([[-0.289293110370636, -0.25726765394210815, -0.9220210909843445, 0.0],
                      [-0.16045163571834564, -0.26527756452560425, -0.9507277011871338, 0.0]], np.float32)


def test_rays_grazing_a_reference_leaf_edge(pt, orc, dev):
    s = pt.Scene().synth(0, seed=0)
    head, prm = s.push(256, 256, frame_index=0, reset=1)
    ro = np.tile(np.array([[0.0, 0.0, 28.0, 0.0]], np.float32), (len(EDGE_RAYS), 1))
    o_hit, o_t, _ = orc.trace(s.packed(), head, prm, ro, EDGE_RAYS)
    assert (o_hit == 0xFFFFFFFF).all()
    for mode in (0, 1):
        dev.set_traversal(mode)
        dev.upload(s)
        hit, t = dev.trace(ro, EDGE_RAYS)
        np.testing.assert_array_equal(hit, o_hit)
        np.testing.assert_array_equal(t, o_t)
    dev.set_traversal(0)


def test_whole_analytic_workload_matches_the_oracle(pt, orc, dev):
    s = pt.Scene().synth(0, seed=0)
    W = H = 256
    frames = 64
    head, prm = s.push(W, H, frame_index=0, reset=1)
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, frames)
    st = dev.stats()
    gpu = dev.read_accum()
    want, c = orc.render(s.packed(), head, prm, W, H, frames)
    print(f"256 x 256 x {head.spp} spp x {frames} frames: GPU {st.extension_rays} + {st.shadow_rays} segments, "
          f"oracle {c.ext_rays} + {c.shadow_rays}")
    assert (st.extension_rays, st.shadow_rays) == (c.ext_rays, c.shadow_rays)
    np.testing.assert_array_equal(gpu, want)
