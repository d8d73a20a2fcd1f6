"""Edge cases of the render call against the oracle: an empty scene (sky only),
images of one pixel and of ragged sizes that are not multiples of a warp or a
block, zero and one bounce, several samples per pixel, the exponential moving
average accumulation, and an accumulation resumed across calls of different
frame counts.  Every case is bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _render_both(dev, orc, s, W, H, frames=1, frame_index=0, reset=1, tweak=None):
    head, prm = s.push(W, H, frame_index=frame_index, reset=reset)
    if tweak:
        tweak(head, prm)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, frames)
    g = dev.read_accum()
    o, _ = orc.render(s.packed(), head, prm, W, H, frames)
    return g, o


def test_empty_scene_renders_the_sky(pt, orc, dev):
    s = pt.Scene()
    env = np.zeros((8, 16, 3), np.float32)
    env[..., 0], env[..., 1], env[..., 2] = 0.25, 0.5, 1.0
    s.env(env)
    g, o = _render_both(dev, orc, s, 24, 16)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
    np.testing.assert_allclose(g[..., :3], np.broadcast_to([0.25, 0.5, 1.0], (16, 24, 3)), rtol=1e-6)
    assert (g[..., 3] == 1.0).all()


def test_empty_scene_without_a_sky_is_black(pt, orc, dev):
    s = pt.Scene()
    s.env(np.zeros((2, 4, 3), np.float32))
    g, o = _render_both(dev, orc, s, 5, 3)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
    assert (g[..., :3] == 0).all()


@pytest.mark.parametrize("W,H", [(1, 1), (1, 37), (33, 7), (257, 3), (31, 33)])
def test_ragged_image_sizes(pt, orc, dev, W, H):
    s = pt.Scene().synth(0, seed=3)
    g, o = _render_both(dev, orc, s, W, H, frames=2, frame_index=5)
    assert g.shape == (H, W, 4)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


@pytest.mark.parametrize("bounces,spp", [(0, 1), (1, 1), (1, 3), (3, 5)])
def test_bounce_and_sample_counts(pt, orc, dev, bounces, spp):
    s = pt.Scene().synth(0, seed=1)

    def tweak(head, prm):
        head.max_bounces = bounces
        head.spp = spp

    g, o = _render_both(dev, orc, s, 40, 24, frame_index=7, tweak=tweak)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
    if bounces == 0:        # the bounce loop runs max_bounces times: nothing is traced
        assert (g[..., :3] == 0).all() and (g[..., 3] == 1).all()
    else:
        assert g[..., :3].mean() > 0.0


def test_ema_accumulation(pt, orc, dev):
    s = pt.Scene().synth(0, seed=2)

    def tweak(head, prm):
        prm.accum_ema_alpha = 0.25

    g, o = _render_both(dev, orc, s, 32, 20, frames=4, frame_index=11, tweak=tweak)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


def test_accumulation_resumed_in_uneven_calls(pt, orc, dev):
    """3 + 1 + 2 frames in three calls equal 6 frames in one call (frame
    indices advancing, no reset after the first call)."""
    s = pt.Scene().synth(0, seed=4)
    W, H = 20, 12
    dev.upload(s)
    dev.set_target(W, H)
    fi = 30
    for k, n in enumerate((3, 1, 2)):
        head, prm = s.push(W, H, frame_index=fi, reset=1 if k == 0 else 0)
        dev.render(head, prm, n)
        fi += n
    g = dev.read_accum()
    head, prm = s.push(W, H, frame_index=30, reset=1)
    o, _ = orc.render(s.packed(), head, prm, W, H, 6)
    assert (g[..., 3] == 6).all()
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


def test_stage_schedules_and_profiling_modes_give_the_same_image(pt, dev):
    """The overlapped schedule (next bounce's closest hits beside this bounce's
    shadow rays), the same with events, the serial schedule and the serial
    schedule with the counting traversal variants agree bit for bit; the event
    modes report kernel times; the counting mode's segment counts equal the
    render's own; other modes are refused."""
    s = pt.Scene().synth(1, seed=2, scale=0.02)
    W, H = 64, 40
    head, prm = s.push(W, H, frame_index=3, reset=1)
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    out = []
    for mode in (0, 1, 2, 3):
        dev.set_profiling(mode)
        dev.render(head, prm, 3)
        out.append(dev.read_accum().copy())
        st = dev.stats()
        assert (st.extend_ms > 0 and st.shadow_ms > 0) == (mode != 0)
    t = dev.traversal_stats()
    dev.set_profiling(0)
    for k in (1, 2, 3):
        assert np.array_equal(out[0].view(np.uint32), out[k].view(np.uint32))
    assert t.ext_segments == st.extension_rays and t.shadow_segments == st.shadow_rays
    assert t.ext_nodes > t.ext_segments and t.ext_tris > 0 and t.ext_aprims > 0
    # every node tested was popped; every entry pushed (plus each walk's root) is popped once
    assert t.ext_pop >= t.ext_nodes and t.ext_push <= t.ext_pop
    assert t.shadow_nodes > 0 and t.shadow_pop >= t.shadow_nodes
    with pytest.raises(pt.PtError):
        dev.set_profiling(4)


def test_denoiser_jitter_on_sample_zero(pt, orc, dev):
    """With the denoiser on, sample 0 of a frame takes the push's sub-pixel
    jitter instead of two random numbers (shaders/PathTrace.slang:5729-5736);
    the engine pushes Halton(2,3) of frame_index % 16 + 1, minus 0.5, each
    frame.  A three-frame call equals three single-frame calls with the
    engine's pushes and the oracle, bit for bit, and a caller's own jitter is
    honoured for a single frame."""
    s = pt.Scene().synth(0, seed=7)
    s.set_cvar("r_denoiser", 1)
    s.set_cvar("r_spp", 2)
    W, H = 40, 24
    head, prm = s.push(W, H, frame_index=5, reset=1)
    assert head.denoiser_enabled == 1 and head.halton_jitter[0] != 0.0
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, 3)
    g = dev.read_accum().copy()
    o, _ = orc.render(s.packed(), head, prm, W, H, 3)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
    for k in range(3):
        h, p = s.push(W, H, frame_index=5 + k, reset=int(k == 0))
        dev.render(h, p, 1)
    assert np.array_equal(dev.read_accum().view(np.uint32), g.view(np.uint32))
    mine = type(head).from_buffer_copy(head)
    mine.halton_jitter[0], mine.halton_jitter[1] = 0.25, -0.125
    dev.render(mine, prm, 1)
    g1 = dev.read_accum().copy()
    o1, _ = orc.render(s.packed(), mine, prm, W, H, 1)
    assert np.array_equal(g1.view(np.uint32), o1.view(np.uint32))
    dev.render(head, prm, 1)
    assert not np.array_equal(g1, dev.read_accum())


def _env_scene(pt):
    """The plain analytic scene under a 64 x 32 environment with a dark band
    (flat stretches in every row's CDF) and a small bright patch (a jump)."""
    s = pt.Scene().synth(0, seed=2)
    rng = np.random.default_rng(7)
    env = rng.uniform(0.0, 0.4, (32, 64, 3)).astype(np.float32)
    env[:, 20:30] = 0.0
    env[5:7, 40:42] = 500.0
    s.env(env)
    return s


def test_env_sampling_with_guide_tables(pt, orc, dev):
    """Env samples through the CDF guide tables pick the texels the full binary
    search picks: the render equals the oracle's bit for bit."""
    s = _env_scene(pt)
    g, o = _render_both(dev, orc, s, 48, 40, frames=3, frame_index=11)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


def test_env_sampling_of_an_unsorted_cdf_takes_the_full_search(pt, orc, dev):
    """A conditional row that is not non-decreasing gets no guide table; the
    full binary search then gives the oracle's texels on the same arrays."""
    import ctypes
    s = _env_scene(pt)
    W, H = 48, 40
    head, prm = s.push(W, H, frame_index=3, reset=1)
    p = s.packed()
    ew, eh = p.env_w, p.env_h
    rgba = np.ctypeslib.as_array(p.env_rgba, (eh * ew * 4,)).copy()
    marg = np.ctypeslib.as_array(p.env_marginal, (eh,)).copy()
    cond = np.ctypeslib.as_array(p.env_conditional, (eh * ew,)).copy().reshape(eh, ew)
    row = int(np.argmax(np.diff(marg, prepend=0.0)))   # the likeliest row
    cond[row, 10], cond[row, 40] = cond[row, 40], cond[row, 10]
    assert (np.diff(cond[row]) < 0).any()
    cond = np.ascontiguousarray(cond.ravel())
    hd = np.ctypeslib.as_array(p.hdri_dir_pmf, (32,)).copy()
    hc = np.ctypeslib.as_array(p.hdri_col, (32,)).copy()
    fp = pt.fptr
    dev.upload(s)
    assert dev.lib.pt_gpu_upload_env(dev.h, fp(rgba), ew, eh, fp(marg), fp(cond), fp(hd), fp(hc),
                                     p.hdri_count) == 0
    dev.set_target(W, H)
    dev.render(head, prm, 2)
    g = dev.read_accum()
    p.env_conditional = cond.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    o, _ = orc.render(p, head, prm, W, H, 2)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
