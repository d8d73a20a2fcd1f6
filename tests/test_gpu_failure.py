"""Failure paths of the device code, exercised without faulting the GPU.

The traversal kernels bound every walk: a per-query loop-iteration cap and, on
the 4-wide trees, a stack of at most 64 entries.  A query that runs into
either limit ends with the best hit found so far, sets the context's error
word and the call returns PT_ERR_KERNEL naming the limit; the context stays
usable.  pt_gpu_set_debug_limits lowers both limits so that an ordinary scene
reaches them.

The accumulation sanitises what a frame produces, as the reference's
accumulate does (shaders/PathTrace.slang:7707-7734): a NaN or infinite frame
channel becomes 0, a negative one is raised to 0, and a previous accumulation
texel holding NaN or Inf restarts the running mean.  These cases are checked
bit for bit against the oracle, which restates those lines."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def limits(dev):
    yield dev
    dev.set_debug_limits(0, 0)


def _bit_exact(a, b):
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_iteration_cap_reports_and_the_context_recovers(pt, orc, dev, limits):
    s = pt.Scene().synth(1, seed=2, scale=0.02)
    W, H = 48, 32
    head, prm = s.push(W, H, frame_index=1, reset=1)
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    dev.set_debug_limits(4, 0)
    with pytest.raises(pt.PtError) as e:
        dev.render(head, prm, 1)
    assert e.value.code == -5 and "iteration cap" in str(e.value)
    dev.set_debug_limits(0, 0)
    dev.render(head, prm, 1)
    o, _ = orc.render(s.packed(), head, prm, W, H, 1)
    assert _bit_exact(dev.read_accum(), o)


def test_stack_limit_reports_and_the_context_recovers(pt, orc, dev, limits):
    s = pt.Scene().synth(1, seed=2, scale=0.02)
    W, H = 48, 32
    head, prm = s.push(W, H, frame_index=1, reset=1)
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    dev.set_debug_limits(0, 4)
    with pytest.raises(pt.PtError) as e:
        dev.render(head, prm, 1)
    assert e.value.code == -5 and "stack overflow" in str(e.value)
    dev.set_debug_limits(0, 0)
    dev.render(head, prm, 1)
    o, _ = orc.render(s.packed(), head, prm, W, H, 1)
    assert _bit_exact(dev.read_accum(), o)


def test_trace_probe_reports_the_iteration_cap(pt, dev, limits):
    s = pt.Scene().synth(0, seed=3)
    dev.set_traversal(0)
    dev.upload(s)
    ro = np.zeros((64, 4), np.float32)
    rd = np.zeros((64, 4), np.float32)
    ro[:, :3] = (0.0, 0.0, 28.0)
    rd[:, 2] = -1.0
    dev.set_debug_limits(2, 0)
    with pytest.raises(pt.PtError) as e:
        dev.trace(ro, rd)
    assert "iteration cap" in str(e.value)
    dev.set_debug_limits(0, 0)
    dev.trace(ro, rd)


def test_debug_limits_are_validated(pt, dev, limits):
    for stack in (1, 3, 65):
        with pytest.raises(pt.PtError):
            dev.set_debug_limits(0, stack)


def test_nan_inf_and_negative_emission_are_sanitised(pt, orc, dev):
    """An emitter whose radiance is (NaN, -5, +Inf): the frame's NaN and Inf
    channels become 0 and its negative channel is raised to 0."""
    s = pt.Scene()
    s.env(np.full((4, 8, 3), 0.2, np.float32))
    s.plane(1, (0.0, 1.0, 0.0), 1.0, 0, (0.6, 0.6, 0.6))              # Lambert floor
    s.sphere(10, 0.0, 0.0, -4.0, 1.0, 0, (0.8, 0.8, 0.8))
    s.emission(10, (float("nan"), -5.0, float("inf")))
    s.sphere(11, 2.2, 0.0, -4.0, 0.8, 0, (0.5, 0.7, 0.9))
    s.camera((0.0, 0.5, 2.0), 0.0, np.radians(-5.0), 55.0)
    W, H = 40, 30
    head, prm = s.push(W, H, frame_index=2, reset=1)
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, 2)
    g = dev.read_accum()
    o, _ = orc.render(s.packed(), head, prm, W, H, 2)
    assert _bit_exact(g, o)
    assert np.isfinite(g).all() and (g[..., :3] >= 0).all()
    # the camera sees the emitter: its pixels are 0 in the NaN and Inf channels
    seen = g[H // 2, W // 2]
    assert seen[0] == 0.0 and seen[2] == 0.0


def test_nan_inf_and_negative_env_texels_are_sanitised(pt, orc, dev):
    s = pt.Scene()
    env = np.full((16, 32, 3), 0.5, np.float32)
    env[4:12, 0:16, 0] = np.nan
    env[4:12, 16:32, 1] = np.inf
    env[0:4, :, 2] = -1.0
    s.env(env)
    W, H = 32, 24
    head, prm = s.push(W, H, frame_index=0, reset=1)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, 1)
    g = dev.read_accum()
    o, _ = orc.render(s.packed(), head, prm, W, H, 1)
    assert _bit_exact(g, o)
    assert np.isfinite(g).all() and (g[..., :3] >= 0).all()


def test_bad_previous_accumulation_restarts_the_mean(pt, orc, dev):
    s = pt.Scene().synth(0, seed=6)
    W, H = 24, 16
    dev.upload(s)
    dev.set_target(W, H)
    prev = np.full((H, W, 4), 0.25, np.float32)
    prev[..., 3] = 3.0
    prev[2, 3, 0] = np.nan
    prev[5, 7, 3] = np.inf
    prev[9, 11, 1] = -np.inf
    dev.write_accum(prev)
    head, prm = s.push(W, H, frame_index=40, reset=0)
    dev.render(head, prm, 2)
    g = dev.read_accum()
    o, _ = orc.render(s.packed(), head, prm, W, H, 2, accum=prev.copy())
    assert _bit_exact(g, o)
    assert g[2, 3, 3] == 2.0 and g[5, 7, 3] == 2.0 and g[9, 11, 3] == 2.0
    assert g[0, 0, 3] == 5.0
