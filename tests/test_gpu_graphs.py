"""CUDA-graph replay of the render waves (pt_gpu_set_render_graphs, off by
default).  A wave's launches are captured once and replayed by later calls with
the same launch parameters; the frame index and the accumulation reset are read
on the device, so a frame loop that advances frame_index replays one graph.
Every image here is compared bit for bit: with the oracle, and with the same
calls launched kernel by kernel."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(dev, s, W, H, frames, frame_index, reset, tweak=None):
    head, prm = s.push(W, H, frame_index=frame_index, reset=reset)
    if tweak:
        tweak(head, prm)
    dev.render(head, prm, frames)
    return head, prm, dev.stats()


@pytest.mark.parametrize("graphs", [True, False])
def test_frame_loop_replays_one_graph(pt, orc, dev, graphs):
    """An engine-style loop: 2 frames per call, frame_index advancing, reset on
    the first call only.  With graphs the first call captures and the others
    replay; the accumulation equals the oracle's over the same calls."""
    s = pt.Scene().synth(0, seed=2)
    W, H, nf, calls = 48, 40, 2, 4
    dev.set_render_graphs(graphs)
    dev.upload(s)
    dev.set_target(W, H)
    acc = np.zeros((H, W, 4), np.float32)
    replays = []
    try:
        for c in range(calls):
            head, prm, st = _call(dev, s, W, H, nf, 100 + nf * c, int(c == 0))
            replays.append(st.graph_replays)
            acc, _ = orc.render(s.packed(), head, prm, W, H, nf, accum=acc)
            g = dev.read_accum()
            assert np.array_equal(g.view(np.uint32), acc.view(np.uint32)), f"call {c}"
    finally:
        dev.set_render_graphs(False)
    assert replays == ([0, 1, 1, 1] if graphs else [0, 0, 0, 0])


def test_changed_calls_are_not_replayed_stale(pt, orc, dev):
    """Calls that change what the launches depend on (the camera, the bounce
    count and so the node list, the samples, the scene) each render their own
    image; a repeat of the last call replays its graph.  (A re-uploaded scene
    may land on the same device addresses, and then its launches are the same
    bytes as before: a replay there is correct too, so only the calls whose
    view or shape changed are required to capture.)"""
    s0 = pt.Scene().synth(0, seed=4)
    s1 = pt.Scene().synth(0, seed=9)
    W, H = 37, 29

    def cam(head, prm):
        head.pos_fovtan[0] += 0.25

    def depth(head, prm):
        head.max_bounces = 2

    def spp(head, prm):
        head.spp = 3

    steps = [(s0, None), (s0, cam), (s0, depth), (s0, spp), (s1, None), (s0, None), (s0, None)]
    dev.set_target(W, H)
    dev.set_render_graphs(True)
    replays = []
    current = None
    try:
        for i, (s, tweak) in enumerate(steps):
            if s is not current:
                dev.upload(s)
                current = s
            head, prm, st = _call(dev, s, W, H, 1, 3, 1, tweak)
            replays.append(st.graph_replays)
            o, _ = orc.render(s.packed(), head, prm, W, H, 1)
            g = dev.read_accum()
            assert np.array_equal(g.view(np.uint32), o.view(np.uint32)), f"step {i}"
    finally:
        dev.set_render_graphs(False)
    assert replays[1:4] == [0, 0, 0] and replays[-1] == 1, replays


def test_two_wave_call_matches_direct_launches(pt, dev):
    """2048 x 1024 at 1 spp: 32 frames fit one wave of path state, so 34 frames
    run two waves (the second of 2 frames, without the reset).  Graph replay,
    first capture and direct launches give the same image; a later call with
    an advanced frame index replays both waves."""
    s = pt.Scene().synth(0, seed=6)
    W, H = 2048, 1024

    def one_spp(head, prm):
        head.spp = 1

    dev.upload(s)
    dev.set_target(W, H)
    imgs = {}
    try:
        for graphs in (False, True):
            dev.set_render_graphs(graphs)
            _call(dev, s, W, H, 34, 0, 1, one_spp)
            _, _, st = _call(dev, s, W, H, 34, 34, 0, one_spp)
            assert st.waves == 2
            assert st.graph_replays == (2 if graphs else 0)
            imgs[graphs] = dev.read_accum()
    finally:
        dev.set_render_graphs(False)
    assert np.array_equal(imgs[True].view(np.uint32), imgs[False].view(np.uint32))
    assert (imgs[True][..., 3] == 68).all()
