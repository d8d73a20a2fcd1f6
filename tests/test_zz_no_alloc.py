"""The allocation-free render entry point (pt_gpu_render_noalloc) against the
ordinary one (pt_gpu_render), through the C-ABI.

pt_gpu_render_noalloc exists for callers that must not allocate device memory
while they render (a fixed device-memory budget reserved up front, a frame loop
that cannot take the implicit synchronisation of cudaMalloc/cudaFree, a host
application that accounts for every device byte): its path state lives in a
fixed array inside the library and the caller supplies the accumulation buffer.
Here the caller-side buffer comes from torch; the entry point itself allocates
nothing.  Two calls in a row must reproduce the ordinary entry point's running
mean exactly (the same tolerance as the other GPU parity tests: bit-exact), and
frames above the stated pixel limit are refused with a clear error.  This file
is collected last and passes alone in a fresh process or after the others."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(pt, dev, head, prm, W, H, frames, buf):
    return pt.load().pt_gpu_render_noalloc(dev.h, ctypes.byref(head), ctypes.byref(prm), W, H, frames,
                                           ctypes.c_void_p(buf.data_ptr()))


# (config, W, H, frames per call): the first two fit one wave of the fixed
# path-state array (65,536 paths); 256 x 256 x 3 frames runs three waves of one
# frame each and 200 x 150 x 5 frames three waves of 2, 2 and 1 frames, so the
# wave loop (frame index offsets, reset on the first wave only) is exercised
@pytest.mark.parametrize("config,W,H,frames", [(0, 64, 48, 2), (1, 96, 54, 2), (0, 256, 256, 3),
                                               (1, 200, 150, 5)])
def test_render_noalloc_matches_render_on_two_calls(pt, dev, config, W, H, frames):
    import torch
    s = pt.Scene().synth(config, seed=21, scale=1.0 if config == 0 else 0.02)
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    head1, prm1 = s.push(W, H, frame_index=4, reset=1)
    head2, prm2 = s.push(W, H, frame_index=4 + frames, reset=0)
    dev.render(head1, prm1, frames)
    want1 = dev.read_accum().copy()
    dev.render(head2, prm2, frames)
    want2 = dev.read_accum().copy()

    buf = torch.full((H, W, 4), float("nan"), dtype=torch.float32, device="cuda")
    assert _noalloc(pt, dev, head1, prm1, W, H, frames, buf) == 0, pt.load().pt_gpu_last_error(dev.h)
    torch.cuda.synchronize()
    got1 = buf.cpu().numpy()
    np.testing.assert_array_equal(got1, want1)
    assert _noalloc(pt, dev, head2, prm2, W, H, frames, buf) == 0, pt.load().pt_gpu_last_error(dev.h)
    torch.cuda.synchronize()
    got2 = buf.cpu().numpy()
    np.testing.assert_array_equal(got2, want2)
    assert (got2[..., 3] == 2 * frames).all()


def test_render_noalloc_rejects_frames_above_the_limit(pt, dev):
    import torch
    s = pt.Scene().synth(0, seed=22)
    dev.upload(s)
    W, H = 512, 256
    head, prm = s.push(W, H, 0, 1)
    buf = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    assert _noalloc(pt, dev, head, prm, W, H, 1, buf) == -1
    assert b"exceed the static scratch limit" in pt.load().pt_gpu_last_error(dev.h)
