"""The reference's golden-image cells rendered on the GPU through the C-ABI
(pt_gpu_render for 64 frames, then pt_gpu_tonemap), on the committed fixture
(tests/reference_cells.py): the HDR accumulation and the 8-bit image must equal
the fp32 oracle's bit for bit, and the GPU image itself must pass the cell's
imgdiff thresholds against the reference's golden PNG."""
import numpy as np
import pytest

from reference_cells import FRAMES, cells, load_cell, passes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scene", cells())
def test_gpu_passes_the_reference_golden_cell(pt, orc, dev, scene, tmp_path):
    s, gold, thr = load_cell(pt, scene, str(tmp_path))
    W, H = int(s.get_cvar("app_window_width")), int(s.get_cvar("app_window_height"))
    head, prm = s.push(W, H, 0, 1)
    exposure, op = s.get_cvar("r_exposure"), int(s.get_cvar("r_tonemap_op"))
    dev.set_traversal(0)
    dev.upload(s)
    dev.set_target(W, H)
    dev.render(head, prm, FRAMES)
    g_acc = dev.read_accum()
    g_img = dev.tonemap(exposure, op, True)
    o_acc, _ = orc.render(s.packed(), head, prm, W, H, FRAMES)
    o_img = orc.tonemap(o_acc, exposure, op, True)
    np.testing.assert_array_equal(g_acc, o_acc)
    np.testing.assert_array_equal(g_img, o_img)
    assert gold.shape == g_img.shape
    ok, st = passes(pt, g_img, gold, thr)
    print(f"{scene}: GPU vs golden mean {st.mean_delta:.3f} max {st.max_delta:.1f} "
          f"over-threshold {st.bad_percent:.3f}%")
    assert ok, (st.mean_delta, st.bad_percent, st.max_delta)
