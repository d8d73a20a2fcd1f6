"""The reference's own image goldens, for the cells whose estimator is this
path's (tests/reference_cells.py describes the cells and the fixture).  Here
the fp32 oracle renders each fixture for 64 frames and its tone map makes the
8-bit image, which must pass the reference's imgdiff thresholds against the
golden PNG.  tests/test_gpu_reference_cells.py renders the same cells on the
GPU, bit for bit equal to these oracle images."""
import pytest

from conftest import load_pkg
from reference_cells import FRAMES, cells, load_cell, passes


@pytest.mark.parametrize("scene", cells())
def test_oracle_passes_the_reference_golden_cell(orc, scene, tmp_path):
    pt = load_pkg()
    s, gold, thr = load_cell(pt, scene, str(tmp_path))
    W, H = int(s.get_cvar("app_window_width")), int(s.get_cvar("app_window_height"))
    head, prm = s.push(W, H, 0, 1)
    acc, _ = orc.render(s.packed(), head, prm, W, H, FRAMES)
    img = orc.tonemap(acc, s.get_cvar("r_exposure"), int(s.get_cvar("r_tonemap_op")), True)
    assert gold.shape == img.shape
    ok, st = passes(pt, img, gold, thr)
    assert ok, (st.mean_delta, st.bad_percent, st.max_delta)
