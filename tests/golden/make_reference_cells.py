"""Regenerates tests/golden/reference_cells.npz: the inputs and golden images of
the reference's golden-image cells whose estimator is this library's path, so
that they can be rendered where the reference tree is absent (the GPU host).

For each cell the fixture holds, byte for byte as the reference ships them:
  * cfg_<scene>:  the scene fixture tests/goldens/scenes/<scene>.cfg;
  * png_<scene>:  the golden tests/goldens/Darwin/<scene>__metal__off.png;
  * thr_<scene>:  the cell's imgdiff thresholds (MAX_DELTA, MEAN_DELTA,
                  FAIL_PERCENT) as registered in tests/CMakeLists.txt:499-1000;
and, once for all cells, the Radiance .hdr environment maps the engine loads:
  * hdr_sunset:        assets/hdri/sunset.hdr (the engine's startup env map);
  * hdr_uniform_gray:  assets/hdri/uniform_gray.hdr (env_glass_furnace's).

Run where the reference tree is present:

    python tests/golden/make_reference_cells.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle  # noqa: E402

# scene: (MAX_DELTA, MEAN_DELTA, FAIL_PERCENT) of its metal/off golden cell
CELLS = {
    "env_glass_furnace": (16.0, 2.0, 1.0),
    "light_tree_200_pts": (32.0, 4.0, 2.0),
    "sdf_smin_row": (32.0, 4.0, 2.0),
    "sdf_fractals": (32.0, 4.0, 2.0),
}
HDRS = {"sunset": "sunset.hdr", "uniform_gray": "uniform_gray.hdr"}


def main():
    ref = oracle.REF_TREE
    if ref is None:
        sys.exit("the reference tree is not present here")
    out = {}
    for scene, thr in CELLS.items():
        cfg = os.path.join(ref, "tests", "goldens", "scenes", scene + ".cfg")
        png = os.path.join(ref, "tests", "goldens", "Darwin", scene + "__metal__off.png")
        out["cfg_" + scene] = np.frombuffer(open(cfg, "rb").read(), np.uint8)
        out["png_" + scene] = np.frombuffer(open(png, "rb").read(), np.uint8)
        out["thr_" + scene] = np.array(thr, np.float64)
    for key, name in HDRS.items():
        out["hdr_" + key] = np.frombuffer(open(os.path.join(ref, "assets", "hdri", name), "rb").read(), np.uint8)
    path = os.path.join(HERE, "reference_cells.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
