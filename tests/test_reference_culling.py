"""The reference walk can drop a true hit at a leaf edge (CPU, oracle only).

The reference tests a primitive only after the slab test of every BVH node on
its path passes (shaders/PathTrace.slang:2321-2329, 2592-2636).  Its node boxes
are not padded, so a ray that grazes a box at an edge can have its slab
interval rounded to empty: the reference then never tests the primitives of
that leaf, even where Moller-Trumbore accepts one.  Two primary rays of the
256 x 256 analytic scene (seed 0) do this at box 2's outer edge: every
triangle tested by brute force gives triangle 25, but the reference walk, and
so the fp32 oracle, reports a miss, and the slab test of the leaf holding
triangle 25 rejects both rays.  The GPU's wide trees reproduce that answer
(tests/test_gpu_north_star.py, test_rays_grazing_a_reference_leaf_edge)."""
import numpy as np

from conftest import first_tested_wins

# the camera at (0, 0, 28); frames 1 and 58 of the scene trace these directions
EDGE_RAYS = np.array([[-0.289293110370636, -0.25726765394210815, -0.9220210909843445, 0.0],
                      [-0.16045163571834564, -0.26527756452560425, -0.9507277011871338, 0.0]], np.float32)
TRIANGLE = 25


def reference_slab(node, ro, rd):
    """The reference's slab test of one node (float32, its operation order),
    with an unbounded best distance."""
    f = np.float32
    lo = node[0:3].view(np.float32)
    hi = node[4:7].view(np.float32)
    inv = np.array([f(1.0) / (d if abs(d) > f(1e-30) else f(1e-30)) for d in rd[:3]], np.float32)
    t0 = ((lo - ro[:3]).astype(f) * inv).astype(f)
    t1 = ((hi - ro[:3]).astype(f) * inv).astype(f)
    tmin = max(max(min(t0[0], t1[0]), min(t0[1], t1[1])), min(t0[2], t1[2]))
    tmax = min(min(max(t0[0], t1[0]), max(t0[1], t1[1])), max(t0[2], t1[2]))
    return bool(tmax >= max(tmin, f(0.0)))


def test_reference_walk_drops_a_true_hit_at_a_leaf_edge(pt, orc):
    s = pt.Scene().synth(0, seed=0)
    head, prm = s.push(256, 256, frame_index=0, reset=1)
    ro = np.tile(np.array([[0.0, 0.0, 28.0, 0.0]], np.float32), (len(EDGE_RAYS), 1))
    o_hit, _, _ = orc.trace(s.packed(), head, prm, ro, EDGE_RAYS)
    assert (o_hit == 0xFFFFFFFF).all()

    arrays = s.arrays()
    bf_hit, bf_t = first_tested_wins(arrays, ro, EDGE_RAYS)
    assert (bf_hit == ((1 << 30) | TRIANGLE)).all()
    assert (bf_t > 28.0).all() and (bf_t < 30.0).all()

    # the reference triangle BVH leaf whose slot range holds triangle 25
    nodes, perm = arrays["tri_bvh"], arrays["tri_perm"]
    slot = int(np.flatnonzero(perm == TRIANGLE)[0])
    leaves = [i for i, n in enumerate(nodes) if n[7] > 0 and n[3] <= slot < n[3] + n[7]]
    assert len(leaves) == 1
    for r in range(len(EDGE_RAYS)):
        assert not reference_slab(nodes[leaves[0]], ro[r], EDGE_RAYS[r])
