"""Regenerates tests/golden/*.npz from the reference's OWN builders
(AnalyticBvh::Build, TriangleBvh::Build, BuildEnvCdf, BuildLightTree), compiled from the
reference sources by `make -C oracle ref` into oracle/_ref.  Run where the
reference tree is present:

    make -C oracle ref && python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))
import oracle  # noqa: E402
from conftest import XorShift32, load_pkg, xorshift_spheres  # noqa: E402

LIGHT_INPUT_DTYPE = load_pkg().LIGHT_INPUT_DTYPE


def tri_soup(n, seed):
    """Random small triangles in [-10, 10]^3 (xorshift32), plus one collinear
    triangle and one with an out-of-range index (the builder must skip it)."""
    rng = XorShift32(seed)
    pos, idx = [], []
    for t in range(n):
        c = [rng.rangef(-10, 10) for _ in range(3)]
        for _ in range(3):
            pos.append([c[k] + rng.rangef(-1, 1) for k in range(3)])
        idx.append([3 * t, 3 * t + 1, 3 * t + 2])
    base = len(pos)
    pos += [[0, 0, 0], [1, 1, 1], [2, 2, 2]]
    idx.append([base, base + 1, base + 2])
    idx.append([0, 1, 10 ** 6])
    return np.array(pos, np.float32), np.array(idx, np.uint32)


def light_inputs(n, seed, coincident=False):
    """Mixed point/spot/sphere/quad lights (xorshift32) with tilted spot and
    quad axes; `coincident`: every light at the same position."""
    rng = XorShift32(seed)
    a = np.zeros(n, LIGHT_INPUT_DTYPE)
    for i in range(n):
        a[i]["type"] = i % 4
        p = [rng.rangef(-10, 10) for _ in range(3)]
        a[i]["pos"] = [1.0, 2.0, 3.0] if coincident else p
        a[i]["radius"] = rng.rangef(0.05, 1.0)
        a[i]["intensity"] = [rng.rangef(0.1, 50) for _ in range(3)]
        d = np.array([rng.rangef(-1, 1), rng.rangef(-1, 0.2), rng.rangef(-1, 1)], np.float64)
        d /= np.linalg.norm(d) + 1e-12
        a[i]["dir"] = d.astype(np.float32)
        a[i]["cos_outer"] = rng.rangef(0.2, 0.95)
        a[i]["u_vec"] = [rng.rangef(-1, 1) for _ in range(3)]
        a[i]["v_half"] = rng.rangef(0.1, 1.5)
    return a


def sdf_clusters(n, seed):
    """Random SDF clusters as SdfNode records (12 words each): single leaves of
    the five bounded shapes and smooth union/subtract/intersect/displace trees."""
    rng = XorShift32(seed)
    out = []
    for c in range(n):
        def leaf():
            shape = int(rng.next() % 5)
            p = [rng.rangef(0.2, 2.0) for _ in range(4)]
            if shape == 2:
                p[3] = rng.rangef(0.0, 0.5)
            node = np.zeros(12, np.float32)
            node[:4].view(np.uint32)[:] = [0, shape, 0, 0]
            node[4:8] = p
            node[8:11] = [rng.rangef(-5, 5) for _ in range(3)]
            return node
        kind = c % 5
        if kind == 0:
            nodes = [leaf()]
        else:
            a, b = leaf(), leaf()
            op = np.zeros(12, np.float32)
            opc = [1, 2, 3, 4][kind - 1]
            op[:4].view(np.uint32)[:] = [opc, 0, 0, 1]
            op[4] = rng.rangef(-0.3, 0.8)
            nodes = [a, b, op]
        arr = np.zeros((8, 12), np.float32)
        arr[:len(nodes)] = nodes
        out.append((arr, len(nodes)))
    return out


def sdf_fractal_clusters(n, seed):
    """Fractal leaves (Mandelbulb 6, Mandelbox 7, Apollonian 8) with bound radii
    that are sometimes non-positive (refused), alone or under a smooth union."""
    rng = XorShift32(seed)
    out = []
    for c in range(n):
        node = np.zeros(12, np.float32)
        node[:4].view(np.uint32)[:] = [0, 6 + c % 3, 0, 0]
        node[4:8] = [rng.rangef(1.0, 9.0), rng.rangef(-0.5, 4.0), 0.0, 0.0]
        node[8:11] = [rng.rangef(-5, 5) for _ in range(3)]
        arr = np.zeros((8, 12), np.float32)
        arr[0] = node
        if c % 4 == 3:      # under a smooth union with a sphere leaf
            arr[1, :4].view(np.uint32)[:] = [0, 0, 0, 0]
            arr[1, 4] = rng.rangef(0.2, 1.5)
            arr[1, 8:11] = [rng.rangef(-5, 5) for _ in range(3)]
            arr[2, :4].view(np.uint32)[:] = [1, 0, 0, 1]
            arr[2, 4] = rng.rangef(0.0, 0.5)
            out.append((arr, 3))
        else:
            out.append((arr, 1))
    return out


def sdf_procedural_clusters(n, seed):
    """A leaf under one procedural op (5 fBm displace, 6 twist, 7 bend,
    8 repeat, 9 limited repeat) with random parameters; the noise octave count
    and the repeat limits are packed into the float words as the reference does."""
    rng = XorShift32(seed)
    out = []
    for c in range(n):
        arr = np.zeros((8, 12), np.float32)
        arr[0, :4].view(np.uint32)[:] = [0, rng.next() % 5, 0, 0]
        arr[0, 4:8] = [rng.rangef(0.2, 2.0) for _ in range(4)]
        arr[0, 8:11] = [rng.rangef(-4, 4) for _ in range(3)]
        op = 5 + c % 5
        arr[1, :4].view(np.uint32)[:] = [op, 0, 0, 0]
        arr[1, 4:8] = [rng.rangef(-0.5, 3.0) for _ in range(4)]
        if op == 5:
            arr[1, 6:7].view(np.uint32)[0] = rng.next() % 9
        if op == 9:
            arr[1, 7:8].view(np.uint32)[0] = (rng.next() % 1024) | ((rng.next() % 1024) << 10) | \
                ((rng.next() % 1024) << 20)
        out.append((arr, 2))
    return out


def main():
    if oracle.load_ref() is None:
        sys.exit("oracle/_ref/libref_builders.so missing: run `make -C oracle ref` first")
    out = {}
    for name, (n, seed) in {"s50": (50, 0xABCDEF01), "s2000": (2000, 0x12345678)}.items():
        cr = xorshift_spheres(n, seed)
        nodes, perm = oracle.ref_analytic_bvh(cr)
        out[f"{name}_cr"], out[f"{name}_nodes"], out[f"{name}_perm"] = cr, nodes, perm
    pos, idx = tri_soup(3000, 0x7A1A5EED)
    nodes, perm = oracle.ref_triangle_bvh(pos, idx)
    out.update(tri_pos=pos, tri_idx=idx, tri_nodes=nodes, tri_perm=perm)
    rng = XorShift32(0xC0FFEE)
    img = np.array([[[rng.rangef(0, 4) for _ in range(3)] for _ in range(32)] for _ in range(16)], np.float32)
    mask = np.zeros((16, 32), np.uint8)
    mask[3:5, 7:10] = 1
    marg, cond, tot = oracle.ref_env_cdf(img)
    margm, condm, totm = oracle.ref_env_cdf(img, mask)
    out.update(env_img=img, env_mask=mask, env_marg=marg, env_cond=cond, env_total=np.float64(tot),
               env_marg_m=margm, env_cond_m=condm, env_total_m=np.float64(totm))
    for name, (n, seed, co) in {"lt1": (1, 5, False), "lt7": (7, 11, False), "lt200": (200, 0x1157, False),
                                "lt16c": (16, 3, True)}.items():
        inp = light_inputs(n, seed, co)
        out[f"{name}_in"], out[f"{name}_nodes"] = inp.view(np.uint8).reshape(n, -1), oracle.ref_light_tree(inp)
    cl = sdf_clusters(60, 0x5DF5EED)
    boxes = []
    for arr, n in cl:
        r = oracle.ref_sdf_aabb(arr, n)
        boxes.append(np.concatenate([r[0], r[1], [1.0]]) if r else np.array([0, 0, 0, 0, 0, 0, 0], np.float32))
    out.update(sdf_nodes=np.stack([a for a, _ in cl]), sdf_counts=np.array([n for _, n in cl], np.uint32),
               sdf_boxes=np.stack(boxes).astype(np.float32))
    cl = sdf_fractal_clusters(24, 0xF4AC7A15)
    boxes = []
    for arr, n in cl:
        r = oracle.ref_sdf_aabb(arr, n)
        boxes.append(np.concatenate([r[0], r[1], [1.0]]) if r else np.array([0, 0, 0, 0, 0, 0, 0], np.float32))
    out.update(sdf_frac_nodes=np.stack([a for a, _ in cl]), sdf_frac_counts=np.array([n for _, n in cl], np.uint32),
               sdf_frac_boxes=np.stack(boxes).astype(np.float32))
    cl = sdf_procedural_clusters(40, 0x9A0CED)
    boxes = []
    for arr, n in cl:
        r = oracle.ref_sdf_aabb(arr, n)
        boxes.append(np.concatenate([r[0], r[1], [1.0]]) if r else np.array([0, 0, 0, 0, 0, 0, 0], np.float32))
    out.update(sdf_proc_nodes=np.stack([a for a, _ in cl]), sdf_proc_counts=np.array([n for _, n in cl], np.uint32),
               sdf_proc_boxes=np.stack(boxes).astype(np.float32))
    np.savez_compressed(os.path.join(HERE, "reference_builders.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_builders.npz"))


if __name__ == "__main__":
    main()
