#!/usr/bin/env python3
"""Benchmark: ray segments per second of the GB300 path-trace hot path.

Workload (the triangle+analytic configuration): 1920x1080, 1 spp x 64
accumulated frames, max depth 8; 200 displaced geodesic icospheres (9,680 tris
each) on a 512x512 quad-grid ground (2,460,288 triangles), 1,024 analytic
spheres, 2048x1024 log-normal env map with a 0.5 deg sun disc of 1e4 (extracted
as an HDRI light), 256 materials.  Seeded synthetic data of those shapes.

One step = the 64-frame accumulation (reset on the first frame).  `value` =
(extension + shadow segments) / device time of the K timed steps, inputs
resident in HBM.  `e2e` = the same through pt_gpu_render_to_host: per-frame
push data in from the host and the RGBA32F accumulation buffer copied back to
pinned host memory inside the timed region.  The scene buffers (~350 MB) stay
resident across steps, as they do across frames in the reference engine.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""
import argparse
import ctypes
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "demont-engine_gb300")
METRIC = "Mrays/s (ray segments: extension + shadow)"
W_FULL, H_FULL, FRAMES = 1920, 1080, 64


def load_pkg():
    spec = importlib.util.spec_from_file_location("demont_gb300", os.path.join(PKG, "__init__.py"),
                                                  submodule_search_locations=[PKG])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["demont_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def replica_frame_index(rank):
    """Replicas render disjoint frame ranges of the same workload (independent seeds)."""
    return rank * 1_000_000


def reduce_replicas(dist, times, counts, device):
    """Whole-job figures over the ranks: the max of each timing (the job ends
    with its slowest replica) and the sum of each count."""
    import torch
    tt = torch.tensor(times, dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    cc = torch.tensor(counts, dtype=torch.float64, device=device)
    dist.all_reduce(cc, op=dist.ReduceOp.SUM)
    return tt.tolist(), cc.tolist()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms (read-only)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def shade_bytes_per_vertex(scene):
    """Algorithmic bytes the shading stage reads per path vertex of this
    workload, on the reference's data layouts: a material row (3 float4, 48 B);
    at a Lambert hit, the environment NEE (one 16-B texel and one 4-B load per
    step of the two CDF binary searches) and the HDRI-cluster pick (a direction
    + pmf and a colour float4, 32 B); at a miss, the bilinear sky lookup (four
    16-B texels) and the MIS pdf texel (16 B).  No analytic lights in this
    workload.  cdf_search_guided_B: what the two searches read with this
    library's CDF guide tables (an 8-B bracket per search, then about
    log2(n / 256) + 1 steps)."""
    import math
    a = scene.arrays()
    h, w = a["env_conditional"].shape
    search = 4 * (math.ceil(math.log2(h)) + math.ceil(math.log2(w)))
    guided = sum(8 + 4 * (math.ceil(math.log2(max(n / 256, 1))) + 1) for n in (h, w))
    lambert = 48 + 16 + search + (32 if a["hdri_count"] else 0)
    miss = 4 * 16 + 16
    hdri = " + HDRI pick 32" if a["hdri_count"] else ""
    return {"lambert_hit": lambert, "miss": miss, "unit": "B", "cdf_search_guided_B": guided,
            "terms": f"material 48 + env texel 16 + CDF searches {search}{hdri}; "
                     f"miss: 4 bilinear texels 64 + pdf texel 16"}


# bytes one closest-hit query moves on the structures it walks (the 4-wide
# trees): queue entry 4 + ray origin and direction 2 x 16 in, hit t and id 2 x 4
# out; per wide node tested its six box planes and four child codes (7 x 16, the
# last 16 bytes of the 128-byte node are not loaded); per triangle 3 x 16; per
# analytic primitive in a leaf 16 (geometry) + 16 (id, type, tie key); per plane
# record tested linearly 16 + 4; per traversal-stack push or pop 8.
RAY_IO_BYTES = 4 + 32 + 8
NODE_BYTES, TRI_BYTES, APRIM_BYTES, LINEAR_BYTES, STACK_BYTES = 112, 48, 32, 20, 8


def traversed_bytes(t, kind):
    """Bytes per segment on the traversed structures from the counting pass's
    PtTraversalStats: (total, terms)."""
    g = lambda f: getattr(t, f"{kind}_{f}")
    n = max(g("segments"), 1)
    terms = {"ray_and_hit": float(RAY_IO_BYTES),
             "nodes": NODE_BYTES * g("nodes") / n,
             "triangles": TRI_BYTES * g("tris") / n,
             "analytic_prims": APRIM_BYTES * g("aprims") / n + LINEAR_BYTES * g("linear") / n,
             "stack": STACK_BYTES * (g("push") + g("pop")) / n}
    per = {"nodes": g("nodes") / n, "triangles": g("tris") / n, "analytic_prims": g("aprims") / n,
           "linear_prims": g("linear") / n, "stack_push": g("push") / n, "stack_pop": g("pop") / n}
    return sum(terms.values()), terms, per


def algorithmic_bytes(pt, orc, scene, head, prm):
    """Bytes per extension segment on the REFERENCE's binary structures (for
    comparison with the trees actually walked): 32 (ray) + 16 (hit) + 32 N_node
    + 52 N_tri + 112 N_prim, N from the oracle walking the reference BVHs on a
    crop of frame 0."""
    _, c = orc.render(scene.packed(), head, prm, W_FULL, H_FULL, 1, crop=(704, 396, 1216, 684))
    n = max(c.ext_rays, 1)
    nn, nt, npr = c.ext_nodes / n, c.ext_tris / n, c.ext_prims / n
    return 32 + 16 + 32 * nn + 52 * nt + 112 * npr, {"nodes": nn, "tris": nt, "prims": npr,
                                                       "sample_segments": int(c.ext_rays)}


def cpu_baseline(pt, orc, scene, head, prm, budget_s=12.0):
    """fp32 oracle (the reference-semantics CPU port) on whole frames of the
    same workload, all host threads, about `budget_s` seconds of CPU work."""
    cores = os.cpu_count() or 1
    acc = np.zeros((H_FULL, W_FULL, 4), np.float32)
    segs, t_used, frames = 0, 0.0, 0
    h0, p0 = head, prm
    while t_used < budget_s and frames < FRAMES:
        h0, p0 = scene.push(W_FULL, H_FULL, frame_index=head.frame_index + frames, reset=int(frames == 0))
        t0 = time.perf_counter()
        _, c = orc.render(scene.packed(), h0, p0, W_FULL, H_FULL, 1, accum=acc, threads=cores)
        t_used += time.perf_counter() - t0
        segs += c.ext_rays + c.shadow_rays
        frames += 1
    out = {"value": segs / t_used / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "port",
           "sample": f"frames 0..{frames - 1} of the 64 (1920x1080, 1 spp each), "
                     f"{segs} segments in {t_used:.1f} s"}
    # the reference's own CPU estimator (Software backend preview: primary hit,
    # sky ambient, one sun shadow ray), restated on the oracle's traversal
    sw_acc = np.zeros((H_FULL, W_FULL, 4), np.float32)
    sw_segs, sw_t, sw_frames = 0, 0.0, 0
    while sw_t < budget_s / 3 and sw_frames < FRAMES:
        h0, p0 = scene.push(W_FULL, H_FULL, frame_index=head.frame_index + sw_frames, reset=int(sw_frames == 0))
        t0 = time.perf_counter()
        _, c = orc.software_preview(scene.packed(), h0, p0, W_FULL, H_FULL, accum=sw_acc, threads=cores)
        sw_t += time.perf_counter() - t0
        sw_segs += c.ext_rays + c.shadow_rays
        sw_frames += 1
    out["software_preview"] = {
        "value": sw_segs / sw_t / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "port",
        "sample": f"{sw_frames} frames 1920x1080 of the reference's Software-backend preview estimator "
                  f"(1 primary + <=1 sun shadow ray per pixel), {sw_segs} segments in {sw_t:.1f} s"}
    return out


def c0_bench(pt, orc, frames=64, steps=3, cpu_budget_s=6.0):
    """The plain analytic configuration: 256x256, 16 spp, depth 8, roulette from
    bounce 3; 64 spheres, 4 boxes (12 triangles each), one 1x1 quad light of
    radiance 15, black environment.  One step = `frames` frames accumulated.
    Beside it the fp32 oracle on all host cores over whole frames of the same
    workload (about `cpu_budget_s` of CPU work)."""
    s = pt.Scene().synth(0, seed=0)
    W = H = 256
    dev = pt.Device(0)
    try:
        dev.upload(s)
        dev.set_target(W, H)
        head, prm = s.push(W, H, frame_index=0, reset=1)
        for _ in range(3):
            dev.render(head, prm, frames)
        t_ms, segs = 0.0, 0
        for _ in range(steps):
            dev.render(head, prm, frames)
            st = dev.stats()
            t_ms += st.gpu_ms
            segs += st.extension_rays + st.shadow_rays
    finally:
        dev.close()
    cores = os.cpu_count() or 1
    acc = np.zeros((H, W, 4), np.float32)
    c_segs, c_t, f = 0, 0.0, 0
    while c_t < cpu_budget_s and f < frames:
        h0, p0 = s.push(W, H, frame_index=f, reset=int(f == 0))
        t0 = time.perf_counter()
        _, c = orc.render(s.packed(), h0, p0, W, H, 1, accum=acc, threads=cores)
        c_t += time.perf_counter() - t0
        c_segs += c.ext_rays + c.shadow_rays
        f += 1
    return {"workload": f"plain analytic 256x256, {head.spp} spp x {frames} frames, depth {head.max_bounces}, "
                        f"roulette from bounce {prm.rr_start}, 64 spheres + 4 boxes, 1 quad light",
            "mrays_s": segs / (t_ms / 1e3) / 1e6, "ms_per_step": t_ms / steps,
            "segments_per_step": segs // steps,
            "cpu_baseline": {"value": c_segs / c_t / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "port",
                             "sample": f"{f} whole frames (256x256, 16 spp each), {c_segs} segments in {c_t:.1f} s"}}


def _tris_at_scale(sc):
    """Triangle count of the synthetic triangle+analytic scene at `scale`
    (mirrors the generator: round(200 s) icospheres of 20 nu^2 tris, nu =
    round(22 sqrt s), plus a round(512 sqrt s)^2-quad ground)."""
    import math
    n_ico = max(1, round(200 * sc))
    nu = max(2, round(22 * math.sqrt(sc)))
    grid = max(2, round(512 * math.sqrt(sc)))
    return n_ico * 20 * nu * nu + 2 * grid * grid


def _scale_for_tris(target):
    lo, hi = 1e-5, 1.0
    for _ in range(60):
        mid = (lo + hi) / 2
        if _tris_at_scale(mid) < target:
            lo = mid
        else:
            hi = mid
    return hi


def batched_workload(pt, n_views=64, n_scenes=8, seed=0x5EED + 2):
    """The batched configuration: n_views square views with sides log-uniform in
    [128, 1024] (rounded to the 8x4 tile), over n_scenes triangle+analytic scenes
    with triangle counts log-uniform in [10k, 1M]; 4 spp, depth 6."""
    import math
    rng = np.random.default_rng(seed)
    scenes, devs, tris = [], [], []
    for k in range(n_scenes):
        target = 10_000 * 100 ** rng.uniform()
        s = pt.Scene().synth(1, seed=100 + k, scale=_scale_for_tris(target))
        s.set_cvar("r_spp", 4)
        s.set_cvar("r_max_bounces", 6)
        d = pt.Device(0)
        d.upload(s)
        scenes.append(s)
        devs.append(d)
        tris.append(_tris_at_scale(_scale_for_tris(target)))
    views = []
    for i in range(n_views):
        side = int(round(128 * 8 ** rng.uniform() / 8)) * 8
        k = i % n_scenes
        yaw = rng.uniform(0, 2 * math.pi)
        dist, hgt = rng.uniform(60, 140), rng.uniform(15, 40)
        pos = (dist * math.sin(yaw), hgt, -dist * math.cos(yaw))
        look_yaw = math.atan2(-pos[0], pos[2])      # forward = (sin yaw, ., -cos yaw) toward the origin
        pitch = -math.atan2(hgt, dist)
        scenes[k].camera(pos, look_yaw, pitch, 45.0)
        head, prm = scenes[k].push(side, side, frame_index=1000 + i, reset=1)
        views.append((k, side, side, head, prm))
    return scenes, devs, views, tris


def batched_bench(pt, steps=3):
    """Plain form (each view rendered by its own pt_gpu_render call, one after the
    other) against the batched form (pt_gpu_batch_render: all views in one
    graph-replayed wavefront, launch shape from the autotuner).  Both produce
    bit-identical images (tests/test_gpu_parity.py), so the image RMSE is equal."""
    scenes, devs, views, tris = batched_workload(pt)
    # plain
    t_plain, s_plain = 0.0, 0
    for _ in range(steps + 1):
        tt, ss = 0.0, 0
        for (k, w, h, head, prm) in views:
            d = devs[k]
            d.set_target(w, h)
            d.render(head, prm, 1)
            st = d.stats()
            tt += st.gpu_ms
            ss += st.extension_rays + st.shadow_rays
        t_plain, s_plain = tt, ss      # keep the last (warm) pass
    batch = pt.Device(0)
    tune = batch.batch_autotune(devs, views)
    default_ms, tuned_ms = batch.batch_tuning_gain()
    for _ in range(2):
        batch.batch_render(devs, views, 1)
    tb, sb = 0.0, 0
    for _ in range(steps):
        batch.batch_render(devs, views, 1)
        st = batch.stats()
        tb += st.gpu_ms
        sb += st.extension_rays + st.shadow_rays
    plain_v = s_plain / (t_plain / 1e3) / 1e6
    batch_v = sb / (tb / 1e3) / 1e6
    out = {"workload": f"{len(views)} views (sides 128..1024 log-uniform), {len(devs)} scenes "
                       f"({min(tris):,}..{max(tris):,} tris), 4 spp, depth 6, 1 frame",
           "pixels": int(sum(w * h for (_, w, h, _, _) in views)),
           "plain_mrays_s": plain_v, "batched_mrays_s": batch_v, "batched_over_plain": batch_v / plain_v,
           "plain_ms_per_frame": t_plain, "batched_ms_per_frame": tb / steps,
           "tuning": {"persistent_blocks_per_sm": tune.persistent_blocks_per_sm,
                      "stream_blocks_per_sm": tune.stream_blocks_per_sm, "cuda_graph": bool(tune.use_graph),
                      "shade_threads": tune.shade_threads, "camera_tile": f"{tune.camera_tile_w}x{32 // tune.camera_tile_w}",
                      "octant_grouping": bool(tune.octant_grouping),
                      "search": "coordinate descent from the default (4, 8, graph, 512, 4x8, no grouping), "
                                "one frame of the batch per candidate",
                      "default_ms_per_frame": default_ms, "tuned_ms_per_frame": tuned_ms,
                      "tuned_over_default": default_ms / tuned_ms if tuned_ms > 0 else None},
           "image_rmse_plain_vs_batched": 0.0}
    batch.close()
    for d in devs:
        d.close()
    return out


def adjoint_bench(pt, fd_params=32, seed=0x5EED + 3):
    """Differentiable render (512x512, 32 spp, depth 6, roulette from bounce 3,
    256 material rows of which 16 emissive, ~200k triangles + 512 spheres).
    Target: 32 frames x 32 spp (1024 spp) with the albedos perturbed by
    N(0, 0.1) and clamped to [0.02, 0.98]; loss = L2 over HDR pixels.  One
    gradient evaluation = pt_gpu_diff_forward + pt_gpu_diff_backward.  Central
    differences (eps 1e-3, common random numbers = the same pixel seeds) on 32
    random parameters, once with the configured roulette and once with it off
    (the per-sample estimator is then smooth in the parameters)."""
    W = H = 512
    sc = pt.Scene().synth(3, seed=0)
    pk = sc.packed()
    nm = pk.material_count
    mats = np.ctypeslib.as_array(pk.materials, (nm * 12,)).reshape(nm, 12).copy()
    tris = pk.tri_count
    dev = pt.Device(0)
    dev.upload(sc)
    dev.set_target(W, H)
    rng = np.random.default_rng(seed)
    tgt_m = mats.copy()
    tgt_m[:, :3] = np.clip(mats[:, :3] + rng.normal(0.0, 0.1, (nm, 3)), 0.02, 0.98).astype(np.float32)
    dev.materials(tgt_m)
    h_t, p_t = sc.push(W, H, frame_index=500, reset=1)
    dev.render(h_t, p_t, 32)
    target = dev.read_accum()[..., :3].astype(np.float64)
    dev.materials(mats)
    head, prm = sc.push(W, H, frame_index=0, reset=1)

    def grad_eval():
        dev.diff_forward(head, prm, 1)
        f = dev.stats()
        img = dev.read_accum()[..., :3].astype(np.float64)
        dl = (2.0 * (img - target)).astype(np.float32)
        ga, ge = dev.diff_backward(dl, nm)
        b = dev.backward_stats()
        return f, b, ga, ge, float(((img - target) ** 2).sum())

    for _ in range(3):
        grad_eval()
    fwd_ms, bwd_ms, n = 0.0, 0.0, 5
    t0 = time.perf_counter()
    for _ in range(n):
        f, b, ga, ge, loss0 = grad_eval()
        fwd_ms += f.gpu_ms
        bwd_ms += b.gpu_ms
    wall = (time.perf_counter() - t0) / n
    fwd_ms /= n
    bwd_ms /= n

    emissive = [r for r in range(nm) if mats[r, 4:7].max() > 0]
    pool = [("a", r, c) for r in range(nm) for c in range(3)] + [("e", r, c) for r in emissive for c in range(3)]
    pick = [pool[i] for i in rng.choice(len(pool), fd_params, replace=False)]

    def fd_check(rr_start):
        """Central differences with common random numbers; under roulette the
        nominal render's survival probabilities are recorded and reused by the
        +-eps renders (pt_gpu_set_roulette_freeze), so that each sample is a
        smooth function of the parameters."""
        p2 = type(prm).from_buffer_copy(prm)
        p2.rr_start = rr_start
        dev.materials(mats)
        dev.diff_forward(head, p2, 1)
        img = dev.read_accum()[..., :3].astype(np.float64)
        ga, ge = dev.diff_backward((2.0 * (img - target)).astype(np.float32), nm)
        frozen = rr_start < head.max_bounces
        if frozen:
            dev.set_roulette_freeze(1)
            dev.render(head, p2, 1)
            dev.set_roulette_freeze(2)

        def loss(m):
            dev.materials(m)
            dev.render(head, p2, 1)
            return float(((dev.read_accum()[..., :3].astype(np.float64) - target) ** 2).sum())

        g_adj, g_fd = [], []
        for kind, r, c in pick:
            col = c if kind == "a" else 4 + c
            mp, mm = mats.copy(), mats.copy()
            mp[r, col] += 1e-3
            mm[r, col] -= 1e-3
            g_fd.append((loss(mp) - loss(mm)) / 2e-3)
            g_adj.append(ga[r, c] if kind == "a" else ge[r, c])
        dev.materials(mats)
        dev.set_roulette_freeze(0)
        g_adj, g_fd = np.array(g_adj), np.array(g_fd)
        rel = np.abs(g_adj - g_fd) / np.maximum(np.abs(g_fd), 1e-30)
        big = np.abs(g_fd) >= 0.01 * np.abs(g_fd).max()
        return {"rr_start": rr_start, "roulette_probabilities_fixed": frozen,
                "rel_l2_error": float(np.linalg.norm(g_adj - g_fd) / max(np.linalg.norm(g_fd), 1e-30)),
                "within_2pct": int((rel <= 0.02).sum()), "params": len(pick),
                "median_rel_error_significant": float(np.median(rel[big])) if big.any() else None,
                "max_rel_error_significant": float(rel[big].max()) if big.any() else None}

    fd_rr = fd_check(int(prm.rr_start))
    fd_smooth = fd_check(int(head.max_bounces))
    out = {"workload": f"512x512, 32 spp, depth 6, roulette from bounce {int(prm.rr_start)}, {tris:,} tris + "
                       f"{pk.prim_count} spheres, {nm} material rows ({len(emissive)} emissive)",
           "params": nm * 3 + len(emissive) * 3,
           "grad_evals_per_s": 1e3 / (fwd_ms + bwd_ms), "grad_evals_per_s_wall": 1.0 / wall,
           "forward_ms": fwd_ms, "backward_ms": bwd_ms, "backward_over_forward": bwd_ms / fwd_ms,
           "loss": loss0, "fd_check": [fd_rr, fd_smooth],
           "fd_equivalent_renders_per_eval": 2 * (nm * 3 + len(emissive) * 3)}
    dev.close()
    return out


def inverse_views(pt, sc, n_views=16, side=384):
    """Cameras of the 16 views: one above each tile of a 4 x 4 tiling of the
    120 x 120 arena, 45 up and 20 back from the tile centre, looking at it,
    the back direction turning by 1/16 of a circle from view to view."""
    import math
    cams = []
    for i in range(n_views):
        cx, cz = -45.0 + 30.0 * (i % 4), -45.0 + 30.0 * (i // 4)
        yaw = 2 * math.pi * (i + 0.5) / n_views
        pos = (cx - 20.0 * math.sin(yaw), 45.0, cz + 20.0 * math.cos(yaw))
        cams.append((pos, yaw, -math.atan2(45.0, 20.0)))
    return cams


def _cam_views(sc, cams, side, frame0, spp, frames_per_wave):
    """One batch view per camera, rendering frames_per_wave frames per wave."""
    out = []
    sc.set_cvar("r_spp", spp)
    for c, (pos, yaw, pitch) in enumerate(cams):
        sc.camera(pos, yaw, pitch, 50.0)
        head, prm = sc.push(side, side, frame_index=frame0 + 100_003 * c, reset=1)
        out.append((side, side, head, prm, frames_per_wave))
    return out


def inverse_bench(pt, steps=200, lr=1e-2, spp=16, seed=0x5EED + 4):
    """Batched inverse rendering: recover 1,024 Lambert albedos from 16 views of
    384x384 of a ~1M-triangle scene.  Target: 2,048 samples per pixel per view
    (16 waves x 8 frames x 16 spp) from hidden albedos U[0.05, 0.95].  Each step
    draws 16 samples per pixel per view as 16 one-spp frames with fresh seeds,
    as two half-views per camera (A: frames 0-7, B: frames 8-15) of 8 frames per
    wave, all in one batched wavefront: one recorded forward and one adjoint
    replay.  The residual of half A's image drives the replay of half B's
    samples and vice versa, so residual and dI/dalbedo never share samples (an
    unbiased gradient of the L2 loss of the mean image).  Then Adam (lr 1e-2)
    on the albedos, clamped to [0.01, 0.99].  Reports the time until the albedo
    RMSE first drops below 0.01 and the RMSE curve."""
    sc = pt.Scene().synth(4, seed=0)
    pk = sc.packed()
    nm = pk.material_count
    mats = np.ctypeslib.as_array(pk.materials, (nm * 12,)).reshape(nm, 12).copy()
    rng = np.random.default_rng(seed)
    hidden = rng.uniform(0.05, 0.95, (nm, 3)).astype(np.float32)
    side, nv = 384, 16
    cams = inverse_views(pt, sc, nv, side)
    scene = pt.Device(0)
    scene.upload(sc)
    batch = pt.Device(0)
    tgt = mats.copy()
    tgt[:, :3] = hidden
    scene.materials(tgt)
    t0 = time.perf_counter()
    tv = _cam_views(sc, cams, side, 1 << 28, 16, 8)
    batch.batch_render([scene], [(0,) + v for v in tv], 16)
    target = [batch.batch_read(i, side, side)[..., :3].copy() for i in range(nv)]
    t_target = time.perf_counter() - t0
    half = spp // 2
    alb = mats[:, :3].astype(np.float64).copy()
    m_t = np.zeros_like(alb)
    v_t = np.zeros_like(alb)
    b1, b2, eps = 0.9, 0.999, 1e-8
    rmse0 = float(np.sqrt(((alb - hidden) ** 2).mean()))
    hist, t_hit, fwd_ms, bwd_ms, losses, host_s = [], None, 0.0, 0.0, [], 0.0
    g0 = None
    t0 = time.perf_counter()
    for k in range(steps):
        cur = mats.copy()
        cur[:, :3] = alb.astype(np.float32)
        scene.materials(cur)
        base = (k + 1) * 4096
        views = (_cam_views(sc, cams, side, base, 1, half) +            # A halves
                 _cam_views(sc, cams, side, base + half, 1, spp - half))   # B halves
        batch.batch_diff_forward(scene, views)
        fwd_ms += batch.stats().gpu_ms
        th = time.perf_counter()
        res, loss = [], 0.0
        for c in range(nv):
            ra = batch.batch_read(c, side, side)[..., :3] - target[c]
            rb = batch.batch_read(nv + c, side, side)[..., :3] - target[c]
            m = 0.5 * (ra + rb)
            loss += float(np.dot(m.ravel().astype(np.float64), m.ravel().astype(np.float64)))
            res.append((ra, rb))
        # L = |mean(I) - T|^2, I = (I_A + I_B) / 2: dL/dI_A = (I - T) taken from the
        # other half (B's residual), and the other way round
        dl = [rb for (ra, rb) in res] + [ra for (ra, rb) in res]
        host_s += time.perf_counter() - th
        ga, _ = batch.batch_diff_backward(dl, nm)
        bwd_ms += batch.backward_stats().gpu_ms
        if g0 is None:
            g0 = np.abs(ga).sum(axis=1)
        m_t = b1 * m_t + (1 - b1) * ga
        v_t = b2 * v_t + (1 - b2) * ga * ga
        mh = m_t / (1 - b1 ** (k + 1))
        vh = v_t / (1 - b2 ** (k + 1))
        alb = np.clip(alb - lr * mh / (np.sqrt(vh) + eps), 0.01, 0.99)
        rmse = float(np.sqrt(((alb - hidden) ** 2).mean()))
        hist.append(rmse)
        losses.append(loss)
        if t_hit is None and rmse < 0.01:
            t_hit = time.perf_counter() - t0
    wall = time.perf_counter() - t0
    err = np.sqrt(((alb - hidden) ** 2).mean(axis=1))
    order = np.argsort(g0)
    q = len(order) // 4
    out = {"workload": f"16 views 384x384, {pk.tri_count:,} tris + {pk.prim_count} spheres, {nm} Lambert rows, "
                       f"{spp} samples/pixel/view/step as {spp} one-spp frames (halves A/B cross-paired), depth 8, "
                       f"Adam lr {lr}, {steps} steps",
           "target_spp": 2048, "target_render_s": t_target,
           "rmse_start": rmse0, "rmse_final": hist[-1], "rmse_min": min(hist),
           "rmse_at": {str(s): hist[s - 1] for s in (10, 25, 50, 100, 150, 200, 300, 400) if s <= steps},
           "time_to_rmse_below_0.01_s": t_hit,
           "steps_to_rmse_below_0.01": (next(i + 1 for i, r in enumerate(hist) if r < 0.01)
                                        if t_hit is not None else None),
           "row_rmse_by_gradient_quartile": [float(np.sqrt((err[order[i * q:(i + 1) * q]] ** 2).mean()))
                                             for i in range(4)],
           "loss_first_last": [losses[0], losses[-1]],
           "wall_s": wall, "step_ms": 1e3 * wall / steps, "host_ms_per_step": 1e3 * host_s / steps,
           "forward_ms_per_step": fwd_ms / steps, "backward_ms_per_step": bwd_ms / steps,
           "paths_per_step": side * side * nv * spp}
    batch.close()
    scene.close()
    return out


def run_reference(args):
    """The reference's CPU implementation of this path is its Slang shader
    (not runnable: no Slang/Vulkan/Metal here) and a reduced Software preview
    tracer that needs Embree + glm (absent); the timed reference arm is
    therefore the oracle's fp32 restatement of the shader on the host cores."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, ROOT)
    pt = load_pkg()
    import oracle as orc
    orc.load()
    scene = pt.Scene().synth(1, seed=0)
    head, prm = scene.push(W_FULL, H_FULL, 0, 1)
    cores = os.cpu_count() or 1
    acc = np.zeros((H_FULL, W_FULL, 4), np.float32)

    def step(i):
        h, p = scene.push(W_FULL, H_FULL, frame_index=i, reset=int(i == 0))
        t0 = time.perf_counter()
        _, c = orc.render(scene.packed(), h, p, W_FULL, H_FULL, 1, accum=acc, threads=cores)
        return time.perf_counter() - t0, c.ext_rays + c.shadow_rays

    for i in range(args.warmup):
        step(i)
    tt, ss = 0.0, 0
    for i in range(args.steps):
        t, s = step(args.warmup + i)
        tt += t
        ss += s
    v = ss / tt / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "triangles+analytic 1920x1080 1spp x64 frames depth 8 (2,460,288 tris, "
                                   "1024 spheres, 2048x1024 env)", "step": "one 1920x1080 1 spp frame of the 64"},
            "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} whole frames after {args.warmup} warm-up frames, {ss} segments"},
            "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--frames", type=int, default=FRAMES)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-c0", action="store_true", help="skip the plain analytic (256x256, 16 spp) leg")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-views leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiable-render leg")
    ap.add_argument("--no-inverse", action="store_true", help="skip the inverse-rendering leg")
    ap.add_argument("--inverse-steps", type=int, default=200)
    ap.add_argument("--traversal", type=int, default=0, choices=[0, 1],
                    help="0: 4-wide SAH trees built on the device (default); 1: the reference BVHs")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    rank, world, local = dist_env()
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        pg = dist
    sys.path.insert(0, ROOT)
    pt = load_pkg()
    scene = pt.Scene().synth(1, seed=0)
    dev = pt.Device(local)
    dev.set_traversal(args.traversal)
    dev.upload(scene)
    accel = dev.accel_info()
    dev.set_target(W_FULL, H_FULL)
    # replicas: each rank renders its own disjoint frame range of the same workload
    head, prm = scene.push(W_FULL, H_FULL, frame_index=replica_frame_index(rank), reset=1)

    def barrier():
        if pg:
            import torch
            torch.cuda.synchronize()
            pg.barrier()

    dev.set_profiling(False)
    for _ in range(args.warmup):
        dev.render(head, prm, args.frames)
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    t_dev, segs, launches, segs_ext, segs_sh = 0.0, 0, 0, 0, 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dev.render(head, prm, args.frames)
        st = dev.stats()
        t_dev += st.gpu_ms / 1e3
        segs += st.extension_rays + st.shadow_rays
        segs_ext += st.extension_rays
        segs_sh += st.shadow_rays
        launches += st.kernel_launches
    t_wall = time.perf_counter() - t0
    barrier()
    clk = clocks.stop()

    # per-kernel device times: the same steps again with the stages serial and
    # CUDA events around every closest-hit / transmittance launch on its stream
    # (in the timed schedule above the next bounce's closest-hit pass overlaps
    # this bounce's shadow rays, so their spans are not each kernel's own time)
    dev.set_profiling(2)
    dev.render(head, prm, args.frames)
    ext, ext_ms, ext_launch, sh_ms, t_serial = 0, 0.0, 0, 0.0, 0.0
    for _ in range(args.steps):
        dev.render(head, prm, args.frames)
        st = dev.stats()
        ext += st.extension_rays
        ext_ms += st.extend_ms
        sh_ms += st.shadow_ms
        ext_launch += st.extend_launches
        t_serial += st.gpu_ms / 1e3
    barrier()
    # what the traversal touched: one step with the counting kernel variants
    # (same images; the counting costs time, so kernel times come from mode 2)
    dev.set_profiling(3)
    dev.render(head, prm, args.frames)
    tstat = dev.traversal_stats()
    barrier()

    # end to end through the C-ABI with host buffers (pinned when torch can pin)
    dev.set_profiling(False)
    try:
        import torch
        host = torch.empty((H_FULL, W_FULL, 4), dtype=torch.float32, pin_memory=True).numpy()
    except Exception:
        host = np.empty((H_FULL, W_FULL, 4), np.float32)
    dev.render_to_host(head, prm, args.frames, host)
    barrier()
    t1 = time.perf_counter()
    e2e_segs = 0
    for _ in range(args.steps):
        dev.render_to_host(head, prm, args.frames, host)
        st = dev.stats()
        e2e_segs += st.extension_rays + st.shadow_rays
    t_e2e = time.perf_counter() - t1
    barrier()

    if pg:
        (t_dev, t_e2e), (segs, e2e_segs, segs_ext, segs_sh) = reduce_replicas(
            pg, [t_dev, t_e2e], [segs, e2e_segs, segs_ext, segs_sh], "cuda")
    if rank != 0:
        if pg:
            pg.destroy_process_group()
        return 0

    import oracle as orc
    orc.load()
    ref_bseg, ref_nbar = algorithmic_bytes(pt, orc, scene, head, prm)
    peak, peak_kind = measured_peak()
    roofline = None
    if tstat.ext_segments:
        launch_ms = ext_ms / max(ext_launch, 1)
        per_launch = ext / max(ext_launch, 1)
        bseg, terms, per = traversed_bytes(tstat, "ext")
        achieved = bseg * per_launch / (launch_ms * 1e-3) / 1e9
        sh_bseg, sh_terms, sh_per = traversed_bytes(tstat, "shadow")
        roofline = {
            "bound": "hbm", "kernel": "k_closest (persistent closest hit, 4-wide SAH trees)",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
            "peak_kind": peak_kind,
            "algorithmic_bytes_per_launch": bseg * per_launch, "avg_launch_ms": launch_ms, "launches": ext_launch,
            "bytes_per_segment": bseg, "bytes_per_segment_terms": terms, "per_segment": per,
            "dram_compulsory_frac": RAY_IO_BYTES * per_launch / (launch_ms * 1e-3) / 1e9 / peak,
            "ref_structure_bytes_per_segment": ref_bseg, "ref_structure_N_per_segment": ref_nbar,
            "shadow_kernel": {"kernel": "k_transmit", "bytes_per_segment": sh_bseg, "bytes_per_segment_terms": sh_terms,
                              "per_segment": sh_per,
                              "achieved_GBs": sh_bseg * tstat.shadow_segments
                              / max(sh_ms / args.steps * 1e-3, 1e-12) / 1e9},
            "shade_bytes_per_vertex": shade_bytes_per_vertex(scene),
            "note": "achieved = bytes the closest-hit kernel moves per segment on the trees it walks (device "
                    "counters of a counting pass: wide nodes, triangles, leaf and plane records, 8-byte stack "
                    "pushes and pops, ray in and hit out) x extension segments per launch / average launch "
                    "time (CUDA events, stages serial).  Most of these bytes are L1/L2 hits: ray in and hit "
                    "out (dram_compulsory_frac) are the only bytes that must reach DRAM; the scene (~350 MB) "
                    "exceeds L2, so part of the node and triangle traffic does too (an ncu capture of one "
                    "launch measures it).  traffic is null: no ncu capture runs inside the bench.",
            "step_share": {"k_closest": ext_ms / max(1e3 * t_serial, 1e-9),
                           "k_transmit": sh_ms / max(1e3 * t_serial, 1e-9),
                           "serial_ms_per_step": 1e3 * t_serial / args.steps}}
    line = {"metric": METRIC, "value": segs / t_dev / 1e6, "unit": "Mrays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps,
            "wall_ms_per_step": 1e3 * t_wall / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "triangles+analytic 1920x1080 1spp x64 frames depth 8 (2,460,288 tris, "
                                   "1024 spheres, 2048x1024 env)", "frames_per_step": args.frames,
                       "parallelism": f"replicas x{world}",
                       "traversal": ("4-wide SAH (device-built, %d nodes, depth %d, build %.1f ms)"
                                     % (accel.mesh_wide_nodes, accel.mesh_wide_depth, accel.mesh_build_ms))
                       if (accel.mesh_wide and args.traversal == 0) else "reference binary BVH",
                       "l2": "no flush: per-wave path state (376 B x up to 64 M paths, ~25 GB at 32 frames "
                             "per wave) and scene (~350 MB) exceed the 129 MB L2"},
            "e2e": {"value": e2e_segs / t_e2e / 1e6, "unit": "Mrays/s",
                    "h2d_bytes_per_step": args.frames * (ctypes.sizeof(pt.PtPushHead) + ctypes.sizeof(pt.PtPathParams)),
                    "d2h_bytes_per_step": W_FULL * H_FULL * 16},
            "segments_per_step": {"extension": int(segs_ext) // args.steps, "shadow": int(segs_sh) // args.steps,
                                  "total": int(segs) // args.steps},
            "gpu_launches": launches,
            "roofline": roofline,
            "clocks": clk}
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(pt, orc, scene, head, prm)
    if world == 1 and not args.no_c0:
        line["c0"] = c0_bench(pt, orc)
    if world == 1 and not args.no_batched:
        dev.close()
        line["batched"] = batched_bench(pt)
    if world == 1 and not args.no_adjoint:
        if dev.h:
            dev.close()
        line["adjoint"] = adjoint_bench(pt)
    if world == 1 and not args.no_inverse:
        if dev.h:
            dev.close()
        line["inverse"] = inverse_bench(pt, steps=args.inverse_steps)
    print(json.dumps(line), flush=True)
    if dev.h:
        dev.close()
    if pg:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
