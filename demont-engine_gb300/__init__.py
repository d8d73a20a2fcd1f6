"""Python mirror of the GB300 path-trace C-ABI (include/pt_gpu.h, include/pt_scene.h).

The product is the shared library ``_build/libdemont_pt.so`` (CUDA kernels for
sm_103a + the C++ host scene builder).  This module only binds it with ctypes
and wraps buffers as numpy arrays; it never computes anything itself, and it
raises when the library is missing instead of falling back to anything.

The directory name contains a hyphen, so it is loaded by path::

    import importlib.util, sys
    spec = importlib.util.spec_from_file_location(
        "demont_gb300", "demont-engine_gb300/__init__.py",
        submodule_search_locations=["demont-engine_gb300"])
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# the in-tree build; DEMONT_PT_LIB names another build of the same library
LIB_PATH = os.environ.get("DEMONT_PT_LIB") or os.path.join(HERE, "_build", "libdemont_pt.so")

PT_OK = 0
ERRORS = {-1: "PT_ERR_INVALID", -2: "PT_ERR_CUDA", -3: "PT_ERR_OOM", -4: "PT_ERR_STATE",
          -5: "PT_ERR_KERNEL", -6: "PT_ERR_UNSUPPORTED"}
HIT_MISS = 0xFFFFFFFF
HIT_TRI = 1 << 30

u32 = ctypes.c_uint32
f32 = ctypes.c_float
P = ctypes.POINTER


class PtPushHead(ctypes.Structure):
    _fields_ = [("pos_fovtan", f32 * 4), ("fwd_aspect", f32 * 4), ("right_xyz", f32 * 4),
                ("up_xyz", f32 * 4), ("frame_index", u32), ("reset_accum", u32),
                ("max_bounces", u32), ("tlas_present", u32), ("prim_count", u32), ("spp", u32),
                ("denoiser_enabled", u32), ("env_map_present", u32), ("halton_jitter", f32 * 2),
                ("env_intensity", f32), ("env_total_luminance", f32)]


class PtPathParams(ctypes.Structure):
    _fields_ = [("refract_budget", f32), ("firefly_clamp", f32), ("mis_enabled", u32),
                ("accum_ema_alpha", f32), ("bvh_params", u32 * 4), ("light_count", u32),
                ("light_tree_enabled", u32), ("light_tree_node_count", u32), ("rr_start", u32),
                ("sun_and_mode", f32 * 4), ("stars", u32), ("sdf_procedural_ops", u32), ("reserved", u32 * 2),
                ("moon_dir_phase", f32 * 4), ("moon_extra", f32 * 4), ("sun_extra", f32 * 4),
                ("sun_extra2", f32 * 4), ("sdf_params", u32 * 4), ("sdf_params_f", f32 * 4)]


class PtBvhNode(ctypes.Structure):
    _fields_ = [("aabb_min", f32 * 3), ("left_first", u32), ("aabb_max", f32 * 3), ("count", u32)]


class PtStats(ctypes.Structure):
    _fields_ = [("extension_rays", ctypes.c_uint64), ("shadow_rays", ctypes.c_uint64),
                ("paths", ctypes.c_uint64), ("frames", u32), ("waves", u32), ("gpu_ms", ctypes.c_double),
                ("extend_ms", ctypes.c_double), ("shadow_ms", ctypes.c_double),
                ("extend_launches", u32), ("shadow_launches", u32), ("kernel_launches", u32),
                ("graph_replays", u32)]


class PtAccelInfo(ctypes.Structure):
    _fields_ = [("traversal", u32), ("mesh_wide", u32), ("prims_wide", u32), ("mesh_wide_nodes", u32),
                ("mesh_wide_depth", u32), ("mesh_binary_nodes", u32), ("prims_wide_nodes", u32),
                ("merged_wide_nodes", u32), ("mesh_build_ms", ctypes.c_double)]


class PtBatchView(ctypes.Structure):
    _fields_ = [("scene", u32), ("width", u32), ("height", u32), ("frames_per_wave", u32),
                ("head", PtPushHead), ("params", PtPathParams)]


class PtBatchTuning(ctypes.Structure):
    _fields_ = [("persistent_blocks_per_sm", u32), ("stream_blocks_per_sm", u32), ("use_graph", u32),
                ("shade_threads", u32), ("camera_tile_w", u32), ("octant_grouping", u32), ("reserved", u32 * 2)]


class PtLightTreeNode(ctypes.Structure):
    _fields_ = [("aabb_min", f32 * 3), ("left_first", u32), ("aabb_max", f32 * 3), ("count", u32),
                ("cone_axis", f32 * 3), ("cone_cos_half", f32), ("intensity", f32), ("pad", f32 * 3)]


class PtLightInput(ctypes.Structure):
    _fields_ = [("type", u32), ("pos", f32 * 3), ("radius", f32), ("intensity", f32 * 3), ("dir", f32 * 3),
                ("cos_outer", f32), ("u_vec", f32 * 3), ("v_half", f32)]


class PtTraversalStats(ctypes.Structure):
    _fields_ = [(f"{k}_{f}", ctypes.c_uint64) for k in ("ext", "shadow")
                for f in ("segments", "nodes", "tris", "aprims", "linear", "push", "pop")]


class PtDiffStats(ctypes.Structure):
    _fields_ = [("max_delta", ctypes.c_double), ("mean_delta", ctypes.c_double), ("rms_delta", ctypes.c_double),
                ("bad_percent", ctypes.c_double), ("total_pixels", ctypes.c_uint64), ("bad_pixels", ctypes.c_uint64)]


class PtPackedScene(ctypes.Structure):
    _fields_ = [("prims", P(f32)), ("prim_count", u32), ("linear_prim_count", u32),
                ("bvh_nodes", P(PtBvhNode)), ("bvh_node_count", u32),
                ("positions", P(f32)), ("vertex_count", u32), ("indices", P(u32)), ("tri_count", u32),
                ("tri_nodes", P(PtBvhNode)), ("tri_node_count", u32), ("tri_perm", P(u32)),
                ("tri_perm_count", u32), ("tri_mat_ids", P(u32)), ("materials", P(f32)),
                ("material_count", u32), ("lights", P(f32)), ("light_count", u32),
                ("env_rgba", P(f32)), ("env_w", u32), ("env_h", u32), ("env_marginal", P(f32)),
                ("env_conditional", P(f32)), ("env_total_luminance", ctypes.c_double),
                ("hdri_count", u32), ("hdri_dir_pmf", P(f32)), ("hdri_col", P(f32)),
                ("env_present", u32), ("prim_mat_ids", P(u32)), ("moon_rgba", P(f32)),
                ("moon_w", u32), ("moon_h", u32), ("light_tree", P(PtLightTreeNode)),
                ("light_tree_node_count", u32), ("sdf_clusters", P(f32)), ("sdf_count", u32)]


# every entry point include/*.h declares, with its ctypes signature
SIGNATURES = {
    # pt_gpu.h
    "pt_gpu_create": (ctypes.c_int, [P(ctypes.c_void_p), ctypes.c_int]),
    "pt_gpu_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pt_gpu_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "pt_gpu_version": (ctypes.c_char_p, []),
    "pt_gpu_upload_prims": (ctypes.c_int, [ctypes.c_void_p, P(f32), u32, u32, P(PtBvhNode), u32]),
    "pt_gpu_upload_mesh": (ctypes.c_int, [ctypes.c_void_p, P(f32), u32, P(u32), u32, P(PtBvhNode), u32,
                                          P(u32), u32, P(u32)]),
    "pt_gpu_upload_materials": (ctypes.c_int, [ctypes.c_void_p, P(f32), u32]),
    "pt_gpu_upload_prim_materials": (ctypes.c_int, [ctypes.c_void_p, P(u32), u32]),
    "pt_gpu_upload_lights": (ctypes.c_int, [ctypes.c_void_p, P(f32), u32]),
    "pt_gpu_upload_env": (ctypes.c_int, [ctypes.c_void_p, P(f32), u32, u32, P(f32), P(f32), P(f32),
                                         P(f32), u32]),
    "pt_gpu_upload_moon": (ctypes.c_int, [ctypes.c_void_p, P(f32), u32, u32]),
    "pt_gpu_upload_light_tree": (ctypes.c_int, [ctypes.c_void_p, P(PtLightTreeNode), u32]),
    "pt_gpu_upload_sdf": (ctypes.c_int, [ctypes.c_void_p, P(f32), u32]),
    "pt_gpu_set_target": (ctypes.c_int, [ctypes.c_void_p, u32, u32]),
    "pt_gpu_read_accum": (ctypes.c_int, [ctypes.c_void_p, P(f32)]),
    "pt_gpu_write_accum": (ctypes.c_int, [ctypes.c_void_p, P(f32)]),
    "pt_gpu_accum_device_ptr": (ctypes.c_int, [ctypes.c_void_p, P(ctypes.c_void_p)]),
    "pt_gpu_render": (ctypes.c_int, [ctypes.c_void_p, P(PtPushHead), P(PtPathParams), u32]),
    "pt_gpu_render_to_host": (ctypes.c_int, [ctypes.c_void_p, P(PtPushHead), P(PtPathParams), u32,
                                             P(f32)]),
    "pt_gpu_get_stats": (ctypes.c_int, [ctypes.c_void_p, P(PtStats)]),
    "pt_gpu_tonemap": (ctypes.c_int, [ctypes.c_void_p, f32, u32, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]),
    "pt_gpu_set_profiling": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "pt_gpu_set_wave_frames": (ctypes.c_int, [ctypes.c_void_p, u32]),
    "pt_gpu_set_traversal": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "pt_gpu_get_traversal_stats": (ctypes.c_int, [ctypes.c_void_p, P(PtTraversalStats)]),
    "pt_gpu_set_debug_limits": (ctypes.c_int, [ctypes.c_void_p, u32, u32]),
    "pt_gpu_set_roulette_freeze": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "pt_gpu_set_render_graphs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "pt_gpu_batch_tuning_gain": (ctypes.c_int, [ctypes.c_void_p, P(ctypes.c_double), P(ctypes.c_double)]),
    "pt_gpu_get_accel_info": (ctypes.c_int, [ctypes.c_void_p, P(PtAccelInfo)]),
    "pt_gpu_batch_render": (ctypes.c_int, [ctypes.c_void_p, P(ctypes.c_void_p), u32, P(PtBatchView), u32, u32]),
    "pt_gpu_batch_read_accum": (ctypes.c_int, [ctypes.c_void_p, u32, P(f32)]),
    "pt_gpu_batch_set_tuning": (ctypes.c_int, [ctypes.c_void_p, P(PtBatchTuning)]),
    "pt_gpu_batch_get_tuning": (ctypes.c_int, [ctypes.c_void_p, P(PtBatchTuning)]),
    "pt_gpu_batch_autotune": (ctypes.c_int, [ctypes.c_void_p, P(ctypes.c_void_p), u32, P(PtBatchView), u32,
                                             P(PtBatchTuning)]),
    "pt_gpu_diff_forward": (ctypes.c_int, [ctypes.c_void_p, P(PtPushHead), P(PtPathParams), u32]),
    "pt_gpu_diff_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                            P(ctypes.c_double), P(ctypes.c_double)]),
    "pt_gpu_diff_get_backward_stats": (ctypes.c_int, [ctypes.c_void_p, P(PtStats)]),
    "pt_gpu_batch_diff_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, P(PtBatchView), u32]),
    "pt_gpu_batch_diff_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                                  P(ctypes.c_double), P(ctypes.c_double)]),
    "pt_gpu_render_noalloc": (ctypes.c_int, [ctypes.c_void_p, P(PtPushHead), P(PtPathParams), u32, u32, u32,
                                             ctypes.c_void_p]),
    "pt_gpu_trace_closest": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, u32,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    # pt_scene.h
    "pt_scene_create": (ctypes.c_int, [P(ctypes.c_void_p)]),
    "pt_scene_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pt_scene_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "pt_scene_clear": (ctypes.c_int, [ctypes.c_void_p]),
    "pt_scene_prim_sphere": (ctypes.c_int, [ctypes.c_void_p, u32, f32, f32, f32, f32, ctypes.c_int, f32,
                                            f32, f32, f32, f32]),
    "pt_scene_prim_plane": (ctypes.c_int, [ctypes.c_void_p, u32, f32, f32, f32, f32, ctypes.c_int, f32,
                                           f32, f32, f32, f32]),
    "pt_scene_prim_set_emission": (ctypes.c_int, [ctypes.c_void_p, u32, f32, f32, f32]),
    "pt_scene_prim_set_orient": (ctypes.c_int, [ctypes.c_void_p, u32, f32, f32, f32, f32]),
    "pt_scene_prim_set_material": (ctypes.c_int, [ctypes.c_void_p, u32, u32]),
    "pt_scene_light_quad": (ctypes.c_int, [ctypes.c_void_p, u32] + [f32] * 14),
    "pt_scene_light_point": (ctypes.c_int, [ctypes.c_void_p, u32] + [f32] * 6),
    "pt_scene_light_sphere": (ctypes.c_int, [ctypes.c_void_p, u32] + [f32] * 7),
    "pt_scene_light_spot": (ctypes.c_int, [ctypes.c_void_p, u32] + [f32] * 11),
    "pt_scene_set_mesh": (ctypes.c_int, [ctypes.c_void_p, P(f32), u32, P(u32), u32, P(u32)]),
    "pt_scene_set_materials": (ctypes.c_int, [ctypes.c_void_p, P(f32), u32]),
    "pt_scene_set_env": (ctypes.c_int, [ctypes.c_void_p, P(f32), u32, u32]),
    "pt_scene_set_moon": (ctypes.c_int, [ctypes.c_void_p, P(f32), u32, u32]),
    "pt_scene_set_camera": (ctypes.c_int, [ctypes.c_void_p, f32, f32, f32, f32, f32, f32]),
    "pt_scene_set_cvar": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_double]),
    "pt_scene_get_cvar": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, P(ctypes.c_double)]),
    "pt_scene_pack": (ctypes.c_int, [ctypes.c_void_p]),
    "pt_scene_packed": (ctypes.c_int, [ctypes.c_void_p, P(PtPackedScene)]),
    "pt_scene_fill_push": (ctypes.c_int, [ctypes.c_void_p, u32, u32, u32, u32, P(PtPushHead),
                                          P(PtPathParams)]),
    "pt_scene_upload": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "pt_scene_exec_cfg": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                         ctypes.c_size_t, P(u32)]),
    "pt_scene_load_cfg": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                         ctypes.c_size_t, P(u32)]),
    "pt_load_radiance_hdr": (ctypes.c_int, [ctypes.c_char_p, P(f32), u32, P(u32), P(u32)]),
    "pt_write_png": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, u32, u32]),
    "pt_write_ppm": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_void_p, u32, u32]),
    "pt_imgdiff": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, u32, u32, ctypes.c_double, P(PtDiffStats),
                                  ctypes.c_void_p]),
    "pt_scene_sdf_leaf": (ctypes.c_int, [ctypes.c_void_p, u32, u32, P(f32), f32, f32, f32, u32, f32, f32, f32]),
    "pt_scene_sdf_combine": (ctypes.c_int, [ctypes.c_void_p, u32, u32, u32, u32, f32, u32, f32, f32, f32]),
    "pt_scene_sdf_wrap": (ctypes.c_int, [ctypes.c_void_p, u32, u32, u32, P(f32), u32, f32, f32, f32]),
    "pt_scene_sdf_remove": (ctypes.c_int, [ctypes.c_void_p, u32]),
    "pt_scene_sdf_clear": (ctypes.c_int, [ctypes.c_void_p]),
    "pt_sdf_cluster_box": (ctypes.c_int, [P(f32), u32, P(f32), P(f32)]),
    "pt_build_light_tree": (ctypes.c_int, [P(PtLightInput), u32, P(PtLightTreeNode), P(u32)]),
    "pt_scene_synth": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_double]),
    "pt_build_analytic_bvh": (ctypes.c_int, [P(f32), u32, P(PtBvhNode), P(u32), P(u32)]),
    "pt_build_triangle_bvh": (ctypes.c_int, [P(f32), u32, P(u32), u32, P(PtBvhNode), P(u32), P(u32),
                                             P(u32)]),
    "pt_build_env_cdf": (ctypes.c_int, [P(f32), u32, u32, P(ctypes.c_uint8), P(f32), P(f32),
                                        P(ctypes.c_double)]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load the product library; raises FileNotFoundError when it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} not found: build it with `python demont-engine_gb300/build.py` "
            "(there is no fallback path)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class PtError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def fptr(a):
    return a.ctypes.data_as(P(f32)) if a is not None else None


def uptr(a):
    return a.ctypes.data_as(P(u32)) if a is not None else None


def nptr(a):
    return a.ctypes.data_as(P(PtBvhNode)) if a is not None else None


def nodes_to_array(nodes_ptr, n):
    """PtBvhNode* -> structured numpy copy (n, 8) of uint32 words."""
    if n == 0:
        return np.zeros((0, 8), np.uint32)
    buf = (ctypes.c_uint32 * (8 * n)).from_address(ctypes.addressof(nodes_ptr.contents))
    return np.frombuffer(buf, dtype=np.uint32).reshape(n, 8).copy()


class Scene:
    """Host scene builder (pt_scene_*): the reference's scene commands, cvars,
    packing rules and the seeded synthetic configs."""

    def __init__(self):
        self.lib = load()
        h = ctypes.c_void_p()
        self._check(self.lib.pt_scene_create(ctypes.byref(h)), h)
        self.h = h

    def _check(self, rc, h=None):
        if rc != PT_OK:
            msg = self.lib.pt_scene_last_error(h if h is not None else self.h)
            raise PtError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.lib.pt_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def synth(self, config_id: int, seed: int = 0, scale: float = 1.0):
        self._check(self.lib.pt_scene_synth(self.h, config_id, seed, scale))
        return self

    def set_cvar(self, name: str, value: float):
        self._check(self.lib.pt_scene_set_cvar(self.h, name.encode(), float(value)))

    def get_cvar(self, name: str) -> float:
        v = ctypes.c_double()
        self._check(self.lib.pt_scene_get_cvar(self.h, name.encode(), ctypes.byref(v)))
        return v.value

    def sphere(self, id, x, y, z, r, mat, rgb, rough=0.0, ior=1.5):
        self._check(self.lib.pt_scene_prim_sphere(self.h, id, x, y, z, r, mat, *rgb, rough, ior))

    def plane(self, id, n, d, mat, rgb, rough=0.0, ior=1.0):
        self._check(self.lib.pt_scene_prim_plane(self.h, id, *n, d, mat, *rgb, rough, ior))

    def emission(self, id, rgb):
        self._check(self.lib.pt_scene_prim_set_emission(self.h, id, *rgb))

    def prim_material(self, id, mat):
        self._check(self.lib.pt_scene_prim_set_material(self.h, id, mat))

    def orient(self, id, q):
        self._check(self.lib.pt_scene_prim_set_orient(self.h, id, *q))

    def light_quad(self, id, pos, n, u, u_half, v_half, rgb):
        self._check(self.lib.pt_scene_light_quad(self.h, id, *pos, *n, *u, u_half, v_half, *rgb))

    def light_point(self, id, pos, rgb):
        self._check(self.lib.pt_scene_light_point(self.h, id, *pos, *rgb))

    def light_sphere(self, id, pos, radius, rgb):
        self._check(self.lib.pt_scene_light_sphere(self.h, id, *pos, radius, *rgb))

    def light_spot(self, id, pos, d, outer_deg, inner_deg, rgb):
        self._check(self.lib.pt_scene_light_spot(self.h, id, *pos, *d, outer_deg, inner_deg, *rgb))

    def mesh(self, positions, indices, mat_ids=None):
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
        idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        mid = None if mat_ids is None else np.ascontiguousarray(mat_ids, np.uint32)
        self._keep_mesh = (pos, idx, mid)
        self._check(self.lib.pt_scene_set_mesh(self.h, fptr(pos), pos.size // 3, uptr(idx),
                                               idx.size // 3, uptr(mid)))

    def materials(self, mats12):
        m = np.ascontiguousarray(mats12, np.float32).reshape(-1)
        self._check(self.lib.pt_scene_set_materials(self.h, fptr(m), m.size // 12))

    def env(self, rgb):
        """rgb: (H, W, 3) float32 lat-long image, or None for no env map."""
        if rgb is None:
            self._check(self.lib.pt_scene_set_env(self.h, None, 0, 0))
            return
        a = np.ascontiguousarray(rgb, np.float32)
        H, W = a.shape[:2]
        self._check(self.lib.pt_scene_set_env(self.h, fptr(a), W, H))

    def moon(self, rgba):
        """Moon surface map (H, W, 4) float32 for the gradient sky, or None."""
        if rgba is None:
            self._check(self.lib.pt_scene_set_moon(self.h, None, 0, 0))
            return
        a = np.ascontiguousarray(rgba, np.float32)
        self._moon_keep = a
        self._check(self.lib.pt_scene_set_moon(self.h, fptr(a), a.shape[1], a.shape[0]))

    def exec_cfg(self, text: str, base_dir: str = "."):
        """Run console/.cfg text; returns (report of skipped lines, count)."""
        buf = ctypes.create_string_buffer(1 << 16)
        n = u32(0)
        rc = self.lib.pt_scene_exec_cfg(self.h, text.encode(), base_dir.encode(), buf, len(buf), ctypes.byref(n))
        self._check(rc)
        return buf.value.decode(), n.value

    def load_cfg(self, path: str, base_dir: str | None = None):
        buf = ctypes.create_string_buffer(1 << 16)
        n = u32(0)
        self._check(self.lib.pt_scene_load_cfg(self.h, path.encode(), base_dir.encode() if base_dir else None,
                                               buf, len(buf), ctypes.byref(n)))
        return buf.value.decode(), n.value

    def sdf_leaf(self, id, shape, params, center, mat, rgb):
        """shape 0 sphere, 1 box, 2 rounded box, 3 torus, 4 capsule; params up to 4 floats."""
        q = (f32 * 4)(*(list(params) + [0.0] * (4 - len(params))))
        self._check(self.lib.pt_scene_sdf_leaf(self.h, id, shape, q, *center, mat, *rgb))

    def sdf_combine(self, id, a, b, op, k, mat, rgb):
        """op 1 smooth union, 2 smooth subtract (b from a), 3 smooth intersect."""
        self._check(self.lib.pt_scene_sdf_combine(self.h, id, a, b, op, k, mat, *rgb))

    def sdf_wrap(self, id, child, op, params, mat, rgb):
        """op 5 fBm displace (amp, freq[, octaves]), 6 twist / 7 bend (rate), 8 repeat
        (px, py, pz), 9 limited repeat (px, py, pz, lx, ly, lz); the child is consumed."""
        q = (f32 * 6)(*(list(params) + [0.0] * (6 - len(params))))
        self._check(self.lib.pt_scene_sdf_wrap(self.h, id, child, op, q, mat, *rgb))

    def camera(self, pos, yaw, pitch, fov_deg):
        self._check(self.lib.pt_scene_set_camera(self.h, *pos, yaw, pitch, fov_deg))

    def packed(self) -> PtPackedScene:
        ps = PtPackedScene()
        self._check(self.lib.pt_scene_packed(self.h, ctypes.byref(ps)))
        return ps

    def push(self, width, height, frame_index=0, reset=1):
        head, prm = PtPushHead(), PtPathParams()
        self._check(self.lib.pt_scene_fill_push(self.h, width, height, frame_index, reset,
                                                ctypes.byref(head), ctypes.byref(prm)))
        return head, prm

    def arrays(self) -> dict:
        """numpy copies of the packed buffers (for tests and inspection)."""
        p = self.packed()

        def f(ptr, n):
            return np.ctypeslib.as_array(ptr, shape=(n,)).copy() if n else np.zeros(0, np.float32)

        def u(ptr, n):
            return np.ctypeslib.as_array(ptr, shape=(n,)).copy() if n else np.zeros(0, np.uint32)

        out = dict(prims=f(p.prims, p.prim_count * 28).reshape(-1, 28),
                   linear=p.linear_prim_count,
                   bvh=nodes_to_array(p.bvh_nodes, p.bvh_node_count),
                   positions=f(p.positions, p.vertex_count * 3).reshape(-1, 3),
                   indices=u(p.indices, p.tri_count * 3).reshape(-1, 3),
                   tri_bvh=nodes_to_array(p.tri_nodes, p.tri_node_count),
                   tri_perm=u(p.tri_perm, p.tri_perm_count),
                   lights=f(p.lights, p.light_count * 20).reshape(-1, 20),
                   env_total=p.env_total_luminance, hdri_count=p.hdri_count)
        if p.env_present:
            out["env_marginal"] = f(p.env_marginal, p.env_h)
            out["env_conditional"] = f(p.env_conditional, p.env_w * p.env_h).reshape(p.env_h, p.env_w)
            out["hdri_dir_pmf"] = f(p.hdri_dir_pmf, 32).reshape(8, 4)
            out["hdri_col"] = f(p.hdri_col, 32).reshape(8, 4)
        return out


def _views_array(views):
    """(scene, width, height, head, params[, frames_per_wave]) tuples -> PtBatchView[]."""
    va = (PtBatchView * len(views))()
    for i, v in enumerate(views):
        va[i].scene, va[i].width, va[i].height = v[0], v[1], v[2]
        va[i].head, va[i].params = v[3], v[4]
        va[i].frames_per_wave = v[5] if len(v) > 5 else 1
    return va


LIGHT_TREE_DTYPE = np.dtype([("aabb_min", "<f4", 3), ("left_first", "<u4"), ("aabb_max", "<f4", 3),
                             ("count", "<u4"), ("cone_axis", "<f4", 3), ("cone_cos_half", "<f4"),
                             ("intensity", "<f4"), ("pad", "<f4", 3)])
LIGHT_INPUT_DTYPE = np.dtype([("type", "<u4"), ("pos", "<f4", 3), ("radius", "<f4"), ("intensity", "<f4", 3),
                              ("dir", "<f4", 3), ("cos_outer", "<f4"), ("u_vec", "<f4", 3), ("v_half", "<f4")])


def build_light_tree(lights: np.ndarray) -> np.ndarray:
    """lights: structured array of LIGHT_INPUT_DTYPE -> nodes (LIGHT_TREE_DTYPE), pt_build_light_tree."""
    lib = load()
    lights = np.ascontiguousarray(lights, LIGHT_INPUT_DTYPE)
    out = np.zeros(max(2 * len(lights) - 1, 1), LIGHT_TREE_DTYPE)
    n = u32(0)
    rc = lib.pt_build_light_tree(lights.ctypes.data_as(P(PtLightInput)), len(lights),
                                 out.ctypes.data_as(P(PtLightTreeNode)), ctypes.byref(n))
    if rc != PT_OK:
        raise PtError(rc, "build_light_tree failed")
    return out[:n.value]


def write_png(path: str, rgba8: np.ndarray):
    a = np.ascontiguousarray(rgba8, np.uint8)
    if load().pt_write_png(path.encode(), a.ctypes.data, a.shape[1], a.shape[0]) != PT_OK:
        raise PtError(-1, f"cannot write {path}")


def write_ppm(path: str, rgba8: np.ndarray):
    a = np.ascontiguousarray(rgba8, np.uint8)
    if load().pt_write_ppm(path.encode(), a.ctypes.data, a.shape[1], a.shape[0]) != PT_OK:
        raise PtError(-1, f"cannot write {path}")


def imgdiff(a: np.ndarray, b: np.ndarray, bad_threshold: float = 0.0, heatmap: bool = False):
    """RGBA8 images -> (PtDiffStats, heat map or None), pt_imgdiff."""
    a = np.ascontiguousarray(a, np.uint8)
    b = np.ascontiguousarray(b, np.uint8)
    st = PtDiffStats()
    hm = np.zeros_like(a) if heatmap else None
    rc = load().pt_imgdiff(a.ctypes.data, b.ctypes.data, a.shape[1], a.shape[0], bad_threshold, ctypes.byref(st),
                           hm.ctypes.data if heatmap else None)
    if rc != PT_OK:
        raise PtError(rc, "imgdiff failed")
    return st, hm


def load_hdr(path: str) -> np.ndarray:
    """Radiance .hdr file -> (H, W, 3) float32 (pt_load_radiance_hdr)."""
    lib = load()
    w, h = u32(0), u32(0)
    if lib.pt_load_radiance_hdr(path.encode(), None, 0, ctypes.byref(w), ctypes.byref(h)) != PT_OK:
        raise PtError(-1, f"cannot read {path}")
    out = np.empty((h.value, w.value, 3), np.float32)
    rc = lib.pt_load_radiance_hdr(path.encode(), fptr(out), out.size, ctypes.byref(w), ctypes.byref(h))
    if rc != PT_OK:
        raise PtError(rc, f"cannot read {path}")
    return out


class Device:
    """One CUDA device context (pt_gpu_*)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        rc = self.lib.pt_gpu_create(ctypes.byref(h), device)
        self.h = h
        if rc != PT_OK:
            msg = self.lib.pt_gpu_last_error(h) if h else b"create failed"
            if h:
                self.lib.pt_gpu_destroy(h)
            self.h = None
            raise PtError(rc, msg.decode())
        self.W = self.H = 0

    def _check(self, rc):
        if rc != PT_OK:
            raise PtError(rc, self.lib.pt_gpu_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.pt_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, scene: Scene):
        self._check(self.lib.pt_scene_upload(scene.h, self.h))

    def upload_moon(self, rgba):
        """Moon surface map (H, W, 4) float32 for the gradient sky's moon disc."""
        a = np.ascontiguousarray(rgba, np.float32)
        self._check(self.lib.pt_gpu_upload_moon(self.h, fptr(a), a.shape[1], a.shape[0]))

    def set_target(self, width, height):
        self._check(self.lib.pt_gpu_set_target(self.h, width, height))
        self.W, self.H = width, height

    def render(self, head, prm, frames=1):
        self._check(self.lib.pt_gpu_render(self.h, ctypes.byref(head), ctypes.byref(prm), frames))

    def render_to_host(self, head, prm, frames, out):
        self._check(self.lib.pt_gpu_render_to_host(self.h, ctypes.byref(head), ctypes.byref(prm),
                                                   frames, fptr(out)))
        return out

    def read_accum(self, out=None):
        if out is None:
            out = np.empty((self.H, self.W, 4), np.float32)
        self._check(self.lib.pt_gpu_read_accum(self.h, fptr(out)))
        return out

    def write_accum(self, a):
        a = np.ascontiguousarray(a, np.float32)
        self._check(self.lib.pt_gpu_write_accum(self.h, fptr(a)))

    def tonemap(self, exposure=1.5, op=0, srgb=False):
        """The accumulation buffer through exposure + tone map -> (H, W, 4) uint8."""
        out = np.empty((self.H, self.W, 4), np.uint8)
        self._check(self.lib.pt_gpu_tonemap(self.h, exposure, op, 1 if srgb else 0, out.ctypes.data, 0))
        return out

    def stats(self) -> PtStats:
        s = PtStats()
        self._check(self.lib.pt_gpu_get_stats(self.h, ctypes.byref(s)))
        return s

    def set_profiling(self, on=True):
        """True/1: events on the overlapped schedule; 2: stages serial (each
        kernel timed alone); 3: as 2 with the counting traversal variants
        (traversal_stats); False/0: off."""
        self._check(self.lib.pt_gpu_set_profiling(self.h, int(on)))

    def set_roulette_freeze(self, mode):
        """1: the next render records its roulette survival probabilities; 2:
        later renders of the same shape reuse them; 0: off (finite differences
        under roulette)."""
        self._check(self.lib.pt_gpu_set_roulette_freeze(self.h, int(mode)))

    def set_render_graphs(self, on=True):
        """Replay each render wave as a cached CUDA graph, or launch every
        kernel directly (default); the images are the same bit for bit."""
        self._check(self.lib.pt_gpu_set_render_graphs(self.h, int(bool(on))))

    def set_debug_limits(self, traverse_cap=0, stack_entries=0):
        """Lower the traversal iteration cap / stack (failure-path tests); 0 = default."""
        self._check(self.lib.pt_gpu_set_debug_limits(self.h, traverse_cap, stack_entries))

    def traversal_stats(self) -> PtTraversalStats:
        """Traversal work of the last render in profiling mode 3."""
        t = PtTraversalStats()
        self._check(self.lib.pt_gpu_get_traversal_stats(self.h, ctypes.byref(t)))
        return t

    def set_traversal(self, mode):
        self._check(self.lib.pt_gpu_set_traversal(self.h, mode))

    def accel_info(self) -> PtAccelInfo:
        a = PtAccelInfo()
        self._check(self.lib.pt_gpu_get_accel_info(self.h, ctypes.byref(a)))
        return a

    def set_wave_frames(self, n):
        self._check(self.lib.pt_gpu_set_wave_frames(self.h, n))

    # ---- batched renders ----
    def batch_render(self, scene_devs, views, frames=1):
        """scene_devs: list of Device (each holding an uploaded scene); views: list of
        (scene index, width, height, head, params)."""
        arr = (ctypes.c_void_p * len(scene_devs))(*[d.h.value if hasattr(d.h, "value") else d.h for d in scene_devs])
        va = _views_array(views)
        self._batch_keep = (arr, va)
        self._check(self.lib.pt_gpu_batch_render(self.h, arr, len(scene_devs), va, len(views), frames))

    def batch_read(self, view, w, h):
        out = np.empty((h, w, 4), np.float32)
        self._check(self.lib.pt_gpu_batch_read_accum(self.h, view, fptr(out)))
        return out

    def batch_autotune(self, scene_devs, views):
        arr = (ctypes.c_void_p * len(scene_devs))(*[d.h.value if hasattr(d.h, "value") else d.h for d in scene_devs])
        va = _views_array(views)
        t = PtBatchTuning()
        self._check(self.lib.pt_gpu_batch_autotune(self.h, arr, len(scene_devs), va, len(views), ctypes.byref(t)))
        return t

    def batch_set_tuning(self, persistent_blocks_per_sm=4, stream_blocks_per_sm=8, use_graph=1, shade_threads=512,
                         camera_tile_w=4, octant_grouping=0):
        t = PtBatchTuning(persistent_blocks_per_sm, stream_blocks_per_sm, use_graph, shade_threads, camera_tile_w,
                          octant_grouping)
        self._check(self.lib.pt_gpu_batch_set_tuning(self.h, ctypes.byref(t)))

    def batch_tuning_gain(self):
        """(default ms, tuned ms) per frame from the last batch_autotune."""
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.pt_gpu_batch_tuning_gain(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    # ---- differentiable renders ----
    def materials(self, mats12):
        """Replace the material table (n x 12 floats: albedo rgb, roughness,
        emission rgb, ior, type, 3 pad) -- the differentiable parameters."""
        m = np.ascontiguousarray(mats12, np.float32).reshape(-1, 12)
        self._check(self.lib.pt_gpu_upload_materials(self.h, fptr(m), m.shape[0]))

    def diff_forward(self, head, prm, frames=1):
        self._check(self.lib.pt_gpu_diff_forward(self.h, ctypes.byref(head), ctypes.byref(prm), frames))

    def diff_backward(self, dl_di, nmat):
        """dl_di: (H, W, 3 or 4) float32 dLoss/dImage.  Returns (grad_albedo,
        grad_emission), each (nmat, 3) float64."""
        g = np.zeros((self.H, self.W, 4), np.float32)
        d = np.asarray(dl_di, np.float32)
        g[..., :3] = d[..., :3]
        ga = np.zeros((nmat, 3), np.float64)
        ge = np.zeros((nmat, 3), np.float64)
        dp = ctypes.POINTER(ctypes.c_double)
        self._check(self.lib.pt_gpu_diff_backward(self.h, g.ctypes.data, 0, ga.ctypes.data_as(dp),
                                                  ge.ctypes.data_as(dp)))
        return ga, ge

    def batch_diff_forward(self, scene_dev, views):
        """views: list of (width, height, head, params[, frames_per_wave]) of the one
        scene held by scene_dev."""
        va = _views_array([(0,) + tuple(v) for v in views])
        self._diff_views = [(v[0], v[1]) for v in views]
        self._check(self.lib.pt_gpu_batch_diff_forward(self.h, scene_dev.h, va, len(views)))

    def batch_diff_backward(self, dl_di_list, nmat):
        """dl_di_list: per view (H, W, 3|4) dLoss/dImage.  Returns (grad_albedo, grad_emission)."""
        parts = []
        for (w, h), d in zip(self._diff_views, dl_di_list):
            g = np.zeros((h, w, 4), np.float32)
            g[..., :3] = np.asarray(d, np.float32)[..., :3]
            parts.append(g.reshape(-1, 4))
        flat = np.ascontiguousarray(np.concatenate(parts, axis=0))
        ga = np.zeros((nmat, 3), np.float64)
        ge = np.zeros((nmat, 3), np.float64)
        dp = ctypes.POINTER(ctypes.c_double)
        self._check(self.lib.pt_gpu_batch_diff_backward(self.h, flat.ctypes.data, 0, ga.ctypes.data_as(dp),
                                                        ge.ctypes.data_as(dp)))
        return ga, ge

    def backward_stats(self) -> PtStats:
        s = PtStats()
        self._check(self.lib.pt_gpu_diff_get_backward_stats(self.h, ctypes.byref(s)))
        return s

    def trace(self, ro4, rd4):
        ro4 = np.ascontiguousarray(ro4, np.float32)
        rd4 = np.ascontiguousarray(rd4, np.float32)
        n = ro4.shape[0]
        hit = np.empty(n, np.uint32)
        t = np.empty(n, np.float32)
        self._check(self.lib.pt_gpu_trace_closest(self.h, ro4.ctypes.data, rd4.ctypes.data, n,
                                                  hit.ctypes.data, t.ctypes.data, 0))
        return hit, t


def material_render_fn(dev: "Device", scene: "Scene", width: int, height: int, frames: int = 1,
                       frame_index: int = 0):
    """A torch.autograd.Function over the differentiable render:
    image = f(albedo, emission), both (n_materials, 3) float tensors, image
    (height, width, 3) float32.  forward uploads the material table with the
    given albedo and emission and runs pt_gpu_diff_forward; backward hands
    dLoss/dImage to pt_gpu_diff_backward (path replay).  Torch is only the
    caller's autograd plumbing here: all rendering runs in the CUDA library."""
    import torch

    packed = scene.packed()
    n = packed.material_count
    base = np.ctypeslib.as_array(packed.materials, (n * 12,)).reshape(n, 12).copy()
    head, prm = scene.push(width, height, frame_index=frame_index, reset=1)

    class _Render(torch.autograd.Function):
        @staticmethod
        def forward(ctx, albedo, emission):
            m = base.copy()
            m[:, 0:3] = albedo.detach().cpu().numpy().astype(np.float32)
            m[:, 4:7] = emission.detach().cpu().numpy().astype(np.float32)
            dev.set_target(width, height)
            dev.materials(m)
            dev.diff_forward(head, prm, frames)
            img = dev.read_accum()[..., :3].copy()
            ctx.dtypes = (albedo.dtype, emission.dtype, albedo.device)
            return torch.from_numpy(img)

        @staticmethod
        def backward(ctx, grad_img):
            ga, ge = dev.diff_backward(grad_img.detach().cpu().numpy().astype(np.float32), n)
            adt, edt, device = ctx.dtypes
            return (torch.from_numpy(ga).to(device=device, dtype=adt),
                    torch.from_numpy(ge).to(device=device, dtype=edt))

    return _Render.apply

