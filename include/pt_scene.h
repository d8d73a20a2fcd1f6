/*
 * pt_scene.h -- C-ABI of the host-side scene builder that feeds pt_gpu.h.
 *
 * It keeps the reference's scene API and packing rules so the GPU path is a
 * drop-in for the reference engine's upload step:
 *   - analytic prims keyed by user id in id order (the reference's
 *     std::map<uint32_t, AnalyticPrim>, src/engine/Engine.h:836), planes
 *     first, finite prims permuted into BVH leaf order, 28 floats per prim
 *     (src/engine/Engine.cpp:4743-5003);
 *   - the binary centroid-median BVHs (src/renderer/AnalyticBvh.cpp:369-486,
 *     src/renderer/TriangleBvh.cpp:33-169), bit-identical trees;
 *   - analytic lights, 20 floats per light (src/engine/Engine.cpp:5235-5330,
 *     commands light_point/spot/sphere/quad at :20308-20420);
 *   - env map: HDRI bright-cluster extraction + env CDF
 *     (src/engine/Engine.cpp:4329-4580, src/renderer/HdrImage.cpp:169-219);
 *   - camera basis (src/renderer/Camera.h:18-30) and the push fill
 *     (src/engine/Engine.cpp:7821-7931, 8640-8676);
 *   - the in-scope cvars with the reference defaults.
 * It also holds the seeded synthetic scene generators used by the benchmark.
 */
#ifndef PT_SCENE_H
#define PT_SCENE_H

#include <stdint.h>
#include "pt_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pt_scene pt_scene;

/* material ids as in the reference (src/engine/Engine.h:187) */
#define PT_MAT_LAMBERT    0
#define PT_MAT_METAL      1
#define PT_MAT_DIELECTRIC 2

int         pt_scene_create(pt_scene** out);
int         pt_scene_destroy(pt_scene* s);
const char* pt_scene_last_error(const pt_scene* s);
int         pt_scene_clear(pt_scene* s);

/* prim_sphere <id> <x> <y> <z> <radius> <mat> <r> <g> <b> [roughness] [ior]
 * (src/engine/Engine.cpp:16783-16832) */
int pt_scene_prim_sphere(pt_scene* s, uint32_t id, float x, float y, float z, float radius,
                         int material, float r, float g, float b, float roughness, float ior);
/* prim_plane <id> <nx> <ny> <nz> <d> <mat> <r> <g> <b> [roughness] [ior]
 * (src/engine/Engine.cpp:16834-16880) */
int pt_scene_prim_plane(pt_scene* s, uint32_t id, float nx, float ny, float nz, float d,
                        int material, float r, float g, float b, float roughness, float ior);
/* per-prim emission (W/sr per channel) and orientation quaternion (xyzw) */
int pt_scene_prim_set_emission(pt_scene* s, uint32_t id, float r, float g, float b);
int pt_scene_prim_set_orient(pt_scene* s, uint32_t id, float qx, float qy, float qz, float qw);
/* Extension: make the prim take albedo, roughness, ior, emission and material
 * type from row `mat` of the material table (the differentiable parameters);
 * 0xFFFFFFFF restores the prim's own record values. */
int pt_scene_prim_set_material(pt_scene* s, uint32_t id, uint32_t mat);

/* light_quad <id> <x y z> <nx ny nz> <ux uy uz> <u_half> <v_half> <r g b>
 * (src/engine/Engine.cpp:20403-20450) */
int pt_scene_light_quad(pt_scene* s, uint32_t id, float x, float y, float z,
                        float nx, float ny, float nz, float ux, float uy, float uz,
                        float u_half, float v_half, float r, float g, float b);
int pt_scene_light_point(pt_scene* s, uint32_t id, float x, float y, float z,
                         float r, float g, float b);
int pt_scene_light_sphere(pt_scene* s, uint32_t id, float x, float y, float z, float radius,
                          float r, float g, float b);
int pt_scene_light_spot(pt_scene* s, uint32_t id, float x, float y, float z,
                        float dx, float dy, float dz, float outer_deg, float inner_deg,
                        float r, float g, float b);

/* Triangle mesh in world space.  mat_ids (nullable) index the material table. */
int pt_scene_set_mesh(pt_scene* s, const float* positions, uint32_t nv,
                      const uint32_t* indices, uint32_t nt, const uint32_t* mat_ids);
/* mats: n records of 12 floats (see pt_gpu_upload_materials) */
int pt_scene_set_materials(pt_scene* s, const float* mats12, uint32_t n);

/* Env map from linear RGB float[3*W*H] (rows top to bottom, the reference's
 * LoadRadianceHdr layout).  Runs the reference's cluster extraction with
 * r_hdri_extract_percentile and builds the masked CDF.  W = H = 0 clears it.
 * A "black env" is an all-zero image: present, total luminance 0. */
int pt_scene_set_env(pt_scene* s, const float* rgb, uint32_t W, uint32_t H);

/* Moon surface map for the gradient sky (the reference engine's moon_map
 * texture): RGBA float[4*W*H].  W = H = 0 clears it. */
int pt_scene_set_moon(pt_scene* s, const float* rgba, uint32_t W, uint32_t H);

/* Camera (src/renderer/Camera.h): position, yaw/pitch (radians), vertical fov (deg). */
int pt_scene_set_camera(pt_scene* s, float x, float y, float z, float yaw, float pitch,
                        float fov_deg);

/* In-scope cvars with the reference defaults (names as in src/engine/Engine.cpp):
 * r_max_bounces 8, r_spp 1, r_mis 1, r_firefly_clamp 10, r_caustics 1,
 * r_refract_bounces 4, r_env_intensity 1, r_accum_ema_alpha 0,
 * r_analytic_bvh_threshold 16, r_hdri_extract_percentile 0.005, r_light_tree 1,
 * r_rr_start 2 (extension), r_denoiser 0; gradient sky (no env map): r_sun_elevation 30,
 * r_sun_azimuth 135 (degrees), r_sun_size 1, r_sun_disc_brightness 1, r_sun_horizon_flatten 1,
 * r_moon_size 1, r_moon_disc_brightness 0.7; output step: r_exposure 1.5, r_tonemap_op 0 (aces);
 * SDF: r_sdf_max_iters 128, r_sdf_epsilon 1e-4, r_sdf_fractal_power 8, r_sdf_fractal_iters 12,
 * r_sdf_de_eps_scale 1, r_sdf_normal_mode 0, r_sdf_displace_octaves 4; r_sdf_procedural_ops 0
 * stands in for the reference's build flags (1: PT_SDF_PROCEDURAL_OPS, ops 5-9 evaluated with
 * central-difference normals; 2: also PT_SDF_AUTODIFF, forward-mode AD normals by r_sdf_normal_mode).
 * Returns PT_ERR_INVALID for unknown names. */
int pt_scene_set_cvar(pt_scene* s, const char* name, double value);
int pt_scene_get_cvar(const pt_scene* s, const char* name, double* value);

/* Pack everything (idempotent; called by the accessors below when dirty). */
int pt_scene_pack(pt_scene* s);

/* Views of the packed buffers (valid until the next mutation). */
typedef struct PtPackedScene {
    const float*     prims;        /* 28 floats per record */
    uint32_t         prim_count;
    uint32_t         linear_prim_count;
    const PtBvhNode* bvh_nodes;
    uint32_t         bvh_node_count;
    const float*     positions;
    uint32_t         vertex_count;
    const uint32_t*  indices;
    uint32_t         tri_count;
    const PtBvhNode* tri_nodes;
    uint32_t         tri_node_count;
    const uint32_t*  tri_perm;
    uint32_t         tri_perm_count;
    const uint32_t*  tri_mat_ids;   /* NULL when the mesh has no material ids */
    const float*     materials;     /* 12 floats per material */
    uint32_t         material_count;
    const float*     lights;        /* 20 floats per light */
    uint32_t         light_count;
    const float*     env_rgba;
    uint32_t         env_w, env_h;
    const float*     env_marginal;
    const float*     env_conditional;
    double           env_total_luminance;
    uint32_t         hdri_count;
    const float*     hdri_dir_pmf;  /* 8 float4 */
    const float*     hdri_col;      /* 8 float4 */
    uint32_t         env_present;
    const uint32_t*  prim_mat_ids;  /* per packed record, NULL when no prim uses the table */
    const float*     moon_rgba;     /* moon surface map (RGBA, moon_w x moon_h), NULL when unset */
    uint32_t         moon_w, moon_h;
    const PtLightTreeNode* light_tree;   /* built over the packed lights, NULL when there are none */
    uint32_t         light_tree_node_count;
    const float*     sdf_clusters;  /* 28 float4 per cluster (pt_gpu_upload_sdf layout), id order */
    uint32_t         sdf_count;
} PtPackedScene;
int pt_scene_packed(pt_scene* s, PtPackedScene* out);

/* Push head + tail for frame `frame_index` of a W x H target. */
int pt_scene_fill_push(pt_scene* s, uint32_t width, uint32_t height, uint32_t frame_index,
                       uint32_t reset_accum, PtPushHead* head, PtPathParams* params);

/* Upload the packed scene into a GPU context (all pt_gpu_upload_* calls). */
int pt_scene_upload(pt_scene* s, pt_gpu_ctx* ctx);

/* ---- scene fixtures in the reference's console (.cfg) syntax ----
 * One command per line; `//` starts a comment, a line starting with `#` is a
 * comment.  Executed (src/engine/Engine.cpp:16783-18060, 20308-20450, 2487-2502):
 *   prim_sphere <id> <x y z> <r> <lambert|metal|dielectric> <r g b> [rough] [ior]
 *   prim_plane <id> <nx ny nz> <d> <material> <r g b>
 *   prim_set_albedo|emission|pos|normal <id> <x y z>, prim_set_roughness|ior|radius|plane_d <id> <v>,
 *   prim_set_material <id> <material>, prim_set_rotation <id> <qx qy qz qw>, prim_remove <id>, prim_clear
 *   light_point|spot|sphere|quad (argument orders as the reference's commands), light_remove <id>, light_clear
 *   cam_pos <x y z>, cam_yaw <deg>, cam_pitch <deg>, cam_fov <deg>
 *   r_sky_mode <gradient|hdri|procedural|hosek>, r_env_map <path.hdr> (relative to base_dir),
 *   sdf_sphere|box|round_box|torus|capsule, sdf_mandelbulb|mandelbox|apollonian,
 *   sdf_smin|sdf_smax|sdf_sdiff, sdf_displace_noise|sdf_twist|sdf_bend|sdf_repeat|
 *   sdf_repeat_limited, sdf_remove, sdf_clear
 *   (argument orders as the reference's commands),
 *   r_denoiser <off|...>, and every numeric cvar of pt_scene_set_cvar (incl. app_window_width/height,
 *   r_capture_seed, r_show_stars).
 * Lines outside the path (water, post-processing, denoiser settings, clouds,
 * SDF, editor, ...) are skipped: `skipped` (nullable, NUL-terminated, truncated
 * to skipped_len) lists each with the reason and *n_skipped counts them.  A
 * malformed in-scope line is reported too; the other lines still run and the
 * call returns PT_ERR_INVALID naming the first bad line. */
int pt_scene_exec_cfg(pt_scene* s, const char* text, const char* base_dir, char* skipped, size_t skipped_len,
                      uint32_t* n_skipped);
/* base_dir NULL: paths relative to the file's directory (the reference engine
 * resolves them against its working directory: pass that). */
int pt_scene_load_cfg(pt_scene* s, const char* path, const char* base_dir, char* skipped, size_t skipped_len,
                      uint32_t* n_skipped);

/* Radiance RGBE .hdr reader (the reference's LoadRadianceHdr contract,
 * src/renderer/HdrImage.cpp:104-167: -Y h +X w layout, adaptive RLE or flat
 * scanlines, value = mantissa * 2^(exponent - 136)).  rgb NULL: size query;
 * else capacity_floats >= 3*w*h. */
int pt_load_radiance_hdr(const char* path, float* rgb, uint32_t capacity_floats, uint32_t* width,
                         uint32_t* height);

/* ---- SDF clusters (src/engine/Engine.cpp:18605-18990 sdf_* commands) ----
 * A leaf cluster: shape 0 sphere (params: r), 1 box (hx hy hz), 2 rounded box
 * (hx hy hz corner_r), 3 torus (R r, XZ plane), 4 capsule (half_h r, along Y),
 * 6 Mandelbulb (power, bound), 7 Mandelbox (scale, bound), 8 Apollonian gasket
 * (scale, bound), at center, material 0/1/2 with albedo.  A combined cluster: op 1 smooth union,
 * 2 smooth subtract (b from a), 3 smooth intersect of clusters a and b with
 * smoothing k; a and b are consumed (the reference's sdf_smin/sdf_sdiff/sdf_smax).
 * Bounding boxes follow ComputeSdfAabb (src/renderer/AnalyticBvh.cpp:335-348). */
int pt_scene_sdf_leaf(pt_scene* s, uint32_t id, uint32_t shape, const float params[4], float x, float y,
                      float z, uint32_t material, float r, float g, float b);
int pt_scene_sdf_combine(pt_scene* s, uint32_t id, uint32_t a, uint32_t b, uint32_t op, float k,
                         uint32_t material, float r, float g, float bl);
/* A wrapped cluster (the reference's sdf_displace_noise / sdf_twist / sdf_bend /
 * sdf_repeat / sdf_repeat_limited, src/engine/Engine.cpp:19095-19400): one op node
 * over the child cluster, which is consumed.  op 5 fBm displace (amp > 0, freq > 0,
 * octaves clamped to 1..6), 6 twist about y (rate rad/m), 7 bend about x (rate rad/m),
 * 8 repetition (periods px py pz; 0 = none on that axis), 9 limited repetition
 * (periods, then integer half-extents 0..1023 per axis).  params: op 5 {amp, freq,
 * octaves}, 6/7 {rate}, 8 {px, py, pz}, 9 {px, py, pz, lx, ly, lz}.  A warp (6-9)
 * over a child that already holds one is refused, as in the reference.  The
 * renderer evaluates these ops only when PtPathParams.sdf_procedural_ops is set. */
int pt_scene_sdf_wrap(pt_scene* s, uint32_t id, uint32_t child, uint32_t op, const float* params,
                      uint32_t material, float r, float g, float b);
int pt_scene_sdf_remove(pt_scene* s, uint32_t id);
int pt_scene_sdf_clear(pt_scene* s);
/* Bounding box of `count` nodes in the reference's SdfNode layout (12 words
 * each: op, shape, child_a, child_b as uint32, params[4], center[3], pad), as
 * the scene builder computes it for a cluster (exposed for parity tests). */
int pt_sdf_cluster_box(const float* nodes12, uint32_t count, float* lo, float* hi);

/* Light-tree builder (src/renderer/LightTree.cpp:BuildLightTree): binary
 * centroid-median tree over the lights, leaves of one light, cone-bounded
 * clusters, bit-identical to the reference's.  One input per light, in light
 * order, with dir and u_vec already rotated by the light's orientation
 * (src/engine/Engine.cpp:5479-5506).  out: capacity 2n - 1 nodes. */
typedef struct PtLightInput {
    uint32_t type;          /* 0 point, 1 spot, 2 sphere, 3 quad */
    float    pos[3];
    float    radius;
    float    intensity[3];
    float    dir[3];
    float    cos_outer;
    float    u_vec[3];
    float    v_half;
} PtLightInput;
int pt_build_light_tree(const PtLightInput* lights, uint32_t n, PtLightTreeNode* out, uint32_t* n_nodes);

/* ---- capture and comparison (r_capture_format png|ppm, src/engine/CaptureFormat.h;
 *      tools/imgdiff/ImgDiff.h) ----
 * rgba8: w*h*4 bytes, rows top to bottom.  The PNG is 8-bit RGBA (stored deflate
 * blocks); the PPM is binary P6 RGB. */
int pt_write_png(const char* path, const uint8_t* rgba8, uint32_t w, uint32_t h);
int pt_write_ppm(const char* path, const uint8_t* rgba8, uint32_t w, uint32_t h);
typedef struct PtDiffStats {
    double   max_delta, mean_delta, rms_delta;   /* per-pixel Euclidean RGBA distance */
    double   bad_percent;                        /* share of pixels above bad_threshold */
    uint64_t total_pixels, bad_pixels;
} PtDiffStats;
/* diff_rgba (nullable): w*h*4 heat map of the distance, scaled to the maximum. */
int pt_imgdiff(const uint8_t* a, const uint8_t* b, uint32_t w, uint32_t h, double bad_threshold,
               PtDiffStats* out, uint8_t* diff_rgba);

/* Seeded synthetic scenes (PCG32 stream, seed 0x5EED + config id):
 *   0: 64 spheres + 4 boxes (12-tri meshes) + one 1x1 quad light (radiance 15), black env;
 *   1: 200 displaced icospheres (nu = 22, 9680 tris each) on a 512x512 quad-grid ground,
 *      1024 spheres, 2048x1024 log-normal env with a 0.5 deg sun disc of 1e4, 256 materials;
 *   3: differentiable-render scene: 512 spheres in [-20,20]^3 and ~200k triangles (20
 *      icospheres, 4 boxes, a 56x56-quad floor) on a 256-row material table of which 16
 *      rows are emissive, the 1x1 quad light, black env; 32 spp, depth 6, no firefly clamp;
 *   4: inverse-rendering scene: config 1's terrain in a 120 x 120 arena with ~1M triangles
 *      (80 icospheres + 340x340-quad ground), 256 spheres, the same env, 1024 Lambert rows
 *      with albedo U[0.2,0.8]; ground patch k (56x56 patches) takes row 389k mod 1024; 16 spp, depth 8,
 *      no firefly clamp.
 * scale (0 < scale <= 1) shrinks the triangle/sphere/env counts for fast tests
 * (1 = the full configuration).  Sets the camera and cvars of the config. */
int pt_scene_synth(pt_scene* s, int config_id, uint64_t seed, double scale);

/* ---- reference builders, exposed for parity tests ---- */
/* AnalyticBvh::Build over (center, radius, prim_id) records (5 x 4 bytes each).
 * nodes_out capacity >= 2n; perm_out capacity n.  Returns node count via *n_nodes. */
int pt_build_analytic_bvh(const float* centers_radii /* 4 floats per prim */, uint32_t n,
                          PtBvhNode* nodes_out, uint32_t* n_nodes, uint32_t* perm_out);
/* TriangleBvh::Build; nodes_out capacity >= 2*nt; perm_out capacity nt. */
int pt_build_triangle_bvh(const float* positions, uint32_t nv, const uint32_t* indices,
                          uint32_t n_index, PtBvhNode* nodes_out, uint32_t* n_nodes,
                          uint32_t* perm_out, uint32_t* n_perm);
/* BuildEnvCdf (mask may be NULL); returns the total in *total. */
int pt_build_env_cdf(const float* rgb, uint32_t W, uint32_t H, const uint8_t* mask,
                     float* marginal, float* conditional, double* total);

#ifdef __cplusplus
}
#endif

#endif /* PT_SCENE_H */
