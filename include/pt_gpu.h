/*
 * pt_gpu.h -- C-ABI of the GB300 path-trace hot path (device side).
 *
 * This library replaces the reference's per-frame `pathtrace` compute
 * dispatch: the RHI plugin call sequence
 *   Device::CreateBuffer/WriteBuffer/CreateTexture/WriteTexture
 *   CommandBuffer::BindComputePipeline("pathtrace") / BindBuffer /
 *   PushConstants / Dispatch / Submit / ReadbackTexture
 * (reference: src/rhi/Device.h:34-91, src/rhi/CommandBuffer.h:15-44,
 *  src/rhi_software/SoftwareDevice.cpp:105-120, src/engine/Engine.cpp:6867-6900,
 *  9580-9582) with a handful of plain C entry points.  All buffers use the
 * reference's own layouts byte for byte, so an engine that already packs
 * them for the reference can hand the same bytes over unchanged.
 *
 * Conventions
 *   - Every call returns an int status: PT_OK (0) or a negative PT_ERR_*.
 *     pt_gpu_last_error(ctx) returns a message for the last failure.
 *   - A context owns one CUDA device's buffers; it is single-threaded per
 *     caller (the reference records and submits from one engine thread).
 *   - Host pointers are plain host memory unless a parameter says "device".
 *   - No torch or CUDA types appear in any signature.
 */
#ifndef PT_GPU_H
#define PT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PT_OK               0
#define PT_ERR_INVALID     -1  /* bad argument (null pointer, size, layout) */
#define PT_ERR_CUDA        -2  /* a CUDA runtime call failed */
#define PT_ERR_OOM         -3  /* device allocation failed */
#define PT_ERR_STATE       -4  /* call made in the wrong state (e.g. no target) */
#define PT_ERR_KERNEL      -5  /* a kernel set its error word (overflow, bad index) */
#define PT_ERR_UNSUPPORTED -6  /* feature not built */

typedef struct pt_gpu_ctx pt_gpu_ctx;

/* The 112-byte push-constant head.  Same fields, order and meaning as the
 * reference's PtPush head (src/rhi_software/SoftwareTracer.cpp:38-56,
 * shaders/PathTrace.slang:643-658, filled at src/engine/Engine.cpp:7821-7931). */
typedef struct PtPushHead {
    float    pos_fovtan[4];   /* camera position xyz, tan(fovY/2) */
    float    fwd_aspect[4];   /* forward xyz, width/height */
    float    right_xyz[4];
    float    up_xyz[4];
    uint32_t frame_index;     /* seeds the per-pixel PCG stream */
    uint32_t reset_accum;     /* 1: start a new running mean */
    uint32_t max_bounces;
    uint32_t tlas_present;    /* must be 0: the hardware-RT branch has no CUDA counterpart */
    uint32_t prim_count;
    uint32_t spp;             /* samples per pixel per frame (0 is treated as 1) */
    uint32_t denoiser_enabled;/* only its RNG effect is honoured: sample 0 uses halton_jitter (a
                                 multi-frame call gives its later frames the engine's jitter of
                                 their frame index, Halton(2,3) of frame_index % 16 + 1 minus 0.5) */
    uint32_t env_map_present;
    float    halton_jitter[2];
    float    env_intensity;
    float    env_total_luminance;
} PtPushHead;

/* The push-constant tail fields the in-scope path reads
 * (shaders/PathTrace.slang:660-1218; engine fill src/engine/Engine.cpp:8640-8676,
 *  7869-7905).  Fields of features outside this library (clouds, water, SDF,
 *  ReSTIR, spectral, DOF, motion blur, denoiser G-buffers) are absent and
 *  behave as the reference does when those features are off. */
typedef struct PtPathParams {
    float    refract_budget;        /* w2j_row1.w: max dielectric hops of a shadow ray (0 = opaque) */
    float    firefly_clamp;         /* w2j_row2.w: clampIndirect ceiling (<= 0 disables) */
    uint32_t mis_enabled;           /* r_mis */
    float    accum_ema_alpha;       /* accum_params.x (r_accum_ema_alpha) */
    uint32_t bvh_params[4];         /* linear_prim_count, analytic BVH node count,
                                       triangle count (0 = no mesh), triangle BVH node count */
    uint32_t light_count;
    uint32_t light_tree_enabled;    /* 1: pick lights through the tree uploaded with
                                       pt_gpu_upload_light_tree (r_light_tree, the reference's
                                       default); 0: uniform pick (one random number) */
    uint32_t light_tree_node_count;
    uint32_t rr_start;              /* Russian roulette starts at bounce b >= rr_start; reference: 2 */
    float    sun_and_mode[4];       /* sun dir xyz, sky mode in w (0 gradient, 1 env map, 2 procedural,
                                       3 Hosek-Wilkie, not built) */
    uint32_t stars;                 /* exposure_pad.y/z: procedural-sky stars (must be 0: not built) */
    uint32_t sdf_procedural_ops;    /* SDF ops 5-9 (fBm displace, twist, bend, repeat, limited repeat):
                                       0 read as empty (the reference's default build); 1 evaluated, with
                                       central-difference normals (built with PT_SDF_PROCEDURAL_OPS=1);
                                       2 evaluated, with forward-mode AD normals where sdf_params_f[3] is 0
                                       (also PT_SDF_AUTODIFF=1); shaders/SdfPrimitives.slang:56-68, 504-1245 */
    uint32_t reserved[2];
    /* gradient sky (no env map): the moon and the sun-disc shape
       (shaders/PathTrace.slang:766, 1222-1241; engine fill src/engine/Engine.cpp:8324-8410) */
    float    moon_dir_phase[4];     /* moon dir xyz (y < -0.1: hidden), phase angle in w */
    float    moon_extra[4];         /* size multiplier, distance ratio, disc brightness, - */
    float    sun_extra[4];          /* size multiplier, distance ratio, vertical flatten (1 = round), - */
    float    sun_extra2[4];         /* sun disc brightness, -, -, - */
    /* SDF clusters (shaders/PathTrace.slang:859-885; engine fill src/engine/Engine.cpp:7940-7981) */
    uint32_t sdf_params[4];         /* cluster count (= uploaded), march step budget, -, fractal DE iterations */
    float    sdf_params_f[4];       /* hit epsilon, fractal default power, fractal epsilon growth per step,
                                       r_sdf_normal_mode (0 forward-mode AD, 1 central differences) */
} PtPathParams;

/* 32-byte BVH node, identical to the reference's BvhNode / TriBvhNode
 * (src/renderer/AnalyticBvh.h:195-201, src/renderer/TriangleBvh.h:325-331). */
typedef struct PtBvhNode {
    float    aabb_min[3];
    uint32_t left_first;      /* internal: left child index (right = +1); leaf: first prim */
    float    aabb_max[3];
    uint32_t count;           /* 0 = internal, >0 = leaf prim count */
} PtBvhNode;

/* Per-frame counters of the last pt_gpu_render call. */
typedef struct PtStats {
    uint64_t extension_rays;  /* closest-hit segments traced (camera + bounce rays) */
    uint64_t shadow_rays;     /* transmittance segments traced (incl. refraction hops) */
    uint64_t paths;           /* camera paths started */
    uint32_t frames;
    uint32_t waves;
    double   gpu_ms;          /* device time of the render, CUDA events */
    double   extend_ms;       /* device time inside the closest-hit kernel */
    double   shadow_ms;       /* device time inside the transmittance kernel */
    uint32_t extend_launches;
    uint32_t shadow_launches;
    uint32_t kernel_launches; /* every kernel this render call launched */
    uint32_t graph_replays;   /* waves replayed from a cached CUDA graph unchanged
                                 (pt_gpu_set_render_graphs); 0 when launched directly */
} PtStats;

/* ---- lifecycle (replaces Device::Create(BackendType), src/rhi/Device.cpp:20-48) ---- */
int         pt_gpu_create(pt_gpu_ctx** out_ctx, int device_ordinal);
int         pt_gpu_destroy(pt_gpu_ctx* ctx);
const char* pt_gpu_last_error(const pt_gpu_ctx* ctx);
/* Library build tag, e.g. "demont-gb300 sm_103a". */
const char* pt_gpu_version(void);

/* ---- scene upload (replaces the buffer writes of Engine::EnsurePrimitivesUploaded,
 *      src/engine/Engine.cpp:4743-5070, bound at slots 5 and 18) ----
 * recs28: n records of 28 floats (7 float4) in the reference packing
 *         (v0 pos|normal,radius|d  v1 albedo,rough  v2 type,mat,ior,asuint(id)
 *          v3 prev_pos  v4 emission  v5 orient quat  v6 texture tiles).
 * linear_count: the first linear_count records are tested linearly (planes).
 * nodes/n_nodes: the analytic BVH over records [linear_count, n); n_nodes 0 =
 *         linear scan of all records (reference bvh_params.y == 0). */
int pt_gpu_upload_prims(pt_gpu_ctx* ctx, const float* recs28, uint32_t n,
                        uint32_t linear_count, const PtBvhNode* nodes, uint32_t n_nodes);

/* ---- mesh upload (replaces Engine::RebuildMeshResources, src/engine/Engine.cpp:3752-3911,
 *      slots 3, 4, 19, 20) ----
 * positions: float[3*nv]; indices: uint32[3*nt]; nodes/perm: the triangle BVH
 * and its permuted triangle ids (src/renderer/TriangleBvh.h).
 * mat_ids (nullable, extension): per-triangle index into the material table of
 * pt_gpu_upload_materials; NULL = the reference's gold metal for every triangle. */
int pt_gpu_upload_mesh(pt_gpu_ctx* ctx, const float* positions, uint32_t nv,
                       const uint32_t* indices, uint32_t nt,
                       const PtBvhNode* nodes, uint32_t n_nodes,
                       const uint32_t* perm, uint32_t n_perm,
                       const uint32_t* mat_ids);

/* ---- mesh material table (extension; the reference meshes are all gold metal,
 *      shaders/PathTrace.slang:2655-2658) ----
 * mats: n records of 12 floats: albedo rgb, roughness, emission rgb, ior,
 *       material type (0 Lambert, 1 metal, 2 dielectric) as float, 3 pad. */
int pt_gpu_upload_materials(pt_gpu_ctx* ctx, const float* mats12, uint32_t n);
/* Extension: per analytic record (n == uploaded record count), the material
 * table row it takes albedo / roughness / ior / emission / type from
 * (0xFFFFFFFF = its own record).  NULL, 0 clears. */
int pt_gpu_upload_prim_materials(pt_gpu_ctx* ctx, const uint32_t* mat_ids, uint32_t n);

/* ---- analytic lights (replaces Engine::EnsureLightsUploaded, src/engine/Engine.cpp:5235-5330,
 *      slot 27): n records of 20 floats (5 float4) in the reference packing. ---- */
int pt_gpu_upload_lights(pt_gpu_ctx* ctx, const float* recs20, uint32_t n);

/* ---- environment (replaces Engine::ReloadEnvMap's uploads, src/engine/Engine.cpp:4329-4600,
 *      slots 9, 10, 11 and the push fields hdri_lights_*) ----
 * rgba: float[4*W*H] texels; marginal: float[H]; conditional: float[W*H]
 * (as built by BuildEnvCdf, src/renderer/HdrImage.cpp:169-219);
 * hdri_dir_pmf / hdri_col: n_hdri (<= 8) float4 each (dir xyz + pmf, flux rgb). */
int pt_gpu_upload_env(pt_gpu_ctx* ctx, const float* rgba, uint32_t W, uint32_t H,
                      const float* marginal, const float* conditional,
                      const float* hdri_dir_pmf, const float* hdri_col, uint32_t n_hdri);

/* ---- light tree (replaces the light_tree_nodes buffer of Engine::EnsureLightsUploaded,
 *      src/engine/Engine.cpp:5420-5545; node layout src/renderer/LightTree.h LightTreeNode) ----
 * 64 bytes per node: node 0 is the root; internal nodes (count 0) have children
 * left_first and left_first + 1; leaves (count 1) hold the light index in
 * left_first.  Used when PtPathParams.light_tree_enabled != 0 and
 * light_tree_node_count equals the uploaded count. */
typedef struct PtLightTreeNode {
    float    aabb_min[3];
    uint32_t left_first;
    float    aabb_max[3];
    uint32_t count;
    float    cone_axis[3];
    float    cone_cos_half;
    float    intensity;
    float    pad[3];
} PtLightTreeNode;
int pt_gpu_upload_light_tree(pt_gpu_ctx* ctx, const PtLightTreeNode* nodes, uint32_t n_nodes);

/* ---- SDF clusters (replaces the sdf_clusters buffer, shaders/PathTrace.slang:2163-2305;
 *      host layout src/renderer/AnalyticBvh.h SdfPrim) ----
 * 28 float4 per cluster: aabb_min + asuint(node_count), aabb_max + asuint(material),
 * albedo + roughness, ior + 3 pad, then 8 nodes of 3 float4: asuint(op, shape,
 * child_a, child_b), params, center + pad.  Nodes are evaluated in order; an op
 * combines earlier nodes (smooth union/subtract/intersect, displace); the last
 * node is the cluster's distance.  A cluster whose last node is a fractal leaf
 * (shape 6 Mandelbulb, 7 Mandelbox, 8 Apollonian gasket; params: power or scale,
 * bound) is marched with the fractal estimator (shaders/SdfFractals.slang).  Hit
 * ids of SDF clusters are 0x80000000 | index (fractals: | accepted step << 20).
 * The procedural ops (5-9) evaluate as empty, as in the reference's default build. */
int pt_gpu_upload_sdf(pt_gpu_ctx* ctx, const float* clusters, uint32_t n_clusters);

/* ---- moon surface map (the moon_map texture of the gradient sky's moon disc,
 *      moonDisc, shaders/PathTrace.slang:3212-3353) ----
 * RGBA32F W x H, lat-long over the moon's near side.  Needed only when a dispatch
 * shows the moon (moon_dir_phase.y >= -0.1 with no env map).  W = H = 0 removes it. */
int pt_gpu_upload_moon(pt_gpu_ctx* ctx, const float* rgba, uint32_t W, uint32_t H);

/* ---- render target: the reference's accum_hdr RGBA32F texture, .a = frame count ---- */
int pt_gpu_set_target(pt_gpu_ctx* ctx, uint32_t width, uint32_t height);
int pt_gpu_read_accum(pt_gpu_ctx* ctx, float* host_rgba);          /* ReadbackTexture */
int pt_gpu_write_accum(pt_gpu_ctx* ctx, const float* host_rgba);   /* resume from a saved state */
int pt_gpu_accum_device_ptr(pt_gpu_ctx* ctx, void** device_ptr);  /* zero-copy view, device memory */

/* ---- per-frame dispatch (replaces Dispatch of "pathtrace"; shaders/PathTrace.slang:5450-7930) ----
 * Renders `frames` consecutive frames: frame f uses frame_index = head->frame_index + f
 * and reset_accum only for f == 0 (each later frame continues the running mean),
 * exactly as `frames` back-to-back reference dispatches would.  Frames are
 * batched into device waves; results do not depend on the batching. */
int pt_gpu_render(pt_gpu_ctx* ctx, const PtPushHead* head, const PtPathParams* params,
                  uint32_t frames);
/* Same as pt_gpu_render, then copies the accumulation buffer to host_rgba
 * (W*H*4 floats).  This is the end-to-end call a host engine makes. */
int pt_gpu_render_to_host(pt_gpu_ctx* ctx, const PtPushHead* head, const PtPathParams* params,
                          uint32_t frames, float* host_rgba);
int pt_gpu_get_stats(pt_gpu_ctx* ctx, PtStats* out);

/* ---- output step (the `output` store of shaders/PathTrace.slang:7925-7929) ----
 * The accumulation buffer times `exposure` (the reference's exposure_state: r_exposure
 * when auto exposure is off) through the tone-map operator (tonemapDispatch,
 * :3466-3607; r_tonemap_op: 0 aces, 1 agx, 2 khronos_pbr_neutral, 3 reinhard,
 * 4 linear), optionally the sRGB OETF (the SPIR-V target's), quantised to RGBA8
 * (round to nearest, alpha 255).  rgba8: width*height*4 bytes, host or device. */
#define PT_TONEMAP_ACES     0
#define PT_TONEMAP_AGX      1
#define PT_TONEMAP_KHRONOS  2
#define PT_TONEMAP_REINHARD 3
#define PT_TONEMAP_LINEAR   4
int pt_gpu_tonemap(pt_gpu_ctx* ctx, float exposure, uint32_t op, int srgb_oetf, uint8_t* rgba8, int on_device);
/* on != 0: record CUDA events around every closest-hit and transmittance
 * launch so PtStats.extend_ms / shadow_ms report their device time.
 *   on == 1: the production schedule, in which the next bounce's closest-hit
 *            pass runs on a second stream while this bounce's shadow rays
 *            run (the two event spans overlap, so each kernel's span includes
 *            time shared with the other);
 *   on == 2: the stages run one after another on one stream, so each span is
 *            the kernel's own device time (for per-kernel timing);
 *   on == 3: as 2, with traversal kernels compiled to also count what they
 *            touch (read with pt_gpu_get_traversal_stats; plain renders with
 *            the wide trees and no procedural SDF cluster; results unchanged,
 *            the counting itself costs time, so take kernel times from mode 2). */
int pt_gpu_set_profiling(pt_gpu_ctx* ctx, int on);

/* Traversal work of the last render in profiling mode 3, summed over its
 * closest-hit (ext_*) and transmittance (shadow_*) launches on the 4-wide
 * trees: segments traced, wide nodes whose four child boxes were tested,
 * triangles and analytic primitives tested in leaves, linear (plane) records
 * tested, and traversal-stack pushes and pops (8-byte entries). */
typedef struct PtTraversalStats {
    uint64_t ext_segments, ext_nodes, ext_tris, ext_aprims, ext_linear, ext_push, ext_pop;
    uint64_t shadow_segments, shadow_nodes, shadow_tris, shadow_aprims, shadow_linear, shadow_push,
             shadow_pop;
} PtTraversalStats;
int pt_gpu_get_traversal_stats(pt_gpu_ctx* ctx, PtTraversalStats* out);

/* Traversal structure: 0 (default) = 4-wide SAH trees built on the device at
 * upload from the same primitives (hit ids and distances still follow the
 * reference's first-tested-wins order exactly, via per-primitive reference
 * ranks, and a hit is kept only where the slab test of its reference BVH leaf
 * passes, as the reference walk requires before it tests the primitive);
 * 1 = walk the uploaded reference BVHs in the reference's own order. */
int pt_gpu_set_traversal(pt_gpu_ctx* ctx, int mode);

/* Failure-path testing: lower the per-query traversal iteration cap (default
 * 4,194,304 loop iterations) and the wide-tree traversal stack (default and
 * maximum 64 entries, minimum 4) so that a normal scene exceeds them.  A query
 * that runs into either limit ends with the best hit found so far and sets the
 * context's error word; the call then returns PT_ERR_KERNEL naming the limit,
 * and the context stays usable.  0 restores a default.  The reference-order
 * walk keeps the reference's own stack rule (children are dropped when its
 * 32 / 64-entry stack is full, with no error). */
int pt_gpu_set_debug_limits(pt_gpu_ctx* ctx, uint32_t traverse_cap, uint32_t stack_entries);

/* CUDA-graph replay of pt_gpu_render's waves (no counterpart in the
 * reference; default off).  With it on and profiling off, each wave's launches
 * are captured once into a CUDA graph and replayed by later calls with the same
 * scene, view, size, sample and bounce counts; the frame index and the
 * accumulation reset are read on the device, so a frame loop that advances
 * frame_index replays the same graph.  A call that changes the launch
 * parameters updates the cached graph in place.  Up to 8 graphs are cached per
 * context.  The images are the same bit for bit either way.  Measured on the
 * 256 x 256, 16 spp analytic scene: +5% at one frame per call, -2.4% at 64
 * frames per call (the time between a wave's launches is the slowest rays'
 * latency, not launch overhead), so direct launches stay the default. */
int pt_gpu_set_render_graphs(pt_gpu_ctx* ctx, int on);

typedef struct PtAccelInfo {
    uint32_t traversal;          /* current mode */
    uint32_t mesh_wide;          /* 1 if the mesh wide tree is in use */
    uint32_t prims_wide;         /* 1 if the analytic wide tree is in use */
    uint32_t mesh_wide_nodes;
    uint32_t mesh_wide_depth;
    uint32_t mesh_binary_nodes;  /* SAH binary nodes before the 4-wide collapse */
    uint32_t prims_wide_nodes;
    uint32_t merged_wide_nodes;  /* nodes of the merged tree over triangles and analytic records (0: none);
                                    renders walk it when both parts are present and no SDF cluster is */
    double   mesh_build_ms;      /* device build time of the mesh wide tree */
} PtAccelInfo;
int pt_gpu_get_accel_info(pt_gpu_ctx* ctx, PtAccelInfo* out);

/* Max number of frames batched into one device wave (default: chosen from the
 * frame size so a wave holds about 64 M paths, ~25 GB of path state, halved
 * while the device cannot hold it). 0 restores the default. */
int pt_gpu_set_wave_frames(pt_gpu_ctx* ctx, uint32_t frames_per_wave);

/* ---- batched render (extension: many views of several scenes in one wavefront) ----
 * Each scene is a context that holds its own uploads; `ctx` owns the batch's
 * path state and one RGBA32F accumulation region per view.  One frame of every
 * view is one device wave: all views' pixels run through the same kernels (the
 * persistent traversal mixes scenes within a warp), and the wave's launch
 * sequence is captured once as a CUDA graph and replayed per frame.  Each view
 * behaves exactly like pt_gpu_render of that view on its scene (bit-identical
 * accumulation), frame f of a view using frame_index = head.frame_index + f and
 * reset_accum only for f == 0.  A view with frames_per_wave = n renders n
 * consecutive frames in every wave (a call with `frames` waves renders
 * frames * n frames of it), which fills the device with fewer, larger views. */
typedef struct PtBatchView {
    uint32_t     scene;      /* index into the scenes array */
    uint32_t     width, height;
    uint32_t     frames_per_wave;   /* consecutive frames of this view in each wave (0 = 1, <= 1024) */
    PtPushHead   head;
    PtPathParams params;
} PtBatchView;

/* Launch shape of batched renders; no knob changes a result. */
typedef struct PtBatchTuning {
    uint32_t persistent_blocks_per_sm;   /* grid of the persistent traversal kernels (1..4) */
    uint32_t stream_blocks_per_sm;       /* grid cap of the streaming kernels (shade/resolve, 1..64) */
    uint32_t use_graph;                  /* 1: replay the captured wave graph; 0: launch the wave directly */
    uint32_t shade_threads;              /* shading-kernel block: 512 (default) or 256 threads */
    uint32_t camera_tile_w;              /* pixels of a 32-pixel camera tile along x: 4 (default), 8, 16, 32 */
    uint32_t octant_grouping;            /* 1: the shading kernel groups each block's next-bounce queue
                                            entries by ray direction octant; 0: path order (default) */
    uint32_t reserved[2];
} PtBatchTuning;

int pt_gpu_batch_render(pt_gpu_ctx* ctx, pt_gpu_ctx* const* scenes, uint32_t n_scenes,
                        const PtBatchView* views, uint32_t n_views, uint32_t frames);
int pt_gpu_batch_read_accum(pt_gpu_ctx* ctx, uint32_t view, float* host_rgba);
int pt_gpu_batch_set_tuning(pt_gpu_ctx* ctx, const PtBatchTuning* tuning);
int pt_gpu_batch_get_tuning(pt_gpu_ctx* ctx, PtBatchTuning* tuning);
/* Tunes every PtBatchTuning knob on this batch by coordinate descent from the
 * default: one knob at a time (persistent grid, streaming grid, shading block,
 * camera tile, octant grouping, graph replay), each candidate timed on one
 * frame of the batch, the fastest kept.  The views' accumulation is reset
 * afterwards by the next render with reset_accum.  Writes the choice to *chosen
 * (nullable); pt_gpu_batch_tuning_gain reports the default's and the chosen
 * shape's frame times from that search. */
int pt_gpu_batch_autotune(pt_gpu_ctx* ctx, pt_gpu_ctx* const* scenes, uint32_t n_scenes,
                          const PtBatchView* views, uint32_t n_views, PtBatchTuning* chosen);
int pt_gpu_batch_tuning_gain(pt_gpu_ctx* ctx, double* default_ms, double* tuned_ms);

/* ---- differentiable render (extension: path-replay adjoint) ----
 * The reference has no derivative path; these two calls are shaped like the
 * forward/backward of a torch.autograd.Function whose inputs are the material
 * table (pt_gpu_upload_materials: per-row albedo and emission) and whose output
 * is the accumulation image.
 *
 * pt_gpu_diff_forward renders exactly like pt_gpu_render (same image, bit for
 * bit) and also records the radiance of every sample (16 B per pixel, frame
 * and sample).  It needs head.reset_accum != 0 and no EMA (the image is the
 * mean of the samples), firefly_clamp <= 0 (the clamp is not differentiable),
 * refract_budget <= 4, a material table of at most 4096 rows, and traversal
 * mode 0.
 *
 * pt_gpu_diff_backward takes dLoss/dImage (width*height RGBA floats, .a
 * ignored; on_device != 0: a 16-byte aligned device pointer) and replays the
 * recorded paths from their stored seeds -- nothing per vertex is stored -- to
 * produce dLoss/d(albedo) and dLoss/d(emission) per material row (3 doubles a
 * row each, nullable).  Per path vertex the albedo factor scales everything the
 * path collects after that vertex's emission, so its derivative is
 * (sample radiance - radiance so far) / albedo; emission's is the throughput;
 * a dielectric crossed by a visible shadow ray contributes that NEE term over
 * its albedo.  Russian-roulette survival probabilities are held fixed (an
 * unbiased gradient of the expected image).  Uploads or a target change after
 * the forward invalidate it (PT_ERR_STATE). */
int pt_gpu_diff_forward(pt_gpu_ctx* ctx, const PtPushHead* head, const PtPathParams* params,
                        uint32_t frames);
int pt_gpu_diff_backward(pt_gpu_ctx* ctx, const float* dl_di_rgba, int on_device,
                         double* grad_albedo, double* grad_emission);
/* Batched form (many views of one scene in one wavefront, one frame each):
 * the gradient of a loss over all views' images.  views[i].scene must be 0
 * (the one scene context); the views' accumulation regions are read with
 * pt_gpu_batch_read_accum.  dl_di_rgba holds every view's dLoss/dImage
 * back to back in view order (sum of width*height RGBA floats). */
int pt_gpu_batch_diff_forward(pt_gpu_ctx* ctx, pt_gpu_ctx* scene, const PtBatchView* views,
                              uint32_t n_views);
int pt_gpu_batch_diff_backward(pt_gpu_ctx* ctx, const float* dl_di_rgba, int on_device,
                               double* grad_albedo, double* grad_emission);
/* PtStats of the last backward replay (pt_gpu_get_stats keeps the forward's). */
int pt_gpu_diff_get_backward_stats(pt_gpu_ctx* ctx, PtStats* out);

/* Finite-difference checks under Russian roulette.  With common random numbers
 * alone, a roulette decision u > p(theta) flips for a few samples when a
 * material parameter moves by eps, and each flip changes its sample by O(1/p):
 * the per-sample finite difference is noise.  mode 1 makes the next
 * pt_gpu_render store every survival probability it draws against (per
 * sample, path vertex); mode 2 makes later pt_gpu_render calls of the same
 * width, height, frame count, spp and depth use those stored probabilities
 * instead of computing them, so that renders at theta +- eps follow the same
 * paths and each sample is a smooth function of the parameters -- the
 * estimator whose gradient pt_gpu_diff_backward computes (it holds the
 * probabilities fixed too).  The image of the recording render is unchanged.
 * mode 0 (default) stops and frees the record.  Memory: 4 bytes per sample
 * and bounce.  PT_ERR_STATE: mode 2 with nothing recorded, or a replaying
 * render of another shape. */
int pt_gpu_set_roulette_freeze(pt_gpu_ctx* ctx, int mode);

/* ---- allocation-free render (no counterpart in the reference) ----
 * For callers that must not allocate device memory while rendering: an engine
 * that reserved its whole device budget up front, a frame loop that cannot
 * afford the implicit synchronisation cudaMalloc/cudaFree may cause, or a
 * plugin whose host application accounts for every device byte.  Same result
 * as pt_gpu_render on the same inputs, but the per-wave path state lives in a
 * fixed file-scope device array inside the library and the caller passes its
 * own accumulation buffer: accum_device = width*height*4 floats of DEVICE
 * memory, 16-byte aligned, read and updated in place (.a = frame count).
 * Nothing in this call allocates (no cudaMalloc, cudaFree or allocating
 * library routine).  The scene must have been uploaded to ctx beforehand.
 * Limits: width*height <= 65536 pixels (e.g. 256 x 256); larger frames return
 * PT_ERR_INVALID.  The array (about 23.5 MiB) is held by every GPU that loads
 * the library until the process exits.  All calls on a device share it and it
 * keeps the last call's contents (each call clears what must start at zero);
 * calls that overlap on the same GPU race and must be serialised.  The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress
 * with that device current): make that first call before any stream capture. */
int pt_gpu_render_noalloc(pt_gpu_ctx* ctx, const PtPushHead* head, const PtPathParams* params,
                          uint32_t width, uint32_t height, uint32_t frames, float* accum_device);

/* ---- parity probe: traceScene for arbitrary rays (shaders/PathTrace.slang:2331-2693) ----
 * ray_o: n float4 (origin xyz, w unused); ray_d: n float4 (direction xyz,
 * w = initial closest distance; <= 0 means the reference's 1e30).
 * hit_id out: 0xFFFFFFFF = miss; (0 << 30 | slot) = analytic record `slot` of the
 * uploaded buffer; (1u << 30 | tri) = original triangle index; (1u << 31 | c) = SDF
 * cluster c (fractal clusters also carry the accepted step << 20), sphere-traced
 * with the reference's defaults (128 steps, epsilon 1e-4, fractal: 12 DE
 * iterations, power 8, epsilon growth 1) and the procedural ops 5-9 off, as in the
 * reference's default build (clusters holding them are never hit here; renders
 * evaluate them under PtPathParams.sdf_procedural_ops).
 * t out: hit distance.
 * on_device != 0: all four pointers are device pointers. */
int pt_gpu_trace_closest(pt_gpu_ctx* ctx, const float* ray_o, const float* ray_d,
                         uint32_t n, uint32_t* hit_id, float* t, int on_device);

#ifdef __cplusplus
}
#endif

#endif /* PT_GPU_H */
