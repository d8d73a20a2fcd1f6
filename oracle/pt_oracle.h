/*
 * pt_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference path tracer (shaders/PathTrace.slang,
 * shaders/PathTraceMath.slang) that the GPU results are verified against.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * it; the product never links or calls it.
 *
 * Two instantiations of one template:
 *   fp32: same operation order as the shader, no FMA contraction, IEEE
 *         division and square root, and the same polynomial sin/cos/atan2/acos
 *         as the GPU kernels -> the GPU image must equal it bit for bit;
 *   fp64: the same algorithm in double precision with libm transcendentals
 *         -> the semantic oracle converged images are compared against.
 * Parity pinning: traversal/BVH/CDF contracts are pinned against the
 * reference's own test cases and against the reference builders compiled from
 * source (oracle/_ref); image-level HDR parity has no reference golden (the
 * reference ships only 8-bit Metal PNGs) and is pinned by the FP64 instance.
 */
#ifndef PT_ORACLE_H
#define PT_ORACLE_H

#include <stdint.h>
#include "../include/pt_scene.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OracleCounters {
    uint64_t rays;          /* closest-hit queries (traceScene calls) */
    uint64_t nodes;         /* BVH nodes fetched (analytic + triangle) */
    uint64_t tris;          /* triangles tested */
    uint64_t prims;         /* analytic records tested */
    uint64_t ext_rays;      /* camera + bounce segments */
    uint64_t shadow_rays;   /* transmittance segments */
    uint64_t ext_nodes;     /* nodes / triangles / records of extension segments only */
    uint64_t ext_tris;
    uint64_t ext_prims;
} OracleCounters;

/* traceScene for n rays (same encoding as pt_gpu_trace_closest). */
int oracle_trace(const PtPackedScene* scene, const PtPushHead* head, const PtPathParams* params,
                 const float* ray_o, const float* ray_d, uint32_t n, uint32_t* hit_id, float* t,
                 int fp64, OracleCounters* counters);

/* Render `frames` frames of a W x H target into accum_rgba (in/out, W*H*4
 * floats), pixels restricted to [x0,x1) x [y0,y1) (pass 0,0,W,H for all).
 * threads <= 0: all hardware threads.  fp64 != 0: double-precision instance
 * (accumulation in double, result rounded to float). */
int oracle_render(const PtPackedScene* scene, const PtPushHead* head, const PtPathParams* params,
                  uint32_t W, uint32_t H, uint32_t frames, float* accum_rgba,
                  uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                  int fp64, int threads, OracleCounters* counters);

/* The extension rays that bounce `bounce` of frame head->frame_index traces
 * (fp32 instance: the rays the GPU render traces, bit for bit), for every
 * sample of every pixel of [x0,x1) x [y0,y1): float4 slot
 * ((y - y0) * (x1 - x0) + (x - x0)) * spp + s of ray_o / ray_d (w = 0).
 * Samples whose path ended earlier keep a zero direction. */
int oracle_capture_rays(const PtPackedScene* scene, const PtPushHead* head, const PtPathParams* params,
                        uint32_t W, uint32_t H, uint32_t bounce, uint32_t x0, uint32_t y0, uint32_t x1,
                        uint32_t y1, float* ray_o, float* ray_d, int threads);

/* The reference's Software-backend preview estimator (primary hit, sky-lit
 * ambient, one sun shadow ray, emission; running mean), for a timed CPU
 * baseline only: one frame into accum_rgba (H x W x 4). */
int oracle_software_preview(const PtPackedScene* scene, const PtPushHead* head, const PtPathParams* params,
                            uint32_t W, uint32_t H, float* accum_rgba, int threads, OracleCounters* counters);
/* Environment importance sampling for n uniform pairs (xu, xv): sampled
 * directions (x, y, z, 0), their pdf as sampled, and pdfEnvMapDir of each. */
int oracle_env_sample(const PtPackedScene* scene, const PtPushHead* head, const PtPathParams* params, uint32_t n,
                      const float* xu, const float* xv, float* dir4, float* pdf, float* pdf_of_dir);
/* Adjoint oracle: dLoss/d(albedo) and dLoss/d(emission) per material-table
 * row (3 doubles a row each) of a render of `frames` frames from reset, for
 * dLoss/dImage = dl_di_rgba (W*H*4 floats, .a ignored).  The paths are the
 * fp32 instance's (the GPU's paths bit for bit); each sample's contributions
 * are differentiated term by term in double (no suffix sums), with the
 * Russian-roulette probabilities held fixed.  -7: firefly clamp enabled. */
int oracle_adjoint(const PtPackedScene* scene, const PtPushHead* head, const PtPathParams* params,
                   uint32_t W, uint32_t H, uint32_t frames, const float* dl_di_rgba, int threads,
                   double* grad_albedo, double* grad_emission);

/* Output step: RGBA8 of n accumulation texels (the kernels' exposure, tone map,
 * optional sRGB OETF and rounding). */
int oracle_tonemap(const float* accum_rgba, uint32_t n, float exposure, uint32_t op, int srgb, uint8_t* out);

/* The polynomial transcendentals shared (by restatement) with the GPU kernels. */
float oracle_sinf(float x);
float oracle_cosf(float x);
float oracle_atan2f(float y, float x);
float oracle_acosf(float x);
uint32_t oracle_pcg_hash(uint32_t x);
float oracle_expf(float x);
float oracle_logf(float x);
float oracle_powf(float x, float y);
float oracle_asinf(float x);

#ifdef __cplusplus
}
#endif

#endif
