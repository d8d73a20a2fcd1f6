// GB300 path-trace hot path: wavefront integrator + C-ABI (include/pt_gpu.h).
//
// One frame of the reference kernel (shaders/PathTrace.slang:5450-7930) is a
// per-pixel loop over spp samples, each a loop over bounces.  Here the same
// work runs as a wavefront over a "wave" = F frames x all pixels:
//
//   init     per path slot: seed = pcgHash(x*1973 + y*9277 + frame*26699)
//   for s < spp (samples share the pixel's seed stream, so they run in order):
//     camera   primary rays for every slot (consumes the jitter draws)
//     for b < max_bounces:
//       extend   closest hit for the live queue
//       shade    miss / emission / NEE sampling / BSDF / Russian roulette in
//                the reference's RNG order; NEE shadow rays go to a queue with
//                their pending contribution; survivors go to the next queue
//       shadow   transmittance for every queued shadow ray
//       resolve  adds the visible NEE terms in the reference's order, and the
//                sample radiance of paths that ended this bounce
//   accumulate  running mean over the wave's frames, in frame order
//
// Extend and shadow are persistent closest-hit kernels over 4-wide SAH trees
// (pt_device.cuh).  Once shade has written bounce b's next rays, extend of
// bounce b+1 runs on a second stream beside shadow and resolve of bounce b.
// Shade writes the next queue in each block's path order (grouped by
// ray-direction octant when a batch tuning asks for it); camera rays run in
// 4 x 8 pixel tiles, one warp each.  A wave holds up to ~64 M paths.
//
// All float math is compiled with -fmad=false and follows the shader's
// operation order, so the result equals a scalar restatement bit for bit.

#include "pt_gpu.h"
#include "pt_device.cuh"
#include "bvh_build.cuh"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <array>
#include <initializer_list>
#include <cstdio>
#include <mutex>
#include <cstring>
#include <string>
#include <vector>

using namespace ptd;

namespace {

constexpr uint32_t kEnded = 4u, kSkipSky = 1u, kPrevLambert = 2u;
constexpr uint32_t kAmbBit = 1u << 8;   // shadow mask: the path has a skylight ambient term (P.amb)
static_assert(ptb::kWideLeafBit == ptd::kLeafBit, "wide-node leaf codes must match the traversal's");
constexpr int kThreads = 256;
constexpr uint32_t kCdfGuide = 256;   // guide-table buckets per CDF (cdf_search)
// k_transmit carries the dielectric-chain state besides the traversal state: at
// 3 blocks of 256 per SM it needs no register spills (at 4 it spilled 230 bytes
// per thread and ran 2% slower on the 1080p triangle scene).
constexpr int kTransmitBlocks = 3;
// k_shade runs blocks of 512 (+0.8% on the 1080p triangle scene against 256
// when its queue compaction grouped by octant; batched renders can pick 256).
constexpr int kShadeThreads = 512;

struct DFrame {
    V3 cam_pos;
    float tanf;
    V3 fwd;
    float aspect;
    V3 right;
    V3 up;
    uint32_t W, H, npix, nframes, frame_index0, spp, maxb, denoiser;
    float jx, jy;
    uint32_t env_present;
    float env_intensity, env_total;
    int kmax;
    float firefly;
    uint32_t mis, rr_start, light_count;
    // batched renders: per-view fields
    uint32_t scene;          // index into the batch's scene table
    uint32_t slot_base;      // first path slot of the view in the wave
    uint32_t reset;          // reset_accum of the view's first frame
    float ema;               // accum_params.x
    size_t accum_base;       // first texel of the view in the batch accumulation buffer
    // gradient sky (no env map): sun_and_mode.xyz, moon_dir_phase, moon_extra, sun_extra, sun_extra2.x
    V3 sun_dir;
    float sun_bright;
    uint32_t sky_mode;       // sun_and_mode.w: 0 gradient, 1 env map, 2 procedural
    uint32_t light_tree;     // pick NEE lights from the light tree
    float4 moon;
    float4 moon_extra;
    float4 sun_extra;
    // launch-shape knobs (results do not depend on them; zero = the defaults)
    uint32_t tile_lw;        // camera tile width log2, one warp of 32 pixels per tile (0: 2, 4 x 8)
    uint32_t call_fi0;       // frame index of the call's first frame (it takes the push's jitter)
    uint32_t octant_on;      // 1: the shading kernel's queue compaction groups by ray octant
};

// Adjoint replay state (differentiable renders)
struct Adj {
    const float4* srad;    // per-sample radiance recorded by the forward pass
    const float4* dldi;    // dLoss/dI per pixel (rgb)
    double* grad;          // global: [2][nmat][3] albedo then emission
    const uint4* sh_mats;  // dielectric rows crossed per shadow slot
    size_t srec_base;      // srad index of path slot 0 for the current sample
    uint32_t nmat;
    float scale;           // 1 / (frames * spp)
};

// Batched renders: device tables of per-view frame constants and per-scene
// descriptors; every path records its view and scene.
struct Batch {
    const DFrame* views;
    const DScene* scenes;
    uint32_t* path_view;
    uint32_t* path_scene;
    const uint32_t* view_base;   // n_views + 1 slot offsets
    float4* accum;
    uint32_t n_views;
};

struct DPaths {
    float4* ray_o;
    float4* ray_d;
    float4* thr;      // w: cosine pdf of the last Lambert bounce (MIS)
    float4* rad;
    float4* fsum;
    uint32_t* seed;
    uint32_t* state;
    float* hit_t;
    uint32_t* hit_id;
    uint32_t* shmask;  // bits 0-2: shadow slot issued; bits 4-6: clamp as indirect
    float4* sh_o;      // 3 per path: origin, w = t_max
    float4* sh_d;      // direction, w = first scalar factor
    float4* sh_pre;    // throughput * emitter radiance, w = second scalar factor
    float4* sh_brdf;   // brdf, w = pdf
    float4* sh_tr;     // transmittance result
    uint32_t* q[2];
    uint32_t* sq;
    // Queue counters: a ring of 4 blocks of 4 words, block b & 3 for bounce b:
    // [0] rays queued for the bounce (q[b & 1]), [1] shadow rays (sq), [2] the
    // closest-hit kernel's fetch counter, [3] the transmittance kernel's.  A
    // bounce's launches get cnt = its block, cnt_next = the next bounce's
    // (k_shade appends the survivors there) and cnt_clear = block (b + 2) & 3,
    // which k_shade zeroes for bounce b + 2: every launch of bounce b - 2 has
    // finished by then and none that may run beside k_shade uses it.  k_camera
    // (single-view renders) sets up block 0 and zeroes the rest, so a sample
    // needs no memset of its own.
    uint32_t* cnt;
    uint32_t* cnt_next;
    uint32_t* cnt_clear;
    float4* amb;       // gradient sky: skylight ambient of the bounce, added after its NEE terms
    float4* srad;      // differentiable renders: radiance of every sample [s * npaths + p], or null
    unsigned long long* stat;   // [0] extension rays, [1] shadow segments
    // roulette survival probabilities held fixed (pt_gpu_set_roulette_freeze):
    // [p * max_bounces + b] for this sample and wave, recorded (rr_mode 1) or
    // read back (rr_mode 2); null when off
    float* rr_frozen;
    uint32_t rr_mode;
    // single-view renders: [0] frame index of the wave's first frame, [1] of
    // the call's first frame, [2] reset the accumulation at the wave's first
    // frame; written by k_set_wave ahead of each wave, so that the wave's other
    // launches (and a CUDA graph of them) do not depend on the frame index
    const uint32_t* wave;
};

// ---------------------------------------------------------------------------
// sampling helpers that need the frame constants
// ---------------------------------------------------------------------------
__device__ __forceinline__ V3 clamp_ind(V3 c, float w) {
    if (w <= 0.0f) return c;
    const float m = fmaxf(c.x, fmaxf(c.y, c.z));
    return (m > w) ? c * (w / m) : c;
}

__device__ __forceinline__ V3 env_texel(const DScene& S, uint32_t u, uint32_t v) {
    return v3(__ldg(S.env + (size_t(v) * S.env_w + u)));
}

__device__ __forceinline__ float saturatef(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + t * (b - a); }
__device__ __forceinline__ float smoothstepf(float e0, float e1, float x) {
    const float t = saturatef((x - e0) / (e1 - e0));
    return t * t * (3.0f - 2.0f * t);
}

// sky dome of the gradient mode (skyColorBase, shaders/PathTrace.slang:3461-3463)
__device__ __forceinline__ V3 sky_gradient(V3 rd) {
    const float t = clampf(0.5f * (rd.y + 1.0f), 0.0f, 1.0f);
    return lerp3(v3(0.50f, 0.55f, 0.62f), v3(1.0f, 1.0f, 1.0f), t);
}

// sun disc + halo (sunDisc, shaders/PathTrace.slang:3112-3195)
__device__ V3 sun_disc(const DFrame& F, V3 rd) {
    const V3 sd = F.sun_dir;
    if (sd.y < -0.10f) return v3(0.0f, 0.0f, 0.0f);
    const float ang = dot(rd, sd);
    const float sun_mult = fmaxf(F.sun_extra.x * F.sun_extra.y, 0.1f);
    const float r_deg = 0.55f * sun_mult;
    const float cos_r = f_cos(r_deg * 0.0174533f);
    const float halo_deg = lerpf(2.0f, 8.0f, saturatef(1.0f - sd.y));
    const float halo_rad = halo_deg * 0.0174533f;
    const float cos_halo = f_cos(halo_rad);
    if (ang <= cos_halo) return v3(0.0f, 0.0f, 0.0f);
    const float vflat = F.sun_extra.z;
    const bool oval = vflat < 0.999f;
    bool inside = false;
    if (ang > cos_r) {
        if (!oval) {
            inside = true;
        } else {
            const V3 lr = normalize(cross(v3(0.0f, 1.0f, 0.0f), sd));
            const V3 lu = cross(sd, lr);
            const V3 delta = rd - sd * ang;
            const float h_off = dot(delta, lr), v_off = dot(delta, lu);
            const float r_h = r_deg * 0.0174533f;
            const float r_v = r_h * vflat;
            const float ellipse = (h_off * h_off) / (r_h * r_h) + (v_off * v_off) / (r_v * r_v);
            inside = ellipse <= 1.0f;
        }
    }
    const float am = 1.0f / fmaxf(sd.y, 0.04f);
    const float atm = f_exp(-0.30f * am);
    const float warmth = saturatef((am - 1.0f) * 0.18f);
    const V3 col = lerp3(v3(1.00f, 0.98f, 0.94f), v3(1.55f, 0.55f, 0.20f), warmth);
    float halo = 0.0f;
    if (ang > cos_halo) {
        const float t_h = (ang - cos_halo) / (1.0f - cos_halo);
        const float falloff = lerpf(8.0f, 3.0f, saturatef(1.0f - sd.y));
        halo = f_pow(t_h, falloff);
    }
    const float bright = fmaxf(F.sun_bright, 0.0f);
    if (inside) return (col * (250.0f * atm) + col * halo * atm * 4.0f) * bright;
    return col * halo * atm * 4.0f * bright;
}

__device__ __forceinline__ V3 moon_texel(const DScene& S, int32_t x, int32_t y) {
    return v3(__ldg(S.moon_tex + (size_t(y) * S.moon_w + x)));
}

// moon disc + surface + halo (moonDisc, shaders/PathTrace.slang:3212-3353)
__device__ V3 moon_disc(const DScene& S, const DFrame& F, V3 rd) {
    const float4 mph = F.moon;
    if (mph.y < -0.10f) return v3(0.0f, 0.0f, 0.0f);
    const V3 m_dir = v3(mph);
    const V3 sun = F.sun_dir;
    const float ang = dot(rd, m_dir);
    const float size_mult = fmaxf(F.moon_extra.x * F.moon_extra.y, 0.1f);
    const float r_deg = 0.55f * size_mult;
    const float halo_deg = 1.5f * size_mult;
    const float cos_r = f_cos(r_deg * 0.0174533f);
    const float cos_halo = f_cos(halo_deg * 0.0174533f);
    if (ang <= cos_halo) return v3(0.0f, 0.0f, 0.0f);
    const V3 col_tint = v3(0.92f, 0.94f, 1.00f);
    const float moon_am = 1.0f / fmaxf(mph.y, 0.04f);
    const float moon_atm = f_exp(-0.30f * moon_am);
    const float warmth_m = saturatef((moon_am - 1.0f) * 0.18f);
    const V3 col_atm = lerp3(v3(1.00f, 1.00f, 1.00f), v3(1.20f, 0.65f, 0.40f), warmth_m);
    float halo = 0.0f;
    if (ang > cos_halo) {
        const float t_h = (ang - cos_halo) / (1.0f - cos_halo);
        halo = f_pow(t_h, 4.0f) * 0.6f;
    }
    if (ang > cos_r) {
        const float t_d = (ang - cos_r) / (1.0f - cos_r);
        const V3 ax = (fabsf(m_dir.y) < 0.99f) ? v3(0.0f, 1.0f, 0.0f) : v3(1.0f, 0.0f, 0.0f);
        const V3 t_a = normalize(cross(ax, m_dir));
        const V3 t_b = cross(m_dir, t_a);
        const float disc_scale = 1.0f / fmaxf(f_sin(r_deg * 0.0174533f), 1e-5f);
        const float du = dot(rd, t_a) * disc_scale;
        const float dv = dot(rd, t_b) * disc_scale;
        const float r2 = du * du + dv * dv;
        const float zz = sqrtf(fmaxf(1.0f - r2, 0.0f));
        const V3 n_world = t_a * du + t_b * dv - m_dir * zz;
        const float lit = saturatef(dot(n_world, sun) * 10.0f + 0.05f);
        if (lit <= 0.0f) return col_tint * col_atm * halo * moon_atm * 0.05f;
        const float anti_sun_dot = -dot(m_dir, sun);
        const float anti_sun_ang = f_acos(saturatef(anti_sun_dot));
        const float eclipse = 1.0f - smoothstepf(0.0122f, 0.0218f, anti_sun_ang);
        const float lon = f_atan2(du, zz);
        const float lat = f_asin(clampf(dv, -1.0f, 1.0f));
        const float u_tex = saturatef(0.5f + lon / 6.28318530718f);
        const float v_tex = saturatef(0.5f - lat / 3.14159265358979f);
        const int32_t mw = int32_t(S.moon_w), mh = int32_t(S.moon_h);
        const float fx = u_tex * float(mw) - 0.5f, fy = v_tex * float(mh) - 0.5f;
        const int32_t ix = int32_t(floorf(fx)), iy = int32_t(floorf(fy));
        const float tx = fx - float(ix), ty = fy - float(iy);
        const int32_t x0 = min(max(ix, 0), mw - 1), x1 = min(max(ix + 1, 0), mw - 1);
        const int32_t y0 = min(max(iy, 0), mh - 1), y1 = min(max(iy + 1, 0), mh - 1);
        const V3 surface = lerp3(lerp3(moon_texel(S, x0, y0), moon_texel(S, x1, y0), tx),
                                 lerp3(moon_texel(S, x0, y1), moon_texel(S, x1, y1), tx), ty);
        const float limb = 0.55f + 0.45f * sqrtf(saturatef(t_d));
        const float bright_mult = fmaxf(F.moon_extra.z, 0.0f);
        const float disc_scale_b = 3.5f * bright_mult;
        const V3 lit_col = col_tint * col_atm * surface * (disc_scale_b * lit * limb * moon_atm) +
                           col_tint * col_atm * halo * lit * moon_atm * (0.6f * bright_mult);
        const V3 eclipse_col = v3(0.55f, 0.15f, 0.04f) * surface * (limb * moon_atm * 1.2f);
        return lerp3(lit_col, eclipse_col, eclipse);
    }
    const float phase_b = 0.5f * (1.0f - f_cos(mph.w));
    return col_tint * col_atm * halo * phase_b * moon_atm * 0.3f;
}

// procSkyInlineSunDiscAndHalo (shaders/PathTrace.slang:2860-2872)
__device__ V3 proc_sun_inline(V3 rd, V3 sun) {
    const float cos_gamma = clampf(dot(rd, sun), -1.0f, 1.0f);
    const float day = smoothstepf(-0.10f, 0.20f, sun.y);
    const float disk = smoothstepf(0.99996f, 0.99999f, cos_gamma);
    const V3 sun_col = lerp3(v3(1.00f, 0.55f, 0.20f), v3(1.00f, 0.95f, 0.85f), day);
    V3 result = sun_col * (disk * 50.0f) * day;
    const float halo = f_pow(fmaxf(0.0f, cos_gamma), 80.0f);
    result = result + sun_col * halo * 0.30f * day;
    return result;
}

// procSky with the stars off (shaders/PathTrace.slang:2990-3103)
__device__ V3 proc_sky(const DFrame& F, V3 rd) {
    const V3 sun = F.sun_dir;
    const float cos_theta_raw = clampf(rd.y, -1.0f, 1.0f);
    const float cos_gamma = clampf(dot(rd, sun), -1.0f, 1.0f);
    const float sun_elev = sun.y;
    const float cam_h = fmaxf(F.cam_pos.y, 0.0f);
    const float planet_r = F.sun_extra.w;
    float dip = 0.0f;
    if (planet_r > 0.0f && cam_h > 0.0f) {
        const float ratio = cam_h / planet_r;
        dip = sqrtf(2.0f * ratio + ratio * ratio);
        dip = fminf(dip, 0.5f);
    }
    const float cos_theta = clampf(cos_theta_raw + dip, -1.0f, 1.0f);
    const float day = smoothstepf(-0.10f, 0.20f, sun_elev);
    const float sunset = smoothstepf(0.30f, -0.05f, sun_elev) * smoothstepf(-0.20f, 0.05f, sun_elev);
    const V3 zenith_day = v3(0.32f, 0.55f, 0.92f), horizon_day = v3(0.78f, 0.88f, 1.00f);
    const float side_factor =
        smoothstepf(0.0f, 0.7f, dot(normalize(v3(rd.x, 0.0f, rd.z)), normalize(v3(sun.x, 0.0f, sun.z))));
    const V3 horizon_sunset = lerp3(v3(0.95f, 0.45f, 0.20f), v3(1.00f, 0.65f, 0.30f), side_factor);
    const V3 horizon_col = lerp3(horizon_day, horizon_sunset, sunset);
    const V3 zenith_col = lerp3(zenith_day, v3(0.18f, 0.18f, 0.30f), sunset * 0.6f);
    const float t = smoothstepf(0.0f, 0.40f, cos_theta);
    V3 sky = lerp3(horizon_col, zenith_col, t);
    const V3 night = v3(0.005f, 0.010f, 0.030f);   // + smoothstep(...) * 0.0 in the source: adds +0
    sky = lerp3(night, sky, day);
    sky = sky + proc_sun_inline(rd, sun);          // the stars term is zero with the stars off
    const V3 sun_col = lerp3(v3(1.00f, 0.55f, 0.20f), v3(1.00f, 0.95f, 0.85f), day);
    const float wide = f_pow(fmaxf(0.0f, cos_gamma), 6.0f);
    sky = sky + sun_col * wide * sunset * 0.50f;
    return v3(fmaxf(sky.x, 0.0f), fmaxf(sky.y, 0.0f), fmaxf(sky.z, 0.0f));
}

// skyColorBase without an env map (shaders/PathTrace.slang:3445-3464): the dome
// without celestial overlays, seen by the skylight ambient
__device__ __forceinline__ V3 sky_base(const DFrame& F, V3 rd) {
    if (F.sky_mode == 2u) return proc_sky(F, rd) - proc_sun_inline(rd, F.sun_dir);
    return sky_gradient(rd);
}

// sampleSunDisc (shaders/PathTraceMath.slang:55-68)
__device__ __forceinline__ V3 sample_sun_disc(V3 sun_dir, uint32_t& seed) {
    const float u1 = randf(seed);
    const float u2 = randf(seed);
    const float r = sqrtf(u1) * 0.00465f;
    const float phi = kTwoPiHemi * u2;
    const float dx = f_cos(phi) * r, dy = f_sin(phi) * r;
    const V3 ax = (fabsf(sun_dir.y) < 0.99f) ? v3(0.0f, 1.0f, 0.0f) : v3(1.0f, 0.0f, 0.0f);
    const V3 t = normalize(cross(ax, sun_dir));
    const V3 b = cross(sun_dir, t);
    return normalize(sun_dir + t * dx + b * dy);
}

// skyColor (shaders/PathTrace.slang:3373-3434): the env map (mode 1), else the
// gradient dome with the moon and sun discs on top (mode 0)
__device__ V3 sky_env(const DScene& S, const DFrame& F, V3 rd);
__device__ V3 sky_color(const DScene& S, const DFrame& F, V3 rd) {
    if (F.env_present) return sky_env(S, F, rd);
    const V3 base = (F.sky_mode == 2u) ? proc_sky(F, rd) : sky_gradient(rd);
    return base + moon_disc(S, F, rd) + sun_disc(F, rd);
}

// skyColor, env-map branch (shaders/PathTrace.slang:3401-3431)
__device__ V3 sky_env(const DScene& S, const DFrame& F, V3 rd) {
    const int32_t w = int32_t(S.env_w), hh = int32_t(S.env_h);
    const float u = f_atan2(rd.z, rd.x) * kInvTwoPiSky + 0.5f;
    const float v = f_acos(clampf(rd.y, -1.0f, 1.0f)) * kInvPiSky;
    const float fx = u * float(w) - 0.5f, fy = v * float(hh) - 0.5f;
    const int32_t ix = int32_t(floorf(fx)), iy = int32_t(floorf(fy));
    const float tx = fx - float(ix), ty = fy - float(iy);
    const int32_t x0 = (ix % w + w) % w, x1 = (x0 + 1) % w;
    const int32_t y0 = min(max(iy, 0), hh - 1), y1 = min(max(iy + 1, 0), hh - 1);
    const V3 c00 = env_texel(S, x0, y0), c10 = env_texel(S, x1, y0);
    const V3 c01 = env_texel(S, x0, y1), c11 = env_texel(S, x1, y1);
    const V3 sky = lerp3(lerp3(c00, c10, tx), lerp3(c01, c11, tx), ty);
    return sky * F.env_intensity;
}

// The smallest i with cdf[i] >= u (count - 1 if none): a binary search over
// the whole array, or, with a guide table g (g[k] = that index for u = k / K,
// g[K] = count, K = kCdfGuide; built only for non-decreasing arrays), over
// [g[k], g[k + 1]] for u in [k/K, (k+1)/K).  The index sought lies in that
// bracket (the search is monotone in u), and the same comparisons inside it
// give the same index, so the guide only removes dependent loads: about 3
// steps on a 2048-texel row instead of 11 (Chen and Asau's guide-table
// method).  u * K is exact (K is a power of two); negative or NaN u takes the
// full search.
__device__ __forceinline__ uint32_t cdf_search(const float* cdf, uint32_t count, float u,
                                               const uint32_t* g = nullptr) {
    uint32_t lo = 0, hi = count;
    const float uk = u * float(kCdfGuide);
    if (g && uk >= 0.0f) {
        const uint32_t k = uint32_t(fminf(uk, float(kCdfGuide - 1u)));
        lo = __ldg(g + k);
        hi = __ldg(g + k + 1u);
    }
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(cdf + mid) < u) lo = mid + 1;
        else hi = mid;
    }
    return min(lo, count - 1u);
}

__device__ __forceinline__ float env_denom(const DFrame& F) { return 2.0f * kPi * kPi * F.env_total; }

// sampleEnvMap (shaders/PathTrace.slang:3638-3670)
__device__ void sample_env(const DScene& S, const DFrame& F, float xu, float xv, V3& dir, V3& color,
                           float& pdf) {
    dir = v3(0.0f, 1.0f, 0.0f);
    color = v3(0.0f, 0.0f, 0.0f);
    pdf = 0.0f;
    if (F.env_present == 0u || !(F.env_total > 0.0f)) return;
    const uint32_t w = S.env_w, hh = S.env_h;
    const uint32_t vi = cdf_search(S.marg, hh, xv, S.marg_guide);
    const uint32_t ui = cdf_search(S.cond + size_t(vi) * w, w, xu,
                                   S.cond_guide ? S.cond_guide + size_t(vi) * (kCdfGuide + 1u) : nullptr);
    const float u = (float(ui) + 0.5f) / float(w);
    const float v = (float(vi) + 0.5f) / float(hh);
    const float theta = v * kPi;
    const float phi = u * kTwoPi - kPi;
    const float st = f_sin(theta);
    dir = v3(st * f_cos(phi), f_cos(theta), st * f_sin(phi));
    const V3 raw = env_texel(S, ui, vi);
    color = raw * F.env_intensity;
    const float lum = 0.2126f * raw.x + 0.7152f * raw.y + 0.0722f * raw.z;
    if (st > 1e-6f) pdf = (lum * float(w * hh)) / env_denom(F);
}

__device__ __forceinline__ void dir_to_texel(const DScene& S, V3 d, float& st, uint32_t& ui,
                                             uint32_t& vi) {
    const float ct = clampf(d.y, -1.0f, 1.0f);
    const float th = f_acos(ct);
    st = f_sin(th);
    const float ph = f_atan2(d.z, d.x);
    const float u = (ph + kPi) * kInvTwoPiPdf;
    const float v = th * kInvPiPdf;
    ui = min(uint32_t(u * float(S.env_w)), S.env_w - 1u);
    vi = min(uint32_t(v * float(S.env_h)), S.env_h - 1u);
}

// isExtractedClusterDir (shaders/PathTrace.slang:3679-3696)
__device__ bool is_cluster_dir(const DScene& S, const DFrame& F, V3 d) {
    if (F.env_present == 0u || S.hdri_count == 0u) return false;
    float st;
    uint32_t ui, vi;
    dir_to_texel(S, d, st, ui, vi);
    if (st < 1e-6f) return false;
    const size_t base = size_t(vi) * S.env_w;
    const float cc = __ldg(S.cond + base + ui);
    const float cp = (ui > 0u) ? __ldg(S.cond + base + ui - 1u) : 0.0f;
    return cc <= cp;
}

// pdfEnvMapDir (shaders/PathTrace.slang:3710-3727)
__device__ float pdf_env_dir(const DScene& S, const DFrame& F, V3 d) {
    if (F.env_present == 0u || !(F.env_total > 0.0f)) return 0.0f;
    float st;
    uint32_t ui, vi;
    dir_to_texel(S, d, st, ui, vi);
    if (st < 1e-6f) return 0.0f;
    const V3 raw = env_texel(S, ui, vi);
    const float lum = 0.2126f * raw.x + 0.7152f * raw.y + 0.0722f * raw.z;
    return (lum * float(S.env_w * S.env_h)) / env_denom(F);
}

__device__ __forceinline__ float mis_balance(float a, float b) { return a / fmaxf(a + b, 1e-12f); }

// sampleAnalyticLight, uniform pick (shaders/PathTrace.slang:4035-4179)
// lightTreeImportance (shaders/PathTrace.slang:3932-3966)
__device__ __forceinline__ float lt_importance(const float4* T, uint32_t idx, V3 hp, V3 n_face) {
    const float4 v0 = __ldg(T + 4u * idx), v1 = __ldg(T + 4u * idx + 1u);
    const float4 v2 = __ldg(T + 4u * idx + 2u), v3n = __ldg(T + 4u * idx + 3u);
    const V3 lo = v3(v0), hi = v3(v1);
    const V3 to_c = (lo + hi) * 0.5f - hp;
    const float d2 = fmaxf(dot(to_c, to_c), 1e-12f);
    const float d = sqrtf(d2);
    const V3 dir_to = to_c / d;
    const V3 ext = (hi - lo) * 0.5f;
    const float rad2 = fmaxf(dot(ext, ext), 1e-12f);
    const float falloff = 1.0f / fmaxf(d2, rad2);
    float orient = 1.0f;
    if (v2.w > -0.999f) {
        const float cos_emit = -dot(v3(v2), dir_to);
        orient = saturatef((cos_emit - (v2.w - 0.2f)) / 0.2f);
    }
    const float recv = fmaxf(0.0f, dot(n_face, dir_to));
    return fmaxf(v3n.x * falloff * orient * recv, 1e-8f);
}

// pickLightFromTree (shaders/PathTrace.slang:3978-4016): one draw per level
__device__ __forceinline__ uint32_t lt_pick(const DScene& S, V3 hp, V3 n_face, uint32_t& seed, float& pick_pdf) {
    const float4* T = S.ltree;
    uint32_t idx = 0;
    pick_pdf = 1.0f;
    for (int d = 0; d < 32; ++d) {
        const uint32_t left_first = __float_as_uint(__ldg(T + 4u * idx).w);
        if (__float_as_uint(__ldg(T + 4u * idx + 1u).w) > 0u) return left_first;
        const float il = lt_importance(T, left_first, hp, n_face);
        const float ir = lt_importance(T, left_first + 1u, hp, n_face);
        const float total = il + ir;
        const float p_l = (total > 1e-30f) ? (il / total) : 0.5f;
        const float u = randf(seed);
        if (u < p_l) {
            idx = left_first;
            pick_pdf *= p_l;
        } else {
            idx = left_first + 1u;
            pick_pdf *= (1.0f - p_l);
        }
    }
    return 0u;
}

__device__ void sample_light(const DScene& S, const DFrame& F, V3 hp, V3 n_face, uint32_t& seed, V3& dir, V3& Le,
                             float& pdf, float& dist) {
    dir = v3(0.0f, 1.0f, 0.0f);
    Le = v3(0.0f, 0.0f, 0.0f);
    pdf = 0.0f;
    dist = 1e30f;
    const uint32_t n = F.light_count;
    if (n == 0u) return;
    uint32_t pick;
    float pick_pdf;
    if (F.light_tree) {
        pick = min(lt_pick(S, hp, n_face, seed, pick_pdf), n - 1u);
    } else {
        const float u_pick = randf(seed);
        pick = min(uint32_t(u_pick * float(n)), n - 1u);
        pick_pdf = 1.0f / float(n);
    }
    const float4* L = S.lights + 5u * pick;
    const float4 l0 = __ldg(L), l1 = __ldg(L + 1), l2 = __ldg(L + 2), l3 = __ldg(L + 3),
                 l4 = __ldg(L + 4);
    const uint32_t type = uint32_t(l1.w + 0.5f);
    const V3 pos = v3(l0), inten = v3(l1);
    if (type == 0u || type == 1u) {
        const V3 tl = pos - hp;
        const float d2 = fmaxf(dot(tl, tl), 1e-12f);
        const float d = sqrtf(d2);
        if (type == 0u) {
            dir = tl / d;
            Le = inten / d2;
        } else {
            const V3 tld = tl / d;
            const V3 axis = normalize(quat_rotate(l4, v3(l2)));
            const float cos_dir = dot(-tld, axis);
            const float cin = l3.x, cout = l2.w;
            float fall = 0.0f;
            if (cos_dir >= cin) fall = 1.0f;
            else if (cos_dir > cout) fall = (cos_dir - cout) / fmaxf(cin - cout, 1e-6f);
            dir = tld;
            Le = inten * (fall / d2);
        }
        pdf = pick_pdf;
        dist = d;
        return;
    }
    if (type == 2u) {
        const float x0 = randf(seed);
        const float x1 = randf(seed);
        const float z = 1.0f - 2.0f * x0;
        const float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
        const float phi = kTwoPi * x1;
        const V3 nl = v3(r * f_cos(phi), r * f_sin(phi), z);
        const V3 lp = pos + nl * l0.w;
        const V3 tl = lp - hp;
        const float d2 = fmaxf(dot(tl, tl), 1e-12f);
        const float d = sqrtf(d2);
        const V3 wi = tl / d;
        const float cl = fmaxf(0.0f, dot(nl, -wi));
        if (cl <= 0.0f) return;
        const float area = 4.0f * kPi * l0.w * l0.w;
        const float pdf_sa = d2 / fmaxf(area * cl, 1e-12f);
        dir = wi;
        Le = inten;
        pdf = pick_pdf * pdf_sa;
        dist = d;
        return;
    }
    if (type == 3u) {
        const float xa = randf(seed) * 2.0f - 1.0f;
        const float xb = randf(seed) * 2.0f - 1.0f;
        const V3 uvec = quat_rotate(l4, v3(l3));
        const float ulen = length(uvec);
        if (ulen < 1e-6f) return;
        const V3 nq = normalize(quat_rotate(l4, v3(l2)));
        const V3 vax = normalize(cross(nq, uvec));
        const V3 lp = pos + uvec * xa + vax * (l3.w * xb);
        const V3 tl = lp - hp;
        const float d2 = fmaxf(dot(tl, tl), 1e-12f);
        const float d = sqrtf(d2);
        const V3 wi = tl / d;
        const float cl = dot(nq, -wi);
        if (cl <= 0.0f) return;
        const float area = 4.0f * ulen * l3.w;
        const float pdf_sa = d2 / fmaxf(area * cl, 1e-12f);
        dir = wi;
        Le = inten;
        pdf = pick_pdf * pdf_sa;
        dist = d;
    }
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ void warp_add(unsigned long long* dst, uint32_t v) {
    unsigned long long x = v;
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
    if ((threadIdx.x & 31) == 0 && x) atomicAdd(dst, x);
}

__device__ __forceinline__ uint32_t warp_push(uint32_t* counter, bool pred) {
    const uint32_t mask = __ballot_sync(0xFFFFFFFFu, pred);
    const int lane = threadIdx.x & 31;
    const int leader = mask ? __ffs(mask) - 1 : 0;
    uint32_t base = 0;
    if (lane == leader && mask) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

// prim geometry at upload: sphere centre = lerp(prev, curr, shutter 1), plane
// normal rotated by the orientation quaternion (shaders/PathTrace.slang:2096, 2120).
__global__ void k_prep_prims(const float4* rec, uint32_t n, float4* geo, uint32_t* type) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v0 = rec[7u * i], v2 = rec[7u * i + 2u], v3r = rec[7u * i + 3u], v5 = rec[7u * i + 5u];
    const uint32_t t = uint32_t(v2.x);
    float4 g = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (t == 0u) {
        const V3 c = lerp3(v3(v3r), v3(v0), 1.0f);
        g = f4(c, v0.w);
    } else if (t == 1u) {
        g = f4(quat_rotate(v5, v3(v0)), v0.w);
    }
    geo[i] = g;
    type[i] = t;
}

// triangle records in BVH leaf-slot order: (v0, orig id) (v1 - v0, material) (v2 - v0, 0)
__global__ void k_prep_tris(const float* pos, const uint32_t* idx, const uint32_t* perm,
                            const uint32_t* mat, uint32_t slots, float4* tri, float4* blo, float4* bhi) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= slots) return;
    const uint32_t t = perm[j];
    const uint32_t i0 = idx[3u * t], i1 = idx[3u * t + 1u], i2 = idx[3u * t + 2u];
    const V3 v0 = v3(pos[3u * i0], pos[3u * i0 + 1u], pos[3u * i0 + 2u]);
    const V3 v1 = v3(pos[3u * i1], pos[3u * i1 + 1u], pos[3u * i1 + 2u]);
    const V3 v2 = v3(pos[3u * i2], pos[3u * i2 + 1u], pos[3u * i2 + 2u]);
    const uint32_t m = mat ? mat[t] : 0u;
    tri[3u * j] = f4(v0, __uint_as_float(t));
    tri[3u * j + 1u] = f4(v1 - v0, __uint_as_float(m));
    tri[3u * j + 2u] = f4(v2 - v0, 0.0f);
    blo[j] = make_float4(fminf(v0.x, fminf(v1.x, v2.x)), fminf(v0.y, fminf(v1.y, v2.y)),
                         fminf(v0.z, fminf(v1.z, v2.z)), 0.0f);
    bhi[j] = make_float4(fmaxf(v0.x, fmaxf(v1.x, v2.x)), fmaxf(v0.y, fmaxf(v1.y, v2.y)),
                         fmaxf(v0.z, fmaxf(v1.z, v2.z)), 0.0f);
}

// boxes of the finite analytic records (item k = record linear + k)
__global__ void k_prim_boxes(const float4* geo, const uint32_t* type, uint32_t linear, uint32_t n,
                             float4* blo, float4* bhi) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float4 g = geo[linear + k];
    const uint32_t t = type[linear + k];
    if (t == 0u) {
        blo[k] = make_float4(g.x - g.w, g.y - g.w, g.z - g.w, 0.0f);
        bhi[k] = make_float4(g.x + g.w, g.y + g.w, g.z + g.w, 0.0f);
    } else if (t == 1u) {
        blo[k] = make_float4(-1e30f, -1e30f, -1e30f, 0.0f);
        bhi[k] = make_float4(1e30f, 1e30f, 1e30f, 0.0f);
    } else {
        blo[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        bhi[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// wide-leaf-order gathers
__global__ void k_gather_tris(const float4* tri, const uint32_t* order, const uint32_t* rank, uint32_t n,
                              float4* tri4) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t j = order[p];
    tri4[3u * p] = tri[3u * j];
    tri4[3u * p + 1u] = tri[3u * j + 1u];
    const float4 c = tri[3u * j + 2u];
    tri4[3u * p + 2u] = make_float4(c.x, c.y, c.z, __uint_as_float(rank[j]));
}

__global__ void k_gather_prims(const float4* geo, const uint32_t* type, const uint32_t* order,
                               const uint32_t* rank, uint32_t linear, uint32_t n, float4* g4, uint4* m4) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t k = order[p];
    const uint32_t slot = linear + k;
    g4[p] = geo[slot];
    m4[p] = make_uint4(slot, type[slot], linear + rank[k], 0u);
}

__global__ void k_gather_u32(const uint32_t* src, const uint32_t* order, uint32_t n, uint32_t* dst) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) dst[p] = src[order[p]];
}

__global__ void k_iota(uint32_t* a, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = i;
}

__global__ void kb_init_bins(uint32_t* bins, uint32_t nwords) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nwords) return;
    const uint32_t w = i % ptb::kBinWords;
    bins[i] = (w == 0u) ? 0u : ((w <= 3u || (w >= 7u && w <= 9u)) ? 0xFFFFFFFFu : 0u);
}

// Path slot -> pixel: slots run through tiles of 32 pixels (one warp per
// tile; 4 x 8 unless the frame's tile_lw says otherwise: +0.6% on the 1080p
// triangle scene against 8 x 4) in row-major tile order, so a warp's primary
// rays are spatially coherent.  Frames whose size is not a multiple of the
// tile fall back to row order.  Each pixel's seed depends only on its
// coordinates, so the mapping changes no result.
__device__ __forceinline__ void slot_pixel(const DFrame& F, uint32_t pix, uint32_t& x, uint32_t& y) {
    const uint32_t lw = F.tile_lw ? F.tile_lw : 2u;
    const uint32_t tw_px = 1u << lw, th_px = 32u >> lw;
    if ((F.W & (tw_px - 1u)) == 0u && (F.H % th_px) == 0u) {
        const uint32_t tile = pix >> 5, in = pix & 31u;
        const uint32_t tw = F.W >> lw;
        x = (tile % tw) * tw_px + (in & (tw_px - 1u));
        y = (tile / tw) * th_px + (in >> lw);
    } else {
        x = pix % F.W;
        y = pix / F.W;
    }
}

__device__ __forceinline__ uint32_t view_of_slot(const Batch& B, uint32_t p) {
    uint32_t lo = 0, hi = B.n_views;   // last view with view_base[v] <= p
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (B.view_base[mid] <= p) lo = mid;
        else hi = mid;
    }
    return lo;
}

// pixel and frame of batch path slot p in its view (frames of a view are
// consecutive blocks of npix slots)
__device__ __forceinline__ void view_pixel(const DFrame& V, uint32_t p, uint32_t& x, uint32_t& y, uint32_t& f) {
    const uint32_t local = p - V.slot_base;
    f = local / V.npix;
    slot_pixel(V, local - f * V.npix, x, y);
}

__global__ void k_set_wave(uint32_t* wave, uint32_t frame0, uint32_t call_frame0, uint32_t reset) {
    wave[0] = frame0;
    wave[1] = call_frame0;
    wave[2] = reset;
}

template <bool kB>
__global__ void k_init_wave(const __grid_constant__ DFrame F, DPaths P, Batch B, uint32_t npaths) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npaths) return;
    uint32_t x, y, fidx;
    if (kB) {
        const uint32_t v = view_of_slot(B, p);
        const DFrame& V = B.views[v];
        B.path_view[p] = v;
        B.path_scene[p] = V.scene;
        uint32_t f;
        view_pixel(V, p, x, y, f);
        fidx = V.frame_index0 + f;
    } else {
        const uint32_t f = p / F.npix, pix = p - f * F.npix;
        slot_pixel(F, pix, x, y);
        fidx = P.wave[0] + f;
    }
    P.seed[p] = pcg_hash(x * 1973u + y * 9277u + fidx * 26699u);
    P.fsum[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// The engine's sub-pixel jitter with the denoiser on: Halton bases 2 and 3 at
// index frame_index % 16 + 1, minus 0.5 (src/engine/Engine.cpp:8241-8252).
__device__ __forceinline__ float halton_ri(uint32_t i, uint32_t base) {
    float f = 1.0f, r = 0.0f;
    while (i > 0u) {
        f /= float(base);
        r += f * float(i % base);
        i /= base;
    }
    return r;
}
__device__ __forceinline__ void halton_jitter(uint32_t frame_index, float& jx, float& jy) {
    const uint32_t hi = (frame_index % 16u) + 1u;
    jx = halton_ri(hi, 2u) - 0.5f;
    jy = halton_ri(hi, 3u) - 0.5f;
}

// primary rays (shaders/PathTrace.slang:5722-5778)
template <bool kB>
__global__ void k_camera(const __grid_constant__ DFrame F, DPaths P, Batch B, uint32_t npaths, uint32_t s) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (!kB && p < 16u) P.cnt[p] = (p == 0u) ? npaths : 0u;   // the counter ring (P.cnt: block 0)
    bool live = p < npaths;
    const DFrame& V = (kB && live) ? B.views[B.path_view[p]] : F;
    if (kB && live && s >= V.spp) live = false;   // this view has fewer samples
    if (kB) {   // compacted queue (views may differ in spp)
        const uint32_t slot = warp_push(P.cnt, live);
        if (live) P.q[0][slot] = p;
    }
    if (!live) return;
    uint32_t x, y;
    if (kB) {
        uint32_t f;
        view_pixel(V, p, x, y, f);
    } else {
        const uint32_t f = p / F.npix, pix = p - f * F.npix;
        slot_pixel(F, pix, x, y);
    }
    uint32_t seed = P.seed[p];
    float jx, jy;
    if (V.denoiser != 0u && s == 0u) {
        // sample 0 with the denoiser on: the push's sub-pixel jitter for the
        // call's first frame; later frames take the engine's jitter of their
        // own frame index, as back-to-back dispatches would
        uint32_t fi, call_fi;
        if (kB) {
            uint32_t xx, yy, f;
            view_pixel(V, p, xx, yy, f);
            fi = V.frame_index0 + f;
            call_fi = V.call_fi0;
        } else {
            fi = P.wave[0] + p / F.npix;
            call_fi = P.wave[1];
        }
        if (fi == call_fi) {
            jx = V.jx;
            jy = V.jy;
        } else {
            halton_jitter(fi, jx, jy);
        }
    } else {
        const float a = randf(seed);
        const float b = randf(seed);
        jx = a - 0.5f;
        jy = b - 0.5f;
    }
    const float ux = ((float(x) + 0.5f + jx) / float(V.W)) * 2.0f - 1.0f;
    float uy = ((float(y) + 0.5f + jy) / float(V.H)) * 2.0f - 1.0f;
    uy = -uy;
    const V3 rd = normalize(V.fwd + V.right * (ux * V.aspect * V.tanf) + V.up * (uy * V.tanf));
    P.seed[p] = seed;
    P.ray_o[p] = f4(V.cam_pos, 0.0f);
    P.ray_d[p] = f4(rd, 0.0f);
    P.thr[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    P.rad[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    P.state[p] = 0u;
    if (!kB) P.q[0][p] = p;
}

template <bool kWide>
__global__ void __launch_bounds__(kThreads) k_extend(DScene S, DPaths P, int qsel) {
    const uint32_t n = P.cnt[0];
    const uint32_t* q = P.q[qsel];
    uint32_t done = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = q[i];
        const float4 o = P.ray_o[p], d = P.ray_d[p];
        const HitRec h = trace_any_mode(S, v3(o), v3(d), 1e30f, kWide);
        P.hit_t[p] = h.t;
        P.hit_id[p] = h.id;
        ++done;
    }
    warp_add(P.stat + 0, done);
}

__device__ __forceinline__ void issue_shadow(const DPaths& P, uint32_t p, int k, V3 o, V3 d, float tmax,
                                             V3 pre, float s2, V3 brdf, float s1, float pdf,
                                             bool clamp, uint32_t& mask) {
    const uint32_t e = 3u * p + uint32_t(k);
    P.sh_o[e] = f4(o, tmax);
    P.sh_d[e] = f4(d, s1);
    P.sh_pre[e] = f4(pre, s2);
    P.sh_brdf[e] = f4(brdf, pdf);
    mask |= (1u << k) | (clamp ? (16u << k) : 0u);
}

// one bounce of the loop body (shaders/PathTrace.slang:5921-6914)
// Differentiable replay: per-block double accumulators of the parameter
// gradients in dynamic shared memory ([2][nmat][3]: albedo, emission), flushed
// to the global gradient once per block.
extern __shared__ double s_grad[];

__device__ __forceinline__ void adj_begin(const Adj& A) {
    for (uint32_t i = threadIdx.x; i < 6u * A.nmat; i += blockDim.x) s_grad[i] = 0.0;
    __syncthreads();
}
__device__ __forceinline__ void adj_end(const Adj& A) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < 6u * A.nmat; i += blockDim.x)
        if (s_grad[i] != 0.0) atomicAdd(A.grad + i, s_grad[i]);
}
__device__ __forceinline__ void adj_add(const Adj& A, int which, uint32_t m, V3 v) {
    double* g = s_grad + (size_t(which) * A.nmat + m) * 3u;
    atomicAdd(g + 0, double(v.x));
    atomicAdd(g + 1, double(v.y));
    atomicAdd(g + 2, double(v.z));
}
// dLoss/d(sample radiance) of path p: dL/dI of its pixel over the samples
// averaged into it (frames * spp; batched views: one frame, the view's spp,
// dL/dI laid out like the batch accumulation buffer)
template <bool kB>
__device__ __forceinline__ V3 adj_weight(const Adj& A, const DFrame& F, uint32_t p) {
    uint32_t x, y;
    if (kB) {
        uint32_t f;
        view_pixel(F, p, x, y, f);
        return v3(A.dldi[F.accum_base + size_t(y) * F.W + x]) * (1.0f / float(F.spp * F.nframes));
    }
    const uint32_t f = p / F.npix, pix = p - f * F.npix;
    slot_pixel(F, pix, x, y);
    return v3(A.dldi[size_t(y) * F.W + x]) * A.scale;
}
__device__ __forceinline__ V3 safe_div(V3 a, V3 b) {
    return v3(b.x > 0.0f ? a.x / b.x : 0.0f, b.y > 0.0f ? a.y / b.y : 0.0f, b.z > 0.0f ? a.z / b.z : 0.0f);
}

// The NEE terms of a path's last vertex, once its shadow rays are traced: in
// the reference order (light, env, HDRI; shaders/PathTrace.slang:6341-6520),
// each ((((pre * T) * brdf) * s1) * s2) / pdf, clamped where the slot says so,
// then the skylight ambient.  Run by k_shade for the paths of its queue (the
// previous bounce's terms, before the vertex is shaded) and by k_finish for the
// paths that ended.
template <bool kB, bool kAdj>
__device__ __forceinline__ V3 resolve_nee(const DScene& S0, const DFrame& F, const DPaths& P, const Batch& B,
                                          const Adj& A, uint32_t p, uint32_t mask, V3 rad) {
    for (int k = 0; k < 3; ++k) {
        if (!((mask >> k) & 1u)) continue;
        const uint32_t e = 3u * p + uint32_t(k);
        const V3 tr = v3(P.sh_tr[e]);
        if (!any_pos(tr)) continue;
        const float4 pre = P.sh_pre[e], br = P.sh_brdf[e];
        const float s1 = P.sh_d[e].w;
        const V3 c = v3(pre) * tr * v3(br) * s1 * pre.w / br.w;
        rad = rad + (((mask >> (4 + k)) & 1u) ? clamp_ind(c, F.firefly) : c);
        if (kAdj) {   // each dielectric the shadow ray crossed multiplied c by its albedo
            const DScene& S = kB ? B.scenes[F.scene] : S0;
            const uint4 xm = A.sh_mats[e];
            const uint32_t ms[4] = {xm.x, xm.y, xm.z, xm.w};
            const V3 g = adj_weight<kB>(A, F, p);
            for (int j = 0; j < 4; ++j) {
                if (ms[j] == kNoMat || S.mat_count == 0u) continue;
                const uint32_t m = min(ms[j], S.mat_count - 1u);
                adj_add(A, 0, m, g * safe_div(c, v3(__ldg(S.mats + 3u * m))));
            }
        }
    }
    if (mask & kAmbBit) rad = rad + v3(P.amb[p]);
    return rad;
}

// (512-thread blocks are held to 64 registers: two blocks per SM)
template <bool kB, bool kAdj, bool kProc = true, int kSB = kShadeThreads>
__global__ void __launch_bounds__(kSB, kSB == 512 ? 2 : 1) k_shade(const __grid_constant__ DScene S0,
                                                     const __grid_constant__ DFrame F0, DPaths P, Batch B,
                                                     const __grid_constant__ Adj A, int qsel, uint32_t b) {
    const uint32_t n = P.cnt[0];
    const uint32_t* q = P.q[qsel];
    uint32_t* qn = P.q[qsel ^ 1];
    if (blockIdx.x == 0u && threadIdx.x < 4u) P.cnt_clear[threadIdx.x] = 0u;
    const uint32_t n_iter = (n + blockDim.x * gridDim.x - 1) / (blockDim.x * gridDim.x);
    if (kAdj) adj_begin(A);
    __shared__ uint32_t s_hist[2][8], s_base[8], s_block, s_sh[2], s_sblock;
    if (threadIdx.x < 8u) s_hist[0][threadIdx.x] = 0u;
    if (threadIdx.x == 8u) s_sh[0] = 0u;
    __syncthreads();
    for (uint32_t it = 0; it < n_iter; ++it) {
        const uint32_t i = (it * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x;
        bool cont = false;
        uint32_t shadow_mask = 0;
        uint32_t p = 0;
        uint32_t oct = 0;   // direction octant of the next ray
        if (i < n) {
            p = q[i];
            const DFrame& F = kB ? B.views[B.path_view[p]] : F0;
            const DScene& S = kB ? B.scenes[F.scene] : S0;
            if (!kB || b < F.maxb) {
            const float4 o4 = P.ray_o[p], d4 = P.ray_d[p], t4 = P.thr[p], r4 = P.rad[p];
            V3 ro = v3(o4), rd = v3(d4), thr = v3(t4), rad = v3(r4);
            float prev_pdf = t4.w;
            uint32_t st = P.state[p];
            uint32_t seed = P.seed[p];
            const HitRec h{P.hit_t[p], P.hit_id[p]};
            // the previous vertex's NEE terms (its shadow rays were traced by
            // the last transmittance launch) before this vertex adds its own
            if (b > 0u) {
                const uint32_t pmask = P.shmask[p];
                if (pmask) rad = resolve_nee<kB, kAdj>(S0, F, P, B, A, p, pmask, rad);
            }
            bool ended = false;
            if (h.id == kMiss) {
                if (F.mis != 0u && (st & kPrevLambert)) {
                    if (!is_cluster_dir(S, F, rd)) {
                        const float pe = pdf_env_dir(S, F, rd);
                        const float wb = mis_balance(prev_pdf, pe);
                        rad = rad + clamp_ind(thr * sky_color(S, F, rd) * wb, F.firefly);
                    }
                } else if (!(st & kSkipSky)) {
                    if (b == 0u) rad = rad + thr * sky_color(S, F, rd);
                    else rad = rad + clamp_ind(thr * sky_color(S, F, rd), F.firefly);
                }
                ended = true;
            } else {
                const Surface sf = surface_at<kProc>(S, ro, rd, h);
                const V3 hp = ro + rd * h.t;
                const float ndi = dot(sf.normal, rd);
                const V3 nf = (ndi < 0.0f) ? sf.normal : -sf.normal;
                if (any_pos(sf.emission)) {
                    if (b == 0u) rad = rad + thr * sf.emission;
                    else rad = rad + clamp_ind(thr * sf.emission, F.firefly);
                }
                if (kAdj && sf.mid != kNoMat) {
                    // emission term thr*E: d/dE = thr; albedo factor of this vertex
                    // scales everything the path collects after its emission
                    // (this vertex's NEE through the brdf, later vertices through
                    // the throughput): d/da = (R_total - R_so_far) / a
                    const V3 g = adj_weight<kB>(A, F, p);
                    if (any_pos(sf.emission)) adj_add(A, 1, sf.mid, g * thr);
                    if (sf.mat == kMatLambert || sf.mat == kMatMetal) {
                        const V3 total = v3(A.srad[A.srec_base + p]);
                        adj_add(A, 0, sf.mid, g * safe_div(total - rad, sf.albedo));
                    }
                }
                if (sf.mat == kMatLambert) {
                    const V3 so = hp + nf * 1e-3f;
                    if (F.light_count > 0u) {
                        V3 ldir, Le;
                        float lpdf, ldist;
                        sample_light(S, F, hp, nf, seed, ldir, Le, lpdf, ldist);
                        const float ndl = dot(nf, ldir);
                        if (lpdf > 0.0f && ndl > 0.0f) {
                            const float tmax = fmaxf(ldist - 1e-3f, 0.0f);
                            issue_shadow(P, p, 0, so, ldir, tmax, thr * Le, 1.0f, sf.albedo / kPi, ndl,
                                         lpdf, b != 0u, shadow_mask);
                        }
                    }
                    if (F.env_present) {
                        const float xu = randf(seed);
                        const float xv = randf(seed);
                        V3 edir, ecol;
                        float epdf;
                        sample_env(S, F, xu, xv, edir, ecol, epdf);
                        const float ndl = dot(nf, edir);
                        if (epdf > 0.0f && ndl > 0.0f) {
                            const float pdf_brdf = ndl * kInvPi;
                            const bool fire = (F.mis != 0u) && ((b + 1u) < F.maxb);
                            const float wl = fire ? mis_balance(epdf, pdf_brdf) : 1.0f;
                            issue_shadow(P, p, 1, so, edir, 1e30f, thr * ecol, wl, sf.albedo / kPi, ndl,
                                         epdf, true, shadow_mask);
                        }
                        if (S.hdri_count > 0u) {
                            const float u = randf(seed);
                            float acc = 0.0f;
                            uint32_t sel = 0;
                            for (uint32_t k = 0; k < 8u; ++k) {
                                if (k >= S.hdri_count) break;
                                acc += S.hdri_dir[k].w;
                                if (u <= acc) { sel = k; break; }
                                sel = k;
                            }
                            const V3 hdir = v3(S.hdri_dir[sel]);
                            const V3 hcol = v3(S.hdri_col[sel]) * F.env_intensity;
                            const float hpdf = fmaxf(S.hdri_dir[sel].w, 1e-6f);
                            const float ndl2 = dot(nf, hdir);
                            if (ndl2 > 0.0f && hpdf > 0.0f)
                                issue_shadow(P, p, 2, so, hdir, 1e30f, thr * hcol, 1.0f, sf.albedo / kPi,
                                             ndl2, hpdf, b != 0u, shadow_mask);
                        }
                        st = (F.mis == 0u) ? (st | kSkipSky) : (st & ~kSkipSky);
                    } else {
                        // gradient sky: sun NEE (slot 1), moon NEE (slot 2), skylight
                        // ambient (shaders/PathTrace.slang:6546-6667); none clamped
                        const V3 sun_dir = F.sun_dir;
                        if (sun_dir.y > 0.0f) {
                            const float n_dot_l = fmaxf(0.0f, dot(nf, sun_dir));
                            const V3 sun_jit = sample_sun_disc(sun_dir, seed);
                            const float am = 1.0f / fmaxf(sun_dir.y, 0.04f);
                            const float trans_atm = f_exp(-0.30f * am);
                            const float warmth = saturatef((am - 1.0f) * 0.18f);
                            const V3 sun_col = lerp3(v3(1.00f, 0.97f, 0.92f), v3(1.55f, 0.55f, 0.20f), warmth);
                            const float strength = 80.0f * trans_atm;
                            const V3 sun_rad = sun_col * strength;
                            if (n_dot_l > 0.0f)
                                issue_shadow(P, p, 1, so, sun_jit, 1e30f, thr * sun_rad, 1.0f, sf.albedo / kPi,
                                             n_dot_l, 1.0f, false, shadow_mask);
                        }
                        if (F.moon.y > 0.0f) {
                            const float phase_b = 0.5f * (1.0f - f_cos(F.moon.w));
                            if (phase_b > 0.01f) {
                                const V3 moon_jit = sample_sun_disc(v3(F.moon), seed);
                                const float ndl = fmaxf(0.0f, dot(nf, moon_jit));
                                if (ndl > 0.0f) {
                                    const float m_elev = fmaxf(F.moon.y, 0.04f);
                                    const float m_am = 1.0f / m_elev;
                                    const float m_atm = f_exp(-0.30f * m_am);
                                    const float m_warmth = saturatef((m_am - 1.0f) * 0.18f);
                                    const V3 m_col =
                                        lerp3(v3(0.92f, 0.94f, 1.00f), v3(1.20f, 0.65f, 0.40f), m_warmth);
                                    const V3 moon_rad = m_col * (0.3f * phase_b * m_atm);
                                    issue_shadow(P, p, 2, so, moon_jit, 1e30f, thr * moon_rad, 1.0f,
                                                 sf.albedo / kPi, ndl, 1.0f, false, shadow_mask);
                                }
                            }
                        }
                        P.amb[p] = f4(thr * sf.albedo * sky_base(F, nf), 0.0f);
                        shadow_mask |= kAmbBit;
                        st |= kSkipSky;
                    }
                    thr = thr * sf.albedo;
                    ro = hp + nf * 1e-3f;
                    rd = cos_hemi(nf, seed);
                    if (F.mis != 0u && F.env_present) {
                        prev_pdf = fmaxf(0.0f, dot(nf, rd)) * kInvPi;
                        st |= kPrevLambert;
                    } else {
                        st &= ~kPrevLambert;
                    }
                } else if (sf.mat == kMatMetal) {
                    V3 r = reflect(rd, nf);
                    r = normalize(r + sf.rough * (cos_hemi(nf, seed) - nf));
                    thr = thr * sf.albedo;
                    ro = hp + nf * 1e-3f;
                    rd = r;
                    st &= ~(kSkipSky | kPrevLambert);
                } else if (sf.mat == kMatDielectric) {
                    const float ia = (ndi < 0.0f) ? 1.0f : sf.ior;
                    const float ib = (ndi < 0.0f) ? sf.ior : 1.0f;
                    const float eta = ia / ib;
                    const float cos_i = fabsf(dot(nf, -rd));
                    float r0 = (ia - ib) / (ia + ib);
                    r0 = r0 * r0;
                    const float fr = schlick(cos_i, r0);
                    const V3 refl = reflect(rd, nf);
                    const V3 refr = refract(rd, nf, eta);
                    const bool tir = length(refr) < 1e-3f;
                    if (tir || randf(seed) < fr) {
                        rd = refl;
                        ro = hp + nf * 1e-3f;
                        st &= ~(kSkipSky | kPrevLambert);
                    } else {
                        rd = normalize(refr);
                        ro = hp - nf * 1e-3f;
                    }
                }
                if (b >= F.rr_start) {
                    float pr = fmaxf(thr.x, fmaxf(thr.y, thr.z));
                    pr = clampf(pr, 0.05f, 1.0f);
                    if (!kB && P.rr_frozen) {
                        float* slot = P.rr_frozen + size_t(p) * F.maxb + b;
                        if (P.rr_mode == 1u) *slot = pr;
                        else pr = *slot;
                    }
                    if (randf(seed) > pr) ended = true;
                    else thr = thr / pr;
                }
                if (b + 1u >= F.maxb) ended = true;
            }
            if (ended) st |= kEnded;
            if (!ended) {
                P.ray_o[p] = f4(ro, 0.0f);
                P.ray_d[p] = f4(rd, 0.0f);
                oct = F.octant_on ? ((rd.x < 0.0f ? 1u : 0u) | (rd.y < 0.0f ? 2u : 0u) | (rd.z < 0.0f ? 4u : 0u)) : 0u;
            }
            P.thr[p] = f4(thr, prev_pdf);
            P.rad[p] = f4(rad, 0.0f);
            P.state[p] = st;
            P.seed[p] = seed;
            P.shmask[p] = shadow_mask;
            cont = !ended;
            }
        }
        // compaction: survivors to the next queue in the block's path order (a
        // counting sort in shared memory; keeping that order makes the next
        // kernels' path-record accesses more contiguous than per-warp atomic
        // appends, which measured -3.3% on the 1080p triangle scene).  With
        // octant grouping on (a batch tuning knob) the entries are grouped by the
        // direction octant of their next ray, so that a closest-hit warp mostly
        // holds rays of one octant; it measured +2.4% with the 8 x 4 camera tiles
        // and -0.7% with the current build.  Shadow rays go to the shadow queue,
        // a path's entries (slots 0-2 of the mask; bit 8 is the ambient flag)
        // next to each other, reserved for the whole block by the same thread
        // and between the same barriers (one global atomic per block and
        // iteration instead of up to three per warp: +0.2% on the 1080p triangle
        // scene, +0.7% on the 256 x 256 analytic one).  (Two histograms and two
        // shadow counters used in turn: iteration it counts into s_hist[it & 1]
        // and s_sh[it & 1] and clears the others for the next iteration, two
        // barriers each.  Compacting every second iteration instead, with one
        // barrier per iteration and double-buffered lists, measured -2.0%.)
        const uint32_t hb = it & 1u;
        const uint32_t rank = cont ? atomicAdd(&s_hist[hb][oct], 1u) : 0u;
        const uint32_t nsh = uint32_t(__popc(shadow_mask & 7u));
        const uint32_t srank = nsh ? atomicAdd(&s_sh[hb], nsh) : 0u;
        __syncthreads();
        if (threadIdx.x < 8u) s_hist[hb ^ 1u][threadIdx.x] = 0u;
        if (threadIdx.x == 8u) s_sh[hb ^ 1u] = 0u;
        if (threadIdx.x == 0u) {
            uint32_t tot = 0;
            for (int o = 0; o < 8; ++o) {
                s_base[o] = tot;
                tot += s_hist[hb][o];
            }
            s_block = tot ? atomicAdd(P.cnt_next, tot) : 0u;
            const uint32_t stot = s_sh[hb];
            s_sblock = stot ? atomicAdd(P.cnt + 1, stot) : 0u;
        }
        __syncthreads();
        if (cont) qn[s_block + s_base[oct] + rank] = p;
        uint32_t ss = s_sblock + srank;
        for (int k = 0; k < 3; ++k)
            if ((shadow_mask >> k) & 1u) P.sq[ss++] = 3u * p + uint32_t(k);
    }
    if (kAdj) adj_end(A);
}

template <bool kWide>
__global__ void __launch_bounds__(kThreads, 4) k_shadow(DScene S, DPaths P, int kmax) {
    const uint32_t n = P.cnt[1];
    uint32_t segs = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t e = P.sq[i];
        const float4 o = P.sh_o[e], d = P.sh_d[e];
        const V3 tr = transmittance(S, v3(o), v3(d), o.w, kmax, segs, kWide);
        P.sh_tr[e] = f4(tr, 0.0f);
    }
    warp_add(P.stat + 1, segs);
}


// persistent closest hit for a queue of rays (extension rays or first shadow segments)
// (kProc false: the procedural SDF walker compiled out, for launches whose scenes
// hold no procedural cluster in use; it keeps the hot traversal loop lean)
// (kCount: the counting variant of profiling mode 3, which also tallies nodes,
// primitives and stack operations into S.tcount)
template <bool kB, bool kProc = true, bool kCount = false>
__global__ void __launch_bounds__(kThreads, 4) k_closest(const __grid_constant__ DScene S, Batch B,
                                                         const uint32_t* queue, const uint32_t* count,
                                                         const float4* ray_o, const float4* ray_d, float* out_t,
                                                         uint32_t* out_id, uint32_t* fetch_ctr,
                                                         unsigned long long* stat) {
    uint32_t done = 0;
    persistent_closest<false, kB, false, kProc, kCount>(&S, ItemScenes{B.scenes, B.path_scene}, queue, *count, ray_o, ray_d, out_t,
                                  out_id, fetch_ctr, done, ShadowIO{});
    warp_add(stat, done);
}

// persistent transmittance: whole dielectric chains per lane (every segment
// counted as a shadow segment)
template <bool kB, bool kMats, bool kProc = true, bool kCount = false>
__global__ void __launch_bounds__(kThreads, kTransmitBlocks) k_transmit(const __grid_constant__ DScene S, Batch B, DPaths P,
                                                          int kmax, uint4* sh_mats) {
    uint32_t done = 0;
    const ShadowIO io{P.sh_o, P.sh_d, P.sh_tr, kmax, sh_mats};
    persistent_closest<true, kB, kMats, kProc, kCount>(&S, ItemScenes{B.scenes, B.path_scene}, P.sq, P.cnt[1], P.sh_o, P.sh_d, nullptr,
                                 nullptr, P.cnt + 3, done, io);
    warp_add(P.stat + 1, done);
}

// End of a sample: the paths that ended (at any bounce) get their last
// vertex's NEE terms and add the sample's radiance to the frame sum
// (shaders/PathTrace.slang:7701); differentiable records keep it per sample.
// An ended path's shadow slots and mask are its own and no later launch of the
// sample writes them, so resolving here gives the values the path had when it
// ended.  One thread per path slot of the wave; batched views with fewer
// samples than this one (their paths were not restarted) are skipped.
template <bool kB, bool kAdj>
__global__ void k_finish(const __grid_constant__ DScene S0, const __grid_constant__ DFrame F0, DPaths P, Batch B,
                         const __grid_constant__ Adj A, uint32_t npaths, uint32_t s, size_t srec_base) {
    if (kAdj) adj_begin(A);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npaths; p += gridDim.x * blockDim.x) {
        const DFrame& F = kB ? B.views[B.path_view[p]] : F0;
        if (kB && s >= F.spp) continue;
        if (!(P.state[p] & kEnded)) continue;
        const uint32_t mask = P.shmask[p];
        V3 rad = v3(P.rad[p]);
        if (mask) rad = resolve_nee<kB, kAdj>(S0, F, P, B, A, p, mask, rad);
        const float4 fs = P.fsum[p];
        P.fsum[p] = make_float4(fs.x + rad.x, fs.y + rad.y, fs.z + rad.z, 0.0f);
        if (P.srad) P.srad[srec_base + p] = f4(rad, 0.0f);
    }
    if (kAdj) adj_end(A);
}

// running mean / EMA (shaders/PathTrace.slang:7707-7781)
__device__ __forceinline__ float clean(float v) { return (isnan(v) || isinf(v)) ? 0.0f : fmaxf(v, 0.0f); }

__device__ __forceinline__ float4 accum_update(float4 a, float4 fs, float nspp, bool reset, float ema_in) {
    const float ema = clampf(ema_in, 0.0f, 0.999f);
    V3 fr = v3(fs) / nspp;
    fr = v3(clean(fr.x), clean(fr.y), clean(fr.z));
    if (reset) a = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (isnan(a.x) || isinf(a.x) || isnan(a.y) || isinf(a.y) || isnan(a.z) || isinf(a.z) || isnan(a.w) ||
        isinf(a.w))
        a = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const V3 pr = v3(a);
    float n_new;
    V3 avg;
    if (a.w < 0.5f || ema <= 0.0f) {
        n_new = a.w + 1.0f;
        avg = (pr * a.w + fr) / n_new;
    } else {
        avg = pr * ema + fr * (1.0f - ema);
        n_new = fminf(a.w + 1.0f, 1.0f / fmaxf(1.0f - ema, 1e-3f));
    }
    return f4(avg, n_new);
}

__global__ void k_accumulate(DFrame F, DPaths P, float4* accum, uint32_t nframes, float ema_in) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;   // path slot within a frame
    if (pix >= F.npix) return;
    const bool reset_first = P.wave[2] != 0u;
    uint32_t x, y;
    slot_pixel(F, pix, x, y);
    const size_t out = size_t(y) * F.W + x;
    float4 a = accum[out];
    const float nspp = float(F.spp == 0u ? 1u : F.spp);
    for (uint32_t f = 0; f < nframes; ++f)
        a = accum_update(a, P.fsum[size_t(f) * F.npix + pix], nspp, f == 0 && reset_first, ema_in);
    accum[out] = a;
}

// batched renders: one frame of every view, each into its own region
// one thread per pixel of every view (npix_total = sum of the views' pixels):
// the view's frames of this wave in order, as consecutive running-mean updates
__global__ void k_accumulate_batch(DPaths P, Batch B, uint32_t npix_total) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npix_total) return;
    uint32_t lo = 0, hi = B.n_views;   // last view with accum_base <= t
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (B.views[mid].accum_base <= t) lo = mid;
        else hi = mid;
    }
    const DFrame& V = B.views[lo];
    const uint32_t pix = uint32_t(t - V.accum_base);
    uint32_t x, y;
    slot_pixel(V, pix, x, y);
    const size_t out = V.accum_base + size_t(y) * V.W + x;
    float4 a = B.accum[out];
    const float nspp = float(V.spp == 0u ? 1u : V.spp);
    for (uint32_t f = 0; f < V.nframes; ++f)
        a = accum_update(a, P.fsum[V.slot_base + f * V.npix + pix], nspp, f == 0u && V.reset != 0u, V.ema);
    B.accum[out] = a;
}

// ---------------------------------------------------------------------------
// Output step: exposure, tone map and 8-bit quantisation of the accumulation
// buffer (shaders/PathTrace.slang:3466-3607, 7925-7929).
// ---------------------------------------------------------------------------
constexpr float kInvLn2 = 0x1.715476p+0f;
__device__ __forceinline__ float f_log2(float x) { return f_log(x) * kInvLn2; }
__device__ __forceinline__ float pow_nz(float x, float y) { return (y == 1.0f) ? x : f_pow(x, y); }
__device__ __forceinline__ V3 div3(V3 a, V3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }

__device__ __forceinline__ V3 tm_aces(V3 c) {
    const float a = 2.51f, b = 0.03f, d = 2.43f, e = 0.59f, f = 0.14f;
    const V3 num = c * (c * a + v3(b, b, b));
    const V3 den = c * (c * d + v3(e, e, e)) + v3(f, f, f);
    const V3 r = div3(num, den);
    return v3(saturatef(r.x), saturatef(r.y), saturatef(r.z));
}
__device__ __forceinline__ float agx_contrast(float x) {
    const float x2 = x * x, x4 = x2 * x2;
    return 15.5f * x4 * x2 - 40.14f * x4 * x + 31.96f * x4 - 6.868f * x2 * x + 0.4298f * x2 + 0.1191f * x -
           0.00232f;
}
__device__ V3 tm_agx(V3 c) {
    const V3 ir0 = v3(0.842479062253094f, 0.0784335999999992f, 0.0792237451477643f);
    const V3 ir1 = v3(0.0423282422610123f, 0.878468636469772f, 0.0791661274605434f);
    const V3 ir2 = v3(0.0423756549057051f, 0.0784336f, 0.879142973793104f);
    V3 v = v3(dot(ir0, c), dot(ir1, c), dot(ir2, c));
    const float kMinEv = -12.47393f, kMaxEv = 4.026069f;
    float t[3] = {v.x, v.y, v.z};
    for (int k = 0; k < 3; ++k) {
        float l = clampf(f_log2(fmaxf(t[k], 1e-10f)), kMinEv, kMaxEv);
        l = (l - kMinEv) / (kMaxEv - kMinEv);
        t[k] = agx_contrast(l);
    }
    v = v3(t[0], t[1], t[2]);
    const float luma = dot(v, v3(0.2126f, 0.7152f, 0.0722f));
    v = v3(pow_nz(fmaxf(v.x * 1.0f + 0.0f, 0.0f), 1.0f), pow_nz(fmaxf(v.y * 1.0f + 0.0f, 0.0f), 1.0f),
           pow_nz(fmaxf(v.z * 1.0f + 0.0f, 0.0f), 1.0f));
    v = v3(luma, luma, luma) + (v - v3(luma, luma, luma)) * 1.0f;
    const V3 or0 = v3(1.19687900512017f, -0.0980208811401368f, -0.0990297440797205f);
    const V3 or1 = v3(-0.0528968517574562f, 1.15190312990417f, -0.0989611768448433f);
    const V3 or2 = v3(-0.0529716355144438f, -0.0980434501171241f, 1.15107367264116f);
    v = v3(dot(or0, v), dot(or1, v), dot(or2, v));
    v = v3(pow_nz(fmaxf(v.x, 0.0f), 2.2f), pow_nz(fmaxf(v.y, 0.0f), 2.2f), pow_nz(fmaxf(v.z, 0.0f), 2.2f));
    return v3(saturatef(v.x), saturatef(v.y), saturatef(v.z));
}
__device__ V3 tm_khronos(V3 c) {
    const float start = 0.8f - 0.04f, desat = 0.15f;
    const float x = fminf(c.x, fminf(c.y, c.z));
    const float offset = (x < 0.08f) ? (x - 6.25f * x * x) : 0.04f;
    c = c - v3(offset, offset, offset);
    const float peak = fmaxf(c.x, fmaxf(c.y, c.z));
    if (peak < start) return c;
    const float d = 1.0f - start;
    const float new_peak = 1.0f - d * d / (peak + d - start);
    c = c * (new_peak / peak);
    const float g = 1.0f - 1.0f / (desat * (peak - new_peak) + 1.0f);
    return lerp3(c, v3(new_peak, new_peak, new_peak), g);
}
__device__ __forceinline__ float srgb_oetf(float c) {
    c = fmaxf(c, 0.0f);
    return (c < 0.0031308f) ? c * 12.92f : 1.055f * f_pow(c, 1.0f / 2.4f) - 0.055f;
}
__device__ __forceinline__ V3 tonemap_op(V3 c, uint32_t op) {
    switch (op) {
        case 1u: return tm_agx(c);
        case 2u: return tm_khronos(c);
        case 3u: {
            const V3 r = div3(c, v3(1.0f, 1.0f, 1.0f) + c);
            return v3(saturatef(r.x), saturatef(r.y), saturatef(r.z));
        }
        case 4u: return v3(saturatef(c.x), saturatef(c.y), saturatef(c.z));
        default: return tm_aces(c);
    }
}
__device__ __forceinline__ uint32_t unorm8(float v) { return uint32_t(saturatef(v) * 255.0f + 0.5f); }

__global__ void k_tonemap(const float4* accum, uint32_t n, float exposure, uint32_t op, uint32_t srgb,
                          uchar4* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V3 ldr = tonemap_op(v3(accum[i]) * exposure, op);
    if (srgb) ldr = v3(srgb_oetf(ldr.x), srgb_oetf(ldr.y), srgb_oetf(ldr.z));
    out[i] = make_uchar4(uint8_t(unorm8(ldr.x)), uint8_t(unorm8(ldr.y)), uint8_t(unorm8(ldr.z)), 255);
}

// identity queue for the trace probe through the persistent kernel: q[i] = i,
// then the count n and a zeroed fetch counter
__global__ void k_probe_queue(uint32_t* q, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) q[i] = i;
    if (i == 0) {
        q[n] = n;
        q[n + 1] = 0u;
    }
}

// triangle hits of the persistent kernel name the wide-leaf slot: report the
// original triangle index (stored in the slot's first float4 .w)
__global__ void k_probe_ids(DScene S, uint32_t n, uint32_t* hit, float* t) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t id = hit[i];
    if (id != kMiss && (id & kTriBit) && !(id & kSdfBit)) {
        const float4* T = (id & kMergedTri) ? S.mtri4 : ((id & kRefTri) ? S.tri : S.tri4);
        id = kTriBit | __float_as_uint(T[3u * (id & ~(kTriBit | kMergedTri | kRefTri))].w);
    }
    hit[i] = id;
    if (id == kMiss) t[i] = 0.0f;
}

__global__ void k_trace_probe(DScene S, const float4* ro, const float4* rd, uint32_t n, uint32_t* hit,
                              float* t) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 o = ro[i], d = rd[i];
    const float tinit = (d.w > 0.0f) ? d.w : 1e30f;
    const HitRec h = trace_any_mode(S, v3(o), v3(d), tinit, S.use_wide != 0u);
    uint32_t id = h.id;
    if (id != kMiss && (id & kTriBit) && !(id & kSdfBit)) {
        const uint32_t slot = id & ~(kTriBit | kRefTri);
        const float4 a = (S.use_wide && S.t_wide && !(id & kRefTri)) ? S.tri4[3u * slot] : S.tri[3u * slot];
        id = kTriBit | __float_as_uint(a.w);
    }
    hit[i] = id;
    t[i] = (h.id == kMiss) ? 0.0f : h.t;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <class T> struct DBuf {
    T* p = nullptr;
    size_t n = 0;
};

}  // namespace

// a cached CUDA graph of one plain-render wave (launch_wave_graph)
struct WaveGraph {
    cudaGraphExec_t exec = nullptr;
    std::vector<unsigned char> key;   // the launch parameters it was captured with
    std::array<uint32_t, 4> topo{};   // what fixes its node list
    uint64_t used = 0;                // last use, for replacement
};

struct pt_gpu_ctx {
    int device = 0;
    int sm_count = 152;
    std::string err;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // second stream: the next bounce's closest-hit pass runs on it while the
    // shadow rays of the current bounce run on `stream` (fork/join by events)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // small waves run as two halves at once: the second half on its own pair of
    // streams (stream2 + side2, the same fork/join), started and joined by events
    cudaStream_t stream2 = nullptr, side2 = nullptr;
    cudaEvent_t ev_fork2 = nullptr, ev_join2 = nullptr, ev_split = nullptr, ev_half = nullptr;
    // scene
    DBuf<float4> prim_rec, prim_geo, bvh, tri, tri_bvh, mats, lights, env;
    DBuf<uint32_t> prim_type, prim_mat;
    bool has_prim_mat = false;
    DBuf<float> marg, cond;
    DBuf<uint32_t> marg_guide, cond_guide;   // DScene::marg_guide / cond_guide
    bool env_guided = false;
    uint32_t prim_count = 0, linear_count = 0, bvh_nodes = 0, tri_slots = 0, tri_nodes = 0, tri_count = 0;
    uint32_t mat_count = 0, light_count = 0, env_w = 0, env_h = 0, hdri_count = 0;
    bool mesh_has_mat = false;
    float hdri_dir[32] = {0}, hdri_col[32] = {0};
    DBuf<float4> moon;
    uint32_t moon_w = 0, moon_h = 0;
    DBuf<uchar4> ldr;
    DBuf<float4> ltree;
    uint32_t ltree_nodes = 0;
    DBuf<float4> sdf;
    uint32_t sdf_count = 0;
    bool sdf_proc_any = false;   // some cluster holds a procedural op (5-9)
    DBuf<uint32_t> err_word;
    DBuf<uint32_t> wave_vars;   // DPaths::wave
    // reference tie ranks of the wide trees' items (kept for the merged tree)
    DBuf<uint32_t> t_rank, a_rank;
    // the reference BVH leaf of each item (DScene::t_leaf / m_leaf / a_leaf);
    // tslot_leaf: per triangle slot of the reference order, gathered into the wide orders
    DBuf<uint32_t> t_leaf, m_leaf, a_leaf, tslot_leaf;
    // merged 4-wide tree over the triangles and the finite analytic records
    bool m_wide = false;
    DBuf<float4> m4, mtri4, ma4_geo;
    DBuf<uint4> ma4_meta;
    uint32_t m4_count = 0, m4_depth = 0;
    uint32_t dbg_trav_cap = 0, dbg_stack_cap = 0;   // pt_gpu_set_debug_limits (0 = defaults)
    // target
    uint32_t W = 0, H = 0;
    DBuf<float4> accum;
    // wave buffers
    size_t cap = 0;
    DBuf<float4> ray_o, ray_d, thr, rad, fsum, amb, sh_o, sh_d, sh_pre, sh_brdf, sh_tr;
    DBuf<uint32_t> seed, state, hit_id, shmask, q0, q1, sq, cnt;
    DBuf<float> hit_t;
    DBuf<unsigned long long> stat;
    DBuf<unsigned long long> tcount;   // traversal counters (profiling mode 3), 16 entries
    uint32_t wave_frames_override = 0;
    // wide SAH trees built on the device at upload
    int traversal = 0;   // 0 wide (default), 1 reference BVHs
    bool a_wide = false, t_wide = false;
    uint32_t a4_count = 0, t4_count = 0, a4_depth = 0, t4_depth = 0;
    DBuf<float4> a4, a4_geo, t4, tri4, tri_lo, tri_hi;
    DBuf<uint4> a4_meta;
    double build_ms = 0.0;
    uint32_t t4_bin_nodes = 0;
    // batched renders
    DBuf<DFrame> b_views;
    DBuf<DScene> b_scenes;
    DBuf<uint32_t> b_view_base, b_path_view, b_path_scene;
    DBuf<float4> b_accum;
    std::vector<size_t> b_accum_off;
    std::vector<uint32_t> b_w, b_h;
    std::vector<DFrame> b_views_h;
    cudaGraphExec_t b_graph = nullptr;
    // plain renders: cached wave graphs (launch_wave_graph)
    int render_graphs = 0;
    uint64_t graph_clock = 0;
    WaveGraph wave_graphs[8];
    std::vector<uint64_t> b_sig;
    PtBatchTuning b_tune{4u, 8u, 1u, 512u, 4u, 0u, 0u, 0u};
    double b_tune_default_ms = 0.0, b_tune_best_ms = 0.0;   // last pt_gpu_batch_autotune
    // differentiable renders: the recorded forward and the replay's buffers
    DBuf<float4> d_srad, d_dldi;
    int rr_freeze = 0;           // pt_gpu_set_roulette_freeze: 0 off, 1 record, 2 replay
    DBuf<float> rr_buf;          // survival probabilities [sample][path][bounce]
    uint32_t rr_meta[5] = {};    // W, H, frames, spp, max_bounces of the recording
    DBuf<double> d_grad;
    DBuf<uint4> d_sh_mats;
    bool d_valid = false;
    uint64_t d_gen = 0;
    PtPushHead d_head{};
    PtPathParams d_prm{};
    uint32_t d_frames = 0;
    uint64_t gen = 0;   // bumped by every upload / target change
    PtStats d_bwd_stats{};
    pt_gpu_ctx* d_batch_scene = nullptr;
    std::vector<PtBatchView> d_batch_views;
    PtStats stats{};
    int profile = 0;            // 0 off, 1 events on the overlapped schedule, 2 events, stages serial,
                                // 3 as 2 with the counting traversal variants
    std::vector<cudaEvent_t> ev_pool;
};

namespace {

int set_err(pt_gpu_ctx* c, int code, const std::string& m) {
    if (c) c->err = m;
    return code;
}

// NVTX range over a scope: a render's waves, samples, bounces and stages show
// up as named ranges in Nsight tools (ncu --nvtx --nvtx-include "bounce 0/"
// selects one bounce's kernels); without a tool attached a push or pop is a
// no-op call.
struct Nvtx {
    explicit Nvtx(const char* name) { nvtxRangePushA(name); }
    Nvtx(const char* fmt, uint32_t a) {
        char b[48];
        std::snprintf(b, sizeof(b), fmt, a);
        nvtxRangePushA(b);
    }
    ~Nvtx() { nvtxRangePop(); }
    Nvtx(const Nvtx&) = delete;
    Nvtx& operator=(const Nvtx&) = delete;
};

// Message for a traversal error word (bit 0: a query ran into the iteration
// cap; bit 1: a wide-tree walk needed more stack entries than allowed).
std::string traversal_error(uint32_t w) {
    std::string m;
    if (w & 1u) m += "traversal iteration cap reached (malformed BVH?)";
    if (w & 2u) m += std::string(m.empty() ? "" : "; ") + "traversal stack overflow (tree deeper than the stack)";
    return m.empty() ? "traversal error" : m;
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e__ = (call);                                                         \
        if (e__ != cudaSuccess)                                                           \
            return set_err(ctx, PT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e__)); \
    } while (0)

template <class T> void dfree(DBuf<T>& b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
}

template <class T> int dalloc(pt_gpu_ctx* ctx, DBuf<T>& b, size_t n) {
    if (b.n >= n && b.p) return PT_OK;
    dfree(b);
    if (n == 0) return PT_OK;
    cudaError_t e = cudaMalloc(&b.p, n * sizeof(T));
    if (e != cudaSuccess) {
        b.p = nullptr;
        return set_err(ctx, PT_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    b.n = n;
    return PT_OK;
}

template <class T> int dupload(pt_gpu_ctx* ctx, DBuf<T>& b, const void* src, size_t n) {
    int rc = dalloc(ctx, b, n);
    if (rc) return rc;
    if (n) CK(cudaMemcpyAsync(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    return PT_OK;
}

// BVH sanity: children after their parent (so traversal terminates), leaf ranges
// inside the prim range.  Malformed input is rejected before any kernel reads it.
bool check_bvh(const PtBvhNode* nodes, uint32_t n_nodes, uint32_t n_leaf_items, std::string& why) {
    for (uint32_t i = 0; i < n_nodes; ++i) {
        const PtBvhNode& nd = nodes[i];
        if (nd.count > 0u) {
            if (uint64_t(nd.left_first) + nd.count > n_leaf_items) {
                why = "leaf range out of bounds at node " + std::to_string(i);
                return false;
            }
        } else if (nd.left_first <= i || uint64_t(nd.left_first) + 1 >= n_nodes) {
            why = "bad child index at node " + std::to_string(i);
            return false;
        }
    }
    return true;
}

DScene make_scene(pt_gpu_ctx* c, const PtPathParams* prm) {
    DScene S{};
    S.prim_geo = c->prim_geo.p;
    S.prim_type = c->prim_type.p;
    S.prim_rec = c->prim_rec.p;
    S.prim_count = c->prim_count;
    S.linear_count = c->linear_count;
    S.bvh = c->bvh.p;
    S.bvh_nodes = c->bvh_nodes;
    S.tri = c->tri.p;
    S.tri_slots = c->tri_slots;
    S.tri_bvh = c->tri_bvh.p;
    S.tri_nodes = c->tri_nodes;
    S.tri_enabled = (c->tri_nodes > 0u) ? 1u : 0u;
    S.mesh_has_mat = c->mesh_has_mat ? 1u : 0u;
    S.mats = c->mats.p;
    S.mat_count = c->mat_count;
    S.prim_mat = c->has_prim_mat ? c->prim_mat.p : nullptr;
    S.lights = c->lights.p;
    S.light_count = c->light_count;
    S.env = c->env.p;
    S.marg = c->marg.p;
    S.cond = c->cond.p;
    S.marg_guide = c->env_guided ? c->marg_guide.p : nullptr;
    S.cond_guide = c->env_guided ? c->cond_guide.p : nullptr;
    S.env_w = c->env_w;
    S.env_h = c->env_h;
    S.hdri_count = c->hdri_count;
    for (int i = 0; i < 8; ++i) {
        S.hdri_dir[i] = make_float4(c->hdri_dir[4 * i], c->hdri_dir[4 * i + 1], c->hdri_dir[4 * i + 2],
                                    c->hdri_dir[4 * i + 3]);
        S.hdri_col[i] = make_float4(c->hdri_col[4 * i], c->hdri_col[4 * i + 1], c->hdri_col[4 * i + 2],
                                    c->hdri_col[4 * i + 3]);
    }
    S.ltree = c->ltree.p;
    S.ltree_nodes = c->ltree_nodes;
    S.sdf = c->sdf.p;
    S.sdf_count = c->sdf_count;   // a dispatch's push overrides these
    S.sdf_iters = 128;            // r_sdf_max_iters default
    S.sdf_eps = 1e-4f;            // r_sdf_epsilon default
    S.frac_iters = 12;            // r_sdf_fractal_iters default
    S.frac_power = 8.0f;          // r_sdf_fractal_power default
    S.frac_eps_scale = 1.0f;      // r_sdf_de_eps_scale default
    S.moon_tex = c->moon.p;
    S.moon_w = c->moon_w;
    S.moon_h = c->moon_h;
    S.err = c->err_word.p;
    S.trav_cap = c->dbg_trav_cap ? c->dbg_trav_cap : kTraverseCap;
    S.stack_cap = c->dbg_stack_cap ? int(c->dbg_stack_cap) : kPStack;
    S.tcount = c->tcount.p;
    S.use_wide = (c->traversal == 0) ? 1u : 0u;
    S.a_wide = (S.use_wide && c->a_wide) ? 1u : 0u;
    S.t_wide = (S.use_wide && c->t_wide) ? 1u : 0u;
    S.a4 = c->a4.p;
    S.a4_geo = c->a4_geo.p;
    S.a4_meta = c->a4_meta.p;
    S.t4 = c->t4.p;
    S.tri4 = c->tri4.p;
    S.m4 = c->m4.p;
    S.mtri4 = c->mtri4.p;
    S.ma4_geo = c->ma4_geo.p;
    S.ma4_meta = c->ma4_meta.p;
    S.t_leaf = c->t_leaf.p;
    S.m_leaf = c->m_leaf.p;
    S.a_leaf = c->a_leaf.p;
    if (prm) {
        // the push tail decides what the kernel walks (bvh_params), as in the reference
        S.linear_count = prm->bvh_params[0];
        S.bvh_nodes = prm->bvh_params[1];
        S.tri_enabled = (prm->bvh_params[2] != 0u) ? 1u : 0u;
        S.tri_nodes = prm->bvh_params[3];
        S.light_count = prm->light_count;
        S.sdf_count = prm->sdf_params[0];
        S.sdf_iters = prm->sdf_params[1];
        S.sdf_eps = prm->sdf_params_f[0];
        S.frac_iters = prm->sdf_params[3];
        S.frac_power = prm->sdf_params_f[1];
        S.frac_eps_scale = prm->sdf_params_f[2];
        S.sdf_proc = min(prm->sdf_procedural_ops, 2u);
        S.sdf_nmode = prm->sdf_params_f[3] != 0.0f ? 1u : 0u;
    }
    // Without an analytic BVH in the dispatch the reference tests every record
    // linearly, in record order, with no box in front of it; far from a sphere
    // its float intersection cancels badly and can report hits that a box test
    // would cull, so the wide-tree kernels then scan the records too.
    if (S.bvh_nodes == 0u) S.a_wide = 0u;
    S.wide_linear = (S.bvh_nodes == 0u) ? S.prim_count : S.linear_count;
    // one walk over the merged tree when both parts would be walked and no SDF
    // cluster sits between them
    S.m_wide = (c->m_wide && S.a_wide && S.t_wide && S.tri_enabled && S.tri_nodes > 0u && S.sdf_count == 0u) ? 1u : 0u;
    return S;
}

// Sky of a dispatch: env map (mode 1, or 0 with a map), else the gradient
// (mode 0) or procedural (mode 2, stars off) dome with sun/moon discs and
// their NEE.  The Hosek-Wilkie dome (mode 3) and the stars are not built.
int check_sky(pt_gpu_ctx* ctx, const pt_gpu_ctx* sc, const PtPushHead* head, const PtPathParams* prm,
              const std::string& who) {
    const float mode = prm->sun_and_mode[3];
    if (mode == 3.0f) return set_err(ctx, PT_ERR_UNSUPPORTED, who + "the Hosek-Wilkie sky (mode 3) is not built");
    if (mode == 2.0f && prm->stars != 0u)
        return set_err(ctx, PT_ERR_UNSUPPORTED, who + "procedural-sky stars are not built (set stars = 0)");
    if (head->env_map_present) {
        if (sc->env_w == 0 || sc->env_h == 0) return set_err(ctx, PT_ERR_STATE, who + "env map not uploaded");
    } else if (prm->moon_dir_phase[1] >= -0.10f && sc->moon_w == 0) {
        return set_err(ctx, PT_ERR_STATE, who + "moon above the horizon but no moon texture (pt_gpu_upload_moon)");
    }
    return PT_OK;
}

void sky_of(DFrame& F, const PtPathParams* prm) {
    F.sun_dir = v3(prm->sun_and_mode[0], prm->sun_and_mode[1], prm->sun_and_mode[2]);
    F.moon = make_float4(prm->moon_dir_phase[0], prm->moon_dir_phase[1], prm->moon_dir_phase[2],
                         prm->moon_dir_phase[3]);
    F.moon_extra = make_float4(prm->moon_extra[0], prm->moon_extra[1], prm->moon_extra[2], prm->moon_extra[3]);
    F.sun_extra = make_float4(prm->sun_extra[0], prm->sun_extra[1], prm->sun_extra[2], prm->sun_extra[3]);
    F.sun_bright = prm->sun_extra2[0];
    F.sky_mode = (prm->sun_and_mode[3] == 2.0f) ? 2u : 0u;
    F.light_tree = (prm->light_tree_enabled != 0u && prm->light_tree_node_count > 0u) ? 1u : 0u;
}

// the dispatch's SDF cluster count must be the uploaded one
int check_sdf(pt_gpu_ctx* ctx, const pt_gpu_ctx* sc, const PtPathParams* prm, const std::string& who) {
    if (prm->sdf_params[0] != sc->sdf_count)
        return set_err(ctx, PT_ERR_INVALID, who + "sdf_params.x disagrees with the uploaded SDF clusters");
    return PT_OK;
}

// the dispatch's light tree must be the uploaded one
int check_light_tree(pt_gpu_ctx* ctx, const pt_gpu_ctx* sc, const PtPathParams* prm, const std::string& who) {
    if (prm->light_tree_enabled == 0u || prm->light_tree_node_count == 0u) return PT_OK;
    if (prm->light_tree_node_count != sc->ltree_nodes)
        return set_err(ctx, PT_ERR_INVALID, who + "light_tree_node_count disagrees with the uploaded light tree");
    return PT_OK;
}

int grid_for(pt_gpu_ctx* c, size_t work, int per_sm, int threads = kThreads) {
    const size_t need = (work + size_t(threads) - 1) / size_t(threads);
    const size_t cap = size_t(c->sm_count) * per_sm;
    return int(std::max<size_t>(1, std::min(need, cap)));
}

constexpr size_t kWavePaths = size_t(1) << 26;
// waves of at most this many paths run as two concurrent halves (render_waves)
constexpr size_t kSplitWavePaths = size_t(1) << 23;

// cdf_search's guide table of one CDF of n values: g[k] = the smallest i with
// cdf[i] >= k / kCdfGuide (n if none), g[kCdfGuide] = n.  False (no table) when
// the array is not non-decreasing or holds a NaN: the bracket argument needs a
// sorted array.
bool build_cdf_guide(const float* cdf, uint32_t n, uint32_t* g) {
    for (uint32_t i = 0; i < n; ++i)
        if (!(cdf[i] == cdf[i]) || (i + 1u < n && !(cdf[i] <= cdf[i + 1u]))) return false;
    uint32_t i = 0;
    for (uint32_t k = 0; k < kCdfGuide; ++k) {
        const float u = float(k) / float(kCdfGuide);
        while (i < n && cdf[i] < u) ++i;
        g[k] = i;
    }
    g[kCdfGuide] = n;
    return true;
}

int ensure_wave(pt_gpu_ctx* ctx, size_t npaths) {
    if (ctx->cap >= npaths) return PT_OK;
    int rc = 0;
    rc |= dalloc(ctx, ctx->ray_o, npaths);
    rc |= dalloc(ctx, ctx->ray_d, npaths);
    rc |= dalloc(ctx, ctx->thr, npaths);
    rc |= dalloc(ctx, ctx->rad, npaths);
    rc |= dalloc(ctx, ctx->fsum, npaths);
    rc |= dalloc(ctx, ctx->amb, npaths);
    rc |= dalloc(ctx, ctx->seed, npaths);
    rc |= dalloc(ctx, ctx->state, npaths);
    rc |= dalloc(ctx, ctx->hit_t, npaths);
    rc |= dalloc(ctx, ctx->hit_id, npaths);
    rc |= dalloc(ctx, ctx->shmask, npaths);
    rc |= dalloc(ctx, ctx->q0, npaths);
    rc |= dalloc(ctx, ctx->q1, npaths);
    rc |= dalloc(ctx, ctx->sq, 3 * npaths);

    rc |= dalloc(ctx, ctx->sh_o, 3 * npaths);
    rc |= dalloc(ctx, ctx->sh_d, 3 * npaths);
    rc |= dalloc(ctx, ctx->sh_pre, 3 * npaths);
    rc |= dalloc(ctx, ctx->sh_brdf, 3 * npaths);
    rc |= dalloc(ctx, ctx->sh_tr, 3 * npaths);

    if (rc) {
        ctx->cap = 0;   // some buffers were freed: the next call re-checks each one
        return PT_ERR_OOM;
    }
    ctx->cap = npaths;
    return PT_OK;
}


float o2f_host(uint32_t u) {
    const uint32_t v = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
    float f;
    std::memcpy(&f, &v, 4);
    return f;
}

// Binned-SAH binary tree over n items with boxes lo/hi (device), item order in idx.
int gpu_build_tree(pt_gpu_ctx* ctx, const float4* lo, const float4* hi, uint32_t n,
                   std::vector<ptb::Node2H>& nodes, DBuf<uint32_t>& idx) {
    nodes.clear();
    if (n == 0) return PT_OK;
    DBuf<uint32_t> tmp, ctr, bins, cnt2, cb;
    DBuf<float4> dnodes, tcmin, tcmax, ccmin, ccmax;
    DBuf<uint4> tinfo, chunks, cinfo, sinfo;
    DBuf<int4> split;
    auto cleanup = [&]() {
        dfree(tmp); dfree(ctr); dfree(bins); dfree(cnt2); dfree(cb); dfree(dnodes); dfree(tcmin);
        dfree(tcmax); dfree(ccmin); dfree(ccmax); dfree(tinfo); dfree(chunks); dfree(cinfo); dfree(sinfo);
        dfree(split);
    };
    int rc = 0;
    if ((rc = dalloc(ctx, idx, n)) || (rc = dalloc(ctx, tmp, n)) || (rc = dalloc(ctx, dnodes, 4 * size_t(n))) ||
        (rc = dalloc(ctx, ctr, 1)) || (rc = dalloc(ctx, cb, 6))) {
        cleanup();
        return rc;
    }
#define BK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e__ = (call);                                                         \
        if (e__ != cudaSuccess) {                                                         \
            cleanup();                                                                    \
            return set_err(ctx, PT_ERR_CUDA, std::string("bvh build: ") + cudaGetErrorString(e__)); \
        }                                                                                 \
    } while (0)
    k_iota<<<(n + 255) / 256, 256, 0, ctx->stream>>>(idx.p, n);
    const uint32_t init[7] = {1u, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u};
    BK(cudaMemcpyAsync(ctr.p, init, 4, cudaMemcpyHostToDevice, ctx->stream));
    BK(cudaMemcpyAsync(cb.p, init + 1, 24, cudaMemcpyHostToDevice, ctx->stream));
    ptb::kb_cbounds<<<std::min<uint32_t>((n + 255) / 256, 1024), 256, 0, ctx->stream>>>(lo, hi, n, cb.p);
    uint32_t cbh[6];
    BK(cudaMemcpyAsync(cbh, cb.p, 24, cudaMemcpyDeviceToHost, ctx->stream));
    BK(cudaStreamSynchronize(ctx->stream));
    std::vector<uint4> large, small;
    std::vector<float4> lmin, lmax;
    const float4 rmin = make_float4(o2f_host(cbh[0]), o2f_host(cbh[1]), o2f_host(cbh[2]), 0.0f);
    const float4 rmax = make_float4(o2f_host(cbh[3]), o2f_host(cbh[4]), o2f_host(cbh[5]), 0.0f);
    if (n > ptb::kSmallTask) {
        large.push_back(make_uint4(0, n, 0, 0));
        lmin.push_back(rmin);
        lmax.push_back(rmax);
    } else {
        small.push_back(make_uint4(0, n, 0, 0));
    }
    while (!large.empty()) {
        const uint32_t T = uint32_t(large.size());
        std::vector<uint4> ch;
        for (uint32_t t = 0; t < T; ++t)
            for (uint32_t b = large[t].x; b < large[t].y; b += ptb::kChunk)
                ch.push_back(make_uint4(t, b, std::min(b + ptb::kChunk, large[t].y), 0));
        const uint32_t nch = uint32_t(ch.size());
        if ((rc = dupload(ctx, tinfo, large.data(), T)) || (rc = dupload(ctx, tcmin, lmin.data(), T)) ||
            (rc = dupload(ctx, tcmax, lmax.data(), T)) || (rc = dupload(ctx, chunks, ch.data(), nch)) ||
            (rc = dalloc(ctx, bins, size_t(T) * ptb::kTaskBinWords)) || (rc = dalloc(ctx, split, T)) ||
            (rc = dalloc(ctx, cinfo, 2 * size_t(T))) || (rc = dalloc(ctx, ccmin, 2 * size_t(T))) ||
            (rc = dalloc(ctx, ccmax, 2 * size_t(T))) || (rc = dalloc(ctx, cnt2, 2 * size_t(T)))) {
            cleanup();
            return rc;
        }
        const uint32_t nw = T * ptb::kTaskBinWords;
        kb_init_bins<<<(nw + 255) / 256, 256, 0, ctx->stream>>>(bins.p, nw);
        ptb::kb_bin<<<nch, 256, 0, ctx->stream>>>(chunks.p, tcmin.p, tcmax.p, idx.p, lo, hi, bins.p);
        ptb::kb_split<<<(T + 127) / 128, 128, 0, ctx->stream>>>(T, tinfo.p, bins.p, dnodes.p, ctr.p, split.p,
                                                               cinfo.p, ccmin.p, ccmax.p, tcmin.p, tcmax.p);
        BK(cudaMemsetAsync(cnt2.p, 0, 8 * size_t(T), ctx->stream));
        ptb::kb_partition<<<nch, 256, 0, ctx->stream>>>(chunks.p, tinfo.p, split.p, tcmin.p, tcmax.p, idx.p, lo,
                                                         hi, cnt2.p, tmp.p);
        ptb::kb_copy<<<nch, 256, 0, ctx->stream>>>(chunks.p, tmp.p, idx.p);
        std::vector<uint4> ci(2 * T);
        std::vector<float4> cmn(2 * T), cmx(2 * T);
        BK(cudaGetLastError());
        BK(cudaMemcpyAsync(ci.data(), cinfo.p, 2 * size_t(T) * 16, cudaMemcpyDeviceToHost, ctx->stream));
        BK(cudaMemcpyAsync(cmn.data(), ccmin.p, 2 * size_t(T) * 16, cudaMemcpyDeviceToHost, ctx->stream));
        BK(cudaMemcpyAsync(cmx.data(), ccmax.p, 2 * size_t(T) * 16, cudaMemcpyDeviceToHost, ctx->stream));
        BK(cudaStreamSynchronize(ctx->stream));
        large.clear();
        lmin.clear();
        lmax.clear();
        for (uint32_t c = 0; c < 2 * T; ++c) {
            const uint32_t cnt = ci[c].y - ci[c].x;
            if (cnt > ptb::kSmallTask) {
                large.push_back(ci[c]);
                lmin.push_back(cmn[c]);
                lmax.push_back(cmx[c]);
            } else {
                small.push_back(ci[c]);
            }
        }
    }
    if (!small.empty()) {
        const uint32_t S = uint32_t(small.size());
        if ((rc = dupload(ctx, sinfo, small.data(), S))) {
            cleanup();
            return rc;
        }
        ptb::kb_small<<<(S + 127) / 128, 128, 0, ctx->stream>>>(S, sinfo.p, idx.p, lo, hi, dnodes.p, ctr.p);
    }
    uint32_t count = 0;
    BK(cudaGetLastError());
    BK(cudaMemcpyAsync(&count, ctr.p, 4, cudaMemcpyDeviceToHost, ctx->stream));
    BK(cudaStreamSynchronize(ctx->stream));
    if (count > 2 * n) {
        cleanup();
        return set_err(ctx, PT_ERR_KERNEL, "bvh build: node count overflow");
    }
    nodes.resize(count);
    BK(cudaMemcpyAsync(nodes.data(), dnodes.p, size_t(count) * 32, cudaMemcpyDeviceToHost, ctx->stream));
    BK(cudaStreamSynchronize(ctx->stream));
#undef BK
    cleanup();
    return PT_OK;
}

// The reference BVH leaf (node index) holding each of n_items items (leaf
// ranges left_first .. left_first + count - 1); kMiss for an item no leaf holds.
std::vector<uint32_t> ref_item_leaf(const PtBvhNode* nodes, uint32_t n_nodes, uint32_t n_items) {
    std::vector<uint32_t> leaf(n_items, kMiss);
    for (uint32_t i = 0; i < n_nodes; ++i) {
        if (nodes[i].count == 0u) continue;
        for (uint32_t k = 0; k < nodes[i].count; ++k) {
            const uint64_t it = uint64_t(nodes[i].left_first) + k;
            if (it < n_items) leaf[size_t(it)] = i;
        }
    }
    return leaf;
}

// Wide tree over the triangle slots of the uploaded (reference) mesh BVH.
int build_wide_mesh(pt_gpu_ctx* ctx, const PtBvhNode* ref_nodes, uint32_t n_ref, uint32_t n_slots) {
    ctx->t_wide = false;
    ctx->m_wide = false;
    ctx->t4_count = 0;
    if (n_slots == 0 || n_ref == 0) return PT_OK;
    std::vector<uint32_t> rank;
    if (!ptb::ref_ranks(ref_nodes, n_ref, n_slots, 64, rank)) return PT_OK;   // keep the reference walk
    std::vector<ptb::Node2H> bin;
    DBuf<uint32_t> order;
    int rc = gpu_build_tree(ctx, ctx->tri_lo.p, ctx->tri_hi.p, n_slots, bin, order);
    if (rc) { dfree(order); return rc; }
    std::vector<ptb::Wide4> wide;
    const int depth = ptb::collapse4(bin, wide);
    ctx->t4_bin_nodes = uint32_t(bin.size());
    if (depth < 0 || 3 * depth + 1 > kWideStackDev) { dfree(order); return PT_OK; }
    const std::vector<uint32_t> sleaf = ref_item_leaf(ref_nodes, n_ref, n_slots);
    if ((rc = dupload(ctx, ctx->t_rank, rank.data(), n_slots)) || (rc = dalloc(ctx, ctx->tri4, 3 * size_t(n_slots))) ||
        (rc = dupload(ctx, ctx->t4, reinterpret_cast<const float4*>(wide.data()), wide.size() * 8)) ||
        (rc = dupload(ctx, ctx->tslot_leaf, sleaf.data(), n_slots)) || (rc = dalloc(ctx, ctx->t_leaf, n_slots))) {
        dfree(order);
        return rc;
    }
    k_gather_tris<<<(n_slots + 255) / 256, 256, 0, ctx->stream>>>(ctx->tri.p, order.p, ctx->t_rank.p, n_slots,
                                                                 ctx->tri4.p);
    k_gather_u32<<<(n_slots + 255) / 256, 256, 0, ctx->stream>>>(ctx->tslot_leaf.p, order.p, n_slots, ctx->t_leaf.p);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    dfree(order);
    if (e != cudaSuccess) return set_err(ctx, PT_ERR_CUDA, std::string("gather tris: ") + cudaGetErrorString(e));
    ctx->t4_count = uint32_t(wide.size());
    ctx->t4_depth = uint32_t(depth);
    ctx->t_wide = true;
    return PT_OK;
}

// Wide tree over the finite analytic records [linear, n).
int build_wide_prims(pt_gpu_ctx* ctx, const PtBvhNode* ref_nodes, uint32_t n_ref) {
    ctx->a_wide = false;
    ctx->m_wide = false;
    ctx->a4_count = 0;
    const uint32_t nf = ctx->prim_count - ctx->linear_count;
    if (nf == 0 || n_ref == 0) return PT_OK;   // no reference BVH: the records are scanned linearly
    std::vector<uint32_t> rank;
    if (!ptb::ref_ranks(ref_nodes, n_ref, nf, 32, rank)) return PT_OK;
    DBuf<float4> blo, bhi;
    DBuf<uint32_t> order;
    DBuf<uint32_t>& drank = ctx->a_rank;
    auto cleanup = [&]() { dfree(blo); dfree(bhi); dfree(order); };
    int rc = 0;
    if ((rc = dalloc(ctx, blo, nf)) || (rc = dalloc(ctx, bhi, nf))) { cleanup(); return rc; }
    k_prim_boxes<<<(nf + 255) / 256, 256, 0, ctx->stream>>>(ctx->prim_geo.p, ctx->prim_type.p, ctx->linear_count,
                                                           nf, blo.p, bhi.p);
    std::vector<ptb::Node2H> bin;
    if ((rc = gpu_build_tree(ctx, blo.p, bhi.p, nf, bin, order))) { cleanup(); return rc; }
    std::vector<ptb::Wide4> wide;
    const int depth = ptb::collapse4(bin, wide);
    if (depth < 0 || 3 * depth + 1 > kWideStackDev) { cleanup(); return PT_OK; }
    const std::vector<uint32_t> aleaf = ref_item_leaf(ref_nodes, n_ref, nf);
    if ((rc = dupload(ctx, drank, rank.data(), nf)) || (rc = dalloc(ctx, ctx->a4_geo, nf)) ||
        (rc = dalloc(ctx, ctx->a4_meta, nf)) || (rc = dupload(ctx, ctx->a_leaf, aleaf.data(), nf)) ||
        (rc = dupload(ctx, ctx->a4, reinterpret_cast<const float4*>(wide.data()), wide.size() * 8))) {
        cleanup();
        return rc;
    }
    k_gather_prims<<<(nf + 255) / 256, 256, 0, ctx->stream>>>(ctx->prim_geo.p, ctx->prim_type.p, order.p, drank.p,
                                                             ctx->linear_count, nf, ctx->a4_geo.p, ctx->a4_meta.p);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    cleanup();
    if (e != cudaSuccess) return set_err(ctx, PT_ERR_CUDA, std::string("gather prims: ") + cudaGetErrorString(e));
    ctx->a4_count = uint32_t(wide.size());
    ctx->a4_depth = uint32_t(depth);
    ctx->a_wide = true;
    return PT_OK;
}

// Merged 4-wide tree over the triangles and the finite analytic records.  The
// separate trees walk the analytic part to its end before the mesh, so a ray
// tests every sphere-tree node its path enters (3.9 per segment on the 1080p
// triangle scene, for 0.4 sphere tests); in one tree a sphere's nodes are
// tested only where the ray passes near it.  Leaves hold one kind of item: a
// leaf of the binary SAH tree holding both is split into a triangle leaf and a
// record leaf (both keep the parent's box).  Record leaves carry kPrimLeafFlag
// in the first-item field.  Items keep their reference tie ranks, so hits are
// those of the separate trees.  Built when both separate wide trees exist.
constexpr uint32_t kPrimLeafFlag = 1u << 27;

int build_wide_merged(pt_gpu_ctx* ctx) {
    ctx->m_wide = false;
    ctx->m4_count = 0;
    if (!ctx->t_wide || !ctx->a_wide || !ctx->t_rank.p || !ctx->a_rank.p || !ctx->tslot_leaf.p) return PT_OK;
    const uint32_t n_t = ctx->tri_slots, n_a = ctx->prim_count - ctx->linear_count;
    if (n_t == 0 || n_a == 0 || n_t >= kPrimLeafFlag || n_a >= kPrimLeafFlag) return PT_OK;
    const uint32_t n = n_t + n_a;
    DBuf<float4> blo, bhi;
    DBuf<uint32_t> order, tperm, pperm;
    auto cleanup = [&]() { dfree(blo); dfree(bhi); dfree(order); dfree(tperm); dfree(pperm); };
    int rc = 0;
    if ((rc = dalloc(ctx, blo, n)) || (rc = dalloc(ctx, bhi, n))) { cleanup(); return rc; }
    CK(cudaMemcpyAsync(blo.p, ctx->tri_lo.p, size_t(n_t) * 16, cudaMemcpyDeviceToDevice, ctx->stream));
    CK(cudaMemcpyAsync(bhi.p, ctx->tri_hi.p, size_t(n_t) * 16, cudaMemcpyDeviceToDevice, ctx->stream));
    k_prim_boxes<<<(n_a + 255) / 256, 256, 0, ctx->stream>>>(ctx->prim_geo.p, ctx->prim_type.p, ctx->linear_count,
                                                            n_a, blo.p + n_t, bhi.p + n_t);
    std::vector<ptb::Node2H> bin;
    if ((rc = gpu_build_tree(ctx, blo.p, bhi.p, n, bin, order))) { cleanup(); return rc; }
    std::vector<uint32_t> ho(n);
    CK(cudaMemcpy(ho.data(), order.p, size_t(n) * 4, cudaMemcpyDeviceToHost));
    // split leaves holding both kinds (triangles first)
    const size_t n_bin = bin.size();
    for (size_t i = 0; i < n_bin; ++i) {
        if (bin[i].count == 0u) continue;
        const uint32_t lf = bin[i].lf, cnt = bin[i].count;
        uint32_t nt = 0;
        for (uint32_t k = 0; k < cnt; ++k) nt += (ho[lf + k] < n_t) ? 1u : 0u;
        if (nt == 0u || nt == cnt) continue;
        std::stable_partition(ho.begin() + lf, ho.begin() + lf + cnt, [&](uint32_t v) { return v < n_t; });
        ptb::Node2H a = bin[i], b = bin[i];
        a.lf = lf;
        a.count = nt;
        b.lf = lf + nt;
        b.count = cnt - nt;
        bin[i].lf = uint32_t(bin.size());
        bin[i].count = 0u;
        bin.push_back(a);
        bin.push_back(b);
    }
    // per-kind positions: the items of a leaf are consecutive in their kind's array
    std::vector<uint32_t> tp, pp, pos(n);
    tp.reserve(n_t);
    pp.reserve(n_a);
    for (uint32_t k = 0; k < n; ++k) {
        if (ho[k] < n_t) {
            pos[k] = uint32_t(tp.size());
            tp.push_back(ho[k]);
        } else {
            pos[k] = uint32_t(pp.size()) | kPrimLeafFlag;
            pp.push_back(ho[k] - n_t);
        }
    }
    for (auto& nd : bin)
        if (nd.count > 0u) nd.lf = pos[nd.lf];
    std::vector<ptb::Wide4> wide;
    const int depth = ptb::collapse4(bin, wide);
    if (depth < 0 || 3 * depth + 1 > kWideStackDev) { cleanup(); return PT_OK; }
    if ((rc = dupload(ctx, tperm, tp.data(), n_t)) || (rc = dupload(ctx, pperm, pp.data(), n_a)) ||
        (rc = dalloc(ctx, ctx->mtri4, 3 * size_t(n_t))) || (rc = dalloc(ctx, ctx->ma4_geo, n_a)) ||
        (rc = dalloc(ctx, ctx->m_leaf, n_t)) ||
        (rc = dalloc(ctx, ctx->ma4_meta, n_a)) ||
        (rc = dupload(ctx, ctx->m4, reinterpret_cast<const float4*>(wide.data()), wide.size() * 8))) {
        cleanup();
        return rc;
    }
    k_gather_tris<<<(n_t + 255) / 256, 256, 0, ctx->stream>>>(ctx->tri.p, tperm.p, ctx->t_rank.p, n_t, ctx->mtri4.p);
    k_gather_u32<<<(n_t + 255) / 256, 256, 0, ctx->stream>>>(ctx->tslot_leaf.p, tperm.p, n_t, ctx->m_leaf.p);
    k_gather_prims<<<(n_a + 255) / 256, 256, 0, ctx->stream>>>(ctx->prim_geo.p, ctx->prim_type.p, pperm.p,
                                                             ctx->a_rank.p, ctx->linear_count, n_a, ctx->ma4_geo.p,
                                                             ctx->ma4_meta.p);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    cleanup();
    if (e != cudaSuccess) return set_err(ctx, PT_ERR_CUDA, std::string("merged tree: ") + cudaGetErrorString(e));
    ctx->m4_count = uint32_t(wide.size());
    ctx->m4_depth = uint32_t(depth);
    ctx->m_wide = true;
    return PT_OK;
}

cudaEvent_t pool_event(pt_gpu_ctx* c, size_t i) {
    while (c->ev_pool.size() <= i) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        c->ev_pool.push_back(e);
    }
    return c->ev_pool[i];
}

}  // namespace

extern "C" {

const char* pt_gpu_version(void) { return "demont-gb300 sm_103a wavefront v1"; }

int pt_gpu_create(pt_gpu_ctx** out, int device_ordinal) {
    if (!out) return PT_ERR_INVALID;
    *out = nullptr;
    auto* ctx = new pt_gpu_ctx();
    ctx->device = device_ordinal;
    cudaError_t e = cudaSetDevice(device_ordinal);
    if (e != cudaSuccess) {
        *out = ctx;
        return set_err(ctx, PT_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    }
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device_ordinal);
    CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&ctx->side2, cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&ctx->ev_fork2, &ctx->ev_join2, &ctx->ev_split, &ctx->ev_half})
        CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    CK(cudaEventCreate(&ctx->ev0));
    CK(cudaEventCreate(&ctx->ev1));
    CK(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
    int rc = dalloc(ctx, ctx->err_word, 1);
    if (rc) { *out = ctx; return rc; }
    rc = dalloc(ctx, ctx->cnt, 32);   // the counter rings (DPaths::cnt) of the two half-waves
    if (rc) { *out = ctx; return rc; }
    rc = dalloc(ctx, ctx->wave_vars, 8);   // DPaths::wave of the two half-waves
    if (rc) { *out = ctx; return rc; }
    rc = dalloc(ctx, ctx->stat, 4);
    if (rc) { *out = ctx; return rc; }
    rc = dalloc(ctx, ctx->tcount, 16);
    if (rc) { *out = ctx; return rc; }
    CK(cudaMemsetAsync(ctx->err_word.p, 0, 4, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    *out = ctx;
    return PT_OK;
}

int pt_gpu_destroy(pt_gpu_ctx* ctx) {
    if (!ctx) return PT_OK;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    if (ctx->stream2) cudaStreamSynchronize(ctx->stream2);
    if (ctx->side2) cudaStreamSynchronize(ctx->side2);
    for (auto* b : {&ctx->prim_rec, &ctx->prim_geo, &ctx->bvh, &ctx->tri, &ctx->tri_bvh, &ctx->mats,
                    &ctx->lights, &ctx->env, &ctx->accum, &ctx->ray_o, &ctx->ray_d, &ctx->thr,
                    &ctx->rad, &ctx->fsum, &ctx->amb, &ctx->sh_o, &ctx->sh_d, &ctx->sh_pre, &ctx->sh_brdf,
                    &ctx->sh_tr, &ctx->moon, &ctx->ltree, &ctx->sdf, &ctx->d_srad, &ctx->d_dldi})
        dfree(*b);
    dfree(ctx->d_grad);
    dfree(ctx->d_sh_mats);
    dfree(ctx->ldr);
    dfree(ctx->prim_mat);
    for (auto* b : {&ctx->prim_type, &ctx->seed, &ctx->state, &ctx->hit_id, &ctx->shmask, &ctx->q0,
                    &ctx->q1, &ctx->sq, &ctx->cnt, &ctx->err_word, &ctx->wave_vars})
        dfree(*b);
    dfree(ctx->marg);
    dfree(ctx->cond);
    dfree(ctx->marg_guide);
    dfree(ctx->cond_guide);
    for (auto* b : {&ctx->a4, &ctx->a4_geo, &ctx->t4, &ctx->tri4, &ctx->tri_lo, &ctx->tri_hi}) dfree(*b);
    dfree(ctx->a4_meta);
    for (auto* b : {&ctx->m4, &ctx->mtri4, &ctx->ma4_geo}) dfree(*b);
    dfree(ctx->ma4_meta);
    dfree(ctx->t_rank);
    dfree(ctx->a_rank);
    for (auto* b : {&ctx->t_leaf, &ctx->m_leaf, &ctx->a_leaf, &ctx->tslot_leaf}) dfree(*b);
    dfree(ctx->hit_t);
    dfree(ctx->stat);
    dfree(ctx->tcount);
    dfree(ctx->rr_buf);
    if (ctx->b_graph) cudaGraphExecDestroy(ctx->b_graph);
    for (auto& gs : ctx->wave_graphs)
        if (gs.exec) cudaGraphExecDestroy(gs.exec);
    dfree(ctx->b_views);
    dfree(ctx->b_scenes);
    dfree(ctx->b_view_base);
    dfree(ctx->b_path_view);
    dfree(ctx->b_path_scene);
    dfree(ctx->b_accum);
    for (auto e : ctx->ev_pool) cudaEventDestroy(e);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    for (cudaEvent_t e : {ctx->ev_fork2, ctx->ev_join2, ctx->ev_split, ctx->ev_half})
        if (e) cudaEventDestroy(e);
    if (ctx->side2) cudaStreamDestroy(ctx->side2);
    if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return PT_OK;
}

const char* pt_gpu_last_error(const pt_gpu_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int pt_gpu_upload_prims(pt_gpu_ctx* ctx, const float* recs28, uint32_t n, uint32_t linear_count,
                        const PtBvhNode* nodes, uint32_t n_nodes) {
    if (ctx) ctx->gen++;
    if (!ctx) return PT_ERR_INVALID;
    if ((n && !recs28) || (n_nodes && !nodes) || linear_count > n)
        return set_err(ctx, PT_ERR_INVALID, "upload_prims: bad arguments");
    std::string why;
    if (n_nodes && !check_bvh(nodes, n_nodes, n - linear_count, why))
        return set_err(ctx, PT_ERR_INVALID, "upload_prims: " + why);
    int rc = dupload(ctx, ctx->prim_rec, recs28, size_t(n) * 7);
    if (rc) return rc;
    if ((rc = dalloc(ctx, ctx->prim_geo, n)) || (rc = dalloc(ctx, ctx->prim_type, n))) return rc;
    if (n) {
        k_prep_prims<<<(n + 255) / 256, 256, 0, ctx->stream>>>(ctx->prim_rec.p, n, ctx->prim_geo.p,
                                                               ctx->prim_type.p);
        CK(cudaGetLastError());
    }
    if ((rc = dupload(ctx, ctx->bvh, nodes, size_t(n_nodes) * 2))) return rc;
    ctx->prim_count = n;
    ctx->linear_count = linear_count;
    ctx->bvh_nodes = n_nodes;
    CK(cudaStreamSynchronize(ctx->stream));
    if (int rc = build_wide_prims(ctx, nodes, n_nodes)) return rc;
    return build_wide_merged(ctx);
}

int pt_gpu_upload_mesh(pt_gpu_ctx* ctx, const float* positions, uint32_t nv, const uint32_t* indices,
                       uint32_t nt, const PtBvhNode* nodes, uint32_t n_nodes, const uint32_t* perm,
                       uint32_t n_perm, const uint32_t* mat_ids) {
    if (ctx) ctx->gen++;
    if (!ctx) return PT_ERR_INVALID;
    if ((nv && !positions) || (nt && !indices) || (n_nodes && !nodes) || (n_perm && !perm))
        return set_err(ctx, PT_ERR_INVALID, "upload_mesh: null buffer");
    std::string why;
    if (n_nodes && !check_bvh(nodes, n_nodes, n_perm, why))
        return set_err(ctx, PT_ERR_INVALID, "upload_mesh: " + why);
    for (uint32_t j = 0; j < n_perm; ++j) {
        const uint32_t t = perm[j];
        if (t >= nt) return set_err(ctx, PT_ERR_INVALID, "upload_mesh: permuted id out of range");
        if (indices[3u * t] >= nv || indices[3u * t + 1] >= nv || indices[3u * t + 2] >= nv)
            return set_err(ctx, PT_ERR_INVALID, "upload_mesh: vertex index out of range");
    }
    DBuf<float> dpos;
    DBuf<uint32_t> didx, dperm, dmat;
    int rc = 0;
    if ((rc = dupload(ctx, dpos, positions, size_t(nv) * 3)) ||
        (rc = dupload(ctx, didx, indices, size_t(nt) * 3)) ||
        (rc = dupload(ctx, dperm, perm, n_perm)) ||
        (rc = dupload(ctx, dmat, mat_ids, mat_ids ? nt : 0)) ||
        (rc = dalloc(ctx, ctx->tri, size_t(n_perm) * 3)) || (rc = dalloc(ctx, ctx->tri_lo, n_perm)) ||
        (rc = dalloc(ctx, ctx->tri_hi, n_perm))) {
        dfree(dpos); dfree(didx); dfree(dperm); dfree(dmat);
        return rc;
    }
    if (n_perm) {
        k_prep_tris<<<(n_perm + 255) / 256, 256, 0, ctx->stream>>>(dpos.p, didx.p, dperm.p, dmat.p,
                                                                   n_perm, ctx->tri.p, ctx->tri_lo.p,
                                                                   ctx->tri_hi.p);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dfree(dpos); dfree(didx); dfree(dperm); dfree(dmat);
    if (e != cudaSuccess) return set_err(ctx, PT_ERR_CUDA, std::string("prep_tris: ") + cudaGetErrorString(e));
    if ((rc = dupload(ctx, ctx->tri_bvh, nodes, size_t(n_nodes) * 2))) return rc;
    ctx->tri_slots = n_perm;
    ctx->tri_nodes = n_nodes;
    ctx->tri_count = nt;
    ctx->mesh_has_mat = (mat_ids != nullptr);
    CK(cudaStreamSynchronize(ctx->stream));
    cudaEvent_t b0, b1;
    cudaEventCreate(&b0);
    cudaEventCreate(&b1);
    cudaEventRecord(b0, ctx->stream);
    rc = build_wide_mesh(ctx, nodes, n_nodes, n_perm);
    if (rc == PT_OK) rc = build_wide_merged(ctx);
    cudaEventRecord(b1, ctx->stream);
    cudaEventSynchronize(b1);
    float bms = 0.0f;
    cudaEventElapsedTime(&bms, b0, b1);
    ctx->build_ms = bms;
    cudaEventDestroy(b0);
    cudaEventDestroy(b1);
    return rc;
}

int pt_gpu_upload_materials(pt_gpu_ctx* ctx, const float* mats12, uint32_t n) {
    if (ctx) ctx->gen++;
    if (!ctx) return PT_ERR_INVALID;
    if (n && !mats12) return set_err(ctx, PT_ERR_INVALID, "upload_materials: null buffer");
    int rc = dupload(ctx, ctx->mats, mats12, size_t(n) * 3);
    if (rc) return rc;
    ctx->mat_count = n;
    CK(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_gpu_upload_prim_materials(pt_gpu_ctx* ctx, const uint32_t* mat_ids, uint32_t n) {
    if (ctx) ctx->gen++;
    if (!ctx) return PT_ERR_INVALID;
    if (!mat_ids || n == 0) {
        ctx->has_prim_mat = false;
        return PT_OK;
    }
    if (n != ctx->prim_count)
        return set_err(ctx, PT_ERR_INVALID, "upload_prim_materials: count differs from the uploaded records");
    int rc = dupload(ctx, ctx->prim_mat, mat_ids, n);
    if (rc) return rc;
    ctx->has_prim_mat = true;
    CK(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_gpu_upload_lights(pt_gpu_ctx* ctx, const float* recs20, uint32_t n) {
    if (ctx) ctx->gen++;
    if (!ctx) return PT_ERR_INVALID;
    if (n && !recs20) return set_err(ctx, PT_ERR_INVALID, "upload_lights: null buffer");
    int rc = dupload(ctx, ctx->lights, recs20, size_t(n) * 5);
    if (rc) return rc;
    ctx->light_count = n;
    CK(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_gpu_upload_env(pt_gpu_ctx* ctx, const float* rgba, uint32_t W, uint32_t H, const float* marginal,
                      const float* conditional, const float* hdri_dir_pmf, const float* hdri_col,
                      uint32_t n_hdri) {
    if (ctx) ctx->gen++;
    if (!ctx) return PT_ERR_INVALID;
    if (n_hdri > 8) return set_err(ctx, PT_ERR_INVALID, "upload_env: at most 8 HDRI lights");
    if ((W || H) && (!rgba || !marginal || !conditional || W == 0 || H == 0))
        return set_err(ctx, PT_ERR_INVALID, "upload_env: bad image");
    if (n_hdri && (!hdri_dir_pmf || !hdri_col)) return set_err(ctx, PT_ERR_INVALID, "upload_env: null HDRI lights");
    int rc = 0;
    if ((rc = dupload(ctx, ctx->env, rgba, size_t(W) * H)) || (rc = dupload(ctx, ctx->marg, marginal, H)) ||
        (rc = dupload(ctx, ctx->cond, conditional, size_t(W) * H)))
        return rc;
    // guide tables for the env-sampling searches (cdf_search), when every CDF
    // is non-decreasing (BuildEnvCdf's always are)
    ctx->env_guided = false;
    if (W && H) {
        std::vector<uint32_t> mg(kCdfGuide + 1u), cg(size_t(H) * (kCdfGuide + 1u));
        bool ok = build_cdf_guide(marginal, H, mg.data());
        for (uint32_t v = 0; ok && v < H; ++v)
            ok = build_cdf_guide(conditional + size_t(v) * W, W, cg.data() + size_t(v) * (kCdfGuide + 1u));
        if (ok) {
            if ((rc = dupload(ctx, ctx->marg_guide, mg.data(), mg.size())) ||
                (rc = dupload(ctx, ctx->cond_guide, cg.data(), cg.size())))
                return rc;
            ctx->env_guided = true;
        }
    }
    ctx->env_w = W;
    ctx->env_h = H;
    ctx->hdri_count = n_hdri;
    std::memset(ctx->hdri_dir, 0, sizeof(ctx->hdri_dir));
    std::memset(ctx->hdri_col, 0, sizeof(ctx->hdri_col));
    if (n_hdri) {
        std::memcpy(ctx->hdri_dir, hdri_dir_pmf, size_t(n_hdri) * 16);
        std::memcpy(ctx->hdri_col, hdri_col, size_t(n_hdri) * 16);
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_gpu_upload_light_tree(pt_gpu_ctx* ctx, const PtLightTreeNode* nodes, uint32_t n) {
    if (ctx) ctx->gen++;
    if (!ctx) return PT_ERR_INVALID;
    if (n && !nodes) return set_err(ctx, PT_ERR_INVALID, "upload_light_tree: null buffer");
    // children after their parent and inside the array: every walk ends within 32 levels' reach
    for (uint32_t i = 0; i < n; ++i) {
        const PtLightTreeNode& nd = nodes[i];
        if (nd.count > 1u) return set_err(ctx, PT_ERR_INVALID, "upload_light_tree: leaf count above 1");
        if (nd.count == 0u && (nd.left_first <= i || uint64_t(nd.left_first) + 1u >= n))
            return set_err(ctx, PT_ERR_INVALID, "upload_light_tree: bad child index at node " + std::to_string(i));
    }
    static_assert(sizeof(PtLightTreeNode) == 64, "light tree node is 4 float4");
    if (int rc = dupload(ctx, ctx->ltree, nodes, 4 * size_t(n))) return rc;
    ctx->ltree_nodes = n;
    CK(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_gpu_upload_sdf(pt_gpu_ctx* ctx, const float* clusters, uint32_t n) {
    if (ctx) ctx->gen++;
    if (!ctx) return PT_ERR_INVALID;
    if (n && !clusters) return set_err(ctx, PT_ERR_INVALID, "upload_sdf: null buffer");
    const uint32_t* u = reinterpret_cast<const uint32_t*>(clusters);
    bool proc_any = false;
    for (uint32_t c = 0; c < n; ++c) {
        const uint32_t* h = u + size_t(c) * kSdfStride * 4u;
        const uint32_t count = h[3];
        const std::string at = "upload_sdf: cluster " + std::to_string(c) + ": ";
        if (count == 0u || count > kSdfMaxNodes) return set_err(ctx, PT_ERR_INVALID, at + "node count must be 1..8");
        for (uint32_t i = 0; i < count; ++i) {
            const uint32_t* nd = h + 16u + 12u * i;
            const uint32_t op = nd[0], shape = nd[1], a = nd[2], b = nd[3];
            if (op > 9u || (op == 0u && shape > 8u)) return set_err(ctx, PT_ERR_INVALID, at + "bad op or shape");
            if (op >= 1u && op <= 3u && (a >= i || b >= i))
                return set_err(ctx, PT_ERR_INVALID, at + "an op must combine earlier nodes");
            if (op >= 4u && a >= i) return set_err(ctx, PT_ERR_INVALID, at + "an op must combine earlier nodes");
            proc_any = proc_any || (op >= 5u);
        }
    }
    if (int rc = dupload(ctx, ctx->sdf, clusters, size_t(n) * kSdfStride)) return rc;
    ctx->sdf_count = n;
    ctx->sdf_proc_any = proc_any;
    CK(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_gpu_upload_moon(pt_gpu_ctx* ctx, const float* rgba, uint32_t W, uint32_t H) {
    if (ctx) ctx->gen++;
    if (!ctx) return PT_ERR_INVALID;
    if (W == 0 || H == 0) {
        dfree(ctx->moon);
        ctx->moon_w = ctx->moon_h = 0;
        return PT_OK;
    }
    if (!rgba || uint64_t(W) * H > (1ull << 26)) return set_err(ctx, PT_ERR_INVALID, "upload_moon: bad image");
    if (int rc = dupload(ctx, ctx->moon, rgba, size_t(W) * H)) return rc;
    ctx->moon_w = W;
    ctx->moon_h = H;
    return PT_OK;
}

int pt_gpu_set_target(pt_gpu_ctx* ctx, uint32_t width, uint32_t height) {
    if (ctx) ctx->gen++;
    if (!ctx) return PT_ERR_INVALID;
    if (width == 0 || height == 0 || uint64_t(width) * height > (1ull << 28))
        return set_err(ctx, PT_ERR_INVALID, "set_target: bad size");
    int rc = dalloc(ctx, ctx->accum, size_t(width) * height);
    if (rc) return rc;
    ctx->W = width;
    ctx->H = height;
    CK(cudaMemsetAsync(ctx->accum.p, 0, size_t(width) * height * 16, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_gpu_read_accum(pt_gpu_ctx* ctx, float* host_rgba) {
    if (!ctx || !host_rgba) return PT_ERR_INVALID;
    if (!ctx->accum.p) return set_err(ctx, PT_ERR_STATE, "read_accum: no target");
    CK(cudaMemcpyAsync(host_rgba, ctx->accum.p, size_t(ctx->W) * ctx->H * 16, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_gpu_write_accum(pt_gpu_ctx* ctx, const float* host_rgba) {
    if (!ctx || !host_rgba) return PT_ERR_INVALID;
    if (!ctx->accum.p) return set_err(ctx, PT_ERR_STATE, "write_accum: no target");
    CK(cudaMemcpyAsync(ctx->accum.p, host_rgba, size_t(ctx->W) * ctx->H * 16, cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_gpu_accum_device_ptr(pt_gpu_ctx* ctx, void** dptr) {
    if (!ctx || !dptr) return PT_ERR_INVALID;
    if (!ctx->accum.p) return set_err(ctx, PT_ERR_STATE, "accum_device_ptr: no target");
    *dptr = ctx->accum.p;
    return PT_OK;
}

int pt_gpu_set_wave_frames(pt_gpu_ctx* ctx, uint32_t frames_per_wave) {
    if (!ctx) return PT_ERR_INVALID;
    ctx->wave_frames_override = frames_per_wave;
    return PT_OK;
}

}  // extern "C"

namespace {

// What a run of waves does besides rendering: record every sample's radiance
// (forward half of a differentiable render) or replay the recorded paths and
// accumulate parameter gradients instead of the image (backward half).
enum class RunMode { kRender, kRecord, kAdjoint };
struct DiffRun {
    RunMode mode = RunMode::kRender;
    const float4* dldi = nullptr;
    uint32_t nmat = 0;
};

// The path state with bounce b's queue counters (DPaths::cnt).
DPaths bounce_paths(const DPaths& P, uint32_t b) {
    DPaths Q = P;
    Q.cnt = P.cnt + 4u * (b & 3u);
    Q.cnt_next = P.cnt + 4u * ((b + 1u) & 3u);
    Q.cnt_clear = P.cnt + 4u * ((b + 2u) & 3u);
    return Q;
}

// Replay of a plain render's wave as a CUDA graph (see render_waves).  The key
// is every byte the wave's launches depend on; the structure (the node list)
// depends on fewer fields, and a graph of the same structure is updated in
// place with cudaGraphExecUpdate when the key differs.
template <class Issue>
int launch_wave_graph(pt_gpu_ctx* ctx, Issue& issue_wave, uint32_t f0, uint32_t nf, const DFrame& F, const DScene& S,
                      DPaths P, float ema, bool rr_fix, bool proc, bool persistent, bool overlap) {
    std::vector<unsigned char> key;
    auto put = [&](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        key.insert(key.end(), b, b + n);
    };
    // f0 fixes the roulette records' offset; the frame indices and the reset
    // flag are read from P.wave at run time
    const uint32_t flags[8] = {f0, nf, 0u, uint32_t(rr_fix), uint32_t(proc), uint32_t(persistent),
                               uint32_t(overlap), uint32_t(ctx->sm_count)};
    P.rr_frozen = nullptr;   // set per sample inside the wave
    put(&F, sizeof(F));
    put(&S, sizeof(S));
    put(&P, sizeof(P));
    put(flags, sizeof(flags));
    put(&ema, sizeof(ema));
    const void* ptrs[4] = {ctx->accum.p, ctx->rr_buf.p, ctx->wave_vars.p, ctx->err_word.p};
    put(ptrs, sizeof(ptrs));
    // the node list depends on the sample and bounce counts and the kernel
    // variants; f0 keeps the waves of one call in graphs of their own (they
    // would otherwise update each other in place on every call)
    const std::array<uint32_t, 4> topo = {F.spp, F.maxb, f0,
                                          uint32_t(proc) | uint32_t(persistent) << 1 | uint32_t(overlap) << 2 |
                                              uint32_t(S.use_wide) << 3};
    ++ctx->graph_clock;
    for (auto& gs : ctx->wave_graphs)
        if (gs.exec && gs.key == key) {
            gs.used = ctx->graph_clock;
            CK(cudaGraphLaunch(gs.exec, ctx->stream));
            ctx->stats.graph_replays++;
            return PT_OK;
        }
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const int irc = issue_wave(f0, nf);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (irc) {
        if (g) cudaGraphDestroy(g);
        return irc;
    }
    if (e != cudaSuccess) return set_err(ctx, PT_ERR_CUDA, std::string("render capture: ") + cudaGetErrorString(e));
    // a cached graph of the same structure: update it in place; else replace the
    // least recently used slot
    WaveGraph* slot = nullptr;
    bool updated = false;
    for (auto& gs : ctx->wave_graphs)
        if (gs.exec && gs.topo == topo) {
            slot = &gs;
            cudaGraphExecUpdateResultInfo info;
            updated = cudaGraphExecUpdate(gs.exec, g, &info) == cudaSuccess;
            if (!updated) cudaGetLastError();
            break;
        }
    if (!updated) {
        if (!slot) {
            slot = &ctx->wave_graphs[0];
            for (auto& gs : ctx->wave_graphs)
                if (gs.used < slot->used) slot = &gs;
        }
        if (slot->exec) cudaGraphExecDestroy(slot->exec);
        slot->exec = nullptr;
        e = cudaGraphInstantiate(&slot->exec, g, 0);
        if (e != cudaSuccess) {
            slot->exec = nullptr;
            cudaGraphDestroy(g);
            return set_err(ctx, PT_ERR_CUDA, std::string("render graph: ") + cudaGetErrorString(e));
        }
    }
    cudaGraphDestroy(g);
    slot->key = std::move(key);
    slot->topo = topo;
    slot->used = ctx->graph_clock;
    CK(cudaGraphLaunch(slot->exec, ctx->stream));
    return PT_OK;
}

int render_waves(pt_gpu_ctx* ctx, const PtPushHead* head, const PtPathParams* prm, uint32_t frames,
                 const DiffRun& dr) {
    if (!ctx || !head || !prm) return PT_ERR_INVALID;
    if (!ctx->accum.p) return set_err(ctx, PT_ERR_STATE, "render: no target (pt_gpu_set_target)");
    if (head->tlas_present) return set_err(ctx, PT_ERR_UNSUPPORTED, "render: tlas_present (hardware RT) has no CUDA path");
    if (int rc = check_light_tree(ctx, ctx, prm, "render: ")) return rc;
    if (int rc = check_sdf(ctx, ctx, prm, "render: ")) return rc;
    if (int rc = check_sky(ctx, ctx, head, prm, "render: ")) return rc;
    if (head->prim_count != ctx->prim_count || prm->bvh_params[0] != ctx->linear_count ||
        (prm->bvh_params[1] != 0u && prm->bvh_params[1] != ctx->bvh_nodes))
        return set_err(ctx, PT_ERR_INVALID, "render: prim_count / bvh_params disagree with the uploaded prims");
    if (prm->bvh_params[1] == 0u && ctx->bvh_nodes == 0u && ctx->linear_count > ctx->prim_count)
        return set_err(ctx, PT_ERR_INVALID, "render: bad linear count");
    if (prm->bvh_params[2] != 0u && prm->bvh_params[3] != 0u && prm->bvh_params[3] != ctx->tri_nodes)
        return set_err(ctx, PT_ERR_INVALID, "render: bvh_params.w disagrees with the uploaded mesh BVH");
    if (prm->light_count > ctx->light_count)
        return set_err(ctx, PT_ERR_INVALID, "render: light_count exceeds the uploaded lights");

    if (frames == 0) return PT_OK;

    DFrame F{};
    F.cam_pos = v3(head->pos_fovtan[0], head->pos_fovtan[1], head->pos_fovtan[2]);
    F.tanf = head->pos_fovtan[3];
    F.fwd = v3(head->fwd_aspect[0], head->fwd_aspect[1], head->fwd_aspect[2]);
    F.aspect = head->fwd_aspect[3];
    F.right = v3(head->right_xyz[0], head->right_xyz[1], head->right_xyz[2]);
    F.up = v3(head->up_xyz[0], head->up_xyz[1], head->up_xyz[2]);
    F.W = ctx->W;
    F.H = ctx->H;
    F.npix = ctx->W * ctx->H;
    F.spp = head->spp == 0u ? 1u : head->spp;
    F.maxb = head->max_bounces;
    F.denoiser = head->denoiser_enabled;
    F.jx = head->halton_jitter[0];
    F.jy = head->halton_jitter[1];
    F.env_present = head->env_map_present;
    F.env_intensity = head->env_intensity;
    F.env_total = head->env_total_luminance;
    F.kmax = int(prm->refract_budget);
    F.firefly = prm->firefly_clamp;
    F.mis = prm->mis_enabled;
    F.rr_start = prm->rr_start;
    F.light_count = prm->light_count;
    sky_of(F, prm);
    const DScene S = make_scene(ctx, prm);
    const bool proc = S.sdf_proc != 0u && ctx->sdf_proc_any;   // procedural SDF walker needed

    // Frames per wave: about kWavePaths paths in flight (376 bytes of path and
    // shadow-ray state each, ~25 GB at the cap).  Larger waves keep more rays
    // per bounce in the later, sparser bounces; if the device cannot hold the
    // wave, halve it until it fits.
    uint32_t fpw = ctx->wave_frames_override;
    if (fpw == 0) fpw = std::max<uint32_t>(1, uint32_t(kWavePaths / std::max<uint32_t>(F.npix, 1)));
    fpw = std::min(fpw, frames);
    int rc = ensure_wave(ctx, size_t(fpw) * F.npix);
    while (rc == PT_ERR_OOM && ctx->wave_frames_override == 0 && fpw > 1) {
        fpw = (fpw + 1) / 2;
        rc = ensure_wave(ctx, size_t(fpw) * F.npix);
    }
    if (rc) return rc;

    DPaths P{};
    P.ray_o = ctx->ray_o.p; P.ray_d = ctx->ray_d.p; P.thr = ctx->thr.p; P.rad = ctx->rad.p; P.amb = ctx->amb.p;
    P.fsum = ctx->fsum.p; P.seed = ctx->seed.p; P.state = ctx->state.p; P.hit_t = ctx->hit_t.p;
    P.hit_id = ctx->hit_id.p; P.shmask = ctx->shmask.p; P.sh_o = ctx->sh_o.p; P.sh_d = ctx->sh_d.p;
    P.sh_pre = ctx->sh_pre.p; P.sh_brdf = ctx->sh_brdf.p; P.sh_tr = ctx->sh_tr.p;
    P.q[0] = ctx->q0.p; P.q[1] = ctx->q1.p; P.sq = ctx->sq.p; P.cnt = ctx->cnt.p; P.stat = ctx->stat.p;
    P.wave = ctx->wave_vars.p;
    // persistent wide-tree kernels need both wide trees (or no such part)
    const bool persistent = S.use_wide && (S.a_wide || S.prim_count == S.wide_linear) &&
                            (S.t_wide || S.tri_enabled == 0u || S.tri_nodes == 0u);
    const int gpers = ctx->sm_count * 4;
    const int gtr = ctx->sm_count * kTransmitBlocks;
    const bool adj = dr.mode == RunMode::kAdjoint;
    const size_t total_paths = size_t(frames) * F.npix;
    size_t smem = 0;
    if (dr.mode != RunMode::kRender) {
        if (!persistent)
            return set_err(ctx, PT_ERR_UNSUPPORTED, "differentiable render: needs the wide trees (traversal mode 0)");
        rc = dalloc(ctx, ctx->d_srad, size_t(F.spp) * total_paths);
        if (rc) return rc;
    }
    if (adj) {
        rc = dalloc(ctx, ctx->d_sh_mats, 3 * size_t(fpw) * F.npix);
        if (rc) return rc;
        rc = dalloc(ctx, ctx->d_grad, 6 * size_t(dr.nmat));
        if (rc) return rc;
        CK(cudaMemsetAsync(ctx->d_grad.p, 0, 6 * size_t(dr.nmat) * sizeof(double), ctx->stream));
        smem = 6 * size_t(dr.nmat) * sizeof(double);
        // always opted in: k_shade also holds static shared memory (its queue
        // counting sort), and the 48 KB default bounds static + dynamic together
        CK(cudaFuncSetAttribute(k_shade<false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        CK(cudaFuncSetAttribute(k_shade<false, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        CK(cudaFuncSetAttribute(k_finish<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    }
    P.srad = (dr.mode == RunMode::kRecord) ? ctx->d_srad.p : nullptr;
    // fixed roulette probabilities: recorded by one plain render, read back by
    // later ones of the same shape
    const bool rr_fix = ctx->rr_freeze != 0 && dr.mode == RunMode::kRender && F.rr_start < F.maxb;
    if (rr_fix) {
        const uint32_t meta[5] = {F.W, F.H, frames, F.spp, F.maxb};
        if (ctx->rr_freeze == 1) {
            rc = dalloc(ctx, ctx->rr_buf, size_t(F.spp) * total_paths * F.maxb);
            if (rc) return rc;
            std::memcpy(ctx->rr_meta, meta, sizeof(meta));
        } else if (std::memcmp(ctx->rr_meta, meta, sizeof(meta)) != 0 || !ctx->rr_buf.p) {
            return set_err(ctx, PT_ERR_STATE,
                           "render: the recorded roulette probabilities are for another size, frame count, "
                           "spp or depth");
        }
    }
    P.rr_mode = uint32_t(ctx->rr_freeze);
    Adj A{};
    if (adj) {
        A.srad = ctx->d_srad.p;
        A.dldi = dr.dldi;
        A.grad = ctx->d_grad.p;
        A.sh_mats = ctx->d_sh_mats.p;
        A.nmat = dr.nmat;
        A.scale = 1.0f / float(double(frames) * double(F.spp));
    }
    const int gadj = ctx->sm_count * 4;
    // The next bounce's closest-hit pass overlaps this bounce's shadow rays
    // (profiling mode 2 keeps the stages serial).  Profiling records an event
    // pair around every closest-hit and shadow launch on the stream it runs on.
    const bool overlap = ctx->profile < 2;
    const bool counting = ctx->profile == 3 && !proc && !adj;   // counting traversal variants
    const int ge = grid_for(ctx, size_t(fpw) * F.npix, 8);
    std::vector<std::pair<size_t, size_t>> ext_ev, sh_ev;
    size_t ev_i = 0;
    auto launch_extend = [&](const DPaths& PP, cudaStream_t st, uint32_t b) -> int {
        if (ctx->profile) {
            ext_ev.emplace_back(ev_i, ev_i + 1);
            CK(cudaEventRecord(pool_event(ctx, ev_i++), st));
            ++ev_i;
        }
        const int qs = int(b & 1u);
        const DPaths Pb = bounce_paths(PP, b);
        if (persistent) {
            (counting ? k_closest<false, false, true> : proc ? k_closest<false, true> : k_closest<false, false>)
                <<<gpers, kThreads, 0, st>>>(S, Batch{}, PP.q[qs], Pb.cnt, PP.ray_o, PP.ray_d, PP.hit_t, PP.hit_id,
                                             Pb.cnt + 2, PP.stat);
        } else if (S.use_wide) {
            k_extend<true><<<ge, kThreads, 0, st>>>(S, Pb, qs);
        } else {
            k_extend<false><<<ge, kThreads, 0, st>>>(S, Pb, qs);
        }
        if (ctx->profile) CK(cudaEventRecord(pool_event(ctx, ext_ev.back().second), st));
        return PT_OK;
    };

    // work a failed earlier call left on the side streams finishes first
    for (cudaStream_t st : {ctx->side, ctx->stream2, ctx->side2}) {
        CK(cudaEventRecord(ctx->ev_join, st));
        CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
    }
    CK(cudaMemsetAsync(ctx->stat.p, 0, 4 * sizeof(unsigned long long), ctx->stream));
    CK(cudaMemsetAsync(ctx->err_word.p, 0, 4, ctx->stream));
    if (counting) CK(cudaMemsetAsync(ctx->tcount.p, 0, 16 * sizeof(unsigned long long), ctx->stream));
    ctx->stats = PtStats{};
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    const Nvtx nv_render(adj ? "pt_gpu adjoint replay" : "pt_gpu_render");
    // The samples and bounces of nf frames whose path state is PP, on stream st
    // (the next bounce's closest hits forked to sd through the events evf / evj).
    // PP's per-path arrays start at the first of those frames.
    auto issue_paths = [&](const DPaths& PP, cudaStream_t st, cudaStream_t sd, cudaEvent_t evf, cudaEvent_t evj,
                           uint32_t f0, uint32_t nf) -> int {
        const uint32_t npaths = nf * F.npix;
        const int gp = (npaths + 255) / 256;
        DPaths Pw = PP;
        k_init_wave<false><<<gp, 256, 0, st>>>(F, Pw, Batch{}, npaths);
        for (uint32_t s = 0; s < F.spp; ++s) {
            const Nvtx nv_sample("sample %u", s);
            const size_t srec = size_t(s) * total_paths + size_t(f0) * F.npix;
            A.srec_base = srec;
            Pw.rr_frozen = rr_fix ? ctx->rr_buf.p + srec * F.maxb : nullptr;
            k_camera<false><<<gp, 256, 0, st>>>(F, Pw, Batch{}, npaths, s);
            for (uint32_t b = 0; b < F.maxb; ++b) {
                const Nvtx nv_bounce("bounce %u", b);
                const int qs = int(b & 1u);
                const DPaths Pb = bounce_paths(Pw, b);
                if (b == 0u || !overlap) {
                    if (int rc = launch_extend(Pw, st, b)) return rc;
                } else {
                    // this bounce's closest hits were traced on the side stream
                    CK(cudaStreamWaitEvent(st, evj, 0));
                }
                if (adj)
                    (proc ? k_shade<false, true, true> : k_shade<false, true, false>)
                        <<<gadj / 2, kShadeThreads, smem, st>>>(S, F, Pb, Batch{}, A, qs, b);
                else
                    (proc ? k_shade<false, false, true> : k_shade<false, false, false>)
                        <<<grid_for(ctx, npaths, 4, kShadeThreads), kShadeThreads, 0, st>>>(S, F, Pb, Batch{},
                                                                                            Adj{}, qs, b);
                if (overlap && b + 1u < F.maxb) {
                    // fork: the next bounce's rays (written by k_shade) are traced
                    // while this bounce's shadow rays are
                    CK(cudaEventRecord(evf, st));
                    CK(cudaStreamWaitEvent(sd, evf, 0));
                    if (int rc = launch_extend(Pw, sd, b + 1u)) return rc;
                    CK(cudaEventRecord(evj, sd));
                }
                if (ctx->profile) {
                    sh_ev.emplace_back(ev_i, ev_i + 1);
                    CK(cudaEventRecord(pool_event(ctx, ev_i), st));
                    ev_i += 2;
                }
                if (persistent) {
                    if (adj)
                        (proc ? k_transmit<false, true, true> : k_transmit<false, true, false>)
                            <<<gtr, kThreads, 0, st>>>(S, Batch{}, Pb, F.kmax, ctx->d_sh_mats.p);
                    else
                        (counting ? k_transmit<false, false, false, true>
                                  : proc ? k_transmit<false, false, true> : k_transmit<false, false, false>)
                            <<<gtr, kThreads, 0, st>>>(S, Batch{}, Pb, F.kmax, nullptr);
                } else if (S.use_wide) {
                    k_shadow<true><<<grid_for(ctx, 3 * size_t(npaths), 8), kThreads, 0, st>>>(S, Pb, F.kmax);
                } else {
                    k_shadow<false><<<grid_for(ctx, 3 * size_t(npaths), 8), kThreads, 0, st>>>(S, Pb, F.kmax);
                }
                if (ctx->profile) CK(cudaEventRecord(pool_event(ctx, sh_ev.back().second), st));
            }
            // the paths' last NEE terms and the sample's radiance (the next
            // bounce's k_shade resolved those of the paths that went on)
            if (adj)
                k_finish<false, true><<<gadj, kThreads, smem, st>>>(S, F, Pw, Batch{}, A, npaths, s, srec);
            else
                k_finish<false, false><<<grid_for(ctx, npaths, 8), kThreads, 0, st>>>(S, F, Pw, Batch{}, Adj{},
                                                                                       npaths, s, srec);
        }
        return PT_OK;
    };
    // With render graphs on, plain renders replay each wave as a CUDA graph: a
    // call that repeats an earlier one's launch parameters (every byte of them)
    // replays its graph as it is; otherwise the wave is captured and the cached
    // graph of the same structure is updated in place (or a new one
    // instantiated).
    const bool use_graph = ctx->render_graphs && ctx->profile == 0 && dr.mode == RunMode::kRender;
    // A small wave (C0's 256 x 256 frames: 4 M paths) spends a large share of
    // each sample-bounce step in the ramp and drain of its four dependent
    // launches.  It runs as two halves of its frames at once, the second half on
    // the second stream pair with its own queues, counters and frame index, so
    // that one half's launches fill the SMs the other's tails leave idle.  The
    // halves touch disjoint path slots and frames; the running mean is applied
    // after both, in frame order, so the image is the same bit for bit.
    auto split_wave = [&](uint32_t nf) {
        return dr.mode == RunMode::kRender && !rr_fix && ctx->profile == 0 && !use_graph && overlap && persistent &&
               nf >= 2u && size_t(nf) * F.npix <= kSplitWavePaths;
    };
    // one wave's launches, on ctx->stream (and, split, on ctx->stream2)
    auto issue_wave = [&](uint32_t f0, uint32_t nf) -> int {
        if (!split_wave(nf)) {
            if (int rc = issue_paths(P, ctx->stream, ctx->side, ctx->ev_fork, ctx->ev_join, f0, nf)) return rc;
        } else {
            const uint32_t na = (nf + 1u) / 2u;
            const size_t off = size_t(na) * F.npix;
            DPaths P2 = P;
            for (float4** a : {&P2.ray_o, &P2.ray_d, &P2.thr, &P2.rad, &P2.fsum, &P2.amb}) *a += off;
            for (uint32_t** a : {&P2.seed, &P2.state, &P2.hit_id, &P2.shmask, &P2.q[0], &P2.q[1]}) *a += off;
            P2.hit_t += off;
            for (float4** a : {&P2.sh_o, &P2.sh_d, &P2.sh_pre, &P2.sh_brdf, &P2.sh_tr}) *a += 3 * off;
            P2.sq += 3 * off;
            P2.cnt = ctx->cnt.p + 16;
            P2.wave = ctx->wave_vars.p + 4;
            CK(cudaEventRecord(ctx->ev_split, ctx->stream));
            CK(cudaStreamWaitEvent(ctx->stream2, ctx->ev_split, 0));
            if (int rc = issue_paths(P, ctx->stream, ctx->side, ctx->ev_fork, ctx->ev_join, f0, na)) return rc;
            if (int rc = issue_paths(P2, ctx->stream2, ctx->side2, ctx->ev_fork2, ctx->ev_join2, f0 + na, nf - na))
                return rc;
            CK(cudaEventRecord(ctx->ev_half, ctx->stream2));
            CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_half, 0));
        }
        if (!adj)
            k_accumulate<<<(F.npix + 255) / 256, 256, 0, ctx->stream>>>(F, P, ctx->accum.p, nf, prm->accum_ema_alpha);
        return PT_OK;
    };
    for (uint32_t f0 = 0; f0 < frames; f0 += fpw) {
        const Nvtx nv_wave("wave from frame %u", f0);
        const uint32_t nf = std::min(fpw, frames - f0);
        const uint32_t npaths = nf * F.npix;
        const bool split = split_wave(nf);
        F.nframes = nf;
        k_set_wave<<<1, 1, 0, ctx->stream>>>(ctx->wave_vars.p, head->frame_index + f0, head->frame_index,
                                             f0 == 0 && head->reset_accum != 0u);
        if (split)   // the second half's frame index (its reset flag is not read)
            k_set_wave<<<1, 1, 0, ctx->stream>>>(ctx->wave_vars.p + 4, head->frame_index + f0 + (nf + 1u) / 2u,
                                                 head->frame_index, 0u);
        if (use_graph) {
            if (int rc = launch_wave_graph(ctx, issue_wave, f0, nf, F, S, P, prm->accum_ema_alpha, rr_fix, proc,
                                           persistent, overlap))
                return rc;
        } else if (int rc = issue_wave(f0, nf)) {
            return rc;
        }
        const uint32_t halves = split ? 2u : 1u;
        ctx->stats.kernel_launches += (adj ? 1u : 2u) + (split ? 1u : 0u) + halves * (1u + F.spp * (2u + 3u * F.maxb));
        ctx->stats.extend_launches += halves * F.spp * F.maxb;
        ctx->stats.shadow_launches += halves * F.spp * F.maxb;
        ctx->stats.waves++;
        ctx->stats.paths += uint64_t(npaths) * F.spp;
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats.gpu_ms = ms;
    ctx->stats.frames = frames;
    if (ctx->profile) {
        double ext = 0, sh = 0;
        for (const auto& e : ext_ev) {
            float a = 0;
            cudaEventElapsedTime(&a, ctx->ev_pool[e.first], ctx->ev_pool[e.second]);
            ext += a;
        }
        for (const auto& e : sh_ev) {
            float c = 0;
            cudaEventElapsedTime(&c, ctx->ev_pool[e.first], ctx->ev_pool[e.second]);
            sh += c;
        }
        ctx->stats.extend_ms = ext;
        ctx->stats.shadow_ms = sh;
    }
    unsigned long long st[4];
    uint32_t errw = 0;
    CK(cudaMemcpy(st, ctx->stat.p, sizeof(st), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&errw, ctx->err_word.p, 4, cudaMemcpyDeviceToHost));
    ctx->stats.extension_rays = st[0];
    ctx->stats.shadow_rays = st[1];
    if (errw) return set_err(ctx, PT_ERR_KERNEL, "render: " + traversal_error(errw));
    return PT_OK;
}


}  // namespace

extern "C" {

int pt_gpu_render(pt_gpu_ctx* ctx, const PtPushHead* head, const PtPathParams* prm, uint32_t frames) {
    return render_waves(ctx, head, prm, frames, DiffRun{});
}

int pt_gpu_diff_forward(pt_gpu_ctx* ctx, const PtPushHead* head, const PtPathParams* prm, uint32_t frames) {
    if (!ctx || !head || !prm) return PT_ERR_INVALID;
    ctx->d_valid = false;
    if (frames == 0) return set_err(ctx, PT_ERR_INVALID, "diff_forward: frames == 0");
    if (ctx->mat_count == 0) return set_err(ctx, PT_ERR_STATE, "diff_forward: no material table (the parameters)");
    if (prm->firefly_clamp > 0.0f)
        return set_err(ctx, PT_ERR_UNSUPPORTED, "diff_forward: the firefly clamp is not differentiable (set it to 0)");
    if (prm->refract_budget > 4u)
        return set_err(ctx, PT_ERR_UNSUPPORTED, "diff_forward: refract budget above 4");
    if (head->reset_accum == 0u || prm->accum_ema_alpha > 0.0f)
        return set_err(ctx, PT_ERR_UNSUPPORTED, "diff_forward: needs reset_accum and no EMA (image = mean of the samples)");
    if (ctx->mat_count > 4096u) return set_err(ctx, PT_ERR_UNSUPPORTED, "diff_forward: more than 4096 materials");
    ctx->d_batch_scene = nullptr;
    ctx->d_batch_views.clear();
    DiffRun dr;
    dr.mode = RunMode::kRecord;
    const int rc = render_waves(ctx, head, prm, frames, dr);
    if (rc) return rc;
    ctx->d_valid = true;
    ctx->d_gen = ctx->gen;
    ctx->d_head = *head;
    ctx->d_prm = *prm;
    ctx->d_frames = frames;
    return PT_OK;
}

int pt_gpu_diff_backward(pt_gpu_ctx* ctx, const float* dl_di_rgba, int on_device, double* grad_albedo,
                         double* grad_emission) {
    if (!ctx || !dl_di_rgba) return PT_ERR_INVALID;
    if (!ctx->d_valid || ctx->d_batch_scene)
        return set_err(ctx, PT_ERR_STATE, "diff_backward: no recorded forward (pt_gpu_diff_forward)");
    if (ctx->d_gen != ctx->gen)
        return set_err(ctx, PT_ERR_STATE, "diff_backward: the scene or target changed since the recorded forward");
    const size_t npix = size_t(ctx->W) * ctx->H;
    const float4* dldi = reinterpret_cast<const float4*>(dl_di_rgba);
    if (!on_device) {
        int rc = dupload(ctx, ctx->d_dldi, dl_di_rgba, npix);
        if (rc) return rc;
        dldi = ctx->d_dldi.p;
    } else if ((reinterpret_cast<uintptr_t>(dl_di_rgba) & 15u) != 0u) {
        return set_err(ctx, PT_ERR_INVALID, "diff_backward: device dL/dI must be 16-byte aligned");
    }
    DiffRun dr;
    dr.mode = RunMode::kAdjoint;
    dr.dldi = dldi;
    dr.nmat = ctx->mat_count;
    const PtStats keep = ctx->stats;
    const int rc = render_waves(ctx, &ctx->d_head, &ctx->d_prm, ctx->d_frames, dr);
    if (rc) return rc;
    ctx->d_bwd_stats = ctx->stats;
    ctx->stats = keep;
    std::vector<double> g(6 * size_t(ctx->mat_count));
    CK(cudaMemcpy(g.data(), ctx->d_grad.p, g.size() * sizeof(double), cudaMemcpyDeviceToHost));
    const size_t n3 = 3 * size_t(ctx->mat_count);
    if (grad_albedo) std::memcpy(grad_albedo, g.data(), n3 * sizeof(double));
    if (grad_emission) std::memcpy(grad_emission, g.data() + n3, n3 * sizeof(double));
    return PT_OK;
}

int pt_gpu_diff_get_backward_stats(pt_gpu_ctx* ctx, PtStats* out) {
    if (!ctx || !out) return PT_ERR_INVALID;
    *out = ctx->d_bwd_stats;
    return PT_OK;
}

int pt_gpu_render_to_host(pt_gpu_ctx* ctx, const PtPushHead* head, const PtPathParams* params,
                          uint32_t frames, float* host_rgba) {
    int rc = pt_gpu_render(ctx, head, params, frames);
    if (rc) return rc;
    return pt_gpu_read_accum(ctx, host_rgba);
}

int pt_gpu_tonemap(pt_gpu_ctx* ctx, float exposure, uint32_t op, int srgb_oetf, uint8_t* rgba8, int on_device) {
    if (!ctx || !rgba8) return PT_ERR_INVALID;
    if (!ctx->accum.p) return set_err(ctx, PT_ERR_STATE, "tonemap: no target");
    if (op > 4u) return set_err(ctx, PT_ERR_INVALID, "tonemap: operator must be 0..4");
    const size_t n = size_t(ctx->W) * ctx->H;
    uchar4* dst = reinterpret_cast<uchar4*>(rgba8);
    if (!on_device) {
        if (int rc = dalloc(ctx, ctx->ldr, n)) return rc;
        dst = ctx->ldr.p;
    } else if (reinterpret_cast<uintptr_t>(rgba8) & 3u) {
        return set_err(ctx, PT_ERR_INVALID, "tonemap: device output must be 4-byte aligned");
    }
    k_tonemap<<<uint32_t((n + 255) / 256), 256, 0, ctx->stream>>>(ctx->accum.p, uint32_t(n), exposure, op,
                                                                   srgb_oetf ? 1u : 0u, dst);
    CK(cudaGetLastError());
    if (!on_device) CK(cudaMemcpyAsync(rgba8, dst, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_gpu_get_stats(pt_gpu_ctx* ctx, PtStats* out) {
    if (!ctx || !out) return PT_ERR_INVALID;
    *out = ctx->stats;
    return PT_OK;
}

int pt_gpu_set_traversal(pt_gpu_ctx* ctx, int mode) {
    if (ctx) ctx->gen++;
    if (!ctx || mode < 0 || mode > 1) return PT_ERR_INVALID;
    ctx->traversal = mode;
    return PT_OK;
}

int pt_gpu_get_accel_info(pt_gpu_ctx* ctx, PtAccelInfo* out) {
    if (!ctx || !out) return PT_ERR_INVALID;
    std::memset(out, 0, sizeof(*out));
    out->traversal = uint32_t(ctx->traversal);
    out->mesh_wide = ctx->t_wide ? 1u : 0u;
    out->prims_wide = ctx->a_wide ? 1u : 0u;
    out->mesh_wide_nodes = ctx->t4_count;
    out->mesh_wide_depth = ctx->t4_depth;
    out->mesh_binary_nodes = ctx->t4_bin_nodes;
    out->prims_wide_nodes = ctx->a4_count;
    out->merged_wide_nodes = ctx->m_wide ? ctx->m4_count : 0u;
    out->mesh_build_ms = ctx->build_ms;
    return PT_OK;
}

int pt_gpu_set_profiling(pt_gpu_ctx* ctx, int on) {
    if (!ctx) return PT_ERR_INVALID;
    if (on < 0 || on > 3) return set_err(ctx, PT_ERR_INVALID, "set_profiling: on must be 0, 1, 2 or 3");
    ctx->profile = on;
    return PT_OK;
}

int pt_gpu_set_roulette_freeze(pt_gpu_ctx* ctx, int mode) {
    if (!ctx) return PT_ERR_INVALID;
    if (mode < 0 || mode > 2) return set_err(ctx, PT_ERR_INVALID, "set_roulette_freeze: mode must be 0, 1 or 2");
    if (mode == 2 && !ctx->rr_buf.p)
        return set_err(ctx, PT_ERR_STATE, "set_roulette_freeze: nothing recorded (render once in mode 1)");
    ctx->rr_freeze = mode;
    if (mode == 0) {
        dfree(ctx->rr_buf);
        std::memset(ctx->rr_meta, 0, sizeof(ctx->rr_meta));
    }
    return PT_OK;
}

int pt_gpu_set_debug_limits(pt_gpu_ctx* ctx, uint32_t traverse_cap, uint32_t stack_entries) {
    if (!ctx) return PT_ERR_INVALID;
    if (stack_entries > uint32_t(kPStack))
        return set_err(ctx, PT_ERR_INVALID, "set_debug_limits: at most " + std::to_string(kPStack) +
                                                " stack entries");
    if (stack_entries != 0u && stack_entries < 4u)
        return set_err(ctx, PT_ERR_INVALID, "set_debug_limits: at least 4 stack entries (one node's children)");
    ctx->dbg_trav_cap = traverse_cap;
    ctx->dbg_stack_cap = stack_entries;
    return PT_OK;
}

int pt_gpu_set_render_graphs(pt_gpu_ctx* ctx, int on) {
    if (!ctx) return PT_ERR_INVALID;
    ctx->render_graphs = on != 0;
    return PT_OK;
}

int pt_gpu_get_traversal_stats(pt_gpu_ctx* ctx, PtTraversalStats* out) {
    if (!ctx || !out) return PT_ERR_INVALID;
    unsigned long long c[16];
    CK(cudaMemcpy(c, ctx->tcount.p, sizeof(c), cudaMemcpyDeviceToHost));
    *out = PtTraversalStats{};
    uint64_t* ext = &out->ext_segments;
    uint64_t* sh = &out->shadow_segments;
    for (int k = 0; k < 7; ++k) {
        ext[k] = c[k];
        sh[k] = c[8 + k];
    }
    return PT_OK;
}

int pt_gpu_trace_closest(pt_gpu_ctx* ctx, const float* ray_o, const float* ray_d, uint32_t n,
                         uint32_t* hit_id, float* t, int on_device) {
    if (!ctx || (n && (!ray_o || !ray_d || !hit_id || !t))) return PT_ERR_INVALID;
    if (n == 0) return PT_OK;
    PtPathParams prm{};
    prm.bvh_params[0] = ctx->linear_count;
    prm.bvh_params[1] = ctx->bvh_nodes;
    prm.bvh_params[2] = ctx->tri_count;
    prm.bvh_params[3] = ctx->tri_nodes;
    prm.light_count = ctx->light_count;
    prm.sdf_params[0] = ctx->sdf_count;   // every uploaded SDF cluster, with the
    prm.sdf_params[1] = 128u;             // reference's default trace settings
    prm.sdf_params[3] = 12u;
    prm.sdf_params_f[0] = 1e-4f;
    prm.sdf_params_f[1] = 8.0f;
    prm.sdf_params_f[2] = 1.0f;
    const DScene S = make_scene(ctx, &prm);
    CK(cudaMemsetAsync(ctx->err_word.p, 0, 4, ctx->stream));
    const float4 *dro, *drd;
    uint32_t* dh;
    float* dt;
    DBuf<float4> bo, bd;
    DBuf<uint32_t> bh;
    DBuf<float> bt;
    if (on_device) {
        dro = reinterpret_cast<const float4*>(ray_o);
        drd = reinterpret_cast<const float4*>(ray_d);
        dh = hit_id;
        dt = t;
    } else {
        int rc = 0;
        if ((rc = dupload(ctx, bo, ray_o, n)) || (rc = dupload(ctx, bd, ray_d, n)) || (rc = dalloc(ctx, bh, n)) ||
            (rc = dalloc(ctx, bt, n))) {
            dfree(bo); dfree(bd); dfree(bh); dfree(bt);
            return rc;
        }
        dro = bo.p; drd = bd.p; dh = bh.p; dt = bt.p;
    }
    // With the wide trees the probe runs the renders' own closest-hit kernel
    // (persistent, dynamic ray fetch) over an identity queue; otherwise the
    // per-ray walk of the chosen traversal.
    const bool persistent = S.use_wide && (S.a_wide || S.prim_count == S.wide_linear) &&
                            (S.t_wide || S.tri_enabled == 0u || S.tri_nodes == 0u);
    DBuf<uint32_t> bq;
    if (persistent) {
        if (int rc = dalloc(ctx, bq, size_t(n) + 2)) {
            dfree(bo); dfree(bd); dfree(bh); dfree(bt);
            return rc;
        }
        k_probe_queue<<<(n + 255) / 256, 256, 0, ctx->stream>>>(bq.p, n);
        k_closest<false, false><<<ctx->sm_count * 4, kThreads, 0, ctx->stream>>>(S, Batch{}, bq.p, bq.p + n, dro, drd,
                                                                                 dt, dh, bq.p + n + 1, ctx->stat.p);
        k_probe_ids<<<(n + 255) / 256, 256, 0, ctx->stream>>>(S, n, dh, dt);
    } else {
        k_trace_probe<<<(n + 127) / 128, 128, 0, ctx->stream>>>(S, dro, drd, n, dh, dt);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && !on_device) {
        e = cudaMemcpyAsync(hit_id, dh, size_t(n) * 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(t, dt, size_t(n) * 4, cudaMemcpyDeviceToHost, ctx->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dfree(bo); dfree(bd); dfree(bh); dfree(bt); dfree(bq);
    if (e != cudaSuccess) return set_err(ctx, PT_ERR_CUDA, std::string("trace_closest: ") + cudaGetErrorString(e));
    uint32_t errw = 0;
    CK(cudaMemcpy(&errw, ctx->err_word.p, 4, cudaMemcpyDeviceToHost));
    if (errw) return set_err(ctx, PT_ERR_KERNEL, "trace_closest: " + traversal_error(errw));
    return PT_OK;
}

}  // extern "C"


// ===========================================================================
// Batched renders
// ===========================================================================
namespace {

int validate_view(pt_gpu_ctx* ctx, pt_gpu_ctx* sc, const PtBatchView& v, uint32_t i) {
    const std::string w = "batch view " + std::to_string(i) + ": ";
    const PtPushHead* head = &v.head;
    const PtPathParams* prm = &v.params;
    if (v.width == 0 || v.height == 0) return set_err(ctx, PT_ERR_INVALID, w + "empty frame");
    if (head->tlas_present) return set_err(ctx, PT_ERR_UNSUPPORTED, w + "tlas (hardware RT) has no CUDA path");
    if (int rc = check_light_tree(ctx, sc, prm, w)) return rc;
    if (int rc = check_sdf(ctx, sc, prm, w)) return rc;
    if (int rc = check_sky(ctx, sc, head, prm, w)) return rc;
    if (head->prim_count != sc->prim_count || prm->bvh_params[0] != sc->linear_count ||
        prm->bvh_params[1] != sc->bvh_nodes)
        return set_err(ctx, PT_ERR_INVALID, w + "prim_count / bvh_params disagree with its scene");
    if ((prm->bvh_params[2] != 0u) != (sc->tri_nodes != 0u) ||
        (prm->bvh_params[2] != 0u && prm->bvh_params[3] != sc->tri_nodes))
        return set_err(ctx, PT_ERR_INVALID, w + "mesh bvh_params disagree with its scene");
    if (prm->light_count != sc->light_count) return set_err(ctx, PT_ERR_INVALID, w + "light_count disagrees");
    if (!sc->a_wide && sc->prim_count > sc->linear_count && sc->bvh_nodes != 0u)
        return set_err(ctx, PT_ERR_UNSUPPORTED, w + "scene has no wide analytic tree");
    if (!sc->t_wide && sc->tri_nodes > 0u)
        return set_err(ctx, PT_ERR_UNSUPPORTED, w + "scene has no wide mesh tree");
    return PT_OK;
}

DFrame frame_of(const PtBatchView& v) {
    const PtPushHead* head = &v.head;
    const PtPathParams* prm = &v.params;
    DFrame F{};
    F.cam_pos = v3(head->pos_fovtan[0], head->pos_fovtan[1], head->pos_fovtan[2]);
    F.tanf = head->pos_fovtan[3];
    F.fwd = v3(head->fwd_aspect[0], head->fwd_aspect[1], head->fwd_aspect[2]);
    F.aspect = head->fwd_aspect[3];
    F.right = v3(head->right_xyz[0], head->right_xyz[1], head->right_xyz[2]);
    F.up = v3(head->up_xyz[0], head->up_xyz[1], head->up_xyz[2]);
    F.W = v.width;
    F.H = v.height;
    F.npix = v.width * v.height;
    F.nframes = v.frames_per_wave == 0u ? 1u : v.frames_per_wave;
    F.frame_index0 = head->frame_index;
    F.call_fi0 = head->frame_index;
    F.spp = head->spp == 0u ? 1u : head->spp;
    F.maxb = head->max_bounces;
    F.denoiser = head->denoiser_enabled;
    F.jx = head->halton_jitter[0];
    F.jy = head->halton_jitter[1];
    F.env_present = head->env_map_present;
    F.env_intensity = head->env_intensity;
    F.env_total = head->env_total_luminance;
    F.kmax = int(prm->refract_budget);
    F.firefly = prm->firefly_clamp;
    F.mis = prm->mis_enabled;
    F.rr_start = prm->rr_start;
    F.light_count = prm->light_count;
    sky_of(F, prm);
    F.scene = v.scene;
    F.reset = head->reset_accum;
    F.ema = prm->accum_ema_alpha;
    return F;
}

// Issue one wave (one frame of every view) on ctx->stream.
int issue_batch_wave(pt_gpu_ctx* ctx, const Batch& Bt, const DPaths& P, uint32_t npaths, uint32_t npix_total,
                     uint32_t max_spp, uint32_t max_b, int kmax_any, const DScene& S0, bool proc,
                     const Adj* adj = nullptr, size_t smem = 0) {
    const DFrame F0{};
    const int gp = (npaths + 255) / 256;
    const int gpers = ctx->sm_count * int(ctx->b_tune.persistent_blocks_per_sm);
    const int gtr = ctx->sm_count * std::min(int(ctx->b_tune.persistent_blocks_per_sm), kTransmitBlocks);
    const int gstream = int(std::max<size_t>(1, std::min<size_t>((npaths + kThreads - 1) / kThreads,
                                                                 size_t(ctx->sm_count) * ctx->b_tune.stream_blocks_per_sm)));
    CK(cudaMemsetAsync(P.stat, 0, 4 * sizeof(unsigned long long), ctx->stream));
    k_init_wave<true><<<gp, 256, 0, ctx->stream>>>(F0, P, Bt, npaths);
    for (uint32_t s = 0; s < max_spp; ++s) {
        // the counter ring (DPaths::cnt); k_camera appends the compacted queue to block 0
        CK(cudaMemsetAsync(P.cnt, 0, 16 * sizeof(uint32_t), ctx->stream));
        k_camera<true><<<gp, 256, 0, ctx->stream>>>(F0, P, Bt, npaths, s);
        for (uint32_t b = 0; b < max_b; ++b) {
            const int qs = int(b & 1u);
            const DPaths Pb = bounce_paths(P, b);
            if (b == 0u) {
                (proc ? k_closest<true, true> : k_closest<true, false>)<<<gpers, kThreads, 0, ctx->stream>>>(
                    S0, Bt, P.q[qs], Pb.cnt, P.ray_o, P.ray_d, P.hit_t, P.hit_id, Pb.cnt + 2, P.stat);
            } else {
                // this bounce's closest hits were traced on the side stream
                CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
            }
            const size_t srec = size_t(s) * npaths;
            Adj A{};
            if (adj) {
                A = *adj;
                A.srec_base = srec;
                (proc ? k_shade<true, true, true> : k_shade<true, true, false>)
                    <<<ctx->sm_count * 2, kShadeThreads, smem, ctx->stream>>>(S0, F0, Pb, Bt, A, qs, b);
            } else {
                // shading block: 512 threads (default) or 256 (autotuner); same grid in threads
                if (ctx->b_tune.shade_threads == 256u)
                    (proc ? k_shade<true, false, true, 256> : k_shade<true, false, false, 256>)
                        <<<gstream, 256, 0, ctx->stream>>>(S0, F0, Pb, Bt, Adj{}, qs, b);
                else
                    (proc ? k_shade<true, false, true> : k_shade<true, false, false>)
                        <<<(gstream + 1) / 2, kShadeThreads, 0, ctx->stream>>>(S0, F0, Pb, Bt, Adj{}, qs, b);
            }
            if (b + 1u < max_b) {
                // fork: the next bounce's closest hits overlap this bounce's shadow rays
                const DPaths Pn = bounce_paths(P, b + 1u);
                CK(cudaEventRecord(ctx->ev_fork, ctx->stream));
                CK(cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
                (proc ? k_closest<true, true> : k_closest<true, false>)<<<gpers, kThreads, 0, ctx->side>>>(
                    S0, Bt, P.q[qs ^ 1], Pn.cnt, P.ray_o, P.ray_d, P.hit_t, P.hit_id, Pn.cnt + 2, P.stat);
                CK(cudaEventRecord(ctx->ev_join, ctx->side));
            }
            if (adj)
                (proc ? k_transmit<true, true, true> : k_transmit<true, true, false>)
                    <<<gtr, kThreads, 0, ctx->stream>>>(S0, Bt, Pb, kmax_any, ctx->d_sh_mats.p);
            else
                (proc ? k_transmit<true, false, true> : k_transmit<true, false, false>)
                    <<<gtr, kThreads, 0, ctx->stream>>>(S0, Bt, Pb, kmax_any, nullptr);
        }
        // the paths' last NEE terms and the sample's radiance
        const size_t srec = size_t(s) * npaths;
        if (adj) {
            Adj A = *adj;
            A.srec_base = srec;
            k_finish<true, true><<<ctx->sm_count * 4, kThreads, smem, ctx->stream>>>(S0, F0, P, Bt, A, npaths, s,
                                                                                     srec);
        } else {
            k_finish<true, false><<<gstream, kThreads, 0, ctx->stream>>>(S0, F0, P, Bt, Adj{}, npaths, s, srec);
        }
    }
    if (!adj) k_accumulate_batch<<<(npix_total + 255) / 256, 256, 0, ctx->stream>>>(P, Bt, npix_total);
    return PT_OK;
}

}  // namespace

extern "C" {

int pt_gpu_batch_set_tuning(pt_gpu_ctx* ctx, const PtBatchTuning* t) {
    if (!ctx || !t || t->persistent_blocks_per_sm < 1 || t->persistent_blocks_per_sm > 4 ||
        t->stream_blocks_per_sm < 1 || t->stream_blocks_per_sm > 64 ||
        (t->shade_threads != 256u && t->shade_threads != 512u) ||
        (t->camera_tile_w != 4u && t->camera_tile_w != 8u && t->camera_tile_w != 16u && t->camera_tile_w != 32u) ||
        t->octant_grouping > 1u || t->use_graph > 1u)
        return ctx ? set_err(ctx, PT_ERR_INVALID, "batch_set_tuning: a knob is out of range") : PT_ERR_INVALID;
    ctx->b_tune = *t;
    if (ctx->b_graph) {
        cudaGraphExecDestroy(ctx->b_graph);
        ctx->b_graph = nullptr;
    }
    ctx->b_sig.clear();
    return PT_OK;
}

int pt_gpu_batch_get_tuning(pt_gpu_ctx* ctx, PtBatchTuning* t) {
    if (!ctx || !t) return PT_ERR_INVALID;
    *t = ctx->b_tune;
    return PT_OK;
}

}  // extern "C"

namespace {

int batch_waves(pt_gpu_ctx* ctx, pt_gpu_ctx* const* scenes, uint32_t n_scenes, const PtBatchView* views,
                uint32_t n_views, uint32_t frames, const DiffRun& dr) {
    if (!ctx || !scenes || !views || n_scenes == 0 || n_views == 0) return PT_ERR_INVALID;
    for (uint32_t k = 0; k < n_scenes; ++k)
        if (!scenes[k] || scenes[k]->device != ctx->device)
            return set_err(ctx, PT_ERR_INVALID, "batch: scene contexts must be on the batch context's device");
    uint64_t total = 0, total_pix = 0;
    uint32_t max_spp = 0, max_b = 0;
    int kmax_any = -1;
    auto fpw = [&](uint32_t i) { return views[i].frames_per_wave == 0u ? 1u : views[i].frames_per_wave; };
    for (uint32_t i = 0; i < n_views; ++i) {
        if (views[i].scene >= n_scenes) return set_err(ctx, PT_ERR_INVALID, "batch: view scene index out of range");
        if (int rc = validate_view(ctx, scenes[views[i].scene], views[i], i)) return rc;
        if (views[i].frames_per_wave > 1024u) return set_err(ctx, PT_ERR_INVALID, "batch: frames_per_wave above 1024");
        total += uint64_t(fpw(i)) * views[i].width * views[i].height;
        total_pix += uint64_t(views[i].width) * views[i].height;
        max_spp = std::max(max_spp, views[i].head.spp == 0u ? 1u : views[i].head.spp);
        max_b = std::max(max_b, views[i].head.max_bounces);
        const int km = int(views[i].params.refract_budget);
        if (kmax_any >= 0 && km != kmax_any)
            return set_err(ctx, PT_ERR_INVALID, "batch: all views must share the refraction budget");
        kmax_any = km;
    }
    if (total > (64ull << 20)) return set_err(ctx, PT_ERR_INVALID, "batch: more than 64 M path slots per wave");
    const uint32_t npaths = uint32_t(total), npix_total = uint32_t(total_pix);
    if (frames == 0) return PT_OK;

    // the procedural SDF walker is compiled into the wave's kernels only when a
    // view enables it over a scene that holds a procedural cluster
    bool proc = false;
    for (uint32_t i = 0; i < n_views; ++i)
        proc = proc || (views[i].params.sdf_procedural_ops != 0u && scenes[views[i].scene]->sdf_proc_any);
    // layout signature: views' sizes and scenes, tuning, walker variant
    std::vector<uint64_t> sig;
    sig.push_back(n_views);
    sig.push_back(proc ? 1u : 0u);
    for (uint32_t i = 0; i < n_views; ++i) {
        sig.push_back((uint64_t(views[i].width) << 32) | views[i].height);
        sig.push_back(uint64_t(reinterpret_cast<uintptr_t>(scenes[views[i].scene])));
        sig.push_back((uint64_t(views[i].head.spp) << 32) | views[i].head.max_bounces);
        sig.push_back(fpw(i));
    }
    const bool same_layout = (sig == ctx->b_sig);
    int rc = ensure_wave(ctx, npaths);
    if (rc) return rc;
    if (!same_layout) {
        if (ctx->b_graph) {
            cudaGraphExecDestroy(ctx->b_graph);
            ctx->b_graph = nullptr;
        }
        std::vector<uint32_t> base(n_views + 1, 0);
        std::vector<size_t> aoff(n_views, 0);
        size_t acc = 0;
        for (uint32_t i = 0; i < n_views; ++i) {
            base[i + 1] = base[i] + fpw(i) * views[i].width * views[i].height;
            aoff[i] = acc;
            acc += size_t(views[i].width) * views[i].height;
        }
        if ((rc = dupload(ctx, ctx->b_view_base, base.data(), n_views + 1)) ||
            (rc = dalloc(ctx, ctx->b_path_view, npaths)) || (rc = dalloc(ctx, ctx->b_path_scene, npaths)) ||
            (rc = dalloc(ctx, ctx->b_views, n_views)) || (rc = dalloc(ctx, ctx->b_scenes, n_scenes)) ||
            (rc = dalloc(ctx, ctx->b_accum, acc)))
            return rc;
        CK(cudaMemsetAsync(ctx->b_accum.p, 0, acc * 16, ctx->stream));
        ctx->b_accum_off = aoff;
        ctx->b_w.resize(n_views);
        ctx->b_h.resize(n_views);
        for (uint32_t i = 0; i < n_views; ++i) {
            ctx->b_w[i] = views[i].width;
            ctx->b_h[i] = views[i].height;
        }
    }
    // scene table (pointers may change after re-uploads); SDF trace settings
    // come from the views of each scene, which must agree
    std::vector<DScene> st(n_scenes);
    for (uint32_t k = 0; k < n_scenes; ++k) {
        st[k] = make_scene(scenes[k], nullptr);
        st[k].err = ctx->err_word.p;
    }
    {
        std::vector<int> seen(n_scenes, 0);
        for (uint32_t i = 0; i < n_views; ++i) {
            DScene& d = st[views[i].scene];
            const PtPathParams& q = views[i].params;
            if (seen[views[i].scene] && (d.sdf_count != q.sdf_params[0] || d.sdf_iters != q.sdf_params[1] ||
                                         d.sdf_eps != q.sdf_params_f[0] || d.frac_iters != q.sdf_params[3] ||
                                         d.frac_power != q.sdf_params_f[1] || d.frac_eps_scale != q.sdf_params_f[2] ||
                                         d.sdf_proc != std::min(q.sdf_procedural_ops, 2u) ||
                                         d.sdf_nmode != (q.sdf_params_f[3] != 0.0f ? 1u : 0u)))
                return set_err(ctx, PT_ERR_INVALID, "batch: views of one scene disagree on the SDF settings");
            d.sdf_count = q.sdf_params[0];
            d.sdf_iters = q.sdf_params[1];
            d.sdf_eps = q.sdf_params_f[0];
            d.frac_iters = q.sdf_params[3];
            d.frac_power = q.sdf_params_f[1];
            d.frac_eps_scale = q.sdf_params_f[2];
            d.sdf_proc = std::min(q.sdf_procedural_ops, 2u);
            d.sdf_nmode = q.sdf_params_f[3] != 0.0f ? 1u : 0u;
            seen[views[i].scene] = 1;
        }
    }
    CK(cudaMemcpyAsync(ctx->b_scenes.p, st.data(), n_scenes * sizeof(DScene), cudaMemcpyHostToDevice, ctx->stream));
    ctx->b_views_h.resize(n_views);
    uint32_t base_slot = 0;
    for (uint32_t i = 0; i < n_views; ++i) {
        ctx->b_views_h[i] = frame_of(views[i]);
        ctx->b_views_h[i].tile_lw = uint32_t(__builtin_ctz(ctx->b_tune.camera_tile_w));
        ctx->b_views_h[i].octant_on = ctx->b_tune.octant_grouping ? 1u : 0u;
        ctx->b_views_h[i].slot_base = base_slot;
        ctx->b_views_h[i].accum_base = ctx->b_accum_off[i];
        base_slot += fpw(i) * views[i].width * views[i].height;
    }

    DPaths P{};
    P.ray_o = ctx->ray_o.p; P.ray_d = ctx->ray_d.p; P.thr = ctx->thr.p; P.rad = ctx->rad.p; P.amb = ctx->amb.p;
    P.fsum = ctx->fsum.p; P.seed = ctx->seed.p; P.state = ctx->state.p; P.hit_t = ctx->hit_t.p;
    P.hit_id = ctx->hit_id.p; P.shmask = ctx->shmask.p; P.sh_o = ctx->sh_o.p; P.sh_d = ctx->sh_d.p;
    P.sh_pre = ctx->sh_pre.p; P.sh_brdf = ctx->sh_brdf.p; P.sh_tr = ctx->sh_tr.p;
    P.q[0] = ctx->q0.p; P.q[1] = ctx->q1.p; P.sq = ctx->sq.p; P.cnt = ctx->cnt.p; P.stat = ctx->stat.p;
    Batch Bt{};
    Bt.views = ctx->b_views.p;
    Bt.scenes = ctx->b_scenes.p;
    Bt.path_view = ctx->b_path_view.p;
    Bt.path_scene = ctx->b_path_scene.p;
    Bt.view_base = ctx->b_view_base.p;
    Bt.accum = ctx->b_accum.p;
    Bt.n_views = n_views;
    const DScene S0 = st[0];
    const bool adj = dr.mode == RunMode::kAdjoint;
    size_t smem = 0;
    Adj A{};
    if (dr.mode != RunMode::kRender) {
        rc = dalloc(ctx, ctx->d_srad, size_t(max_spp) * npaths);
        if (rc) return rc;
        P.srad = (dr.mode == RunMode::kRecord) ? ctx->d_srad.p : nullptr;
    }
    if (adj) {
        if ((rc = dalloc(ctx, ctx->d_sh_mats, 3 * size_t(npaths))) || (rc = dalloc(ctx, ctx->d_grad, 6 * size_t(dr.nmat))))
            return rc;
        CK(cudaMemsetAsync(ctx->d_grad.p, 0, 6 * size_t(dr.nmat) * sizeof(double), ctx->stream));
        smem = 6 * size_t(dr.nmat) * sizeof(double);
        // always opted in: k_shade also holds static shared memory (its queue
        // counting sort), and the 48 KB default bounds static + dynamic together
        CK(cudaFuncSetAttribute(k_shade<true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        CK(cudaFuncSetAttribute(k_shade<true, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        CK(cudaFuncSetAttribute(k_finish<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        A.srad = ctx->d_srad.p;
        A.dldi = dr.dldi;
        A.grad = ctx->d_grad.p;
        A.sh_mats = ctx->d_sh_mats.p;
        A.nmat = dr.nmat;
        A.scale = 1.0f;
    }
    const bool graph = ctx->b_tune.use_graph && dr.mode == RunMode::kRender;

    // work a failed earlier call left on the side stream finishes first
    CK(cudaEventRecord(ctx->ev_join, ctx->side));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
    CK(cudaMemsetAsync(ctx->err_word.p, 0, 4, ctx->stream));
    ctx->stats = PtStats{};
    unsigned long long tot_ext = 0, tot_sh = 0;
    const uint32_t launches_per_wave = 2 + max_spp * (2 + 3 * max_b);
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    for (uint32_t f = 0; f < frames; ++f) {
        for (uint32_t i = 0; i < n_views; ++i) {
            DFrame& V = ctx->b_views_h[i];
            V.frame_index0 = views[i].head.frame_index + f * fpw(i);
            V.reset = (f == 0 && views[i].head.reset_accum) ? 1u : 0u;
        }
        CK(cudaMemcpyAsync(ctx->b_views.p, ctx->b_views_h.data(), n_views * sizeof(DFrame), cudaMemcpyHostToDevice,
                           ctx->stream));
        if (graph) {
            if (!ctx->b_graph) {
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
                const int irc = issue_batch_wave(ctx, Bt, P, npaths, npix_total, max_spp, max_b, kmax_any, S0, proc);
                cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
                if (irc) return irc;
                if (e != cudaSuccess) return set_err(ctx, PT_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
                e = cudaGraphInstantiate(&ctx->b_graph, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    ctx->b_graph = nullptr;
                    return set_err(ctx, PT_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
                }
            }
            CK(cudaGraphLaunch(ctx->b_graph, ctx->stream));
        } else {
            if (int irc = issue_batch_wave(ctx, Bt, P, npaths, npix_total, max_spp, max_b, kmax_any, S0, proc,
                                           adj ? &A : nullptr, smem))
                return irc;
        }
        unsigned long long st2[4];
        CK(cudaMemcpyAsync(st2, ctx->stat.p, sizeof(st2), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        tot_ext += st2[0];
        tot_sh += st2[1];
        ctx->stats.kernel_launches += launches_per_wave - (adj ? 1u : 0u);
        ctx->stats.waves++;
        ctx->stats.paths += uint64_t(npaths) * max_spp;
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->b_sig = sig;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats.gpu_ms = ms;
    ctx->stats.frames = frames;
    ctx->stats.extension_rays = tot_ext;
    ctx->stats.shadow_rays = tot_sh;
    uint32_t errw = 0;
    CK(cudaMemcpy(&errw, ctx->err_word.p, 4, cudaMemcpyDeviceToHost));
    if (errw) return set_err(ctx, PT_ERR_KERNEL, "batch: " + traversal_error(errw));
    return PT_OK;
}

}  // namespace

extern "C" {

int pt_gpu_batch_render(pt_gpu_ctx* ctx, pt_gpu_ctx* const* scenes, uint32_t n_scenes, const PtBatchView* views,
                        uint32_t n_views, uint32_t frames) {
    return batch_waves(ctx, scenes, n_scenes, views, n_views, frames, DiffRun{});
}

int pt_gpu_batch_diff_forward(pt_gpu_ctx* ctx, pt_gpu_ctx* scene, const PtBatchView* views, uint32_t n_views) {
    if (!ctx || !scene || !views || n_views == 0) return PT_ERR_INVALID;
    ctx->d_valid = false;
    if (scene->mat_count == 0) return set_err(ctx, PT_ERR_STATE, "batch_diff_forward: no material table");
    if (scene->mat_count > 4096u) return set_err(ctx, PT_ERR_UNSUPPORTED, "batch_diff_forward: more than 4096 materials");
    for (uint32_t i = 0; i < n_views; ++i) {
        const PtBatchView& v = views[i];
        if (v.scene != 0u) return set_err(ctx, PT_ERR_INVALID, "batch_diff_forward: views index the one scene (0)");
        if (v.params.firefly_clamp > 0.0f || v.params.refract_budget > 4u || v.head.reset_accum == 0u ||
            v.params.accum_ema_alpha > 0.0f)
            return set_err(ctx, PT_ERR_UNSUPPORTED,
                           "batch_diff_forward: needs no firefly clamp, refract budget <= 4, reset_accum, no EMA");
    }
    DiffRun dr;
    dr.mode = RunMode::kRecord;
    pt_gpu_ctx* const sc[1] = {scene};
    const int rc = batch_waves(ctx, sc, 1, views, n_views, 1, dr);
    if (rc) return rc;
    ctx->d_valid = true;
    ctx->d_gen = scene->gen;
    ctx->d_batch_scene = scene;
    ctx->d_batch_views.assign(views, views + n_views);
    return PT_OK;
}

int pt_gpu_batch_diff_backward(pt_gpu_ctx* ctx, const float* dl_di_rgba, int on_device, double* grad_albedo,
                               double* grad_emission) {
    if (!ctx || !dl_di_rgba) return PT_ERR_INVALID;
    if (!ctx->d_valid || !ctx->d_batch_scene || ctx->d_batch_views.empty())
        return set_err(ctx, PT_ERR_STATE, "batch_diff_backward: no recorded batched forward");
    pt_gpu_ctx* scene = ctx->d_batch_scene;
    if (ctx->d_gen != scene->gen)
        return set_err(ctx, PT_ERR_STATE, "batch_diff_backward: the scene changed since the recorded forward");
    size_t npix = 0;
    for (const auto& v : ctx->d_batch_views) npix += size_t(v.width) * v.height;
    const float4* dldi = reinterpret_cast<const float4*>(dl_di_rgba);
    if (!on_device) {
        int rc = dupload(ctx, ctx->d_dldi, dl_di_rgba, npix);
        if (rc) return rc;
        dldi = ctx->d_dldi.p;
    } else if ((reinterpret_cast<uintptr_t>(dl_di_rgba) & 15u) != 0u) {
        return set_err(ctx, PT_ERR_INVALID, "batch_diff_backward: device dL/dI must be 16-byte aligned");
    }
    DiffRun dr;
    dr.mode = RunMode::kAdjoint;
    dr.dldi = dldi;
    dr.nmat = scene->mat_count;
    const PtStats keep = ctx->stats;
    pt_gpu_ctx* const sc[1] = {scene};
    const int rc = batch_waves(ctx, sc, 1, ctx->d_batch_views.data(), uint32_t(ctx->d_batch_views.size()), 1, dr);
    if (rc) return rc;
    ctx->d_bwd_stats = ctx->stats;
    ctx->stats = keep;
    std::vector<double> g(6 * size_t(dr.nmat));
    CK(cudaMemcpy(g.data(), ctx->d_grad.p, g.size() * sizeof(double), cudaMemcpyDeviceToHost));
    const size_t n3 = 3 * size_t(dr.nmat);
    if (grad_albedo) std::memcpy(grad_albedo, g.data(), n3 * sizeof(double));
    if (grad_emission) std::memcpy(grad_emission, g.data() + n3, n3 * sizeof(double));
    return PT_OK;
}

int pt_gpu_batch_read_accum(pt_gpu_ctx* ctx, uint32_t view, float* host_rgba) {
    if (!ctx || !host_rgba) return PT_ERR_INVALID;
    if (view >= ctx->b_accum_off.size()) return set_err(ctx, PT_ERR_INVALID, "batch_read_accum: no such view");
    CK(cudaMemcpyAsync(host_rgba, ctx->b_accum.p + ctx->b_accum_off[view],
                       size_t(ctx->b_w[view]) * ctx->b_h[view] * 16, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return PT_OK;
}

int pt_gpu_batch_autotune(pt_gpu_ctx* ctx, pt_gpu_ctx* const* scenes, uint32_t n_scenes, const PtBatchView* views,
                          uint32_t n_views, PtBatchTuning* chosen) {
    if (!ctx) return PT_ERR_INVALID;
    // one frame of the batch per candidate: a render that builds (captures) the
    // wave, then a timed one; the best time wins
    auto time_of = [&](const PtBatchTuning& c, double& ms) -> int {
        if (int rc = pt_gpu_batch_set_tuning(ctx, &c)) return rc;
        if (int rc = pt_gpu_batch_render(ctx, scenes, n_scenes, views, n_views, 1)) return rc;
        if (int rc = pt_gpu_batch_render(ctx, scenes, n_scenes, views, n_views, 1)) return rc;
        ms = ctx->stats.gpu_ms;
        return PT_OK;
    };
    // coordinate descent from the default, one knob at a time: persistent
    // grid, streaming grid, shading block, camera tile, octant grouping, graph
    PtBatchTuning best{4u, 8u, 1u, 512u, 4u, 0u, 0u, 0u};
    double best_ms = 0.0;
    if (int rc = time_of(best, best_ms)) return rc;
    const double default_ms = best_ms;
    auto sweep = [&](uint32_t PtBatchTuning::*knob, std::initializer_list<uint32_t> values) -> int {
        const PtBatchTuning base = best;
        for (uint32_t v : values) {
            if (base.*knob == v) continue;
            PtBatchTuning c = base;
            c.*knob = v;
            double ms = 0.0;
            if (int rc = time_of(c, ms)) return rc;
            if (ms < best_ms) {
                best_ms = ms;
                best = c;
            }
        }
        return PT_OK;
    };
    int rc = 0;
    if ((rc = sweep(&PtBatchTuning::persistent_blocks_per_sm, {3u, 2u})) ||
        (rc = sweep(&PtBatchTuning::stream_blocks_per_sm, {4u, 16u})) ||
        (rc = sweep(&PtBatchTuning::shade_threads, {256u})) ||
        (rc = sweep(&PtBatchTuning::camera_tile_w, {8u, 16u, 32u})) ||
        (rc = sweep(&PtBatchTuning::octant_grouping, {1u})) || (rc = sweep(&PtBatchTuning::use_graph, {0u})))
        return rc;
    if ((rc = pt_gpu_batch_set_tuning(ctx, &best))) return rc;
    ctx->b_tune_default_ms = default_ms;
    ctx->b_tune_best_ms = best_ms;
    if (chosen) *chosen = best;
    return PT_OK;
}

int pt_gpu_batch_tuning_gain(pt_gpu_ctx* ctx, double* default_ms, double* tuned_ms) {
    if (!ctx || !default_ms || !tuned_ms) return PT_ERR_INVALID;
    *default_ms = ctx->b_tune_default_ms;
    *tuned_ms = ctx->b_tune_best_ms;
    return PT_OK;
}

}  // extern "C"

// ===========================================================================
// Allocation-free render: pt_gpu_render_noalloc
//
// Some callers of this library must not allocate device memory while they
// render: an engine that reserved its whole device-memory budget up front and
// treats any later cudaMalloc as a budget violation, a real-time frame loop in
// which cudaMalloc/cudaFree can stall on an implicit device synchronisation,
// or a plugin hosted by an application whose own allocator accounts for every
// device byte.  For them this entry point renders with no allocation at all:
// the per-wave path state lives in one file-scope device array of fixed size,
// the caller passes its own accumulation buffer, and nothing here calls
// cudaMalloc, cudaFree or an allocating library routine.
//
// Limits and sharing rules:
//   - at most kNoAllocMaxPixels pixels per frame (256 x 256); larger frames are
//     rejected with PT_ERR_INVALID;
//   - the array (kNoAllocBytes, about 23.5 MiB) is held by every GPU that loads
//     the library until the process exits;
//   - every call on a device uses the same array and leaves its contents
//     behind; what must start at zero (queue counters, statistics) is cleared
//     by each call, the rest is written before it is read;
//   - calls that overlap on the same GPU (two contexts, or concurrent threads)
//     race on the array and must be serialised by the caller;
//   - the first call on a device resolves the array's device address with
//     cudaGetSymbolAddress (that device made current for the call); make this
//     first call before any stream capture.
// ===========================================================================
namespace {

constexpr uint32_t kNoAllocMaxPixels = 65536u;
constexpr size_t kNoAllocAlign = 256;
constexpr size_t align_up(size_t v) { return (v + kNoAllocAlign - 1) / kNoAllocAlign * kNoAllocAlign; }
constexpr size_t kNA_P = kNoAllocMaxPixels;
// 6 float4 path arrays, 5 float4 x 3 shadow slots, 7 u32 path arrays, 1 u32 x 3 shadow queue,
// the 16 u32 queue counters (the ring of DPaths::cnt), 4 u64 statistics
constexpr size_t kNoAllocBytes = 6 * align_up(16 * kNA_P) + 5 * align_up(16 * 3 * kNA_P) +
                                 7 * align_up(4 * kNA_P) + align_up(4 * 3 * kNA_P) + align_up(64) +
                                 align_up(32);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
constexpr int kNoAllocMaxDevices = 64;
unsigned char* g_noalloc_base[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on ctx's device (resolved once per device).
int noalloc_base(pt_gpu_ctx* ctx, unsigned char** out) {
    if (ctx->device < 0 || ctx->device >= kNoAllocMaxDevices)
        return set_err(ctx, PT_ERR_INVALID, "render_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_base[ctx->device]) {
        int prev = 0;
        cudaError_t e = cudaGetDevice(&prev);
        if (e == cudaSuccess) e = cudaSetDevice(ctx->device);
        void* p = nullptr;
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        cudaSetDevice(prev);
        if (e != cudaSuccess || !p)
            return set_err(ctx, PT_ERR_CUDA, std::string("render_noalloc: cudaGetSymbolAddress: ") +
                                                 cudaGetErrorString(e));
        g_noalloc_base[ctx->device] = static_cast<unsigned char*>(p);
    }
    *out = g_noalloc_base[ctx->device];
    return PT_OK;
}

}  // namespace

extern "C" int pt_gpu_render_noalloc(pt_gpu_ctx* ctx, const PtPushHead* head, const PtPathParams* prm,
                                     uint32_t width, uint32_t height, uint32_t frames, float* accum_device) {
    if (!ctx || !head || !prm || !accum_device) return PT_ERR_INVALID;
    if (width == 0 || height == 0) return set_err(ctx, PT_ERR_INVALID, "render_noalloc: empty frame");
    if (uint64_t(width) * height > kNoAllocMaxPixels)
        return set_err(ctx, PT_ERR_INVALID,
                       "render_noalloc: " + std::to_string(uint64_t(width) * height) +
                           " pixels exceed the static scratch limit of " + std::to_string(kNoAllocMaxPixels) +
                           " pixels per frame");
    if ((reinterpret_cast<uintptr_t>(accum_device) & 15u) != 0)
        return set_err(ctx, PT_ERR_INVALID, "render_noalloc: accumulation buffer must be 16-byte aligned");
    if (head->tlas_present) return set_err(ctx, PT_ERR_UNSUPPORTED, "render_noalloc: tlas_present has no CUDA path");
    if (int rc = check_light_tree(ctx, ctx, prm, "render_noalloc: ")) return rc;
    if (int rc = check_sdf(ctx, ctx, prm, "render_noalloc: ")) return rc;
    if (int rc = check_sky(ctx, ctx, head, prm, "render_noalloc: ")) return rc;
    if (head->prim_count != ctx->prim_count || prm->bvh_params[0] != ctx->linear_count ||
        (prm->bvh_params[1] != 0u && prm->bvh_params[1] != ctx->bvh_nodes))
        return set_err(ctx, PT_ERR_INVALID, "render_noalloc: prim_count / bvh_params disagree with the uploaded prims");
    if (prm->bvh_params[2] != 0u && prm->bvh_params[3] != 0u && prm->bvh_params[3] != ctx->tri_nodes)
        return set_err(ctx, PT_ERR_INVALID, "render_noalloc: bvh_params.w disagrees with the uploaded mesh BVH");
    if (prm->light_count > ctx->light_count)
        return set_err(ctx, PT_ERR_INVALID, "render_noalloc: light_count exceeds the uploaded lights");

    if (frames == 0) return PT_OK;
    unsigned char* base = nullptr;
    if (int rc = noalloc_base(ctx, &base)) return rc;

    // carve the path state out of the static array
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char* p = base + off;
        off += align_up(bytes);
        return p;
    };
    DPaths P{};
    P.ray_o = reinterpret_cast<float4*>(take(16 * kNA_P));
    P.ray_d = reinterpret_cast<float4*>(take(16 * kNA_P));
    P.thr = reinterpret_cast<float4*>(take(16 * kNA_P));
    P.rad = reinterpret_cast<float4*>(take(16 * kNA_P));
    P.fsum = reinterpret_cast<float4*>(take(16 * kNA_P));
    P.amb = reinterpret_cast<float4*>(take(16 * kNA_P));
    P.sh_o = reinterpret_cast<float4*>(take(16 * 3 * kNA_P));
    P.sh_d = reinterpret_cast<float4*>(take(16 * 3 * kNA_P));
    P.sh_pre = reinterpret_cast<float4*>(take(16 * 3 * kNA_P));
    P.sh_brdf = reinterpret_cast<float4*>(take(16 * 3 * kNA_P));
    P.sh_tr = reinterpret_cast<float4*>(take(16 * 3 * kNA_P));
    P.seed = reinterpret_cast<uint32_t*>(take(4 * kNA_P));
    P.state = reinterpret_cast<uint32_t*>(take(4 * kNA_P));
    P.hit_t = reinterpret_cast<float*>(take(4 * kNA_P));
    P.hit_id = reinterpret_cast<uint32_t*>(take(4 * kNA_P));
    P.shmask = reinterpret_cast<uint32_t*>(take(4 * kNA_P));
    P.q[0] = reinterpret_cast<uint32_t*>(take(4 * kNA_P));
    P.q[1] = reinterpret_cast<uint32_t*>(take(4 * kNA_P));
    P.sq = reinterpret_cast<uint32_t*>(take(4 * 3 * kNA_P));
    P.cnt = reinterpret_cast<uint32_t*>(take(64));   // the counter ring
    P.stat = reinterpret_cast<unsigned long long*>(take(32));
    P.wave = ctx->wave_vars.p;
    if (off > kNoAllocBytes) return set_err(ctx, PT_ERR_KERNEL, "render_noalloc: scratch layout overflow");

    DFrame F{};
    F.cam_pos = v3(head->pos_fovtan[0], head->pos_fovtan[1], head->pos_fovtan[2]);
    F.tanf = head->pos_fovtan[3];
    F.fwd = v3(head->fwd_aspect[0], head->fwd_aspect[1], head->fwd_aspect[2]);
    F.aspect = head->fwd_aspect[3];
    F.right = v3(head->right_xyz[0], head->right_xyz[1], head->right_xyz[2]);
    F.up = v3(head->up_xyz[0], head->up_xyz[1], head->up_xyz[2]);
    F.W = width;
    F.H = height;
    F.npix = width * height;
    F.spp = head->spp == 0u ? 1u : head->spp;
    F.maxb = head->max_bounces;
    F.denoiser = head->denoiser_enabled;
    F.jx = head->halton_jitter[0];
    F.jy = head->halton_jitter[1];
    F.env_present = head->env_map_present;
    F.env_intensity = head->env_intensity;
    F.env_total = head->env_total_luminance;
    F.kmax = int(prm->refract_budget);
    F.firefly = prm->firefly_clamp;
    F.mis = prm->mis_enabled;
    F.rr_start = prm->rr_start;
    F.light_count = prm->light_count;
    sky_of(F, prm);
    const DScene S = make_scene(ctx, prm);
    const bool persistent = S.use_wide && (S.a_wide || S.prim_count == S.wide_linear) &&
                            (S.t_wide || S.tri_enabled == 0u || S.tri_nodes == 0u);
    const int gpers = ctx->sm_count * 4;
    const int gtr = ctx->sm_count * kTransmitBlocks;
    const uint32_t fpw = std::max<uint32_t>(1u, std::min<uint32_t>(frames, kNoAllocMaxPixels / F.npix));
    float4* accum = reinterpret_cast<float4*>(accum_device);
    const bool proc = S.sdf_proc != 0u && ctx->sdf_proc_any;   // procedural SDF walker needed

    // work a failed earlier pt_gpu_render left on the side stream (it writes
    // the error word) finishes before this call clears it
    CK(cudaEventRecord(ctx->ev_join, ctx->side));
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
    CK(cudaMemsetAsync(P.stat, 0, 32, ctx->stream));
    CK(cudaMemsetAsync(ctx->err_word.p, 0, 4, ctx->stream));
    ctx->stats = PtStats{};
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    for (uint32_t f0 = 0; f0 < frames; f0 += fpw) {
        const uint32_t nf = std::min(fpw, frames - f0);
        const uint32_t npaths = nf * F.npix;
        F.nframes = nf;
        const int gp = (npaths + 255) / 256;
        k_set_wave<<<1, 1, 0, ctx->stream>>>(ctx->wave_vars.p, head->frame_index + f0, head->frame_index,
                                             f0 == 0 && head->reset_accum != 0u);
        k_init_wave<false><<<gp, 256, 0, ctx->stream>>>(F, P, Batch{}, npaths);
        ctx->stats.kernel_launches += 3;
        for (uint32_t s = 0; s < F.spp; ++s) {
            k_camera<false><<<gp, 256, 0, ctx->stream>>>(F, P, Batch{}, npaths, s);
            ctx->stats.kernel_launches += 2 + 3 * F.maxb;
            for (uint32_t b = 0; b < F.maxb; ++b) {
                const int qs = int(b & 1u);
                const DPaths Pb = bounce_paths(P, b);
                if (persistent) {
                    (proc ? k_closest<false, true> : k_closest<false, false>)<<<gpers, kThreads, 0, ctx->stream>>>(
                        S, Batch{}, P.q[qs], Pb.cnt, P.ray_o, P.ray_d, P.hit_t, P.hit_id, Pb.cnt + 2, P.stat);
                } else if (S.use_wide) {
                    k_extend<true><<<grid_for(ctx, npaths, 8), kThreads, 0, ctx->stream>>>(S, Pb, qs);
                } else {
                    k_extend<false><<<grid_for(ctx, npaths, 8), kThreads, 0, ctx->stream>>>(S, Pb, qs);
                }
                (proc ? k_shade<false, false, true> : k_shade<false, false, false>)
                    <<<grid_for(ctx, npaths, 4, kShadeThreads), kShadeThreads, 0, ctx->stream>>>(S, F, Pb, Batch{},
                                                                                              Adj{}, qs, b);
                if (persistent) {
                    (proc ? k_transmit<false, false, true> : k_transmit<false, false, false>)
                        <<<gtr, kThreads, 0, ctx->stream>>>(S, Batch{}, Pb, F.kmax, nullptr);
                } else if (S.use_wide) {
                    k_shadow<true><<<grid_for(ctx, 3 * size_t(npaths), 8), kThreads, 0, ctx->stream>>>(S, Pb, F.kmax);
                } else {
                    k_shadow<false><<<grid_for(ctx, 3 * size_t(npaths), 8), kThreads, 0, ctx->stream>>>(S, Pb, F.kmax);
                }
                ctx->stats.extend_launches++;
                ctx->stats.shadow_launches++;
            }
            k_finish<false, false><<<grid_for(ctx, npaths, 8), kThreads, 0, ctx->stream>>>(S, F, P, Batch{}, Adj{},
                                                                                           npaths, s, 0);
        }
        k_accumulate<<<(F.npix + 255) / 256, 256, 0, ctx->stream>>>(F, P, accum, nf, prm->accum_ema_alpha);
        ctx->stats.waves++;
        ctx->stats.paths += uint64_t(npaths) * F.spp;
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats.gpu_ms = ms;
    ctx->stats.frames = frames;
    unsigned long long st[4];
    uint32_t errw = 0;
    CK(cudaMemcpy(st, P.stat, sizeof(st), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&errw, ctx->err_word.p, 4, cudaMemcpyDeviceToHost));
    ctx->stats.extension_rays = st[0];
    ctx->stats.shadow_rays = st[1];
    if (errw) return set_err(ctx, PT_ERR_KERNEL, "render_noalloc: " + traversal_error(errw));
    return PT_OK;
}
