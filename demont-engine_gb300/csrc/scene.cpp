// Host-side scene builder: the reference engine's scene API and upload
// packing rules, restated in C++ so the GPU path is a drop-in for the
// reference's `pathtrace` dispatch.  See include/pt_scene.h for the API.
//
// Compiled with -ffp-contract=off: every float expression here must round
// exactly as written so that BVH boxes, centroids and packed records are
// bit-identical to what the reference builds from the same inputs.

#include "pt_scene.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <numbers>
#include <numeric>
#include <string>
#include <utility>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Binary centroid-median BVH builders.
//
// Same algorithm as the reference (src/renderer/AnalyticBvh.cpp:369-486,
// src/renderer/TriangleBvh.cpp:33-169): top-down, split the range at
// count/2 after std::nth_element on the widest centroid axis, leaf <= 4,
// left child then right child appended, left child index in left_first.
// std::nth_element is the C++ standard library's selection routine; calling
// it on the same keys in the same order reproduces the reference's
// permutation exactly, so the trees are bit-identical.
// ---------------------------------------------------------------------------
constexpr uint32_t kMaxLeafSize = 4;

inline void aabb_reset(float (&mn)[3], float (&mx)[3]) {
    const float inf = std::numeric_limits<float>::infinity();
    mn[0] = mn[1] = mn[2] = inf;
    mx[0] = mx[1] = mx[2] = -inf;
}

struct SphereItem {      // one finite analytic prim: center + bounding radius
    float center[3];
    float radius;
    uint32_t prim_id;
    float centroid[3];
};

struct TriItem {
    float aabb_min[3];
    float aabb_max[3];
    float centroid[3];
    uint32_t prim_id;
};

template <typename Item, typename BoxFn>
uint32_t build_recursive(std::vector<Item>& work, std::vector<PtBvhNode>& nodes,
                         uint32_t node_idx, uint32_t first, uint32_t count, BoxFn include_box) {
    float bn[3], bx[3];
    aabb_reset(bn, bx);
    for (uint32_t i = 0; i < count; ++i) include_box(bn, bx, work[first + i]);
    for (int a = 0; a < 3; ++a) {
        nodes[node_idx].aabb_min[a] = bn[a];
        nodes[node_idx].aabb_max[a] = bx[a];
    }
    if (count <= kMaxLeafSize) {
        nodes[node_idx].left_first = first;
        nodes[node_idx].count = count;
        return 1;
    }
    float cmn[3], cmx[3];
    aabb_reset(cmn, cmx);
    for (uint32_t i = 0; i < count; ++i) {
        const float* c = work[first + i].centroid;
        for (int a = 0; a < 3; ++a) {
            if (c[a] < cmn[a]) cmn[a] = c[a];
            if (c[a] > cmx[a]) cmx[a] = c[a];
        }
    }
    int axis = 0;
    float widest = cmx[0] - cmn[0];
    for (int a = 1; a < 3; ++a) {
        const float w = cmx[a] - cmn[a];
        if (w > widest) { widest = w; axis = a; }
    }
    if (widest > 0.0f) {
        Item* begin = work.data() + first;
        std::nth_element(begin, begin + count / 2, begin + count,
                         [axis](const Item& a, const Item& b) {
                             return a.centroid[axis] < b.centroid[axis];
                         });
    }
    const uint32_t left_count = count / 2;
    const uint32_t right_count = count - left_count;
    const uint32_t left_idx = static_cast<uint32_t>(nodes.size());
    nodes[node_idx].left_first = left_idx;
    nodes[node_idx].count = 0;
    nodes.push_back(PtBvhNode{});
    nodes.push_back(PtBvhNode{});
    uint32_t emitted = 1;
    emitted += build_recursive(work, nodes, left_idx, first, left_count, include_box);
    emitted += build_recursive(work, nodes, left_idx + 1, first + left_count, right_count, include_box);
    return emitted;
}

void build_sphere_bvh(const std::vector<SphereItem>& in, std::vector<PtBvhNode>& nodes,
                      std::vector<uint32_t>& perm) {
    nodes.clear();
    perm.clear();
    if (in.empty()) return;
    std::vector<SphereItem> work = in;
    for (auto& w : work) {
        w.centroid[0] = w.center[0];
        w.centroid[1] = w.center[1];
        w.centroid[2] = w.center[2];
    }
    nodes.reserve(2 * work.size());
    nodes.push_back(PtBvhNode{});
    build_recursive(work, nodes, 0, 0, static_cast<uint32_t>(work.size()),
                    [](float (&mn)[3], float (&mx)[3], const SphereItem& w) {
                        for (int i = 0; i < 3; ++i) {
                            if (w.center[i] - w.radius < mn[i]) mn[i] = w.center[i] - w.radius;
                            if (w.center[i] + w.radius > mx[i]) mx[i] = w.center[i] + w.radius;
                        }
                    });
    perm.reserve(work.size());
    for (const auto& w : work) perm.push_back(w.prim_id);
}

void build_tri_bvh(const float* pos, uint32_t nv, const uint32_t* idx, uint32_t n_index,
                   std::vector<PtBvhNode>& nodes, std::vector<uint32_t>& perm) {
    nodes.clear();
    perm.clear();
    if (n_index == 0 || (n_index % 3u) != 0u) return;
    const uint32_t nt = n_index / 3u;
    std::vector<TriItem> work;
    work.reserve(nt);
    for (uint32_t t = 0; t < nt; ++t) {
        const uint32_t i0 = idx[3u * t + 0u], i1 = idx[3u * t + 1u], i2 = idx[3u * t + 2u];
        if (i0 >= nv || i1 >= nv || i2 >= nv) continue;   // reference skips bad triangles
        const float* v0 = pos + 3u * i0;
        const float* v1 = pos + 3u * i1;
        const float* v2 = pos + 3u * i2;
        TriItem w{};
        for (int a = 0; a < 3; ++a) {
            w.aabb_min[a] = std::min(v0[a], std::min(v1[a], v2[a]));
            w.aabb_max[a] = std::max(v0[a], std::max(v1[a], v2[a]));
            w.centroid[a] = (v0[a] + v1[a] + v2[a]) * (1.0f / 3.0f);
        }
        w.prim_id = t;
        work.push_back(w);
    }
    if (work.empty()) return;
    nodes.reserve(2 * work.size());
    nodes.push_back(PtBvhNode{});
    build_recursive(work, nodes, 0, 0, static_cast<uint32_t>(work.size()),
                    [](float (&mn)[3], float (&mx)[3], const TriItem& w) {
                        for (int i = 0; i < 3; ++i) {
                            if (w.aabb_min[i] < mn[i]) mn[i] = w.aabb_min[i];
                            if (w.aabb_max[i] > mx[i]) mx[i] = w.aabb_max[i];
                        }
                    });
    perm.reserve(work.size());
    for (const auto& w : work) perm.push_back(w.prim_id);
}

// ---------------------------------------------------------------------------
// Env map: luminance-CDF builder (src/renderer/HdrImage.cpp:169-219).
// Row conditional = prefix of lum*sin(theta) in double, normalised per row;
// marginal = prefix of row sums normalised by the total, last entry forced
// to 1 when the total is positive.
// ---------------------------------------------------------------------------
double env_cdf(const float* rgb, uint32_t W, uint32_t H, const uint8_t* mask,
               float* marginal, float* conditional) {
    for (uint32_t v = 0; v < H; ++v) marginal[v] = 0.0f;
    double total = 0.0;
    for (uint32_t v = 0; v < H; ++v) {
        const double sin_theta = std::sin(std::numbers::pi * (double(v) + 0.5) / double(H));
        double row_sum = 0.0;
        for (uint32_t u = 0; u < W; ++u) {
            const size_t pi = size_t(v) * W + u;
            const float r = rgb[pi * 3 + 0], g = rgb[pi * 3 + 1], b = rgb[pi * 3 + 2];
            const float lum_raw = 0.2126f * r + 0.7152f * g + 0.0722f * b;
            const float lum = (mask && mask[pi]) ? 0.0f : lum_raw;
            row_sum += double(lum) * sin_theta;
            conditional[pi] = float(row_sum);
        }
        const double norm = (row_sum > 0.0) ? (1.0 / row_sum) : 0.0;
        for (uint32_t u = 0; u < W; ++u) {
            const size_t pi = size_t(v) * W + u;
            conditional[pi] = float(double(conditional[pi]) * norm);
        }
        marginal[v] = float(row_sum);
        total += row_sum;
    }
    const double norm = (total > 0.0) ? (1.0 / total) : 0.0;
    double prefix = 0.0;
    for (uint32_t v = 0; v < H; ++v) {
        prefix += marginal[v];
        marginal[v] = float(prefix * norm);
    }
    if (H > 0 && total > 0.0) marginal[H - 1] = 1.0f;
    return total;
}

struct HdriLight {
    float dir[3];
    float irradiance[3];
    float luminance;
    float pmf;
};

// HDRI bright-cluster extraction (src/engine/Engine.cpp:4371-4545): mark the
// top `top_frac` luminance pixels (threshold >= 5% of peak and >= 0.5), flood
// fill 4-connected clusters (u wraps), keep the <= 8 brightest clusters with
// >= 3 pixels as directional lights with a luminance pmf, and leave only the
// kept clusters masked out of the CDF.
void extract_hdri(const float* rgb, uint32_t W, uint32_t H, double top_frac,
                  std::vector<uint8_t>& light_mask, std::vector<HdriLight>& lights) {
    const size_t N = size_t(W) * H;
    light_mask.assign(N, 0u);
    lights.clear();
    std::vector<float> lums(N);
    float peak = 0.0f;
    for (size_t pi = 0; pi < N; ++pi) {
        const float lum = 0.2126f * rgb[pi * 3 + 0] + 0.7152f * rgb[pi * 3 + 1] +
                          0.0722f * rgb[pi * 3 + 2];
        lums[pi] = lum;
        if (lum > peak) peak = lum;
    }
    constexpr float kMinPeakLum = 0.5f;
    if (peak > kMinPeakLum) {
        if (top_frac < 1e-6) top_frac = 1e-6;
        if (top_frac > 0.5) top_frac = 0.5;
        const size_t k_idx = N - std::max<size_t>(1, size_t(double(N) * top_frac));
        std::vector<float> sorted = lums;
        std::nth_element(sorted.begin(), sorted.begin() + k_idx, sorted.end());
        float thresh = sorted[k_idx];
        if (thresh < 0.05f * peak) thresh = 0.05f * peak;
        if (thresh < kMinPeakLum) thresh = kMinPeakLum;
        for (size_t pi = 0; pi < N; ++pi)
            if (lums[pi] >= thresh) light_mask[pi] = 1u;
    }

    const double kTwoPiSq = 2.0 * std::numbers::pi * std::numbers::pi;
    const double dOmega_unit = kTwoPiSq / double(N);
    struct Acc {
        double cdir[3] = {0, 0, 0};
        double cw = 0.0;
        double flux[3] = {0, 0, 0};
        double lum = 0.0;
        uint32_t pixels = 0;
    };
    std::vector<Acc> clusters;
    std::vector<uint32_t> cid_of(N, 0u);
    std::vector<std::pair<uint32_t, uint32_t>> stack;
    for (uint32_t v0 = 0; v0 < H; ++v0) {
        for (uint32_t u0 = 0; u0 < W; ++u0) {
            const size_t p0 = size_t(v0) * W + u0;
            if (!light_mask[p0] || cid_of[p0] != 0u) continue;
            const uint32_t cid = uint32_t(clusters.size()) + 1u;
            clusters.emplace_back();
            stack.clear();
            stack.emplace_back(u0, v0);
            cid_of[p0] = cid;
            while (!stack.empty()) {
                auto [u, v] = stack.back();
                stack.pop_back();
                Acc& acc = clusters[cid - 1];
                const size_t pi = size_t(v) * W + u;
                const double theta = std::numbers::pi * (double(v) + 0.5) / double(H);
                const double sint = std::sin(theta), cost = std::cos(theta);
                const double dOmega = dOmega_unit * sint;
                const double phi = 2.0 * std::numbers::pi * (double(u) + 0.5) / double(W) -
                                   std::numbers::pi;
                const float r = rgb[pi * 3 + 0], g = rgb[pi * 3 + 1], b = rgb[pi * 3 + 2];
                const double lum = 0.2126 * r + 0.7152 * g + 0.0722 * b;
                const double wdir = lum * dOmega;
                acc.cdir[0] += (sint * std::cos(phi)) * wdir;
                acc.cdir[1] += cost * wdir;
                acc.cdir[2] += (sint * std::sin(phi)) * wdir;
                acc.cw += wdir;
                acc.flux[0] += double(r) * dOmega;
                acc.flux[1] += double(g) * dOmega;
                acc.flux[2] += double(b) * dOmega;
                acc.lum += lum * dOmega;
                acc.pixels += 1u;
                const uint32_t um = (u == 0u) ? (W - 1u) : (u - 1u);
                const uint32_t up = (u + 1u >= W) ? 0u : (u + 1u);
                auto try_push = [&](uint32_t uu, uint32_t vv) {
                    const size_t pp = size_t(vv) * W + uu;
                    if (light_mask[pp] && cid_of[pp] == 0u) {
                        cid_of[pp] = cid;
                        stack.emplace_back(uu, vv);
                    }
                };
                try_push(um, v);
                try_push(up, v);
                if (v > 0) try_push(u, v - 1u);
                if (v + 1u < H) try_push(u, v + 1u);
            }
        }
    }
    std::vector<uint32_t> order(clusters.size());
    std::iota(order.begin(), order.end(), 0u);
    std::sort(order.begin(), order.end(),
              [&](uint32_t a, uint32_t b) { return clusters[a].lum > clusters[b].lum; });
    std::vector<uint8_t> keep(clusters.size() + 1u, 0u);
    double total_lum = 0.0;
    for (uint32_t i : order) {
        if (lights.size() >= 8) break;
        const Acc& c = clusters[i];
        if (c.pixels < 3u || c.cw <= 0.0) continue;
        keep[i + 1u] = 1u;
        HdriLight L{};
        // normalize in double as v * (1 / sqrt(dot(v, v)))
        const double d2 = (c.cdir[0] * c.cdir[0] + c.cdir[1] * c.cdir[1]) + c.cdir[2] * c.cdir[2];
        const double inv = 1.0 / std::sqrt(d2);
        for (int a = 0; a < 3; ++a) {
            L.dir[a] = float(c.cdir[a] * inv);
            L.irradiance[a] = float(c.flux[a]);
        }
        L.luminance = float(c.lum);
        total_lum += c.lum;
        lights.push_back(L);
    }
    if (total_lum > 0.0) {
        const float inv_total = float(1.0 / total_lum);
        for (auto& L : lights) L.pmf = L.luminance * inv_total;
    }
    for (size_t pi = 0; pi < N; ++pi) {
        const uint32_t c = cid_of[pi];
        if (c != 0u && !keep[c]) light_mask[pi] = 0u;
    }
}

// ---------------------------------------------------------------------------
// PCG32 (O'Neill 2014, pcg32_random_r / pcg32_srandom_r) for the synthetic
// scene generators.
// ---------------------------------------------------------------------------
struct Pcg32 {
    uint64_t state = 0, inc = 1;
    Pcg32(uint64_t initstate, uint64_t initseq) {
        inc = (initseq << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
    uint32_t next() {
        const uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        const uint32_t xorshifted = uint32_t(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = uint32_t(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((0u - rot) & 31u));
    }
    float unit() { return float(next() >> 8) * (1.0f / 16777216.0f); }
    float range(float lo, float hi) { return lo + (hi - lo) * unit(); }
    double gauss() {   // Box-Muller, double precision
        double u1 = (double(next() >> 8) + 0.5) * (1.0 / 16777216.0);
        double u2 = double(next() >> 8) * (1.0 / 16777216.0);
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * std::numbers::pi * u2);
    }
};

// Integer lattice hash for value noise (Wang-style mix), in [0, 1).
inline float lattice(int32_t x, int32_t y, int32_t z, uint32_t seed) {
    uint32_t h = uint32_t(x) * 0x8da6b343u ^ uint32_t(y) * 0xd8163841u ^ uint32_t(z) * 0xcb1ab31fu ^ seed;
    h ^= h >> 16; h *= 0x7feb352du; h ^= h >> 15; h *= 0x846ca68bu; h ^= h >> 16;
    return float(h >> 8) * (1.0f / 16777216.0f);
}

float value_noise(float px, float py, float pz, uint32_t seed) {
    const float fx = std::floor(px), fy = std::floor(py), fz = std::floor(pz);
    const int32_t ix = int32_t(fx), iy = int32_t(fy), iz = int32_t(fz);
    auto fade = [](float t) { return t * t * (3.0f - 2.0f * t); };
    const float tx = fade(px - fx), ty = fade(py - fy), tz = fade(pz - fz);
    float c[2][2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int d = 0; d < 2; ++d) c[a][b][d] = lattice(ix + a, iy + b, iz + d, seed);
    auto lerp = [](float a, float b, float t) { return a + t * (b - a); };
    const float x00 = lerp(c[0][0][0], c[1][0][0], tx), x10 = lerp(c[0][1][0], c[1][1][0], tx);
    const float x01 = lerp(c[0][0][1], c[1][0][1], tx), x11 = lerp(c[0][1][1], c[1][1][1], tx);
    return lerp(lerp(x00, x10, ty), lerp(x01, x11, ty), tz);
}

// ---------------------------------------------------------------------------
// Scene state
// ---------------------------------------------------------------------------
struct Prim {
    uint8_t type = 0;       // 0 sphere, 1 plane
    uint8_t material = 0;
    float pos[3] = {0, 0, 0};
    float radius_or_d = 0.5f;
    float albedo[3] = {1, 1, 1};
    float roughness = 0.0f;
    float ior = 1.5f;
    float prev[3] = {0, 0, 0};
    float emission[3] = {0, 0, 0};
    float orient[4] = {0, 0, 0, 1};
    uint32_t tex[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
    uint32_t mat_id = 0xFFFFFFFFu;   // extension: material-table row
};

struct Light {
    uint32_t type = 0;      // 0 point, 1 spot, 2 sphere, 3 quad
    float pos[3] = {0, 0, 0};
    float radius = 0.0f;
    float intensity[3] = {1, 1, 1};
    float dir[3] = {0, -1, 0};
    float cos_outer = 0.0f;
    float cos_inner = 0.0f;
    float u_vec[3] = {0, 0, 0};
    float v_half = 0.0f;
    float orient[4] = {0, 0, 0, 1};
};

struct SdfNodeH {
    uint32_t op = 0, shape = 0, a = 0, b = 0;
    float params[4] = {0, 0, 0, 0};
    float center[3] = {0, 0, 0};
};
struct SdfClusterH {
    SdfNodeH nodes[8];
    uint32_t count = 0, material = 0;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    float albedo[3] = {0.7f, 0.7f, 0.7f};
    float roughness = 0.0f, ior = 1.5f;
};

struct CVar {
    const char* name;
    double value;
};

}  // namespace

struct pt_scene {
    std::string err;
    std::map<uint32_t, Prim> prims;
    std::map<uint32_t, Light> lights;
    std::vector<float> mesh_pos;
    std::vector<uint32_t> mesh_idx;
    std::vector<uint32_t> mesh_mat;
    bool mesh_has_mat = false;
    std::vector<float> materials;
    std::vector<float> env_rgb;
    uint32_t env_w = 0, env_h = 0;
    bool env_present = false;
    std::vector<float> moon_rgba;
    uint32_t moon_w = 0, moon_h = 0;
    std::map<uint32_t, SdfClusterH> sdf;
    std::vector<float> packed_sdf;
    float cam_pos[3] = {0.0f, 1.5f, 4.0f};
    float cam_yaw = 0.0f, cam_pitch = -0.20f, cam_fov = 60.0f;
    std::vector<CVar> cvars = {
        {"r_max_bounces", 8},        {"r_spp", 1},
        {"r_mis", 1},                {"r_firefly_clamp", 10},
        {"r_caustics", 1},           {"r_refract_bounces", 4},
        {"r_env_intensity", 1},      {"r_accum_ema_alpha", 0},
        {"r_analytic_bvh_threshold", 16},
        {"r_hdri_extract_percentile", 0.005},
        {"r_light_tree", 1},         {"r_rr_start", 2},
        {"r_denoiser", 0},
        {"r_sun_elevation", 30},     {"r_sun_azimuth", 135},
        {"r_sun_size", 1},           {"r_sun_disc_brightness", 1},
        {"r_sun_horizon_flatten", 1},
        {"r_moon_size", 1},          {"r_moon_disc_brightness", 0.7},
        {"r_sky_mode", 1},           {"r_show_stars", 0},
        {"r_planet_radius", 6378137.0},
        {"r_exposure", 1.5},         {"r_tonemap_op", 0},
        {"r_sdf_max_iters", 128},    {"r_sdf_epsilon", 1e-4},
        {"r_sdf_fractal_power", 8},  {"r_sdf_fractal_iters", 12},
        {"r_sdf_de_eps_scale", 1},   {"r_sdf_normal_mode", 0},
        {"r_sdf_displace_octaves", 4}, {"r_sdf_procedural_ops", 0},
        {"r_capture_seed", 0},
        {"app_window_width", 0},     {"app_window_height", 0},
    };

    // packed state
    bool dirty_prims = true, dirty_mesh = true, dirty_lights = true, dirty_env = true;
    std::vector<float> packed_prims;
    std::vector<uint32_t> packed_prim_mats;
    bool any_prim_mat = false;
    uint32_t linear_count = 0;
    std::vector<PtBvhNode> bvh;
    std::vector<PtBvhNode> tri_bvh;
    std::vector<uint32_t> tri_perm;
    std::vector<float> packed_lights;
    std::vector<PtLightTreeNode> light_tree;
    std::vector<float> env_rgba, env_marg, env_cond;
    double env_total = 0.0;
    std::vector<HdriLight> hdri;
    float hdri_dir[32] = {0};
    float hdri_col[32] = {0};

    double cvar(const char* n) const {
        for (const auto& c : cvars)
            if (std::strcmp(c.name, n) == 0) return c.value;
        return 0.0;
    }
};

namespace {

int fail(pt_scene* s, const std::string& m) {
    if (s) s->err = m;
    return PT_ERR_INVALID;
}

void pack_prims(pt_scene* s) {
    struct Ref { const Prim* p; uint32_t id; };
    std::vector<Ref> inf, fin;
    for (const auto& [id, p] : s->prims) {
        if (p.type == 1u) inf.push_back({&p, id});
        else fin.push_back({&p, id});
    }
    uint32_t threshold = 16u;
    {
        const double t = s->cvar("r_analytic_bvh_threshold");
        if (t > 0) threshold = uint32_t(t);
    }
    std::vector<uint32_t> order(fin.size());
    std::iota(order.begin(), order.end(), 0u);
    s->bvh.clear();
    if (!fin.empty() && uint32_t(fin.size()) >= threshold) {
        std::vector<SphereItem> items(fin.size());
        for (uint32_t i = 0; i < fin.size(); ++i) {
            const Prim& p = *fin[i].p;
            items[i] = SphereItem{{p.pos[0], p.pos[1], p.pos[2]}, p.radius_or_d, i, {0, 0, 0}};
        }
        build_sphere_bvh(items, s->bvh, order);
    }
    s->linear_count = uint32_t(inf.size());
    const size_t count = s->prims.size();
    s->packed_prims.assign(count * 28, 0.0f);
    auto pack = [&](size_t out, const Prim& p, uint32_t id) {
        float* o = s->packed_prims.data() + out * 28;
        o[0] = p.pos[0]; o[1] = p.pos[1]; o[2] = p.pos[2]; o[3] = p.radius_or_d;
        o[4] = p.albedo[0]; o[5] = p.albedo[1]; o[6] = p.albedo[2]; o[7] = p.roughness;
        o[8] = float(p.type); o[9] = float(p.material); o[10] = p.ior;
        std::memcpy(&o[11], &id, 4);
        o[12] = p.prev[0]; o[13] = p.prev[1]; o[14] = p.prev[2]; o[15] = 0.0f;
        o[16] = p.emission[0]; o[17] = p.emission[1]; o[18] = p.emission[2]; o[19] = 0.0f;
        o[20] = p.orient[0]; o[21] = p.orient[1]; o[22] = p.orient[2]; o[23] = p.orient[3];
        std::memcpy(&o[24], p.tex, 16);
    };
    for (size_t i = 0; i < inf.size(); ++i) pack(i, *inf[i].p, inf[i].id);
    for (size_t i = 0; i < order.size(); ++i) pack(s->linear_count + i, *fin[order[i]].p, fin[order[i]].id);
    s->packed_prim_mats.assign(count, 0xFFFFFFFFu);
    s->any_prim_mat = false;
    for (size_t i = 0; i < inf.size(); ++i) s->packed_prim_mats[i] = inf[i].p->mat_id;
    for (size_t i = 0; i < order.size(); ++i) s->packed_prim_mats[s->linear_count + i] = fin[order[i]].p->mat_id;
    for (uint32_t m : s->packed_prim_mats) s->any_prim_mat = s->any_prim_mat || (m != 0xFFFFFFFFu);
    s->dirty_prims = false;
}

void pack_mesh(pt_scene* s) {
    build_tri_bvh(s->mesh_pos.data(), uint32_t(s->mesh_pos.size() / 3), s->mesh_idx.data(),
                  uint32_t(s->mesh_idx.size()), s->tri_bvh, s->tri_perm);
    s->dirty_mesh = false;
}

// ---- light tree (src/renderer/LightTree.cpp:BuildLightTree, restated) ----
struct LtLeaf {
    float lo[3], hi[3], axis[3];
    float cos_half;
    float power;       // scalar luminance x emitter area
    uint32_t light;
};

LtLeaf lt_leaf(const PtLightInput& L, uint32_t id) {
    LtLeaf s{};
    s.light = id;
    if (L.type == 0u || L.type == 1u) {          // point, spot: a 1 mm box
        for (int k = 0; k < 3; ++k) {
            s.lo[k] = L.pos[k] - 1e-3f;
            s.hi[k] = L.pos[k] + 1e-3f;
        }
    } else if (L.type == 2u) {                    // sphere
        const float r = std::max(L.radius, 1e-3f);
        for (int k = 0; k < 3; ++k) {
            s.lo[k] = L.pos[k] - r;
            s.hi[k] = L.pos[k] + r;
        }
    } else {                                      // quad: |u| + v_half per axis
        const float vh = std::fabs(L.v_half);
        for (int k = 0; k < 3; ++k) {
            const float ext = std::fabs(L.u_vec[k]) + vh;
            s.lo[k] = L.pos[k] - ext;
            s.hi[k] = L.pos[k] + ext;
        }
    }
    if (L.type == 0u || L.type == 2u) {           // emits in every direction
        s.axis[0] = 0.0f; s.axis[1] = 1.0f; s.axis[2] = 0.0f;
        s.cos_half = -1.0f;
    } else {
        for (int k = 0; k < 3; ++k) s.axis[k] = L.dir[k];
        s.cos_half = (L.type == 1u) ? L.cos_outer : 0.0f;   // quads: the front hemisphere
    }
    float lum = 0.2126f * L.intensity[0] + 0.7152f * L.intensity[1] + 0.0722f * L.intensity[2];
    if (L.type == 2u) {
        const float r = std::max(L.radius, 1e-3f);
        lum *= 4.0f * 3.14159265358979f * r * r;
    } else if (L.type == 3u) {
        const float ul = std::sqrt(L.u_vec[0] * L.u_vec[0] + L.u_vec[1] * L.u_vec[1] + L.u_vec[2] * L.u_vec[2]);
        lum *= 4.0f * ul * std::fabs(L.v_half);
    }
    s.power = lum;
    return s;
}

// smallest cone holding both cones (axis, cosine of the half angle; -1 = sphere)
void lt_cone_union(const float* a, float ca, const float* b, float cb, float* out, float& cout) {
    auto keep = [&](const float* ax, float c) {
        out[0] = ax[0]; out[1] = ax[1]; out[2] = ax[2];
        cout = c;
    };
    if (ca <= -0.999f || cb <= -0.999f) return keep(a, -1.0f);
    float d = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    d = std::min(std::max(d, -1.0f), 1.0f);
    const float td = std::acos(d);
    const float ta = std::acos(std::clamp(ca, -1.0f, 1.0f));
    const float tb = std::acos(std::clamp(cb, -1.0f, 1.0f));
    if (td + tb <= ta) return keep(a, ca);
    if (td + ta <= tb) return keep(b, cb);
    const float tc = 0.5f * (ta + tb + td);
    if (tc >= 3.14159265358979f) return keep(a, -1.0f);
    cout = std::cos(tc);
    const float rot = tc - ta;
    const float cr = std::cos(rot), sr = std::sin(rot);
    float perp[3] = {b[0] - d * a[0], b[1] - d * a[1], b[2] - d * a[2]};
    const float pl = std::sqrt(perp[0] * perp[0] + perp[1] * perp[1] + perp[2] * perp[2]);
    if (!(pl > 1e-6f)) {
        out[0] = a[0]; out[1] = a[1]; out[2] = a[2];
        if (d < 0.0f) cout = -1.0f;
        return;
    }
    const float inv = 1.0f / pl;
    for (float& v : perp) v *= inv;
    for (int k = 0; k < 3; ++k) out[k] = cr * a[k] + sr * perp[k];
    const float al = std::sqrt(out[0] * out[0] + out[1] * out[1] + out[2] * out[2]);
    if (al > 1e-6f) {
        const float ia = 1.0f / al;
        for (int k = 0; k < 3; ++k) out[k] *= ia;
    }
}

void lt_build(std::vector<LtLeaf>& lv, std::vector<PtLightTreeNode>& nodes, uint32_t b, uint32_t e, uint32_t dst) {
    const uint32_t n = e - b;
    if (n == 1) {
        PtLightTreeNode& o = nodes[dst];
        const LtLeaf& l = lv[b];
        for (int k = 0; k < 3; ++k) {
            o.aabb_min[k] = l.lo[k];
            o.aabb_max[k] = l.hi[k];
            o.cone_axis[k] = l.axis[k];
        }
        o.cone_cos_half = l.cos_half;
        o.intensity = l.power;
        o.left_first = l.light;
        o.count = 1u;
        return;
    }
    float cmin[3], cmax[3];
    for (int k = 0; k < 3; ++k) {
        cmin[k] = std::numeric_limits<float>::infinity();
        cmax[k] = -std::numeric_limits<float>::infinity();
    }
    for (uint32_t i = b; i < e; ++i)
        for (int k = 0; k < 3; ++k) {
            const float c = 0.5f * (lv[i].lo[k] + lv[i].hi[k]);
            cmin[k] = std::min(cmin[k], c);
            cmax[k] = std::max(cmax[k], c);
        }
    int axis = 0;
    float widest = cmax[0] - cmin[0];
    for (int k = 1; k < 3; ++k)
        if (cmax[k] - cmin[k] > widest) {
            widest = cmax[k] - cmin[k];
            axis = k;
        }
    const uint32_t mid = b + n / 2;
    if (!(widest < 1e-6f))
        std::nth_element(lv.begin() + b, lv.begin() + mid, lv.begin() + e, [axis](const LtLeaf& x, const LtLeaf& y) {
            return 0.5f * (x.lo[axis] + x.hi[axis]) < 0.5f * (y.lo[axis] + y.hi[axis]);
        });
    const uint32_t left = uint32_t(nodes.size());
    nodes.emplace_back();
    nodes.emplace_back();
    lt_build(lv, nodes, b, mid, left);
    lt_build(lv, nodes, mid, e, left + 1u);
    PtLightTreeNode& o = nodes[dst];
    const PtLightTreeNode& l = nodes[left];
    const PtLightTreeNode& r = nodes[left + 1u];
    for (int k = 0; k < 3; ++k) {
        o.aabb_min[k] = std::min(l.aabb_min[k], r.aabb_min[k]);
        o.aabb_max[k] = std::max(l.aabb_max[k], r.aabb_max[k]);
    }
    o.intensity = l.intensity + r.intensity;
    lt_cone_union(l.cone_axis, l.cone_cos_half, r.cone_axis, r.cone_cos_half, o.cone_axis, o.cone_cos_half);
    o.left_first = left;
    o.count = 0u;
}

void light_tree_of(const std::vector<PtLightInput>& in, std::vector<PtLightTreeNode>& nodes) {
    nodes.clear();
    if (in.empty()) return;
    std::vector<LtLeaf> lv;
    lv.reserve(in.size());
    for (uint32_t i = 0; i < in.size(); ++i) lv.push_back(lt_leaf(in[i], i));
    nodes.reserve(2 * in.size());
    nodes.emplace_back();
    lt_build(lv, nodes, 0u, uint32_t(lv.size()), 0u);
}

// rotate v by the unit quaternion q (xyzw), in the engine's operation order
void quat_rot_host(const float* q, const float* v, float* out) {
    const float cx = q[1] * v[2] - q[2] * v[1] + q[3] * v[0];
    const float cy = q[2] * v[0] - q[0] * v[2] + q[3] * v[1];
    const float cz = q[0] * v[1] - q[1] * v[0] + q[3] * v[2];
    out[0] = v[0] + 2.0f * (q[1] * cz - q[2] * cy);
    out[1] = v[1] + 2.0f * (q[2] * cx - q[0] * cz);
    out[2] = v[2] + 2.0f * (q[0] * cy - q[1] * cx);
}

void pack_lights(pt_scene* s) {
    std::vector<PtLightInput> in;
    in.reserve(s->lights.size());
    for (const auto& [id, L] : s->lights) {
        PtLightInput li{};
        li.type = L.type;
        quat_rot_host(L.orient, L.dir, li.dir);
        quat_rot_host(L.orient, L.u_vec, li.u_vec);
        for (int k = 0; k < 3; ++k) {
            li.pos[k] = L.pos[k];
            li.intensity[k] = L.intensity[k];
        }
        li.radius = L.radius;
        li.cos_outer = L.cos_outer;
        li.v_half = L.v_half;
        in.push_back(li);
    }
    light_tree_of(in, s->light_tree);
    s->packed_lights.assign(s->lights.size() * 20, 0.0f);
    size_t i = 0;
    for (const auto& [id, L] : s->lights) {
        float* o = s->packed_lights.data() + i * 20;
        o[0] = L.pos[0]; o[1] = L.pos[1]; o[2] = L.pos[2]; o[3] = L.radius;
        o[4] = L.intensity[0]; o[5] = L.intensity[1]; o[6] = L.intensity[2]; o[7] = float(L.type);
        o[8] = L.dir[0]; o[9] = L.dir[1]; o[10] = L.dir[2]; o[11] = L.cos_outer;
        o[12] = (L.type == 1u) ? L.cos_inner : L.u_vec[0];
        o[13] = L.u_vec[1]; o[14] = L.u_vec[2]; o[15] = L.v_half;
        o[16] = L.orient[0]; o[17] = L.orient[1]; o[18] = L.orient[2]; o[19] = L.orient[3];
        ++i;
    }
    s->dirty_lights = false;
}

void pack_env(pt_scene* s) {
    s->env_rgba.clear();
    s->env_marg.clear();
    s->env_cond.clear();
    s->hdri.clear();
    s->env_total = 0.0;
    std::memset(s->hdri_dir, 0, sizeof(s->hdri_dir));
    std::memset(s->hdri_col, 0, sizeof(s->hdri_col));
    if (s->env_present) {
        const uint32_t W = s->env_w, H = s->env_h;
        std::vector<uint8_t> mask;
        extract_hdri(s->env_rgb.data(), W, H, s->cvar("r_hdri_extract_percentile"), mask, s->hdri);
        s->env_marg.resize(H);
        s->env_cond.resize(size_t(W) * H);
        s->env_total = env_cdf(s->env_rgb.data(), W, H, mask.data(), s->env_marg.data(),
                               s->env_cond.data());
        s->env_rgba.resize(size_t(W) * H * 4);
        for (size_t pi = 0; pi < size_t(W) * H; ++pi) {
            s->env_rgba[pi * 4 + 0] = s->env_rgb[pi * 3 + 0];
            s->env_rgba[pi * 4 + 1] = s->env_rgb[pi * 3 + 1];
            s->env_rgba[pi * 4 + 2] = s->env_rgb[pi * 3 + 2];
            s->env_rgba[pi * 4 + 3] = 1.0f;
        }
        for (size_t i = 0; i < s->hdri.size(); ++i) {
            const HdriLight& L = s->hdri[i];
            s->hdri_dir[i * 4 + 0] = L.dir[0]; s->hdri_dir[i * 4 + 1] = L.dir[1];
            s->hdri_dir[i * 4 + 2] = L.dir[2]; s->hdri_dir[i * 4 + 3] = L.pmf;
            s->hdri_col[i * 4 + 0] = L.irradiance[0]; s->hdri_col[i * 4 + 1] = L.irradiance[1];
            s->hdri_col[i * 4 + 2] = L.irradiance[2]; s->hdri_col[i * 4 + 3] = 0.0f;
        }
    }
    s->dirty_env = false;
}

// ---------------------------------------------------------------------------
// Synthetic scenes
// ---------------------------------------------------------------------------
struct MatDraw { int type; float albedo[3]; float rough; float ior; };

MatDraw draw_material(Pcg32& rng) {
    MatDraw m{};
    const uint32_t k = std::min<uint32_t>(uint32_t(rng.unit() * 3.0f), 2u);
    m.type = int(k);
    m.rough = 0.0f;
    m.ior = 1.5f;
    if (k == 0) {
        for (int a = 0; a < 3; ++a) m.albedo[a] = rng.range(0.05f, 0.95f);
    } else if (k == 1) {
        for (int a = 0; a < 3; ++a) m.albedo[a] = rng.range(0.5f, 1.0f);
        m.rough = rng.range(0.0f, 0.3f);
    } else {
        m.albedo[0] = m.albedo[1] = m.albedo[2] = 1.0f;
        m.ior = rng.range(1.3f, 1.7f);
    }
    return m;
}

void add_box(std::vector<float>& pos, std::vector<uint32_t>& idx, std::vector<uint32_t>& mat,
             const float c[3], const float h[3], uint32_t mat_id) {
    const uint32_t base = uint32_t(pos.size() / 3);
    for (int k = 0; k < 8; ++k) {
        pos.push_back(c[0] + ((k & 1) ? h[0] : -h[0]));
        pos.push_back(c[1] + ((k & 2) ? h[1] : -h[1]));
        pos.push_back(c[2] + ((k & 4) ? h[2] : -h[2]));
    }
    static const uint32_t faces[12][3] = {
        {0, 2, 1}, {1, 2, 3}, {4, 5, 6}, {5, 7, 6},   // -z, +z
        {0, 1, 4}, {1, 5, 4}, {2, 6, 3}, {3, 6, 7},   // -y, +y
        {0, 4, 2}, {2, 4, 6}, {1, 3, 5}, {3, 7, 5},   // -x, +x
    };
    for (const auto& f : faces) {
        idx.push_back(base + f[0]);
        idx.push_back(base + f[1]);
        idx.push_back(base + f[2]);
        mat.push_back(mat_id);
    }
}

// Geodesic icosphere of frequency nu with shared vertices (10 nu^2 + 2 of them,
// 20 nu^2 triangles), radially displaced by 3-octave value noise.
void add_icosphere(std::vector<float>& pos, std::vector<uint32_t>& idx, std::vector<uint32_t>& mat,
                   const float c[3], float radius, uint32_t nu, float amp, uint32_t noise_seed,
                   uint32_t mat_id) {
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    const double V[12][3] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0},
                             {0, -1, t}, {0, 1, t}, {0, -1, -t}, {0, 1, -t},
                             {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    static const int F[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11},
                                 {1, 5, 9}, {5, 11, 4}, {11, 10, 2}, {10, 7, 6}, {7, 1, 8},
                                 {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8}, {3, 8, 9},
                                 {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    const uint32_t base = uint32_t(pos.size() / 3);
    std::vector<std::array<double, 3>> dirs;
    auto emit = [&](double x, double y, double z) {
        const double l = std::sqrt(x * x + y * y + z * z);
        dirs.push_back({x / l, y / l, z / l});
        return uint32_t(dirs.size() - 1);
    };
    for (int i = 0; i < 12; ++i) emit(V[i][0], V[i][1], V[i][2]);
    std::map<std::pair<int, int>, uint32_t> edge_start;   // (lo, hi) -> first interior point
    auto edge_point = [&](int a, int b, uint32_t k) -> uint32_t {   // point k of nu along a->b
        if (k == 0) return uint32_t(a);
        if (k == nu) return uint32_t(b);
        const int lo = std::min(a, b), hi = std::max(a, b);
        auto it = edge_start.find({lo, hi});
        if (it == edge_start.end()) {
            const uint32_t first = uint32_t(dirs.size());
            for (uint32_t j = 1; j < nu; ++j) {
                const double w = double(j) / double(nu);
                emit(V[lo][0] * (1 - w) + V[hi][0] * w, V[lo][1] * (1 - w) + V[hi][1] * w,
                     V[lo][2] * (1 - w) + V[hi][2] * w);
            }
            it = edge_start.emplace(std::make_pair(lo, hi), first).first;
        }
        const uint32_t j = (a == lo) ? k : nu - k;
        return it->second + (j - 1);
    };
    for (const auto& f : F) {
        const int A = f[0], B = f[1], C = f[2];
        // grid point (i, j): i steps along A->B, j along A->C, i + j <= nu
        std::vector<uint32_t> grid((nu + 1) * (nu + 1), 0u);
        for (uint32_t i = 0; i <= nu; ++i) {
            for (uint32_t j = 0; i + j <= nu; ++j) {
                uint32_t id;
                if (j == 0) id = edge_point(A, B, i);
                else if (i == 0) id = edge_point(A, C, j);
                else if (i + j == nu) id = edge_point(B, C, j);
                else {
                    const double wa = double(nu - i - j) / nu, wb = double(i) / nu, wc = double(j) / nu;
                    id = emit(V[A][0] * wa + V[B][0] * wb + V[C][0] * wc,
                              V[A][1] * wa + V[B][1] * wb + V[C][1] * wc,
                              V[A][2] * wa + V[B][2] * wb + V[C][2] * wc);
                }
                grid[i * (nu + 1) + j] = id;
            }
        }
        for (uint32_t i = 0; i < nu; ++i) {
            for (uint32_t j = 0; i + j < nu; ++j) {
                const uint32_t p00 = grid[i * (nu + 1) + j], p10 = grid[(i + 1) * (nu + 1) + j],
                               p01 = grid[i * (nu + 1) + j + 1];
                idx.push_back(base + p00); idx.push_back(base + p10); idx.push_back(base + p01);
                mat.push_back(mat_id);
                if (i + j + 1 < nu) {
                    const uint32_t p11 = grid[(i + 1) * (nu + 1) + j + 1];
                    idx.push_back(base + p10); idx.push_back(base + p11); idx.push_back(base + p01);
                    mat.push_back(mat_id);
                }
            }
        }
    }
    for (const auto& d : dirs) {
        const float px = float(d[0]) * 2.0f, py = float(d[1]) * 2.0f, pz = float(d[2]) * 2.0f;
        const float n = (value_noise(px, py, pz, noise_seed) +
                         0.5f * value_noise(2 * px, 2 * py, 2 * pz, noise_seed + 1) +
                         0.25f * value_noise(4 * px, 4 * py, 4 * pz, noise_seed + 2)) / 1.75f;
        const float r = radius * (1.0f + amp * (2.0f * n - 1.0f));
        pos.push_back(c[0] + float(d[0]) * r);
        pos.push_back(c[1] + float(d[1]) * r);
        pos.push_back(c[2] + float(d[2]) * r);
    }
}

void push_material(std::vector<float>& mats, const MatDraw& m) {
    const float rec[12] = {m.albedo[0], m.albedo[1], m.albedo[2], m.rough, 0, 0, 0, m.ior,
                           float(m.type), 0, 0, 0};
    mats.insert(mats.end(), rec, rec + 12);
}

void set_cv(pt_scene* s, const char* n, double v) { pt_scene_set_cvar(s, n, v); }

void synth_c0(pt_scene* s, uint64_t seed, double scale) {
    Pcg32 rng(0x5EEDull + 0ull, seed);
    const uint32_t n_spheres = std::max<uint32_t>(1, uint32_t(std::lround(64 * scale)));
    for (uint32_t i = 0; i < n_spheres; ++i) {
        const float cx = rng.range(-10, 10), cy = rng.range(-10, 10), cz = rng.range(-10, 10);
        const float r = float(0.2 * std::pow(10.0, double(rng.unit())));
        const MatDraw m = draw_material(rng);
        pt_scene_prim_sphere(s, 1 + i, cx, cy, cz, r, m.type, m.albedo[0], m.albedo[1], m.albedo[2],
                             m.rough, m.ior);
    }
    std::vector<float> pos, mats;
    std::vector<uint32_t> idx, mid;
    for (uint32_t b = 0; b < 4; ++b) {
        const float h[3] = {rng.range(0.5f, 3.0f), rng.range(0.5f, 3.0f), rng.range(0.5f, 3.0f)};
        const float c[3] = {rng.range(-10, 10), rng.range(-10, 10), rng.range(-10, 10)};
        push_material(mats, draw_material(rng));
        add_box(pos, idx, mid, c, h, b);
    }
    pt_scene_set_materials(s, mats.data(), uint32_t(mats.size() / 12));
    pt_scene_set_mesh(s, pos.data(), uint32_t(pos.size() / 3), idx.data(), uint32_t(idx.size() / 3),
                      mid.data());
    pt_scene_light_quad(s, 1, 0, 12, 0, 0, -1, 0, 1, 0, 0, 0.5f, 0.5f, 15, 15, 15);
    std::vector<float> black(8 * 4 * 3, 0.0f);
    pt_scene_set_env(s, black.data(), 8, 4);
    pt_scene_set_camera(s, 0, 0, 28, 0, 0, 45);
    set_cv(s, "r_max_bounces", 8);
    set_cv(s, "r_spp", 16);
    set_cv(s, "r_rr_start", 3);
    set_cv(s, "r_mis", 1);
    set_cv(s, "r_caustics", 1);
    set_cv(s, "r_refract_bounces", 4);
    set_cv(s, "r_firefly_clamp", 10);
    set_cv(s, "r_light_tree", 0);
}

// Differentiable-render scene: the analytic scene above grown to 512 spheres
// in [-20,20]^3 plus ~200k triangles (20 displaced icospheres of 9,680
// triangles, 4 boxes and a 56x56-quad floor), all on a 256-row material table
// drawn like the analytic scene's materials; 16 rows (every 16th) are
// emissive Lambert rows.  512x512, 32 spp, depth 6, roulette from bounce 3,
// no firefly clamp.
void synth_c3(pt_scene* s, uint64_t seed, double scale) {
    Pcg32 rng(0x5EEDull + 3ull, seed);
    const double lin = std::sqrt(scale);
    std::vector<float> mats;
    for (uint32_t i = 0; i < 256; ++i) {
        MatDraw m = draw_material(rng);
        if (i % 16u == 0u) m.type = 0;
        if (m.type == 0 && m.albedo[0] == 1.0f) m.albedo[0] = m.albedo[1] = m.albedo[2] = 0.5f;
        push_material(mats, m);
        if (i % 16u == 0u) {
            for (int a = 0; a < 3; ++a) {
                float& al = mats[mats.size() - 12 + a];
                if (al > 0.95f) al = rng.range(0.05f, 0.95f);
                mats[mats.size() - 12 + 4 + a] = rng.range(1.0f, 4.0f);
            }
        }
    }
    const uint32_t n_spheres = std::max<uint32_t>(1, uint32_t(std::lround(512 * scale)));
    for (uint32_t i = 0; i < n_spheres; ++i) {
        const float cx = rng.range(-20, 20), cy = rng.range(-20, 20), cz = rng.range(-20, 20);
        const float r = float(0.2 * std::pow(10.0, double(rng.unit())));
        const uint32_t row = std::min<uint32_t>(uint32_t(rng.unit() * 256.0f), 255u);
        const float* m = mats.data() + 12 * size_t(row);
        pt_scene_prim_sphere(s, 1 + i, cx, cy, cz, r, int(m[8]), m[0], m[1], m[2], m[3], m[7]);
        pt_scene_prim_set_material(s, 1 + i, row);
    }
    std::vector<float> pos;
    std::vector<uint32_t> idx, mid;
    const uint32_t n_ico = std::max<uint32_t>(1, uint32_t(std::lround(20 * scale)));
    const uint32_t nu = std::max<uint32_t>(2, uint32_t(std::lround(22 * lin)));
    for (uint32_t k = 0; k < n_ico; ++k) {
        const float r = rng.range(1.5f, 3.5f);
        const float c[3] = {rng.range(-16, 16), rng.range(-16, 16), rng.range(-16, 16)};
        const uint32_t row = std::min<uint32_t>(uint32_t(rng.unit() * 256.0f), 255u);
        add_icosphere(pos, idx, mid, c, r, nu, 0.1f, 3000u + 7u * k, row);
    }
    for (uint32_t b = 0; b < 4; ++b) {
        const float h[3] = {rng.range(0.5f, 3.0f), rng.range(0.5f, 3.0f), rng.range(0.5f, 3.0f)};
        const float c[3] = {rng.range(-20, 20), rng.range(-20, 20), rng.range(-20, 20)};
        add_box(pos, idx, mid, c, h, std::min<uint32_t>(uint32_t(rng.unit() * 256.0f), 255u));
    }
    const uint32_t grid = std::max<uint32_t>(2, uint32_t(std::lround(56 * lin)));
    const uint32_t floor_row = 1;
    const uint32_t fb = uint32_t(pos.size() / 3);
    for (uint32_t j = 0; j <= grid; ++j)
        for (uint32_t i = 0; i <= grid; ++i) {
            pos.push_back(-25.0f + 50.0f * float(i) / float(grid));
            pos.push_back(-20.5f);
            pos.push_back(-25.0f + 50.0f * float(j) / float(grid));
        }
    for (uint32_t j = 0; j < grid; ++j)
        for (uint32_t i = 0; i < grid; ++i) {
            const uint32_t a = fb + j * (grid + 1) + i, b = a + 1, c = a + grid + 1, d = c + 1;
            idx.insert(idx.end(), {a, c, b, b, c, d});
            mid.push_back(floor_row);
            mid.push_back(floor_row);
        }
    pt_scene_set_materials(s, mats.data(), uint32_t(mats.size() / 12));
    pt_scene_set_mesh(s, pos.data(), uint32_t(pos.size() / 3), idx.data(), uint32_t(idx.size() / 3),
                      mid.data());
    pt_scene_light_quad(s, 1, 0, 24, 0, 0, -1, 0, 1, 0, 0, 0.5f, 0.5f, 15, 15, 15);
    std::vector<float> black(8 * 4 * 3, 0.0f);
    pt_scene_set_env(s, black.data(), 8, 4);
    pt_scene_set_camera(s, 0, 0, 56, 0, 0, 45);
    set_cv(s, "r_max_bounces", 6);
    set_cv(s, "r_spp", 32);
    set_cv(s, "r_rr_start", 3);
    set_cv(s, "r_mis", 1);
    set_cv(s, "r_caustics", 1);
    set_cv(s, "r_refract_bounces", 4);
    set_cv(s, "r_firefly_clamp", 0);
    set_cv(s, "r_light_tree", 0);
}

// env: log-normal radiance per texel (mu 0, sigma 1.5) + 0.5 deg sun disc of
// 1e4 at elevation 40 deg, azimuth 30 deg
void set_sky_env(pt_scene* s, Pcg32& rng, uint32_t envw, uint32_t envh) {
    std::vector<float> rgb(size_t(envw) * envh * 3);
    const double sun_el = 40.0 * std::numbers::pi / 180.0, sun_az = 30.0 * std::numbers::pi / 180.0;
    const double sd[3] = {std::cos(sun_el) * std::cos(sun_az), std::sin(sun_el),
                          std::cos(sun_el) * std::sin(sun_az)};
    const double cos_disc = std::cos(0.25 * std::numbers::pi / 180.0);
    for (uint32_t v = 0; v < envh; ++v) {
        const double theta = std::numbers::pi * (v + 0.5) / envh;
        for (uint32_t u = 0; u < envw; ++u) {
            const double phi = 2.0 * std::numbers::pi * (u + 0.5) / envw - std::numbers::pi;
            const double d[3] = {std::sin(theta) * std::cos(phi), std::cos(theta),
                                 std::sin(theta) * std::sin(phi)};
            float L0 = float(std::exp(1.5 * rng.gauss()));
            if (d[0] * sd[0] + d[1] * sd[1] + d[2] * sd[2] >= cos_disc) L0 = 1e4f;
            const size_t pi = size_t(v) * envw + u;
            rgb[pi * 3 + 0] = L0;
            rgb[pi * 3 + 1] = L0;
            rgb[pi * 3 + 2] = L0;
        }
    }
    pt_scene_set_env(s, rgb.data(), envw, envh);
}

// Inverse-rendering scene: the procedural terrain scene in a 120 x 120 arena,
// ~1M triangles (80 displaced icospheres of 9,680 triangles + a 340x340-quad
// ground), 256 spheres and the log-normal + sun env, on 1,024 Lambert material
// rows with albedos U[0.2, 0.8].  The ground is cut into 56 x 56 patches that
// take the rows in a scattered order, every row on 3-4 patches, so an object
// covering a patch hides no row; icospheres and spheres take random rows.  Depth 8, roulette from bounce 2, no firefly clamp.
void synth_c4(pt_scene* s, uint64_t seed, double scale) {
    Pcg32 rng(0x5EEDull + 4ull, seed);
    const double lin = std::sqrt(scale);
    const uint32_t n_ico = std::max<uint32_t>(1, uint32_t(std::lround(80 * scale)));
    const uint32_t nu = std::max<uint32_t>(2, uint32_t(std::lround(22 * lin)));
    const uint32_t grid = std::max<uint32_t>(32, uint32_t(std::lround(340 * lin)));
    const uint32_t n_sph = std::max<uint32_t>(1, uint32_t(std::lround(256 * scale)));
    uint32_t envw = std::max<uint32_t>(16, uint32_t(std::lround(2048 * lin)));
    envw &= ~1u;
    const uint32_t envh = envw / 2;
    constexpr uint32_t kRows = 1024, kPatches = 56;
    std::vector<float> mats;
    for (uint32_t i = 0; i < kRows; ++i) {
        MatDraw m{0, {rng.range(0.2f, 0.8f), rng.range(0.2f, 0.8f), rng.range(0.2f, 0.8f)}, 0.0f, 1.5f};
        push_material(mats, m);
    }
    std::vector<float> pos;
    std::vector<uint32_t> idx, mid;
    const float L = 60.0f;
    for (uint32_t j = 0; j <= grid; ++j)
        for (uint32_t i = 0; i <= grid; ++i) {
            pos.push_back(-L + 2.0f * L * float(i) / float(grid));
            pos.push_back(0.0f);
            pos.push_back(-L + 2.0f * L * float(j) / float(grid));
        }
    for (uint32_t j = 0; j < grid; ++j)
        for (uint32_t i = 0; i < grid; ++i) {
            const uint32_t a = j * (grid + 1) + i, b = a + 1, c = a + grid + 1, d = c + 1;
            idx.insert(idx.end(), {a, c, b, b, c, d});
            // patch k takes row (389 k) mod 1024: every row covers 3-4 patches
            // about 18 patch rows apart, so no row is hidden by one object
            const uint32_t k = (j * kPatches / grid) * kPatches + (i * kPatches / grid);
            const uint32_t row = (k * 389u) % kRows;
            mid.push_back(row);
            mid.push_back(row);
        }
    for (uint32_t k = 0; k < n_ico; ++k) {
        const float r = rng.range(1.5f, 4.0f);
        const float c[3] = {rng.range(-52, 52), r, rng.range(-52, 52)};
        add_icosphere(pos, idx, mid, c, r, nu, 0.1f, 5000u + 7u * k,
                      std::min<uint32_t>(uint32_t(rng.unit() * float(kRows)), kRows - 1u));
    }
    pt_scene_set_materials(s, mats.data(), uint32_t(mats.size() / 12));
    pt_scene_set_mesh(s, pos.data(), uint32_t(pos.size() / 3), idx.data(), uint32_t(idx.size() / 3),
                      mid.data());
    for (uint32_t i = 0; i < n_sph; ++i) {
        const float r = float(0.3 * std::pow(5.0, double(rng.unit())));
        const float cx = rng.range(-55, 55), cz = rng.range(-55, 55);
        const uint32_t row = std::min<uint32_t>(uint32_t(rng.unit() * float(kRows)), kRows - 1u);
        const float* m = mats.data() + 12 * size_t(row);
        pt_scene_prim_sphere(s, 1 + i, cx, r, cz, r, 0, m[0], m[1], m[2], 0.0f, 1.5f);
        pt_scene_prim_set_material(s, 1 + i, row);
    }
    set_sky_env(s, rng, envw, envh);
    pt_scene_set_camera(s, 0.0f, 45.0f, 70.0f, 0.0f, -0.57f, 45.0f);
    set_cv(s, "r_max_bounces", 8);
    set_cv(s, "r_spp", 16);
    set_cv(s, "r_rr_start", 2);
    set_cv(s, "r_mis", 1);
    set_cv(s, "r_caustics", 1);
    set_cv(s, "r_refract_bounces", 4);
    set_cv(s, "r_firefly_clamp", 0);
    set_cv(s, "r_light_tree", 0);
}

void synth_c1(pt_scene* s, uint64_t seed, double scale) {
    Pcg32 rng(0x5EEDull + 1ull, seed);
    const double lin = std::sqrt(scale);
    const uint32_t n_ico = std::max<uint32_t>(1, uint32_t(std::lround(200 * scale)));
    const uint32_t nu = std::max<uint32_t>(2, uint32_t(std::lround(22 * lin)));
    const uint32_t grid = std::max<uint32_t>(2, uint32_t(std::lround(512 * lin)));
    const uint32_t n_sph = std::max<uint32_t>(1, uint32_t(std::lround(1024 * scale)));
    uint32_t envw = std::max<uint32_t>(16, uint32_t(std::lround(2048 * lin)));
    envw &= ~1u;
    const uint32_t envh = envw / 2;

    std::vector<float> mats;
    push_material(mats, MatDraw{0, {0.5f, 0.5f, 0.5f}, 0.0f, 1.5f});   // ground
    for (uint32_t i = 1; i < 256; ++i) push_material(mats, draw_material(rng));

    std::vector<float> pos;
    std::vector<uint32_t> idx, mid;
    // ground: grid x grid quads over [-120, 120]^2 at y = 0
    const float L = 120.0f;
    for (uint32_t j = 0; j <= grid; ++j)
        for (uint32_t i = 0; i <= grid; ++i) {
            pos.push_back(-L + 2.0f * L * float(i) / float(grid));
            pos.push_back(0.0f);
            pos.push_back(-L + 2.0f * L * float(j) / float(grid));
        }
    for (uint32_t j = 0; j < grid; ++j)
        for (uint32_t i = 0; i < grid; ++i) {
            const uint32_t a = j * (grid + 1) + i, b = a + 1, c = a + grid + 1, d = c + 1;
            idx.insert(idx.end(), {a, c, b, b, c, d});
            mid.push_back(0);
            mid.push_back(0);
        }
    for (uint32_t k = 0; k < n_ico; ++k) {
        const float r = rng.range(1.5f, 4.0f);
        const float c[3] = {rng.range(-100, 100), r, rng.range(-100, 100)};
        add_icosphere(pos, idx, mid, c, r, nu, 0.1f, 1000u + 7u * k, 1u + (k % 255u));
    }
    pt_scene_set_materials(s, mats.data(), uint32_t(mats.size() / 12));
    pt_scene_set_mesh(s, pos.data(), uint32_t(pos.size() / 3), idx.data(), uint32_t(idx.size() / 3),
                      mid.data());
    for (uint32_t i = 0; i < n_sph; ++i) {
        const float r = float(0.3 * std::pow(5.0, double(rng.unit())));
        const float cx = rng.range(-110, 110), cz = rng.range(-110, 110);
        const MatDraw m = draw_material(rng);
        pt_scene_prim_sphere(s, 1 + i, cx, r, cz, r, m.type, m.albedo[0], m.albedo[1], m.albedo[2],
                             m.rough, m.ior);
    }
    set_sky_env(s, rng, envw, envh);
    pt_scene_set_camera(s, 0.0f, 30.0f, 150.0f, 0.0f, -0.197f, 45.0f);
    set_cv(s, "r_max_bounces", 8);
    set_cv(s, "r_spp", 1);
    set_cv(s, "r_rr_start", 2);
    set_cv(s, "r_mis", 1);
    set_cv(s, "r_caustics", 1);
    set_cv(s, "r_refract_bounces", 4);
    set_cv(s, "r_firefly_clamp", 10);
    set_cv(s, "r_light_tree", 0);
}

}  // namespace

// ===========================================================================
// C-ABI
// ===========================================================================
extern "C" {

int pt_scene_create(pt_scene** out) {
    if (!out) return PT_ERR_INVALID;
    *out = new pt_scene();
    return PT_OK;
}

int pt_scene_destroy(pt_scene* s) {
    delete s;
    return PT_OK;
}

const char* pt_scene_last_error(const pt_scene* s) { return s ? s->err.c_str() : "null scene"; }

int pt_scene_clear(pt_scene* s) {
    if (!s) return PT_ERR_INVALID;
    auto cv = s->cvars;
    *s = pt_scene();
    s->cvars = cv;
    return PT_OK;
}

int pt_scene_prim_sphere(pt_scene* s, uint32_t id, float x, float y, float z, float radius,
                         int material, float r, float g, float b, float roughness, float ior) {
    if (!s) return PT_ERR_INVALID;
    if (material < 0 || material > 2) return fail(s, "prim_sphere: unknown material");
    if (!(radius > 0.0f)) return fail(s, "prim_sphere: radius must be > 0");
    Prim p{};
    p.type = 0;
    p.material = uint8_t(material);
    p.pos[0] = x; p.pos[1] = y; p.pos[2] = z;
    p.prev[0] = x; p.prev[1] = y; p.prev[2] = z;
    p.radius_or_d = radius;
    p.albedo[0] = r; p.albedo[1] = g; p.albedo[2] = b;
    p.roughness = roughness;
    p.ior = ior;
    s->prims[id] = p;
    s->dirty_prims = true;
    return PT_OK;
}

int pt_scene_prim_plane(pt_scene* s, uint32_t id, float nx, float ny, float nz, float d,
                        int material, float r, float g, float b, float roughness, float ior) {
    if (!s) return PT_ERR_INVALID;
    if (material < 0 || material > 2) return fail(s, "prim_plane: unknown material");
    const float len = std::sqrt(nx * nx + ny * ny + nz * nz);
    if (!(len > 0.0f)) return fail(s, "prim_plane: zero normal");
    nx /= len; ny /= len; nz /= len;
    Prim p{};
    p.type = 1;
    p.material = uint8_t(material);
    p.pos[0] = nx; p.pos[1] = ny; p.pos[2] = nz;
    p.prev[0] = nx; p.prev[1] = ny; p.prev[2] = nz;
    p.radius_or_d = d;
    p.albedo[0] = r; p.albedo[1] = g; p.albedo[2] = b;
    p.roughness = roughness;
    p.ior = ior;
    s->prims[id] = p;
    s->dirty_prims = true;
    return PT_OK;
}

int pt_scene_prim_set_emission(pt_scene* s, uint32_t id, float r, float g, float b) {
    if (!s) return PT_ERR_INVALID;
    auto it = s->prims.find(id);
    if (it == s->prims.end()) return fail(s, "prim_set_emission: unknown id");
    it->second.emission[0] = r; it->second.emission[1] = g; it->second.emission[2] = b;
    s->dirty_prims = true;
    return PT_OK;
}

int pt_scene_prim_set_orient(pt_scene* s, uint32_t id, float qx, float qy, float qz, float qw) {
    if (!s) return PT_ERR_INVALID;
    auto it = s->prims.find(id);
    if (it == s->prims.end()) return fail(s, "prim_set_rotation: unknown id");
    it->second.orient[0] = qx; it->second.orient[1] = qy;
    it->second.orient[2] = qz; it->second.orient[3] = qw;
    s->dirty_prims = true;
    return PT_OK;
}

int pt_scene_prim_set_material(pt_scene* s, uint32_t id, uint32_t mat) {
    if (!s) return PT_ERR_INVALID;
    auto it = s->prims.find(id);
    if (it == s->prims.end()) return fail(s, "prim_set_material: unknown id");
    it->second.mat_id = mat;
    s->dirty_prims = true;
    return PT_OK;
}

int pt_scene_light_quad(pt_scene* s, uint32_t id, float x, float y, float z, float nx, float ny,
                        float nz, float ux, float uy, float uz, float u_half, float v_half,
                        float r, float g, float b) {
    if (!s) return PT_ERR_INVALID;
    const float nlen = std::sqrt(nx * nx + ny * ny + nz * nz);
    if (nlen < 1e-6f) return fail(s, "light_quad: normal magnitude is zero");
    nx /= nlen; ny /= nlen; nz /= nlen;
    const float ndu = nx * ux + ny * uy + nz * uz;
    float uxo = ux - nx * ndu, uyo = uy - ny * ndu, uzo = uz - nz * ndu;
    const float ulen = std::sqrt(uxo * uxo + uyo * uyo + uzo * uzo);
    if (ulen < 1e-6f) return fail(s, "light_quad: u-axis collinear with normal");
    uxo /= ulen; uyo /= ulen; uzo /= ulen;
    if (u_half <= 0.0f || v_half <= 0.0f) return fail(s, "light_quad: u_half and v_half must be > 0");
    Light L{};
    L.type = 3;
    L.pos[0] = x; L.pos[1] = y; L.pos[2] = z;
    L.dir[0] = nx; L.dir[1] = ny; L.dir[2] = nz;
    L.u_vec[0] = uxo * u_half; L.u_vec[1] = uyo * u_half; L.u_vec[2] = uzo * u_half;
    L.v_half = v_half;
    L.intensity[0] = r; L.intensity[1] = g; L.intensity[2] = b;
    s->lights[id] = L;
    s->dirty_lights = true;
    return PT_OK;
}

int pt_scene_light_point(pt_scene* s, uint32_t id, float x, float y, float z, float r, float g,
                         float b) {
    if (!s) return PT_ERR_INVALID;
    Light L{};
    L.type = 0;
    L.pos[0] = x; L.pos[1] = y; L.pos[2] = z;
    L.intensity[0] = r; L.intensity[1] = g; L.intensity[2] = b;
    s->lights[id] = L;
    s->dirty_lights = true;
    return PT_OK;
}

int pt_scene_light_sphere(pt_scene* s, uint32_t id, float x, float y, float z, float radius,
                          float r, float g, float b) {
    if (!s) return PT_ERR_INVALID;
    if (!(radius > 0.0f)) return fail(s, "light_sphere: radius must be > 0");
    Light L{};
    L.type = 2;
    L.pos[0] = x; L.pos[1] = y; L.pos[2] = z;
    L.radius = radius;
    L.intensity[0] = r; L.intensity[1] = g; L.intensity[2] = b;
    s->lights[id] = L;
    s->dirty_lights = true;
    return PT_OK;
}

int pt_scene_light_spot(pt_scene* s, uint32_t id, float x, float y, float z, float dx, float dy,
                        float dz, float outer_deg, float inner_deg, float r, float g, float b) {
    if (!s) return PT_ERR_INVALID;
    const float dlen = std::sqrt(dx * dx + dy * dy + dz * dz);
    if (dlen < 1e-6f) return fail(s, "light_spot: direction magnitude is zero");
    dx /= dlen; dy /= dlen; dz /= dlen;
    const float deg2rad = std::numbers::pi_v<float> / 180.0f;
    Light L{};
    L.type = 1;
    L.pos[0] = x; L.pos[1] = y; L.pos[2] = z;
    L.dir[0] = dx; L.dir[1] = dy; L.dir[2] = dz;
    L.intensity[0] = r; L.intensity[1] = g; L.intensity[2] = b;
    L.cos_outer = std::cos(outer_deg * deg2rad);
    L.cos_inner = std::cos(inner_deg * deg2rad);
    s->lights[id] = L;
    s->dirty_lights = true;
    return PT_OK;
}

int pt_scene_set_mesh(pt_scene* s, const float* positions, uint32_t nv, const uint32_t* indices,
                      uint32_t nt, const uint32_t* mat_ids) {
    if (!s) return PT_ERR_INVALID;
    if ((nv && !positions) || (nt && !indices)) return fail(s, "set_mesh: null buffer");
    s->mesh_pos.assign(positions, positions + size_t(nv) * 3);
    s->mesh_idx.assign(indices, indices + size_t(nt) * 3);
    s->mesh_has_mat = (mat_ids != nullptr);
    if (mat_ids) s->mesh_mat.assign(mat_ids, mat_ids + nt);
    else s->mesh_mat.clear();
    s->dirty_mesh = true;
    return PT_OK;
}

int pt_scene_set_materials(pt_scene* s, const float* mats12, uint32_t n) {
    if (!s) return PT_ERR_INVALID;
    if (n && !mats12) return fail(s, "set_materials: null buffer");
    s->materials.assign(mats12, mats12 + size_t(n) * 12);
    return PT_OK;
}

int pt_scene_set_env(pt_scene* s, const float* rgb, uint32_t W, uint32_t H) {
    if (!s) return PT_ERR_INVALID;
    if (W == 0 || H == 0) {
        s->env_present = false;
        s->env_rgb.clear();
        s->env_w = s->env_h = 0;
    } else {
        if (!rgb) return fail(s, "set_env: null image");
        s->env_rgb.assign(rgb, rgb + size_t(W) * H * 3);
        s->env_w = W;
        s->env_h = H;
        s->env_present = true;
    }
    s->dirty_env = true;
    return PT_OK;
}

int pt_scene_set_moon(pt_scene* s, const float* rgba, uint32_t W, uint32_t H) {
    if (!s) return PT_ERR_INVALID;
    if (W == 0 || H == 0) {
        s->moon_rgba.clear();
        s->moon_w = s->moon_h = 0;
        return PT_OK;
    }
    if (!rgba) return fail(s, "set_moon: null image");
    s->moon_rgba.assign(rgba, rgba + size_t(W) * H * 4);
    s->moon_w = W;
    s->moon_h = H;
    return PT_OK;
}

int pt_scene_set_camera(pt_scene* s, float x, float y, float z, float yaw, float pitch,
                        float fov_deg) {
    if (!s) return PT_ERR_INVALID;
    s->cam_pos[0] = x; s->cam_pos[1] = y; s->cam_pos[2] = z;
    s->cam_yaw = yaw;
    const float lim = 85.0f * 0.01745329251994329576923690768489f;
    s->cam_pitch = std::min(std::max(pitch, -lim), lim);
    s->cam_fov = fov_deg;
    return PT_OK;
}

int pt_scene_set_cvar(pt_scene* s, const char* name, double value) {
    if (!s || !name) return PT_ERR_INVALID;
    for (auto& c : s->cvars) {
        if (std::strcmp(c.name, name) == 0) {
            if (c.value != value) {
                c.value = value;
                if (std::strcmp(name, "r_analytic_bvh_threshold") == 0) s->dirty_prims = true;
                if (std::strcmp(name, "r_hdri_extract_percentile") == 0) s->dirty_env = true;
            }
            return PT_OK;
        }
    }
    return fail(s, std::string("unknown cvar ") + name);
}

int pt_scene_get_cvar(const pt_scene* s, const char* name, double* value) {
    if (!s || !name || !value) return PT_ERR_INVALID;
    for (const auto& c : s->cvars) {
        if (std::strcmp(c.name, name) == 0) {
            *value = c.value;
            return PT_OK;
        }
    }
    return PT_ERR_INVALID;
}

int pt_scene_pack(pt_scene* s) {
    if (!s) return PT_ERR_INVALID;
    if (s->dirty_prims) pack_prims(s);
    if (s->dirty_mesh) pack_mesh(s);
    if (s->dirty_lights) pack_lights(s);
    if (s->dirty_env) pack_env(s);
    return PT_OK;
}

int pt_scene_packed(pt_scene* s, PtPackedScene* o) {
    if (!s || !o) return PT_ERR_INVALID;
    pt_scene_pack(s);
    std::memset(o, 0, sizeof(*o));
    o->prims = s->packed_prims.data();
    o->prim_count = uint32_t(s->prims.size());
    o->linear_prim_count = s->linear_count;
    o->bvh_nodes = s->bvh.data();
    o->bvh_node_count = uint32_t(s->bvh.size());
    o->positions = s->mesh_pos.data();
    o->vertex_count = uint32_t(s->mesh_pos.size() / 3);
    o->indices = s->mesh_idx.data();
    o->tri_count = uint32_t(s->mesh_idx.size() / 3);
    o->tri_nodes = s->tri_bvh.data();
    o->tri_node_count = uint32_t(s->tri_bvh.size());
    o->tri_perm = s->tri_perm.data();
    o->tri_perm_count = uint32_t(s->tri_perm.size());
    o->tri_mat_ids = s->mesh_has_mat ? s->mesh_mat.data() : nullptr;
    o->materials = s->materials.data();
    o->material_count = uint32_t(s->materials.size() / 12);
    o->lights = s->packed_lights.data();
    o->light_count = uint32_t(s->lights.size());
    o->env_present = s->env_present ? 1u : 0u;
    s->packed_sdf.clear();
    for (const auto& [id, c] : s->sdf) {   // 28 float4 per cluster, id order
        float blk[112] = {0};
        auto u2f = [](uint32_t u) {
            float f;
            std::memcpy(&f, &u, 4);
            return f;
        };
        for (int k = 0; k < 3; ++k) {
            blk[k] = c.lo[k];
            blk[4 + k] = c.hi[k];
            blk[8 + k] = c.albedo[k];
        }
        blk[3] = u2f(c.count);
        blk[7] = u2f(c.material);
        blk[11] = c.roughness;
        blk[12] = c.ior;
        for (uint32_t i = 0; i < 8; ++i) {
            const SdfNodeH& n = c.nodes[i];
            float* q = blk + 16 + 12 * i;
            q[0] = u2f(n.op); q[1] = u2f(n.shape); q[2] = u2f(n.a); q[3] = u2f(n.b);
            for (int k = 0; k < 4; ++k) q[4 + k] = n.params[k];
            for (int k = 0; k < 3; ++k) q[8 + k] = n.center[k];
        }
        s->packed_sdf.insert(s->packed_sdf.end(), blk, blk + 112);
    }
    o->sdf_clusters = s->packed_sdf.empty() ? nullptr : s->packed_sdf.data();
    o->sdf_count = uint32_t(s->sdf.size());
    o->light_tree = s->light_tree.empty() ? nullptr : s->light_tree.data();
    o->light_tree_node_count = uint32_t(s->light_tree.size());
    o->moon_rgba = s->moon_rgba.empty() ? nullptr : s->moon_rgba.data();
    o->moon_w = s->moon_w;
    o->moon_h = s->moon_h;
    o->env_rgba = s->env_rgba.data();
    o->env_w = s->env_w;
    o->env_h = s->env_h;
    o->env_marginal = s->env_marg.data();
    o->env_conditional = s->env_cond.data();
    o->env_total_luminance = s->env_total;
    o->hdri_count = uint32_t(s->hdri.size());
    o->hdri_dir_pmf = s->hdri_dir;
    o->hdri_col = s->hdri_col;
    o->prim_mat_ids = s->any_prim_mat ? s->packed_prim_mats.data() : nullptr;
    return PT_OK;
}

int pt_scene_fill_push(pt_scene* s, uint32_t width, uint32_t height, uint32_t frame_index,
                       uint32_t reset_accum, PtPushHead* head, PtPathParams* params) {
    if (!s || !head || !params || width == 0 || height == 0) return PT_ERR_INVALID;
    pt_scene_pack(s);
    std::memset(head, 0, sizeof(*head));
    std::memset(params, 0, sizeof(*params));
    // Camera basis (src/renderer/Camera.h:18-30): glm float math,
    // normalize(v) = v * inversesqrt(dot(v, v)).
    const float cp = std::cos(s->cam_pitch);
    const float fwd[3] = {std::sin(s->cam_yaw) * cp, std::sin(s->cam_pitch),
                          -std::cos(s->cam_yaw) * cp};
    auto normalize = [](float v[3]) {
        const float inv = 1.0f / std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
        v[0] *= inv; v[1] *= inv; v[2] *= inv;
    };
    // right = normalize(cross(fwd, (0,1,0)))
    float right[3] = {fwd[1] * 0.0f - fwd[2] * 1.0f, fwd[2] * 0.0f - fwd[0] * 0.0f,
                      fwd[0] * 1.0f - fwd[1] * 0.0f};
    normalize(right);
    float up[3] = {right[1] * fwd[2] - right[2] * fwd[1], right[2] * fwd[0] - right[0] * fwd[2],
                   right[0] * fwd[1] - right[1] * fwd[0]};
    normalize(up);
    const float fov_tan = std::tan(s->cam_fov * 0.01745329251994329576923690768489f * 0.5f);
    head->pos_fovtan[0] = s->cam_pos[0]; head->pos_fovtan[1] = s->cam_pos[1];
    head->pos_fovtan[2] = s->cam_pos[2]; head->pos_fovtan[3] = fov_tan;
    head->fwd_aspect[0] = fwd[0]; head->fwd_aspect[1] = fwd[1]; head->fwd_aspect[2] = fwd[2];
    head->fwd_aspect[3] = float(width) / float(height);
    head->right_xyz[0] = right[0]; head->right_xyz[1] = right[1]; head->right_xyz[2] = right[2];
    head->up_xyz[0] = up[0]; head->up_xyz[1] = up[1]; head->up_xyz[2] = up[2];
    head->frame_index = frame_index;
    head->reset_accum = reset_accum ? 1u : 0u;
    head->max_bounces = uint32_t(std::max(0.0, s->cvar("r_max_bounces")));
    head->tlas_present = 0;
    head->prim_count = uint32_t(s->prims.size());
    {
        int n = int(s->cvar("r_spp"));
        if (n < 1) n = 1;
        if (n > 32) n = 32;
        head->spp = uint32_t(n);
    }
    head->denoiser_enabled = s->cvar("r_denoiser") != 0.0 ? 1u : 0u;
    if (head->denoiser_enabled) {
        // the engine's sub-pixel jitter: Halton bases 2 and 3 at index
        // frame_index % 16 + 1, minus 0.5 (src/engine/Engine.cpp:8241-8252)
        auto radical_inverse = [](uint32_t i, uint32_t base) {
            float f = 1.0f, r = 0.0f;
            while (i > 0u) {
                f /= float(base);
                r += f * float(i % base);
                i /= base;
            }
            return r;
        };
        const uint32_t hi = (frame_index % 16u) + 1u;
        head->halton_jitter[0] = radical_inverse(hi, 2u) - 0.5f;
        head->halton_jitter[1] = radical_inverse(hi, 3u) - 0.5f;
    }
    head->env_map_present = s->env_present ? 1u : 0u;
    head->env_intensity = float(s->cvar("r_env_intensity"));
    head->env_total_luminance = float(s->env_total);

    const bool caustics = s->cvar("r_caustics") != 0.0;
    int rb = int(s->cvar("r_refract_bounces"));
    rb = std::min(std::max(rb, 0), 16);
    params->refract_budget = caustics ? float(rb) : 0.0f;
    float ff = float(s->cvar("r_firefly_clamp"));
    params->firefly_clamp = ff < 0.0f ? 0.0f : ff;
    params->mis_enabled = s->cvar("r_mis") != 0.0 ? 1u : 0u;
    float ema = float(s->cvar("r_accum_ema_alpha"));
    params->accum_ema_alpha = std::min(std::max(ema, 0.0f), 0.999f);
    params->bvh_params[0] = s->linear_count;
    params->bvh_params[1] = uint32_t(s->bvh.size());
    const bool mesh = !s->tri_bvh.empty();
    params->bvh_params[2] = mesh ? uint32_t(s->mesh_idx.size() / 3) : 0u;
    params->bvh_params[3] = mesh ? uint32_t(s->tri_bvh.size()) : 0u;
    params->light_count = uint32_t(s->lights.size());
    {
        const bool tree = s->cvar("r_light_tree") != 0.0 && !s->light_tree.empty();
        params->light_tree_enabled = tree ? 1u : 0u;
        params->light_tree_node_count = tree ? uint32_t(s->light_tree.size()) : 0u;
    }
    params->rr_start = uint32_t(std::max(0.0, s->cvar("r_rr_start")));
    // Sky (src/engine/Engine.cpp:8304-8470, 8533-8545): env map -> mode 1, else the
    // gradient dome (mode 0, the reference's fallback for "hdri" without a map).
    // The sun comes from r_sun_elevation / r_sun_azimuth (the non-astronomical
    // driver); the moon is hidden (it is placed only by the astronomical date
    // driver, which is not part of this path); distance ratios are the mean 1.0.
    const float elev_deg = float(s->cvar("r_sun_elevation"));
    const float azim_deg = float(s->cvar("r_sun_azimuth"));
    const float elev_r = elev_deg * 0.01745329251994329576923690768489f;
    const float azim_r = azim_deg * 0.01745329251994329576923690768489f;
    const float ce = std::cos(elev_r), se = std::sin(elev_r);
    params->sun_and_mode[0] = ce * std::sin(azim_r);
    params->sun_and_mode[1] = se;
    params->sun_and_mode[2] = -ce * std::cos(azim_r);
    {
        // r_sky_mode: 0 gradient, 1 hdri (gradient when no map is loaded), 2 procedural,
        // 3 hosek; the env map is bound only in hdri mode (Engine.cpp:8533-8545)
        int mode = int(s->cvar("r_sky_mode"));
        if (mode < 0 || mode > 3) mode = 1;
        if (mode == 1 && !s->env_present) mode = 0;
        params->sun_and_mode[3] = float(mode);
        head->env_map_present = (mode == 1) ? 1u : 0u;
        params->stars = (mode == 2 && s->cvar("r_show_stars") != 0.0) ? 1u : 0u;
    }
    params->moon_dir_phase[0] = 0.0f;
    params->moon_dir_phase[1] = -1.0f;
    params->moon_dir_phase[2] = 0.0f;
    params->moon_dir_phase[3] = 0.0f;
    params->moon_extra[0] = std::clamp(float(s->cvar("r_moon_size")), 0.1f, 50.0f);
    params->moon_extra[1] = 1.0f;
    params->moon_extra[2] = std::clamp(float(s->cvar("r_moon_disc_brightness")), 0.0f, 5.0f);
    params->moon_extra[3] = std::clamp(float(s->cvar("r_sun_disc_brightness")), 0.0f, 5.0f);
    params->sun_extra[0] = std::clamp(float(s->cvar("r_sun_size")), 0.1f, 50.0f);
    params->sun_extra[1] = 1.0f;
    float vflat = 1.0f;
    if (s->cvar("r_sun_horizon_flatten") != 0.0) {
        // atmospheric refraction R(h) = 1 / tan(h + 7.31 / (h + 4.4)) arcmin
        // (Saemundsson 1986) at the real disc's upper and lower limb
        constexpr float kRealSunRadiusDeg = 0.265f;
        auto refraction = [](float h_deg) {
            const float h = std::max(h_deg, -1.5f);
            return 1.0f / std::tan((h + 7.31f / (h + 4.4f)) * 3.14159265358979323846f / 180.0f);
        };
        const float lift = (refraction(elev_deg - kRealSunRadiusDeg) - refraction(elev_deg + kRealSunRadiusDeg)) / 60.0f;
        vflat = std::clamp(1.0f - lift / (2.0f * kRealSunRadiusDeg), 0.5f, 1.0f);
    }
    params->sun_extra[2] = vflat;
    params->sun_extra[3] = std::max(float(s->cvar("r_planet_radius")), 0.0f);
    params->sun_extra2[0] = params->moon_extra[3];
    {   // SDF trace settings (Engine.cpp:7940-7981)
        int it = int(s->cvar("r_sdf_max_iters"));
        it = std::min(std::max(it, 1), 256);
        float eps = float(s->cvar("r_sdf_epsilon"));
        if (eps < 1e-7f) eps = 1e-7f;
        const float power = std::min(std::max(float(s->cvar("r_sdf_fractal_power")), 2.0f), 64.0f);
        const int fit = std::min(std::max(int(s->cvar("r_sdf_fractal_iters")), 1), 32);
        const float de_sc = std::max(float(s->cvar("r_sdf_de_eps_scale")), 0.0f);
        const int nm = std::min(std::max(int(s->cvar("r_sdf_normal_mode")), 0), 1);
        params->sdf_params[0] = uint32_t(s->sdf.size());
        params->sdf_params[1] = uint32_t(it);
        params->sdf_params[3] = uint32_t(fit);
        params->sdf_params_f[0] = eps;
        params->sdf_params_f[1] = power;
        params->sdf_params_f[2] = de_sc;
        params->sdf_params_f[3] = float(nm);
        params->sdf_procedural_ops = uint32_t(std::min(std::max(int(s->cvar("r_sdf_procedural_ops")), 0), 2));
    }
    return PT_OK;
}

int pt_scene_synth(pt_scene* s, int config_id, uint64_t seed, double scale) {
    if (!s) return PT_ERR_INVALID;
    if (!(scale > 0.0) || scale > 1.0) return fail(s, "synth: scale must be in (0, 1]");
    pt_scene_clear(s);
    if (config_id == 0) synth_c0(s, seed, scale);
    else if (config_id == 1) synth_c1(s, seed, scale);
    else if (config_id == 3) synth_c3(s, seed, scale);
    else if (config_id == 4) synth_c4(s, seed, scale);
    else return fail(s, "synth: unknown config id");
    return pt_scene_pack(s);
}

int pt_scene_upload(pt_scene* s, pt_gpu_ctx* ctx) {
    if (!s || !ctx) return PT_ERR_INVALID;
    PtPackedScene p;
    pt_scene_packed(s, &p);
    int rc = pt_gpu_upload_prims(ctx, p.prims, p.prim_count, p.linear_prim_count, p.bvh_nodes,
                                 p.bvh_node_count);
    if (rc) return rc;
    rc = pt_gpu_upload_materials(ctx, p.materials, p.material_count);
    if (rc) return rc;
    rc = pt_gpu_upload_prim_materials(ctx, p.prim_mat_ids, p.prim_mat_ids ? p.prim_count : 0);
    if (rc) return rc;
    rc = pt_gpu_upload_mesh(ctx, p.positions, p.vertex_count, p.indices, p.tri_count, p.tri_nodes,
                            p.tri_node_count, p.tri_perm, p.tri_perm_count, p.tri_mat_ids);
    if (rc) return rc;
    rc = pt_gpu_upload_lights(ctx, p.lights, p.light_count);
    if (rc) return rc;
    rc = pt_gpu_upload_light_tree(ctx, p.light_tree, p.light_tree_node_count);
    if (rc) return rc;
    rc = pt_gpu_upload_sdf(ctx, p.sdf_clusters, p.sdf_count);
    if (rc) return rc;
    if (p.env_present)
        rc = pt_gpu_upload_env(ctx, p.env_rgba, p.env_w, p.env_h, p.env_marginal, p.env_conditional,
                               p.hdri_dir_pmf, p.hdri_col, p.hdri_count);
    else
        rc = pt_gpu_upload_env(ctx, nullptr, 0, 0, nullptr, nullptr, nullptr, nullptr, 0);
    if (rc) return rc;
    return pt_gpu_upload_moon(ctx, p.moon_rgba, p.moon_w, p.moon_h);
}

int pt_build_analytic_bvh(const float* cr, uint32_t n, PtBvhNode* nodes_out, uint32_t* n_nodes,
                          uint32_t* perm_out) {
    if ((n && (!cr || !nodes_out || !perm_out)) || !n_nodes) return PT_ERR_INVALID;
    std::vector<SphereItem> items(n);
    for (uint32_t i = 0; i < n; ++i)
        items[i] = SphereItem{{cr[4 * i], cr[4 * i + 1], cr[4 * i + 2]}, cr[4 * i + 3], i, {0, 0, 0}};
    std::vector<PtBvhNode> nodes;
    std::vector<uint32_t> perm;
    build_sphere_bvh(items, nodes, perm);
    std::copy(nodes.begin(), nodes.end(), nodes_out);
    std::copy(perm.begin(), perm.end(), perm_out);
    *n_nodes = uint32_t(nodes.size());
    return PT_OK;
}

int pt_build_triangle_bvh(const float* positions, uint32_t nv, const uint32_t* indices,
                          uint32_t n_index, PtBvhNode* nodes_out, uint32_t* n_nodes,
                          uint32_t* perm_out, uint32_t* n_perm) {
    if (!n_nodes || !n_perm) return PT_ERR_INVALID;
    std::vector<PtBvhNode> nodes;
    std::vector<uint32_t> perm;
    build_tri_bvh(positions, nv, indices, n_index, nodes, perm);
    if (!nodes.empty() && (!nodes_out || !perm_out)) return PT_ERR_INVALID;
    std::copy(nodes.begin(), nodes.end(), nodes_out);
    std::copy(perm.begin(), perm.end(), perm_out);
    *n_nodes = uint32_t(nodes.size());
    *n_perm = uint32_t(perm.size());
    return PT_OK;
}

int pt_build_env_cdf(const float* rgb, uint32_t W, uint32_t H, const uint8_t* mask,
                     float* marginal, float* conditional, double* total) {
    if (!rgb || !marginal || !conditional || !total) return PT_ERR_INVALID;
    *total = env_cdf(rgb, W, H, mask, marginal, conditional);
    return PT_OK;
}

}  // extern "C"

// ===========================================================================
// SDF clusters: bounding boxes (src/renderer/AnalyticBvh.cpp ComputeSdfAabb,
// restated) and the sdf_* commands.
// ===========================================================================
namespace {

bool sdf_leaf_box(const SdfNodeH& n, float* mn, float* mx) {
    const float* q = n.params;
    switch (n.shape) {
        case 0: {
            if (q[0] <= 0.0f) return false;
            for (int k = 0; k < 3; ++k) { mn[k] = -q[0]; mx[k] = q[0]; }
            return true;
        }
        case 1: {
            if (q[0] <= 0.0f || q[1] <= 0.0f || q[2] <= 0.0f) return false;
            for (int k = 0; k < 3; ++k) { mn[k] = -q[k]; mx[k] = q[k]; }
            return true;
        }
        case 2: {
            const float h[3] = {q[0] + q[3], q[1] + q[3], q[2] + q[3]};
            if (h[0] <= 0.0f || h[1] <= 0.0f || h[2] <= 0.0f) return false;
            for (int k = 0; k < 3; ++k) { mn[k] = -h[k]; mx[k] = h[k]; }
            return true;
        }
        case 3: {
            if (q[0] <= 0.0f || q[1] <= 0.0f) return false;
            mn[0] = -(q[0] + q[1]); mn[1] = -q[1]; mn[2] = -(q[0] + q[1]);
            mx[0] = q[0] + q[1];    mx[1] = q[1];  mx[2] = q[0] + q[1];
            return true;
        }
        case 4: {
            if (q[0] < 0.0f || q[1] <= 0.0f) return false;
            mn[0] = -q[1]; mn[1] = -q[0] - q[1]; mn[2] = -q[1];
            mx[0] = q[1];  mx[1] = q[0] + q[1];  mx[2] = q[1];
            return true;
        }
        case 6:
        case 7:
        case 8: {   // fractal leaves: +-bound
            if (q[1] <= 0.0f) return false;
            for (int k = 0; k < 3; ++k) { mn[k] = -q[1]; mx[k] = q[1]; }
            return true;
        }
        default:
            return false;   // planes are unbounded
    }
}

bool sdf_node_box(const SdfClusterH& c, uint32_t i, float* mn, float* mx, int depth = 0) {
    if (i >= c.count || depth > 8) return false;   // a deeper chain than 8 nodes has a cycle
    const SdfNodeH& n = c.nodes[i];
    auto widen = [&](float k) {
        for (int j = 0; j < 3; ++j) { mn[j] -= k; mx[j] += k; }
    };
    if (n.op == 0) {
        if (!sdf_leaf_box(n, mn, mx)) return false;
        for (int j = 0; j < 3; ++j) { mn[j] += n.center[j]; mx[j] += n.center[j]; }
        return true;
    }
    float an[3], ax[3], bn[3], bx[3];
    if (!sdf_node_box(c, n.a, an, ax, depth + 1)) return false;
    if (n.op == 4) {   // displace
        for (int j = 0; j < 3; ++j) { mn[j] = an[j]; mx[j] = ax[j]; }
        widen(std::abs(n.params[0]));
        return true;
    }
    // The procedural ops (bounded on the host in every build, whether or not
    // the renderer evaluates them): the child's box widened by the noise
    // band's largest sum, or re-bounded around the warp axis / repetition.
    if (n.op == 5) {   // displace by fBm noise: |amp| x sum of the octave amplitudes
        for (int j = 0; j < 3; ++j) { mn[j] = an[j]; mx[j] = ax[j]; }
        uint32_t oct = 0;
        std::memcpy(&oct, &n.params[2], 4);
        oct = std::min(std::max(oct, 1u), 6u);
        const float sum_scale = 2.0f * (1.0f - std::ldexp(1.0f, -int(oct)));
        widen(std::abs(n.params[0]) * sum_scale);
        return true;
    }
    if (n.op == 6 || n.op == 7) {   // twist about y / bend about x: a cylinder around the axis
        const int u = (n.op == 6) ? 0 : 1, w = 2, keep = (n.op == 6) ? 1 : 0;
        const float ru = std::max(std::abs(an[u]), std::abs(ax[u]));
        const float rw = std::max(std::abs(an[w]), std::abs(ax[w]));
        const float r = std::sqrt(ru * ru + rw * rw);
        mn[u] = -r; mx[u] = r;
        mn[w] = -r; mx[w] = r;
        mn[keep] = an[keep]; mx[keep] = ax[keep];
        return true;
    }
    if (n.op == 8 || n.op == 9) {   // repetition: unbounded (1000 m), or the limited cells' span
        uint32_t packed = 0;
        std::memcpy(&packed, &n.params[3], 4);
        const int lim[3] = {int(packed & 0x3FFu), int((packed >> 10) & 0x3FFu), int((packed >> 20) & 0x3FFu)};
        for (int j = 0; j < 3; ++j) {
            if (n.params[j] > 1e-6f) {
                if (n.op == 8) {
                    mn[j] = -1000.0f;
                    mx[j] = 1000.0f;
                } else {
                    const float span = float(lim[j]) * n.params[j];
                    mn[j] = an[j] - span;
                    mx[j] = ax[j] + span;
                }
            } else {
                mn[j] = an[j];
                mx[j] = ax[j];
            }
        }
        return true;
    }
    if (n.op > 3) return false;
    if (!sdf_node_box(c, n.b, bn, bx, depth + 1)) return false;
    if (n.op == 2) {   // subtract: a's box
        for (int j = 0; j < 3; ++j) { mn[j] = an[j]; mx[j] = ax[j]; }
    } else {
        bool disjoint = false;
        for (int j = 0; j < 3; ++j) {
            if (n.op == 1) {
                mn[j] = std::min(an[j], bn[j]);
                mx[j] = std::max(ax[j], bx[j]);
            } else {
                mn[j] = std::max(an[j], bn[j]);
                mx[j] = std::min(ax[j], bx[j]);
                if (mn[j] > mx[j]) disjoint = true;
            }
        }
        if (disjoint)   // an empty intersection keeps the union box
            for (int j = 0; j < 3; ++j) {
                mn[j] = std::min(an[j], bn[j]);
                mx[j] = std::max(ax[j], bx[j]);
            }
    }
    widen(std::max(0.0f, n.params[0]));
    return true;
}

bool sdf_box(SdfClusterH& c) {
    if (c.count == 0 || c.count > 8) return false;
    return sdf_node_box(c, c.count - 1u, c.lo, c.hi);
}

}  // namespace

extern "C" {

int pt_scene_sdf_leaf(pt_scene* s, uint32_t id, uint32_t shape, const float params[4], float x, float y,
                      float z, uint32_t material, float r, float g, float b) {
    if (!s || !params) return PT_ERR_INVALID;
    if (material > 2u) return fail(s, "sdf: material must be 0, 1 or 2");
    if (shape > 8u || shape == 5u)
        return fail(s, "sdf: shape must be 0..4 (sphere, box, rounded box, torus, capsule) or 6..8 (fractals)");
    if (shape >= 6u && params[0] < 0.0f) return fail(s, "sdf: fractal power/scale must be >= 0");
    if (shape == 2u && (!(params[0] > 0.0f) || !(params[1] > 0.0f) || !(params[2] > 0.0f) || params[3] < 0.0f))
        return fail(s, "sdf_round_box: half-extents must be > 0 and corner_r >= 0");
    SdfClusterH c{};
    c.count = 1;
    c.material = material;
    c.albedo[0] = r; c.albedo[1] = g; c.albedo[2] = b;
    SdfNodeH& n = c.nodes[0];
    n.op = 0;
    n.shape = shape;
    for (int k = 0; k < 4; ++k) n.params[k] = params[k];
    n.center[0] = x; n.center[1] = y; n.center[2] = z;
    if (!sdf_box(c)) return fail(s, "sdf: degenerate parameters");
    s->sdf[id] = c;
    return PT_OK;
}

int pt_scene_sdf_combine(pt_scene* s, uint32_t id, uint32_t a, uint32_t b, uint32_t op, float k, uint32_t material,
                         float r, float g, float bl) {
    if (!s) return PT_ERR_INVALID;
    if (op < 1u || op > 3u) return fail(s, "sdf: op must be 1 (union), 2 (subtract) or 3 (intersect)");
    if (material > 2u) return fail(s, "sdf: material must be 0, 1 or 2");
    if (a == b) return fail(s, "sdf: the two children must differ");
    auto ia = s->sdf.find(a), ib = s->sdf.find(b);
    if (ia == s->sdf.end() || ib == s->sdf.end()) return fail(s, "sdf: child cluster not found");
    const SdfClusterH A = ia->second, B = ib->second;
    for (const SdfClusterH* X : {&A, &B})
        for (uint32_t i = 0; i < X->count; ++i)
            if (X->nodes[i].op == 0u && X->nodes[i].shape >= 6u)
                return fail(s, "sdf: fractal leaves cannot take part in smooth operations");
    if (A.count + B.count + 1u > 8u) return fail(s, "sdf: more than 8 nodes");
    SdfClusterH c{};
    for (uint32_t i = 0; i < A.count; ++i) c.nodes[i] = A.nodes[i];
    for (uint32_t i = 0; i < B.count; ++i) {
        SdfNodeH nb = B.nodes[i];
        if (nb.op != 0u) {
            nb.a += A.count;
            nb.b += A.count;
        }
        c.nodes[A.count + i] = nb;
    }
    SdfNodeH& o = c.nodes[A.count + B.count];
    o.op = op;
    o.a = A.count - 1u;
    o.b = A.count + B.count - 1u;
    o.params[0] = k;
    c.count = A.count + B.count + 1u;
    c.material = material;
    c.albedo[0] = r; c.albedo[1] = g; c.albedo[2] = bl;
    if (!sdf_box(c)) return fail(s, "sdf: bounding box failed");
    s->sdf.erase(a);
    s->sdf.erase(b);
    s->sdf[id] = c;
    return PT_OK;
}

int pt_scene_sdf_wrap(pt_scene* s, uint32_t id, uint32_t child, uint32_t op, const float* params,
                      uint32_t material, float r, float g, float b) {
    if (!s || !params) return PT_ERR_INVALID;
    if (op < 5u || op > 9u) return fail(s, "sdf: wrap op must be 5 (noise), 6 (twist), 7 (bend), 8 or 9 (repeat)");
    if (material > 2u) return fail(s, "sdf: material must be 0, 1 or 2");
    auto ia = s->sdf.find(child);
    if (ia == s->sdf.end()) return fail(s, "sdf: child cluster not found");
    const SdfClusterH A = ia->second;
    float q[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (op == 5u) {   // amp, freq, octaves (clamped 1..6, stored as the bits of params[2])
        if (!(params[0] > 0.0f) || !(params[1] > 0.0f)) return fail(s, "sdf_displace_noise: amp and freq must be > 0");
        const float oct = std::min(std::max(params[2], 1.0f), 6.0f);
        const uint32_t ou = uint32_t(int(oct));
        q[0] = params[0];
        q[1] = params[1];
        std::memcpy(&q[2], &ou, 4);
    } else if (op == 6u || op == 7u) {
        q[0] = params[0];
    } else {
        for (int k = 0; k < 3; ++k) q[k] = params[k];
        if (op == 9u) {   // half-extents in 10-bit lanes of params[3]
            uint32_t pk = 0;
            for (int k = 0; k < 3; ++k) {
                const float l = params[3 + k];
                if (!(l >= 0.0f && l <= 1023.0f) || l != std::floor(l))
                    return fail(s, "sdf_repeat_limited: limits must be integers in 0..1023");
                pk |= (uint32_t(l) & 0x3FFu) << (10 * k);
            }
            std::memcpy(&q[3], &pk, 4);
        }
    }
    if (op >= 6u)
        for (uint32_t i = 0; i < A.count; ++i)
            if (A.nodes[i].op >= 6u && A.nodes[i].op <= 9u)
                return fail(s, "sdf: the child already contains a warp (a warp applies only at the cluster root)");
    if (A.count + 1u > 8u) return fail(s, "sdf: more than 8 nodes");
    SdfClusterH c{};
    for (uint32_t i = 0; i < A.count; ++i) c.nodes[i] = A.nodes[i];
    SdfNodeH& o = c.nodes[A.count];
    o.op = op;
    o.a = A.count - 1u;
    for (int k = 0; k < 4; ++k) o.params[k] = q[k];
    c.count = A.count + 1u;
    c.material = material;
    c.albedo[0] = r; c.albedo[1] = g; c.albedo[2] = b;
    if (!sdf_box(c)) return fail(s, "sdf: bounding box failed");
    s->sdf.erase(child);
    s->sdf[id] = c;
    return PT_OK;
}

int pt_scene_sdf_remove(pt_scene* s, uint32_t id) {
    if (!s) return PT_ERR_INVALID;
    return s->sdf.erase(id) ? PT_OK : fail(s, "sdf_remove: unknown id");
}

int pt_scene_sdf_clear(pt_scene* s) {
    if (!s) return PT_ERR_INVALID;
    s->sdf.clear();
    return PT_OK;
}

// test hook: the bounding box of a raw cluster (the reference's SdfPrim node
// layout), for pinning against ComputeSdfAabb
int pt_sdf_cluster_box(const float* nodes12, uint32_t count, float* lo, float* hi) {
    if (!nodes12 || !lo || !hi || count == 0 || count > 8) return PT_ERR_INVALID;
    SdfClusterH c{};
    c.count = count;
    for (uint32_t i = 0; i < count; ++i) {
        const float* q = nodes12 + 12 * i;
        std::memcpy(&c.nodes[i].op, q + 0, 4);
        std::memcpy(&c.nodes[i].shape, q + 1, 4);
        std::memcpy(&c.nodes[i].a, q + 2, 4);
        std::memcpy(&c.nodes[i].b, q + 3, 4);
        for (int k = 0; k < 4; ++k) c.nodes[i].params[k] = q[4 + k];
        for (int k = 0; k < 3; ++k) c.nodes[i].center[k] = q[8 + k];
    }
    if (!sdf_box(c)) return PT_ERR_INVALID;
    for (int k = 0; k < 3; ++k) {
        lo[k] = c.lo[k];
        hi[k] = c.hi[k];
    }
    return PT_OK;
}

}  // extern "C"

// ===========================================================================
// Radiance .hdr (RGBE) loader and the .cfg scene-fixture front end.
// ===========================================================================
namespace {

bool read_line(std::FILE* f, std::string& out) {
    out.clear();
    int c;
    while ((c = std::fgetc(f)) != EOF) {
        if (c == '\n') return true;
        out.push_back(char(c));
    }
    return !out.empty();
}

// One scanline of RGBE quadruples: adaptive run-length (marker 2 2 hi lo, then
// each of the 4 components as runs (byte > 128: count - 128 copies of the next
// byte) or literals (byte = count raw bytes)), or flat quadruples otherwise.
bool read_scanline(std::FILE* f, uint32_t width, std::vector<uint8_t>& q) {
    q.assign(size_t(width) * 4, 0);
    if (width < 8 || width > 0x7fff) return std::fread(q.data(), 1, q.size(), f) == q.size();
    uint8_t m[4];
    if (std::fread(m, 1, 4, f) != 4) return false;
    if (m[0] != 2 || m[1] != 2 || (m[2] & 0x80) != 0) {
        std::memcpy(q.data(), m, 4);
        return std::fread(q.data() + 4, 1, q.size() - 4, f) == q.size() - 4;
    }
    if (((uint32_t(m[2]) << 8) | m[3]) != width) return false;
    for (int c = 0; c < 4; ++c) {
        uint32_t x = 0;
        while (x < width) {
            int lead = std::fgetc(f);
            if (lead == EOF) return false;
            const bool run = lead > 128;
            const uint32_t n = run ? uint32_t(lead - 128) : uint32_t(lead);
            if (n == 0 || x + n > width) return false;
            if (run) {
                const int v = std::fgetc(f);
                if (v == EOF) return false;
                for (uint32_t i = 0; i < n; ++i) q[size_t(x + i) * 4 + c] = uint8_t(v);
            } else {
                for (uint32_t i = 0; i < n; ++i) {
                    const int v = std::fgetc(f);
                    if (v == EOF) return false;
                    q[size_t(x + i) * 4 + c] = uint8_t(v);
                }
            }
            x += n;
        }
    }
    return true;
}

bool load_hdr(const char* path, std::vector<float>& rgb, uint32_t& W, uint32_t& H, std::string& why) {
    std::FILE* f = std::fopen(path, "rb");
    if (!f) {
        why = std::string("cannot open ") + path;
        return false;
    }
    std::string line;
    bool ok = read_line(f, line) && (line.find("RADIANCE") != std::string::npos ||
                                      line.find("RGBE") != std::string::npos);
    if (!ok) why = "not a Radiance HDR file";
    while (ok && read_line(f, line)) {
        if (line.empty()) break;
        if (line.rfind("FORMAT=", 0) == 0 && line.substr(7) != "32-bit_rle_rgbe") {
            why = "unsupported FORMAT (only 32-bit_rle_rgbe)";
            ok = false;
        }
    }
    int h = 0, w = 0;
    if (ok && !(read_line(f, line) && std::sscanf(line.c_str(), "-Y %d +X %d", &h, &w) == 2 && w > 0 && h > 0 &&
                uint64_t(w) * uint64_t(h) <= (1ull << 28))) {
        why = "only -Y h +X w resolution lines are supported";
        ok = false;
    }
    if (ok) {
        W = uint32_t(w);
        H = uint32_t(h);
        rgb.assign(size_t(W) * H * 3, 0.0f);
        std::vector<uint8_t> q;
        for (uint32_t y = 0; y < H && ok; ++y) {
            if (!read_scanline(f, W, q)) {
                why = "scanline " + std::to_string(y) + " is truncated or malformed";
                ok = false;
                break;
            }
            float* row = rgb.data() + size_t(y) * W * 3;
            for (uint32_t x = 0; x < W; ++x) {
                const uint8_t* e = q.data() + size_t(x) * 4;
                // the format's value: mantissa * 2^(exponent - 136), zero exponent = black
                const float sc = e[3] ? std::ldexp(1.0f, int(e[3]) - 136) : 0.0f;
                row[3 * x + 0] = float(e[0]) * sc;
                row[3 * x + 1] = float(e[1]) * sc;
                row[3 * x + 2] = float(e[2]) * sc;
            }
        }
    }
    std::fclose(f);
    return ok;
}

bool to_f(const std::string& t, float& v) {
    if (t.empty()) return false;
    char* e = nullptr;
    v = std::strtof(t.c_str(), &e);
    return e && *e == '\0';
}
bool to_u(const std::string& t, uint32_t& v) {
    if (t.empty() || t[0] == '-') return false;
    char* e = nullptr;
    const unsigned long long x = std::strtoull(t.c_str(), &e, 10);
    if (!e || *e != '\0' || x > 0xFFFFFFFFull) return false;
    v = uint32_t(x);
    return true;
}
// lambert / metal / dielectric -> 0 / 1 / 2; water -> -2 (not part of this path); else -1
int to_mat(const std::string& m) {
    if (m == "lambert") return PT_MAT_LAMBERT;
    if (m == "metal") return PT_MAT_METAL;
    if (m == "dielectric") return PT_MAT_DIELECTRIC;
    if (m == "water") return -2;
    return -1;
}

}  // namespace

extern "C" {

int pt_load_radiance_hdr(const char* path, float* rgb, uint32_t capacity_floats, uint32_t* width,
                         uint32_t* height) {
    if (!path || !width || !height) return PT_ERR_INVALID;
    std::vector<float> img;
    uint32_t W = 0, H = 0;
    std::string why;
    if (!load_hdr(path, img, W, H, why)) return PT_ERR_INVALID;
    *width = W;
    *height = H;
    if (rgb) {
        if (capacity_floats < img.size()) return PT_ERR_INVALID;
        std::memcpy(rgb, img.data(), img.size() * sizeof(float));
    }
    return PT_OK;
}

int pt_scene_exec_cfg(pt_scene* s, const char* text, const char* base_dir, char* skipped, size_t skipped_len,
                      uint32_t* n_skipped) {
    if (!s || !text) return PT_ERR_INVALID;
    std::string report, first_error;
    uint32_t nskip = 0, nerr = 0, lineno = 0;
    auto skip = [&](const std::string& line, const char* why) {
        ++nskip;
        report += line + "    # " + why + "\n";
    };
    auto bad = [&](const std::string& line, const std::string& why) {
        ++nerr;
        if (first_error.empty()) first_error = "cfg line " + std::to_string(lineno) + ": " + why + ": " + line;
        report += line + "    # ERROR: " + why + "\n";
    };
    const char* p = text;
    while (*p) {
        const char* e = std::strchr(p, '\n');
        std::string line = e ? std::string(p, size_t(e - p)) : std::string(p);
        p = e ? e + 1 : p + line.size();
        ++lineno;
        const size_t cpos = line.find("//");
        if (cpos != std::string::npos) line.resize(cpos);
        while (!line.empty() && (line.back() == '\r' || line.back() == ' ' || line.back() == '\t')) line.pop_back();
        size_t b = 0;
        while (b < line.size() && (line[b] == ' ' || line[b] == '\t')) ++b;
        line = line.substr(b);
        if (line.empty() || line[0] == '#') continue;
        std::vector<std::string> tok;
        {
            size_t i = 0;
            while (i < line.size()) {
                while (i < line.size() && (line[i] == ' ' || line[i] == '\t')) ++i;
                size_t j = i;
                while (j < line.size() && line[j] != ' ' && line[j] != '\t') ++j;
                if (j > i) tok.push_back(line.substr(i, j - i));
                i = j;
            }
        }
        const std::string& cmd = tok[0];
        const size_t na = tok.size() - 1;
        auto F = [&](size_t k, float& v) { return k < tok.size() && to_f(tok[k], v); };
        auto U = [&](size_t k, uint32_t& v) { return k < tok.size() && to_u(tok[k], v); };
        float f[16] = {0};
        uint32_t id = 0;
        auto floats = [&](size_t first, size_t n) {
            for (size_t k = 0; k < n; ++k)
                if (!F(first + k, f[k])) return false;
            return true;
        };
        auto find_prim = [&](Prim*& pr) {
            if (!U(1, id)) return false;
            auto it = s->prims.find(id);
            if (it == s->prims.end()) return false;
            pr = &it->second;
            return true;
        };
        if (cmd == "prim_sphere" || cmd == "prim_plane") {
            const bool sph = cmd == "prim_sphere";
            if ((sph && (na < 9 || na > 11)) || (!sph && na != 9)) { bad(line, "wrong argument count"); continue; }
            const int m = to_mat(tok[6]);
            if (m == -2) { skip(line, "water material: not part of this path"); continue; }
            float rough = 0.0f, ior = 1.5f;
            if (!U(1, id) || !floats(2, 4) || m < 0 || !F(7, f[4]) || !F(8, f[5]) || !F(9, f[6]) ||
                (na >= 10 && !F(10, rough)) || (na >= 11 && !F(11, ior))) {
                bad(line, "malformed arguments");
                continue;
            }
            const int rc = sph ? pt_scene_prim_sphere(s, id, f[0], f[1], f[2], f[3], m, f[4], f[5], f[6], rough, ior)
                               : pt_scene_prim_plane(s, id, f[0], f[1], f[2], f[3], m, f[4], f[5], f[6], 0.0f, 1.0f);
            if (rc) bad(line, s->err);
        } else if (cmd == "prim_set_albedo" || cmd == "prim_set_emission" || cmd == "prim_set_pos" ||
                   cmd == "prim_set_normal") {
            Prim* pr = nullptr;
            if (na != 4 || !find_prim(pr) || !floats(2, 3)) { bad(line, "malformed arguments or unknown id"); continue; }
            if (cmd == "prim_set_albedo") {
                std::memcpy(pr->albedo, f, 12);
            } else if (cmd == "prim_set_emission") {
                std::memcpy(pr->emission, f, 12);
            } else {
                if (cmd == "prim_set_normal" && pr->type != 1) { bad(line, "not a plane"); continue; }
                if (pr->type == 1) {
                    const float len = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
                    if (len < 1e-6f) { bad(line, "zero-length normal"); continue; }
                    for (int k = 0; k < 3; ++k) f[k] /= len;
                }
                std::memcpy(pr->pos, f, 12);
                std::memcpy(pr->prev, f, 12);
            }
            s->dirty_prims = true;
        } else if (cmd == "prim_set_roughness" || cmd == "prim_set_ior" || cmd == "prim_set_radius" ||
                   cmd == "prim_set_plane_d") {
            Prim* pr = nullptr;
            if (na != 2 || !find_prim(pr) || !F(2, f[0])) { bad(line, "malformed arguments or unknown id"); continue; }
            if (cmd == "prim_set_roughness") {
                pr->roughness = std::min(std::max(f[0], 0.0f), 1.0f);
            } else if (cmd == "prim_set_ior") {
                pr->ior = std::min(std::max(f[0], 1.0f), 2.4f);
            } else if (cmd == "prim_set_radius") {
                if (pr->type != 0 || !(f[0] > 0.0f)) { bad(line, "not a sphere or radius <= 0"); continue; }
                pr->radius_or_d = f[0];
            } else {
                if (pr->type != 1) { bad(line, "not a plane"); continue; }
                pr->radius_or_d = f[0];
            }
            s->dirty_prims = true;
        } else if (cmd == "prim_set_material") {
            Prim* pr = nullptr;
            const int m = na == 2 ? to_mat(tok[2]) : -1;
            if (m == -2) { skip(line, "water material: not part of this path"); continue; }
            if (na != 2 || !find_prim(pr) || m < 0) { bad(line, "malformed arguments or unknown id"); continue; }
            pr->material = uint8_t(m);
            s->dirty_prims = true;
        } else if (cmd == "prim_set_rotation") {
            Prim* pr = nullptr;
            if (na != 5 || !find_prim(pr) || !floats(2, 4)) { bad(line, "malformed arguments or unknown id"); continue; }
            const float mag = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2] + f[3] * f[3]);
            if (mag < 1e-6f) { bad(line, "zero-magnitude quaternion"); continue; }
            const float inv = 1.0f / mag;
            for (int k = 0; k < 4; ++k) pr->orient[k] = f[k] * inv;
            s->dirty_prims = true;
        } else if (cmd == "prim_remove" || cmd == "light_remove") {
            if (na != 1 || !U(1, id)) { bad(line, "malformed id"); continue; }
            if (cmd == "prim_remove") {
                if (!s->prims.erase(id)) { bad(line, "unknown id"); continue; }
                s->dirty_prims = true;
            } else {
                if (!s->lights.erase(id)) { bad(line, "unknown id"); continue; }
                s->dirty_lights = true;
            }
        } else if (cmd == "prim_clear") {
            s->prims.clear();
            s->dirty_prims = true;
        } else if (cmd == "light_clear") {
            s->lights.clear();
            s->dirty_lights = true;
        } else if (cmd == "light_point" || cmd == "light_spot" || cmd == "light_sphere" || cmd == "light_quad") {
            const size_t want = cmd == "light_point" ? 7 : cmd == "light_spot" ? 12 : cmd == "light_sphere" ? 8 : 15;
            if (na != want || !U(1, id) || !floats(2, want - 1)) { bad(line, "malformed arguments"); continue; }
            int rc;
            if (cmd == "light_point") {
                rc = pt_scene_light_point(s, id, f[0], f[1], f[2], f[3], f[4], f[5]);
            } else if (cmd == "light_spot") {
                rc = pt_scene_light_spot(s, id, f[0], f[1], f[2], f[3], f[4], f[5], f[6], f[7], f[8], f[9], f[10]);
            } else if (cmd == "light_sphere") {
                rc = pt_scene_light_sphere(s, id, f[0], f[1], f[2], f[3], f[4], f[5], f[6]);
            } else {
                rc = pt_scene_light_quad(s, id, f[0], f[1], f[2], f[3], f[4], f[5], f[6], f[7], f[8], f[9], f[10],
                                         f[11], f[12], f[13]);
            }
            if (rc) bad(line, s->err);
        } else if (cmd == "sdf_sphere" || cmd == "sdf_box" || cmd == "sdf_round_box" || cmd == "sdf_torus" ||
                   cmd == "sdf_capsule") {
            // params first, then the center (the reference's argument orders)
            const uint32_t shape = cmd == "sdf_sphere" ? 0u : cmd == "sdf_box" ? 1u : cmd == "sdf_round_box" ? 2u
                                 : cmd == "sdf_torus" ? 3u : 4u;
            const size_t np = shape == 0u ? 1 : shape == 1u ? 3 : shape == 2u ? 4 : 2;
            const size_t want = 1 + np + 3 + 1 + 3;
            const int m = na == want ? to_mat(tok[1 + np + 3 + 1]) : -1;
            float prm4[4] = {0, 0, 0, 0};
            if (na != want || !U(1, id) || !floats(2, np + 3) || m < 0) { bad(line, "malformed arguments"); continue; }
            for (size_t k = 0; k < np; ++k) prm4[k] = f[k];
            float rgb[3];
            if (!F(want - 2, rgb[0]) || !F(want - 1, rgb[1]) || !F(want, rgb[2])) { bad(line, "bad colour"); continue; }
            if (pt_scene_sdf_leaf(s, id, shape, prm4, f[np], f[np + 1], f[np + 2], uint32_t(m), rgb[0], rgb[1], rgb[2]))
                bad(line, s->err);
        } else if (cmd == "sdf_smin" || cmd == "sdf_smax" || cmd == "sdf_sdiff") {
            uint32_t a = 0, bb = 0;
            float k = 0.0f;
            const int m = na == 8 ? to_mat(tok[5]) : -1;
            if (na != 8 || !U(1, id) || !U(2, a) || !U(3, bb) || !F(4, k) || m < 0 || !floats(6, 3)) {
                bad(line, "malformed arguments");
                continue;
            }
            const uint32_t op = cmd == "sdf_smin" ? 1u : cmd == "sdf_sdiff" ? 2u : 3u;
            if (pt_scene_sdf_combine(s, id, a, bb, op, k, uint32_t(m), f[0], f[1], f[2])) bad(line, s->err);
        } else if (cmd == "sdf_remove") {
            if (na != 1 || !U(1, id) || pt_scene_sdf_remove(s, id)) { bad(line, "unknown id"); continue; }
        } else if (cmd == "sdf_clear") {
            pt_scene_sdf_clear(s);
        } else if (cmd == "sdf_mandelbulb" || cmd == "sdf_mandelbox" || cmd == "sdf_apollonian") {
            // <id> <power|scale> <bound> <x y z> <material> <r g b>
            const int m = na == 10 ? to_mat(tok[7]) : -1;
            if (na != 10 || !U(1, id) || !floats(2, 5) || m < 0) { bad(line, "malformed arguments"); continue; }
            float rgb[3];
            if (!F(8, rgb[0]) || !F(9, rgb[1]) || !F(10, rgb[2])) { bad(line, "bad colour"); continue; }
            const uint32_t shape = cmd == "sdf_mandelbulb" ? 6u : cmd == "sdf_mandelbox" ? 7u : 8u;
            const float prm4[4] = {f[0], f[1], 0.0f, 0.0f};
            if (pt_scene_sdf_leaf(s, id, shape, prm4, f[2], f[3], f[4], uint32_t(m), rgb[0], rgb[1], rgb[2]))
                bad(line, s->err);
        } else if (cmd == "sdf_displace_noise" || cmd == "sdf_twist" || cmd == "sdf_bend" || cmd == "sdf_repeat" ||
                   cmd == "sdf_repeat_limited") {
            // <id> <child> <op args> <material> <r g b>; displace_noise's octaves are
            // optional (default r_sdf_displace_octaves)
            const uint32_t op = cmd == "sdf_displace_noise" ? 5u : cmd == "sdf_twist" ? 6u : cmd == "sdf_bend" ? 7u
                              : cmd == "sdf_repeat" ? 8u : 9u;
            const size_t nop = op == 5u ? (na == 9 ? 3 : 2) : op <= 7u ? 1 : op == 8u ? 3 : 6;
            const size_t want = 2 + nop + 4;
            uint32_t child = 0;
            const int m = na == want ? to_mat(tok[3 + nop]) : -1;
            if (na != want || !U(1, id) || !U(2, child) || !floats(3, nop) || m < 0) {
                bad(line, "malformed arguments");
                continue;
            }
            float prm[6] = {f[0], f[1], f[2], f[3], f[4], f[5]};
            if (op == 5u && nop == 2) prm[2] = float(s->cvar("r_sdf_displace_octaves"));
            float rgb[3];
            if (!F(want - 2, rgb[0]) || !F(want - 1, rgb[1]) || !F(want, rgb[2])) { bad(line, "bad colour"); continue; }
            if (pt_scene_sdf_wrap(s, id, child, op, prm, uint32_t(m), rgb[0], rgb[1], rgb[2])) bad(line, s->err);
        } else if (cmd.rfind("sdf_", 0) == 0) {
            skip(line, "SDF command outside the path");
        } else if (cmd == "cam_pos") {
            if (na != 3 || !floats(1, 3)) { bad(line, "want x y z"); continue; }
            std::memcpy(s->cam_pos, f, 12);
        } else if (cmd == "cam_yaw" || cmd == "cam_pitch" || cmd == "cam_fov") {
            if (na != 1 || !F(1, f[0])) { bad(line, "want one number"); continue; }
            constexpr float kRad = 0.01745329251994329576923690768489f;
            if (cmd == "cam_yaw") s->cam_yaw = f[0] * kRad;
            else if (cmd == "cam_fov") s->cam_fov = f[0];
            else pt_scene_set_camera(s, s->cam_pos[0], s->cam_pos[1], s->cam_pos[2], s->cam_yaw, f[0] * kRad, s->cam_fov);
        } else if (cmd == "r_sky_mode") {
            const std::string v = na == 1 ? tok[1] : "";
            const int mode = v == "gradient" ? 0 : v == "hdri" ? 1 : v == "procedural" ? 2 : v == "hosek" ? 3 : -1;
            if (mode < 0) { bad(line, "want gradient|hdri|procedural|hosek"); continue; }
            pt_scene_set_cvar(s, "r_sky_mode", mode);
        } else if (cmd == "r_env_map") {
            std::string path = na >= 1 ? line.substr(line.find(tok[1])) : std::string();
            if (path.size() >= 2 && path.front() == '"' && path.back() == '"') path = path.substr(1, path.size() - 2);
            if (path.empty()) {   // r_env_map "" : no env map
                pt_scene_set_env(s, nullptr, 0, 0);
                continue;
            }
            if (path[0] != '/' && base_dir && *base_dir) path = std::string(base_dir) + "/" + path;
            std::vector<float> img;
            uint32_t W = 0, H = 0;
            std::string why;
            if (!load_hdr(path.c_str(), img, W, H, why)) { bad(line, why); continue; }
            pt_scene_set_env(s, img.data(), W, H);
        } else if (cmd == "r_tonemap_op") {
            const std::string v = na == 1 ? tok[1] : "";
            const int op = v == "aces" ? 0 : v == "agx" ? 1 : v == "khronos_pbr_neutral" ? 2 : v == "reinhard" ? 3
                         : v == "linear" ? 4 : -1;
            if (op < 0) { bad(line, "want aces|agx|khronos_pbr_neutral|reinhard|linear"); continue; }
            pt_scene_set_cvar(s, "r_tonemap_op", op);
        } else if (cmd == "r_denoiser") {
            if (na != 1) { bad(line, "want one value"); continue; }
            pt_scene_set_cvar(s, "r_denoiser", (tok[1] == "off" || tok[1] == "0") ? 0.0 : 1.0);
        } else {
            double have = 0.0;
            if (pt_scene_get_cvar(s, cmd.c_str(), &have) == PT_OK) {   // an in-scope numeric cvar
                if (na != 1 || !F(1, f[0])) { bad(line, "want one number"); continue; }
                pt_scene_set_cvar(s, cmd.c_str(), f[0]);
            } else if (cmd.rfind("r_", 0) == 0 || cmd.rfind("app_", 0) == 0 || cmd.rfind("cam_", 0) == 0 ||
                       cmd.rfind("pt_", 0) == 0) {
                skip(line, "setting outside the path tracer's inputs");
            } else {
                skip(line, "command outside this path");
            }
        }
    }
    if (n_skipped) *n_skipped = nskip;
    if (skipped && skipped_len) {
        const size_t n = std::min(report.size(), skipped_len - 1);
        std::memcpy(skipped, report.data(), n);
        skipped[n] = '\0';
    }
    if (nerr) return fail(s, first_error + (nerr > 1 ? " (+" + std::to_string(nerr - 1) + " more)" : ""));
    return PT_OK;
}

int pt_scene_load_cfg(pt_scene* s, const char* path, const char* base_dir, char* skipped, size_t skipped_len,
                      uint32_t* n_skipped) {
    if (!s || !path) return PT_ERR_INVALID;
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return fail(s, std::string("load_cfg: cannot open ") + path);
    std::string text;
    char buf[4096];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
    std::fclose(f);
    std::string dir = base_dir ? std::string(base_dir) : std::string(path);
    if (!base_dir) {
        const size_t slash = dir.find_last_of('/');
        dir = (slash == std::string::npos) ? std::string(".") : dir.substr(0, slash);
    }
    return pt_scene_exec_cfg(s, text.c_str(), dir.c_str(), skipped, skipped_len, n_skipped);
}

}  // extern "C"

extern "C" int pt_build_light_tree(const PtLightInput* lights, uint32_t n, PtLightTreeNode* out, uint32_t* n_nodes) {
    if ((n && (!lights || !out)) || !n_nodes) return PT_ERR_INVALID;
    std::vector<PtLightInput> in(lights, lights + n);
    std::vector<PtLightTreeNode> nodes;
    light_tree_of(in, nodes);
    if (!nodes.empty()) std::memcpy(out, nodes.data(), nodes.size() * sizeof(PtLightTreeNode));
    *n_nodes = uint32_t(nodes.size());
    return PT_OK;
}

// ===========================================================================
// Capture and image comparison (the reference's r_capture_format png|ppm,
// src/engine/CaptureFormat.h, and tools/imgdiff/ImgDiff.h's metrics).
// ===========================================================================
namespace {

uint32_t crc32_of(const uint8_t* p, size_t n, uint32_t crc = 0) {
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? (0xEDB88320u ^ (c >> 1)) : (c >> 1);
            table[i] = c;
        }
        init = true;
    }
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return ~crc;
}

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
    v.push_back(uint8_t(x >> 24));
    v.push_back(uint8_t(x >> 16));
    v.push_back(uint8_t(x >> 8));
    v.push_back(uint8_t(x));
}

void png_chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data) {
    put_be32(out, uint32_t(data.size()));
    std::vector<uint8_t> td(type, type + 4);
    td.insert(td.end(), data.begin(), data.end());
    out.insert(out.end(), td.begin(), td.end());
    put_be32(out, crc32_of(td.data(), td.size()));
}

}  // namespace

extern "C" {

int pt_write_png(const char* path, const uint8_t* rgba8, uint32_t w, uint32_t h) {
    if (!path || !rgba8 || w == 0 || h == 0) return PT_ERR_INVALID;
    // scanlines with filter byte 0, wrapped in a zlib stream of stored deflate blocks
    std::vector<uint8_t> raw;
    raw.reserve(size_t(h) * (size_t(w) * 4 + 1));
    for (uint32_t y = 0; y < h; ++y) {
        raw.push_back(0);
        raw.insert(raw.end(), rgba8 + size_t(y) * w * 4, rgba8 + size_t(y + 1) * w * 4);
    }
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t pos = 0;
    do {
        const size_t n = std::min<size_t>(65535, raw.size() - pos);
        z.push_back((pos + n == raw.size()) ? 1 : 0);
        z.push_back(uint8_t(n));
        z.push_back(uint8_t(n >> 8));
        z.push_back(uint8_t(~n));
        z.push_back(uint8_t(~n >> 8));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
        pos += n;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;   // Adler-32 of the uncompressed data
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put_be32(z, (b << 16) | a);
    std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, w);
    put_be32(ihdr, h);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});   // 8-bit RGBA, deflate, no filter, no interlace
    png_chunk(png, "IHDR", ihdr);
    png_chunk(png, "IDAT", z);
    png_chunk(png, "IEND", {});
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return PT_ERR_INVALID;
    const bool ok = std::fwrite(png.data(), 1, png.size(), f) == png.size();
    return (std::fclose(f) == 0 && ok) ? PT_OK : PT_ERR_INVALID;
}

int pt_write_ppm(const char* path, const uint8_t* rgba8, uint32_t w, uint32_t h) {
    if (!path || !rgba8 || w == 0 || h == 0) return PT_ERR_INVALID;
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return PT_ERR_INVALID;
    std::fprintf(f, "P6\n%u %u\n255\n", w, h);
    std::vector<uint8_t> rgb(size_t(w) * h * 3);
    for (size_t i = 0; i < size_t(w) * h; ++i)
        for (int c = 0; c < 3; ++c) rgb[3 * i + c] = rgba8[4 * i + c];
    const bool ok = std::fwrite(rgb.data(), 1, rgb.size(), f) == rgb.size();
    return (std::fclose(f) == 0 && ok) ? PT_OK : PT_ERR_INVALID;
}

// per-pixel Euclidean distance over the four 8-bit channels; mean, RMS, max and
// the share above bad_threshold; diff (nullable) = the distance as a heat map
int pt_imgdiff(const uint8_t* a, const uint8_t* b, uint32_t w, uint32_t h, double bad_threshold,
               PtDiffStats* out, uint8_t* diff_rgba) {
    if (!a || !b || !out) return PT_ERR_INVALID;
    *out = PtDiffStats{};
    const uint64_t n = uint64_t(w) * h;
    out->total_pixels = n;
    if (n == 0) return PT_OK;
    std::vector<double> dist(n);
    double sum = 0.0, sum2 = 0.0, mx = 0.0;
    uint64_t bad = 0;
    for (uint64_t i = 0; i < n; ++i) {
        int s2 = 0;
        for (int c = 0; c < 4; ++c) {
            const int d = int(a[4 * i + c]) - int(b[4 * i + c]);
            s2 += d * d;
        }
        const double d = std::sqrt(double(s2));
        dist[i] = d;
        sum += d;
        sum2 += d * d;
        mx = std::max(mx, d);
        if (d > bad_threshold) ++bad;
    }
    out->max_delta = mx;
    out->mean_delta = sum / double(n);
    out->rms_delta = std::sqrt(sum2 / double(n));
    out->bad_pixels = bad;
    out->bad_percent = 100.0 * double(bad) / double(n);
    if (diff_rgba) {
        const double scale = mx > 0.0 ? 1.0 / mx : 0.0;
        for (uint64_t i = 0; i < n; ++i) {
            const double t = std::clamp(dist[i] * scale, 0.0, 1.0);
            double r, g, bl;   // black -> purple -> orange -> yellow
            if (t < 0.33) {
                const double u = t / 0.33;
                r = u * 128.0, g = 0.0, bl = u * 192.0;
            } else if (t < 0.66) {
                const double u = (t - 0.33) / 0.33;
                r = 128.0 + u * 127.0, g = u * 80.0, bl = 192.0 * (1.0 - u);
            } else {
                const double u = (t - 0.66) / 0.34;
                r = 255.0, g = 80.0 + u * 175.0, bl = u * 100.0;
            }
            diff_rgba[4 * i + 0] = uint8_t(std::clamp(r, 0.0, 255.0) + 0.5);
            diff_rgba[4 * i + 1] = uint8_t(std::clamp(g, 0.0, 255.0) + 0.5);
            diff_rgba[4 * i + 2] = uint8_t(std::clamp(bl, 0.0, 255.0) + 0.5);
            diff_rgba[4 * i + 3] = 255;
        }
    }
    return PT_OK;
}

}  // extern "C"
