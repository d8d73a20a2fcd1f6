// Device-side math, traversal and sampling for the path-trace wavefront.
//
// Semantics follow shaders/PathTrace.slang and shaders/PathTraceMath.slang
// (citations inline).  Built with -fmad=false and IEEE division/sqrt, so
// every expression rounds exactly as written; sin/cos/atan2/acos/asin/exp/
// log/pow are the polynomial versions below (not libdevice), which makes the
// whole render reproducible bit for bit by a CPU restatement that evaluates
// the same expressions.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ptd {

// ---------------------------------------------------------------------------
// small vector type
// ---------------------------------------------------------------------------
struct V3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 v3(float4 a) { return V3{a.x, a.y, a.z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float length(V3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ V3 normalize(V3 a) {
    const float inv = 1.0f / sqrtf(dot(a, a));
    return a * inv;
}
__device__ __forceinline__ bool any_pos(V3 a) { return a.x > 0.0f || a.y > 0.0f || a.z > 0.0f; }
__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + t * (b - a); }
__device__ __forceinline__ V3 lerp3(V3 a, V3 b, float t) { return a + t * (b - a); }
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
__device__ __forceinline__ float lerpf_(float a, float b, float t) { return a + t * (b - a); }
// HLSL reflect(i, n) = i - 2 dot(n, i) n; refract per the HLSL/GLSL definition.
__device__ __forceinline__ V3 reflect(V3 i, V3 n) { return i - (2.0f * dot(n, i)) * n; }
__device__ __forceinline__ V3 refract(V3 i, V3 n, float eta) {
    const float c = dot(n, i);
    const float k = 1.0f - (eta * eta) * (1.0f - c * c);
    if (k < 0.0f) return {0.0f, 0.0f, 0.0f};
    return eta * i - (eta * c + sqrtf(k)) * n;
}
__device__ __forceinline__ float4 f4(V3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

// ---------------------------------------------------------------------------
// Polynomial transcendentals.  sin/cos: Cody-Waite reduction by pi/2 (3-part
// constant), Taylor series of sin to r^9 and cos to r^10 on |r| <= pi/4.
// atan: Taylor series to w^17 on |w| <= tan(pi/8), atan(z) = pi/4 +
// atan((z-1)/(z+1)) above; acos(x) = atan2(sqrt((1-x)(1+x)), x).
// ---------------------------------------------------------------------------
constexpr float kPio2Hi = 0x1.92p+0f;
constexpr float kPio2Mid = 0x1.fb54p-12f;
constexpr float kPio2Lo = 0x1.10b462p-30f;
constexpr float kTwoOverPi = 0x1.45f306p-1f;
constexpr float kPiF = 0x1.921fb6p+1f;
constexpr float kPio2F = 0x1.921fb6p+0f;
constexpr float kPio4F = 0x1.921fb6p-1f;
constexpr float kTanPi8 = 0x1.a8279ap-2f;
constexpr float kS1 = float(-1.0 / 6.0), kS2 = float(1.0 / 120.0), kS3 = float(-1.0 / 5040.0),
                kS4 = float(1.0 / 362880.0);
constexpr float kC1 = -0.5f, kC2 = float(1.0 / 24.0), kC3 = float(-1.0 / 720.0),
                kC4 = float(1.0 / 40320.0), kC5 = float(-1.0 / 3628800.0);
constexpr float kA1 = float(-1.0 / 3.0), kA2 = float(1.0 / 5.0), kA3 = float(-1.0 / 7.0),
                kA4 = float(1.0 / 9.0), kA5 = float(-1.0 / 11.0), kA6 = float(1.0 / 13.0),
                kA7 = float(-1.0 / 15.0), kA8 = float(1.0 / 17.0);

__device__ __forceinline__ float poly_sin(float r) {
    const float r2 = r * r;
    float p = kS4;
    p = p * r2 + kS3;
    p = p * r2 + kS2;
    p = p * r2 + kS1;
    return r + (r * r2) * p;
}
__device__ __forceinline__ float poly_cos(float r) {
    const float r2 = r * r;
    float q = kC5;
    q = q * r2 + kC4;
    q = q * r2 + kC3;
    q = q * r2 + kC2;
    q = q * r2 + kC1;
    return 1.0f + r2 * q;
}
__device__ __forceinline__ float reduce_pio2(float x, int& quadrant) {
    const float k = rintf(x * kTwoOverPi);
    float r = x - k * kPio2Hi;
    r = r - k * kPio2Mid;
    r = r - k * kPio2Lo;
    quadrant = int(k) & 3;
    return r;
}
__device__ __forceinline__ float f_sin(float x) {
    int q;
    const float r = reduce_pio2(x, q);
    if (q == 0) return poly_sin(r);
    if (q == 1) return poly_cos(r);
    if (q == 2) return -poly_sin(r);
    return -poly_cos(r);
}
__device__ __forceinline__ float f_cos(float x) {
    int q;
    const float r = reduce_pio2(x, q);
    if (q == 0) return poly_cos(r);
    if (q == 1) return -poly_sin(r);
    if (q == 2) return -poly_cos(r);
    return poly_sin(r);
}
__device__ __forceinline__ float atan_poly(float w) {
    const float w2 = w * w;
    float p = kA8;
    p = p * w2 + kA7;
    p = p * w2 + kA6;
    p = p * w2 + kA5;
    p = p * w2 + kA4;
    p = p * w2 + kA3;
    p = p * w2 + kA2;
    p = p * w2 + kA1;
    return w + (w * w2) * p;
}
__device__ __forceinline__ float atan_unit(float z) {
    if (z > kTanPi8) return kPio4F + atan_poly((z - 1.0f) / (z + 1.0f));
    return atan_poly(z);
}
__device__ __forceinline__ float f_atan2(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    if (ax == 0.0f && ay == 0.0f) return (x < 0.0f) ? kPiF : 0.0f;
    const bool swap = ay > ax;
    const float z = swap ? (ax / ay) : (ay / ax);
    float a = atan_unit(z);
    if (swap) a = kPio2F - a;
    if (x < 0.0f) a = kPiF - a;
    if (y < 0.0f) a = -a;
    return a;
}
__device__ __forceinline__ float f_acos(float x) {
    const float s = sqrtf((1.0f - x) * (1.0f + x));
    return f_atan2(s, x);
}

// exp, log, pow, asin (procedural sky).  exp: Cody-Waite reduction by ln 2
// (k = rint(x log2 e), r = x - k ln2_hi - k ln2_lo, |r| <= ln2 / 2) and the
// Taylor series of e^r to degree 8, scaled by 2^k.  log: x = m 2^e with m in
// [sqrt(1/2), sqrt(2)), log m = 2 atanh(s), s = (m - 1) / (m + 1), odd series to
// s^11.  pow(x, y) = exp(y log x) for x > 0.  asin(x) = atan2(x, sqrt(1 - x^2)).
constexpr float kLog2E = 0x1.715476p+0f;
constexpr float kLn2Hi = 0x1.62e4p-1f;            // 16 significant bits: k * hi exact for |k| < 256
constexpr float kLn2Lo = 0x1.7f7d1cp-20f;         // float(ln 2 - hi)
constexpr float kLn2F = 0x1.62e43p-1f;
constexpr float kSqrtHalf = 0x1.6a09e6p-1f;
constexpr float kE2 = 0.5f, kE3 = float(1.0 / 6.0), kE4 = float(1.0 / 24.0), kE5 = float(1.0 / 120.0),
                kE6 = float(1.0 / 720.0), kE7 = float(1.0 / 5040.0), kE8 = float(1.0 / 40320.0);
constexpr float kL3 = float(1.0 / 3.0), kL5 = float(1.0 / 5.0), kL7 = float(1.0 / 7.0), kL9 = float(1.0 / 9.0),
                kL11 = float(1.0 / 11.0);

__device__ __forceinline__ float f_exp(float x) {
    if (!(x < 88.7f)) return (x != x) ? x : __int_as_float(0x7f800000);
    if (x < -103.0f) return 0.0f;
    const float k = rintf(x * kLog2E);
    float r = x - k * kLn2Hi;
    r = r - k * kLn2Lo;
    float p = kE8;
    p = p * r + kE7;
    p = p * r + kE6;
    p = p * r + kE5;
    p = p * r + kE4;
    p = p * r + kE3;
    p = p * r + kE2;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    const int ki = int(k);
    // 2^k in two exact steps (k may leave the normal exponent range)
    const int k1 = ki / 2, k2 = ki - k1;
    return (p * __int_as_float((127 + k1) << 23)) * __int_as_float((127 + k2) << 23);
}
__device__ __forceinline__ float f_log(float x) {
    if (!(x > 0.0f)) return (x == 0.0f) ? __int_as_float(0xff800000) : __int_as_float(0x7fc00000);
    if (x == __int_as_float(0x7f800000)) return x;
    int e;
    float m = frexpf(x, &e);   // x = m 2^e, m in [0.5, 1)
    if (m < kSqrtHalf) {
        m = m * 2.0f;
        e -= 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = kL11;
    p = p * s2 + kL9;
    p = p * s2 + kL7;
    p = p * s2 + kL5;
    p = p * s2 + kL3;
    const float lm = 2.0f * s + (2.0f * s) * (s2 * p);
    return float(e) * kLn2F + lm;
}
__device__ __forceinline__ float f_pow(float x, float y) {
    if (y == 0.0f || x == 1.0f) return 1.0f;
    if (x == 0.0f) return (y > 0.0f) ? 0.0f : __int_as_float(0x7f800000);
    if (x < 0.0f) return __int_as_float(0x7fc00000);
    return f_exp(y * f_log(x));
}
__device__ __forceinline__ float f_asin(float x) {
    const float c = sqrtf((1.0f - x) * (1.0f + x));
    return f_atan2(x, c);
}

// shader literal constants, rounded once to float
constexpr float kPi = float(3.14159265358979);
constexpr float kTwoPi = float(6.28318530717958);
constexpr float kInvPi = float(1.0 / 3.14159265358979);
constexpr float kTwoPiHemi = float(6.28318530718);
constexpr float kInvTwoPiSky = float(1.0 / 6.28318530718);
constexpr float kInvPiSky = float(1.0 / 3.14159265359);
constexpr float kInvTwoPiPdf = float(1.0 / 6.28318530717958);
constexpr float kInvPiPdf = float(1.0 / 3.14159265358979);

// ---------------------------------------------------------------------------
// PCG (shaders/PathTraceMath.slang:16-24)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pcg_hash(uint32_t x) {
    x = x * 747796405u + 2891336453u;
    x = ((x >> ((x >> 28u) + 4u)) ^ x) * 277803737u;
    return (x >> 22u) ^ x;
}
__device__ __forceinline__ float randf(uint32_t& seed) {
    seed = pcg_hash(seed);
    return float(seed & 0x00FFFFFFu) / 16777216.0f;
}

// q * v * q^-1 (shaders/PathTrace.slang:2028-2031)
__device__ __forceinline__ V3 quat_rotate(float4 q, V3 v) {
    const V3 u = v3(q.x, q.y, q.z);
    return v + 2.0f * cross(u, cross(u, v) + q.w * v);
}

// ---------------------------------------------------------------------------
// Scene in HBM
// ---------------------------------------------------------------------------
constexpr uint32_t kMatLambert = 0u, kMatMetal = 1u, kMatDielectric = 2u;
constexpr uint32_t kMiss = 0xFFFFFFFFu;
constexpr uint32_t kTriBit = 1u << 30;
constexpr uint32_t kMergedTri = 1u << 29;   // with kTriBit: the slot is in the merged tree's triangle order
constexpr uint32_t kRefTri = 1u << 28;      // with kTriBit: the slot is in the reference BVH's order (S.tri)
constexpr uint32_t kTraverseCap = 1u << 22;   // loop-iteration cap per query (error word if hit)

struct DScene {
    // analytic records: geo = sphere (centre at shutter 1, radius) / plane (rotated n, d)
    const float4* prim_geo;
    const uint32_t* prim_type;
    const float4* prim_rec;      // 7 float4 per record, the reference packing
    uint32_t prim_count, linear_count;
    const float4* bvh;           // 2 float4 per node (reference 32-byte node)
    uint32_t bvh_nodes;
    // triangles in BVH leaf-slot order: (v0, orig id) (e1, material) (e2, 0)
    const float4* tri;
    uint32_t tri_slots;
    const float4* tri_bvh;
    uint32_t tri_nodes;
    uint32_t tri_enabled;        // bvh_params.z != 0
    uint32_t mesh_has_mat;
    const float4* mats;          // 3 float4 per material
    uint32_t mat_count;
    const uint32_t* prim_mat;    // extension: material-table row per analytic record (nullable)
    const float4* lights;        // 5 float4 per light
    uint32_t light_count;
    const float4* env;           // W*H texels
    const float* marg;
    const float* cond;
    // guide tables of the CDFs (kCdfGuide + 1 entries per array: the marginal,
    // then row by row), or null: cdf_search's bracket for u in [k/K, (k+1)/K)
    const uint32_t* marg_guide;
    const uint32_t* cond_guide;
    uint32_t env_w, env_h;
    uint32_t hdri_count;
    float4 hdri_dir[8];
    float4 hdri_col[8];
    const float4* moon_tex;      // moon surface map (gradient sky), W*H texels, or null
    uint32_t moon_w, moon_h;
    const float4* ltree;         // light tree, 4 float4 per node (LightTreeNode layout)
    uint32_t ltree_nodes;
    const float4* sdf;           // SDF clusters, 28 float4 each (4 header + 8 nodes x 3)
    uint32_t sdf_count, sdf_iters;
    float sdf_eps;
    uint32_t frac_iters;         // fractal leaves: DE iterations, default power, epsilon growth per step
    float frac_power, frac_eps_scale;
    uint32_t sdf_proc;           // 1, 2: evaluate the procedural ops 5-9 (0: they read as empty);
                                 // 2: normals by forward-mode AD unless sdf_nmode says central
    uint32_t sdf_nmode;          // r_sdf_normal_mode: 0 forward-mode AD, 1 central differences
    uint32_t* err;               // error word: bit 0 traversal cap, bit 1 stack overflow
    uint32_t trav_cap;           // loop iterations allowed per query (default kTraverseCap)
    int stack_cap;               // wide-tree traversal stack entries allowed (default and maximum 64)
    // 4-wide SAH trees (128-byte nodes: child boxes SoA, child, count)
    uint32_t use_wide;           // traversal mode: 1 wide SAH trees, 0 the reference BVHs
    uint32_t a_wide, t_wide;     // 1: walk the wide tree for that part
    uint32_t wide_linear;        // records the wide-tree kernels test linearly: the planes when the
                                 // dispatch walks an analytic BVH, else every record (the reference
                                 // scans them all in order when bvh_params.y == 0)
    const float4* a4;            // analytic wide nodes (8 float4 each)
    const float4* a4_geo;        // finite analytic prims in wide-leaf order
    const uint4* a4_meta;        // (record slot, type, tie key, 0)
    const float4* t4;            // mesh wide nodes
    const float4* tri4;          // triangles in wide-leaf order: (v0, orig id) (e1, material) (e2, tie rank)
    // merged 4-wide tree over the triangles and the finite analytic records
    // (record leaves flagged by bit 27 of the first-item field), with its own
    // item orders; walked instead of the two trees when m_wide is set
    uint32_t m_wide;
    const float4* m4;
    const float4* mtri4;
    const float4* ma4_geo;
    const uint4* ma4_meta;
    // the reference BVH leaf (node index) that holds each item, or kMiss for an
    // item no reference leaf holds: triangles in wide-leaf order (t_leaf) and in
    // the merged tree's order (m_leaf), analytic records by record index minus
    // linear_count (a_leaf); null when not built
    const uint32_t* t_leaf;
    const uint32_t* m_leaf;
    const uint32_t* a_leaf;
    // traversal counters of the counting kernel variants (profiling mode 3), or null:
    // [0..7] extension segments, [8..15] shadow segments, each (segments, wide nodes
    // tested, triangles tested, analytic prims tested in wide leaves, linear prims
    // tested, stack pushes, stack pops, -)
    unsigned long long* tcount;
};

// Per-lane traversal counters of the counting variants.
struct TravCount {
    uint32_t seg = 0, nodes = 0, tris = 0, aprims = 0, linear = 0, push = 0, pop = 0;
};
__device__ __forceinline__ void tcount_flush(unsigned long long* out, const TravCount& c) {
    const uint32_t v[7] = {c.seg, c.nodes, c.tris, c.aprims, c.linear, c.push, c.pop};
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        unsigned long long x = v[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
        if ((threadIdx.x & 31) == 0 && x) atomicAdd(out + k, x);
    }
}

struct HitRec {
    float t;
    uint32_t id;
};

// slab test (shaders/PathTrace.slang:2321-2329)
__device__ __forceinline__ bool slab(V3 ro, V3 inv, float4 lo, float4 hi, float tmax) {
    const float t0x = (lo.x - ro.x) * inv.x, t1x = (hi.x - ro.x) * inv.x;
    const float t0y = (lo.y - ro.y) * inv.y, t1y = (hi.y - ro.y) * inv.y;
    const float t0z = (lo.z - ro.z) * inv.z, t1z = (hi.z - ro.z) * inv.z;
    const float tmin = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z));
    const float tmx = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
    return tmx >= fmaxf(tmin, 0.0f) && tmin <= tmax;
}
__device__ __forceinline__ V3 safe_inv(V3 rd) {
    const float sx = (fabsf(rd.x) > 1e-30f) ? rd.x : 1e-30f;
    const float sy = (fabsf(rd.y) > 1e-30f) ? rd.y : 1e-30f;
    const float sz = (fabsf(rd.z) > 1e-30f) ? rd.z : 1e-30f;
    return v3(1.0f / sx, 1.0f / sy, 1.0f / sz);
}

// testAnalyticPrim geometry part (shaders/PathTrace.slang:2066-2161,
// PathTraceMath.slang:194-214).  Updates best t / id on a strictly closer hit.
__device__ __forceinline__ void test_prim(const DScene& S, uint32_t idx, V3 ro, V3 rd, HitRec& h) {
    const float4 g = __ldg(S.prim_geo + idx);
    const uint32_t type = __ldg(S.prim_type + idx);
    float t;
    if (type == 0u) {
        const V3 oc = ro - v3(g);
        const float b = dot(oc, rd);
        const float k = dot(oc, oc) - g.w * g.w;
        float hh = b * b - k;
        if (hh < 0.0f) return;
        hh = sqrtf(hh);
        const float t0 = -b - hh, t1 = -b + hh;
        t = (t0 > 1e-3f) ? t0 : t1;
    } else if (type == 1u) {
        const V3 n = v3(g);
        const float denom = dot(rd, n);
        if (fabsf(denom) < 1e-4f) return;
        t = -(dot(ro, n) + g.w) / denom;
    } else {
        return;
    }
    if (t > 1e-3f && t < h.t) {
        h.t = t;
        h.id = idx;
    }
}

// traceScene closest hit (shaders/PathTrace.slang:2331-2693): planes linearly,
// analytic BVH (stack 32, right child popped first), then the triangle BVH
// (stack 64) which only replaces the analytic hit when strictly closer.
// parts: bit 0 analytic records, bit 1 triangle mesh.
// ---------------------------------------------------------------------------
// SDF clusters (shaders/SdfPrimitives.slang, the reference's default build:
// the phase-1 ops; shaders/PathTrace.slang:2177-2305 for the layout and the
// per-cluster sphere trace).  A cluster is <= 8 nodes evaluated in order,
// leaves at `center` with shape parameters, ops combining earlier nodes.
// ---------------------------------------------------------------------------
constexpr uint32_t kSdfBit = 0x80000000u;      // hit id kind: SDF cluster
constexpr uint32_t kSdfStride = 28u;            // float4 per cluster
constexpr uint32_t kSdfMaxNodes = 8u;

__device__ __forceinline__ float len2(float x, float y) { return sqrtf(x * x + y * y); }
__device__ __forceinline__ float signf(float x) { return (x > 0.0f) ? 1.0f : ((x < 0.0f) ? -1.0f : 0.0f); }

__device__ __forceinline__ float sd_leaf(V3 p, uint32_t shape, float4 q) {
    switch (shape) {
        case 0u: return length(p) - q.x;                                        // sphere
        case 1u:                                                                // box
        case 2u: {                                                              // rounded box
            const V3 d = v3(fabsf(p.x) - q.x, fabsf(p.y) - q.y, fabsf(p.z) - q.z);
            const float o = length(v3(fmaxf(d.x, 0.0f), fmaxf(d.y, 0.0f), fmaxf(d.z, 0.0f))) +
                            fminf(fmaxf(d.x, fmaxf(d.y, d.z)), 0.0f);
            return shape == 1u ? o : o - q.w;
        }
        case 3u: return len2(len2(p.x, p.z) - q.x, p.y) - q.y;               // torus (XZ plane)
        case 4u: {                                                              // capsule along Y
            const float y = clampf(p.y, -q.x, q.x);
            return length(v3(p.x, p.y - y, p.z)) - q.y;
        }
        case 5u: return dot(p, v3(q)) + q.w;                                    // plane
        default: return 1e30f;
    }
}

__device__ __forceinline__ V3 sd_leaf_normal(V3 p, uint32_t shape, float4 q) {
    switch (shape) {
        case 0u: {
            const float l = length(p);
            return l > 1e-12f ? p / l : v3(0.0f, 1.0f, 0.0f);
        }
        case 1u:
        case 2u: {
            const V3 d = v3(fabsf(p.x) - q.x, fabsf(p.y) - q.y, fabsf(p.z) - q.z);
            const V3 sg = v3(signf(p.x), signf(p.y), signf(p.z));
            if (fmaxf(d.x, fmaxf(d.y, d.z)) > 0.0f) {
                const V3 m = v3(fmaxf(d.x, 0.0f), fmaxf(d.y, 0.0f), fmaxf(d.z, 0.0f));
                const float lm = length(m);
                if (lm < 1e-12f) return sg * v3(0.0f, 1.0f, 0.0f);
                return (m / lm) * sg;
            }
            V3 n = v3(0.0f, 0.0f, 0.0f);
            if (d.x > d.y && d.x > d.z) n.x = sg.x;
            else if (d.y > d.z) n.y = sg.y;
            else n.z = sg.z;
            return n;
        }
        case 3u: {
            const float lxz = len2(p.x, p.z);
            if (lxz < 1e-12f) return v3(0.0f, signf(p.y), 0.0f);
            const float k = q.x / lxz;
            const V3 d = p - v3(p.x * k, 0.0f, p.z * k);
            const float ld = length(d);
            return ld > 1e-12f ? d / ld : v3(0.0f, 1.0f, 0.0f);
        }
        case 4u: {
            const float y = clampf(p.y, -q.x, q.x);
            const V3 d = p - v3(0.0f, y, 0.0f);
            const float l = length(d);
            return l > 1e-12f ? d / l : v3(0.0f, 1.0f, 0.0f);
        }
        case 5u: return v3(q);
        default: return v3(0.0f, 1.0f, 0.0f);
    }
}

struct SdfNodeD {
    uint32_t op, shape, a, b;
    float4 q;
    V3 c;
};

__device__ __forceinline__ SdfNodeD sdf_node(const float4* C, uint32_t i) {
    const float4 n0 = __ldg(C + 4u + 3u * i), n1 = __ldg(C + 5u + 3u * i), n2 = __ldg(C + 6u + 3u * i);
    return SdfNodeD{__float_as_uint(n0.x), __float_as_uint(n0.y), __float_as_uint(n0.z), __float_as_uint(n0.w),
                    n1, v3(n2)};
}

// sdfClusterDist: node i's value from its leaf or from earlier nodes
__device__ float sdf_dist(const float4* C, uint32_t count, V3 p) {
    float d[kSdfMaxNodes];
    for (uint32_t i = 0; i < kSdfMaxNodes; ++i) {
        if (i >= count) break;
        const SdfNodeD n = sdf_node(C, i);
        float v;
        if (n.op == 0u) {
            v = sd_leaf(p - n.c, n.shape, n.q);
        } else if (n.op >= 1u && n.op <= 4u) {
            const float da = d[min(n.a, i - 1u)], db = d[min(n.b, i - 1u)], k = n.q.x;
            if (n.op == 1u) {            // smooth union
                if (k <= 0.0f) v = fminf(da, db);
                else {
                    const float h = clampf(0.5f + 0.5f * (db - da) / k, 0.0f, 1.0f);
                    v = lerpf_(db, da, h) - k * h * (1.0f - h);
                }
            } else if (n.op == 2u) {     // smooth subtract
                if (k <= 0.0f) v = fmaxf(da, -db);
                else {
                    const float h = clampf(0.5f - 0.5f * (db + da) / k, 0.0f, 1.0f);
                    v = lerpf_(da, -db, h) + k * h * (1.0f - h);
                }
            } else if (n.op == 3u) {     // smooth intersect
                if (k <= 0.0f) v = fmaxf(da, db);
                else {
                    const float h = clampf(0.5f - 0.5f * (db - da) / k, 0.0f, 1.0f);
                    v = lerpf_(db, da, h) + k * h * (1.0f - h);
                }
            } else {                     // displace
                v = da + k;
            }
        } else {
            v = 1e30f;                   // procedural ops: compiled out of the reference's default build
        }
        d[i] = v;
    }
    return count > 0u ? d[count - 1u] : 1e30f;
}

// sdfClusterNormal: analytic gradients carried through the same node order
__device__ V3 sdf_normal(const float4* C, uint32_t count, V3 p) {
    float d[kSdfMaxNodes];
    V3 g[kSdfMaxNodes];
    for (uint32_t i = 0; i < kSdfMaxNodes; ++i) {
        if (i >= count) break;
        const SdfNodeD n = sdf_node(C, i);
        float v;
        V3 gr;
        if (n.op == 0u) {
            const V3 pl = p - n.c;
            v = sd_leaf(pl, n.shape, n.q);
            gr = sd_leaf_normal(pl, n.shape, n.q);
        } else if (n.op >= 1u && n.op <= 4u) {
            const uint32_t ia = min(n.a, i - 1u), ib = min(n.b, i - 1u);
            const float da = d[ia], db = d[ib], k = n.q.x;
            if (n.op == 1u) {
                if (k <= 0.0f) {
                    v = fminf(da, db);
                    gr = (da < db) ? g[ia] : g[ib];
                } else {
                    const float h = clampf(0.5f + 0.5f * (db - da) / k, 0.0f, 1.0f);
                    v = lerpf_(db, da, h) - k * h * (1.0f - h);
                    gr = normalize(lerp3(g[ib], g[ia], h));
                }
            } else if (n.op == 2u) {
                if (k <= 0.0f) {
                    v = fmaxf(da, -db);
                    gr = (da > -db) ? g[ia] : -g[ib];
                } else {
                    const float h = clampf(0.5f - 0.5f * (db + da) / k, 0.0f, 1.0f);
                    v = lerpf_(da, -db, h) + k * h * (1.0f - h);
                    gr = normalize(lerp3(g[ia], -g[ib], h));
                }
            } else if (n.op == 3u) {
                if (k <= 0.0f) {
                    v = fmaxf(da, db);
                    gr = (da > db) ? g[ia] : g[ib];
                } else {
                    const float h = clampf(0.5f - 0.5f * (db - da) / k, 0.0f, 1.0f);
                    v = lerpf_(db, da, h) + k * h * (1.0f - h);
                    gr = normalize(lerp3(g[ib], g[ia], h));
                }
            } else {
                v = da + k;
                gr = g[ia];
            }
        } else {
            v = 1e30f;
            gr = v3(0.0f, 1.0f, 0.0f);
        }
        d[i] = v;
        g[i] = gr;
    }
    return count > 0u ? g[count - 1u] : v3(0.0f, 1.0f, 0.0f);
}

// ---- procedural ops 5-9 (shaders/SdfPrimitives.slang:504-1245): the
// reference's PT_SDF_PROCEDURAL_OPS=1 build without PT_SDF_AUTODIFF, so the
// normal of a procedural cluster is the 6-tap central difference ----
__device__ __forceinline__ uint32_t sdf_hash32(uint32_t x) {   // sdfHash32 (lowbias32 mixing)
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float sdf_hash3(uint32_t x, uint32_t y, uint32_t z) {   // sdfHash3, in [0, 1)
    uint32_t h = sdf_hash32(x);
    h = sdf_hash32(h ^ y);
    h = sdf_hash32(h ^ z);
    return __uint2float_rn(h) * (1.0f / 4294967296.0f);
}
// lattice cell of an integral float, as a two's-complement word (saturated to int range)
__device__ __forceinline__ uint32_t sdf_cell(float x) {
    return uint32_t(int(fminf(fmaxf(x, -2147483648.0f), 2147483520.0f)));
}
// sdfValueNoise3: quintic-smoothstep trilinear mix of hashed lattice values, and
// (grad non-null) its analytic gradient
__device__ __forceinline__ float sdf_value_noise(V3 p, V3* grad = nullptr) {
    const V3 ip = v3(floorf(p.x), floorf(p.y), floorf(p.z));
    const V3 f = p - ip;
    const uint32_t ix = sdf_cell(ip.x), iy = sdf_cell(ip.y), iz = sdf_cell(ip.z);
    const V3 u = f * f * f * (f * (f * 6.0f - v3(15.0f, 15.0f, 15.0f)) + v3(10.0f, 10.0f, 10.0f));
    const float n000 = sdf_hash3(ix, iy, iz), n100 = sdf_hash3(ix + 1u, iy, iz);
    const float n010 = sdf_hash3(ix, iy + 1u, iz), n110 = sdf_hash3(ix + 1u, iy + 1u, iz);
    const float n001 = sdf_hash3(ix, iy, iz + 1u), n101 = sdf_hash3(ix + 1u, iy, iz + 1u);
    const float n011 = sdf_hash3(ix, iy + 1u, iz + 1u), n111 = sdf_hash3(ix + 1u, iy + 1u, iz + 1u);
    const float k0 = n000, k1 = n100 - n000, k2 = n010 - n000, k3 = n001 - n000;
    const float k4 = n000 - n100 - n010 + n110;
    const float k5 = n000 - n010 - n001 + n011;
    const float k6 = n000 - n100 - n001 + n101;
    const float k7 = -n000 + n100 + n010 + n001 - n110 - n011 - n101 + n111;
    if (grad) {
        const V3 du = 30.0f * f * f * (f * (f - v3(2.0f, 2.0f, 2.0f)) + v3(1.0f, 1.0f, 1.0f));
        *grad = v3(du.x * (k1 + k4 * u.y + k6 * u.z + k7 * u.y * u.z), du.y * (k2 + k4 * u.x + k5 * u.z + k7 * u.x * u.z),
                   du.z * (k3 + k5 * u.y + k6 * u.x + k7 * u.x * u.y));
    }
    return k0 + k1 * u.x + k2 * u.y + k3 * u.z + k4 * u.x * u.y + k5 * u.y * u.z + k6 * u.z * u.x +
           k7 * u.x * u.y * u.z;
}
// sdfFbm3: at most 6 octaves, each re-centred to [-1, 1]; (grad non-null) the
// gradient summed through the octaves
__device__ __forceinline__ float sdf_fbm(V3 p, uint32_t octaves, V3* grad = nullptr) {
    float v = 0.0f, amp = 1.0f, frq = 1.0f;
    V3 g = v3(0.0f, 0.0f, 0.0f);
    const uint32_t o = min(octaves, 6u);
    for (uint32_t i = 0; i < o; ++i) {
        V3 gn;
        const float vn = sdf_value_noise(p * frq, grad ? &gn : nullptr);
        v += amp * (2.0f * vn - 1.0f);
        if (grad) g = g + amp * 2.0f * gn * frq;
        amp *= 0.5f;
        frq *= 2.0f;
    }
    if (grad) *grad = g;
    return v;
}
// sdfClusterDistProcN: the phase-1 walker over nodes [0, nc) plus the fBm
// displacement band; a warp below the root reads as empty (1e30)
__device__ float sdf_dist_proc(const float4* C, uint32_t nc, V3 p) {
    float d[kSdfMaxNodes];
    for (uint32_t i = 0; i < kSdfMaxNodes; ++i) {
        if (i >= nc) break;
        const SdfNodeD n = sdf_node(C, i);
        float v;
        if (n.op == 0u) {
            v = sd_leaf(p - n.c, n.shape, n.q);
        } else if (n.op >= 1u && n.op <= 5u) {
            const float da = d[min(n.a, i - 1u)], db = d[min(n.b, i - 1u)], k = n.q.x;
            if (n.op == 1u) {
                if (k <= 0.0f) v = fminf(da, db);
                else {
                    const float h = clampf(0.5f + 0.5f * (db - da) / k, 0.0f, 1.0f);
                    v = lerpf_(db, da, h) - k * h * (1.0f - h);
                }
            } else if (n.op == 2u) {
                if (k <= 0.0f) v = fmaxf(da, -db);
                else {
                    const float h = clampf(0.5f - 0.5f * (db + da) / k, 0.0f, 1.0f);
                    v = lerpf_(da, -db, h) + k * h * (1.0f - h);
                }
            } else if (n.op == 3u) {
                if (k <= 0.0f) v = fmaxf(da, db);
                else {
                    const float h = clampf(0.5f - 0.5f * (db - da) / k, 0.0f, 1.0f);
                    v = lerpf_(db, da, h) + k * h * (1.0f - h);
                }
            } else if (n.op == 4u) {
                v = da + k;
            } else {   // displace by amp x fBm(freq p), octaves as the bits of params.z
                v = da + k * sdf_fbm(p * n.q.y, __float_as_uint(n.q.z));
            }
        } else {
            v = 1e30f;
        }
        d[i] = v;
    }
    return nc > 0u ? d[nc - 1u] : 1e30f;
}
// sdfClusterDistWarped: a warp at the root moves the point once, then the
// child sub-tree [0, child + 1) is walked; twist and bend halve the distance.
// One walker call for every branch (x 1.0 leaves a distance unchanged).
__device__ float sdf_dist_warped(const float4* C, uint32_t count, V3 p) {
    const SdfNodeD r = sdf_node(C, count > 0u ? count - 1u : 0u);
    V3 q = p;
    uint32_t nc = count;
    float scale = 1.0f;
    if (r.op == 6u) {   // twist about the world y axis
        const float c = f_cos(r.q.x * p.y), s = f_sin(r.q.x * p.y);
        q = v3(c * p.x - s * p.z, p.y, s * p.x + c * p.z);
        scale = 0.5f;
    } else if (r.op == 7u) {   // bend about the world x axis
        const float c = f_cos(r.q.x * p.x), s = f_sin(r.q.x * p.x);
        q = v3(p.x, c * p.y - s * p.z, s * p.y + c * p.z);
        scale = 0.5f;
    } else if (r.op == 8u || r.op == 9u) {   // repetition, unbounded or clamped to +-limit cells
        const uint32_t pk = __float_as_uint(r.q.w);
        const float per[3] = {r.q.x, r.q.y, r.q.z};
        const float lim[3] = {float(pk & 0x3FFu), float((pk >> 10) & 0x3FFu), float((pk >> 20) & 0x3FFu)};
        float w[3] = {p.x, p.y, p.z};
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            if (per[j] > 1e-6f) {
                float idx = roundf(w[j] / per[j]);
                if (r.op == 9u) idx = clampf(idx, -lim[j], lim[j]);
                w[j] = w[j] - per[j] * idx;
            }
        }
        q = v3(w[0], w[1], w[2]);
    }
    if (r.op >= 6u && r.op <= 9u) nc = min(r.a + 1u, kSdfMaxNodes);
    return scale * sdf_dist_proc(C, nc, q);
}
// sdfClusterHasProcedural
__device__ __forceinline__ bool sdf_has_proc(const float4* C, uint32_t count) {
    for (uint32_t i = 0; i < kSdfMaxNodes; ++i) {
        if (i >= count) break;
        const uint32_t op = __float_as_uint(__ldg(C + 4u + 3u * i).x);
        if (op >= 5u && op <= 9u) return true;
    }
    return false;
}
// sdfClusterNormalCentral: 6-tap central differences of step h (the taps in
// a loop, so that the walker is compiled once)
__device__ __noinline__ V3 sdf_normal_central(const float4* C, uint32_t count, V3 p, float h) {
    float d[6];
#pragma unroll 1
    for (int k = 0; k < 6; ++k) {
        const V3 e = v3(k < 2 ? h : 0.0f, (k >> 1) == 1 ? h : 0.0f, k >= 4 ? h : 0.0f);   // axis k / 2
        d[k] = sdf_dist_warped(C, count, (k & 1) ? p - e : p + e);
    }
    const V3 g = v3(d[0] - d[1], d[2] - d[3], d[4] - d[5]);
    const float l = length(g);
    return l > 1e-12f ? g / l : v3(0.0f, 1.0f, 0.0f);
}

// sdfClusterDistDN: the forward-mode AD walker over nodes [0, nc), value and
// gradient per node (smooth ops blend the children's gradients unnormalised)
__device__ V3 sdf_dual_proc(const float4* C, uint32_t nc, V3 p) {
    float vv[kSdfMaxNodes];
    V3 vg[kSdfMaxNodes];
    for (uint32_t i = 0; i < kSdfMaxNodes; ++i) {
        if (i >= nc) break;
        const SdfNodeD n = sdf_node(C, i);
        float rv;
        V3 rg;
        if (n.op == 0u) {
            const V3 pl = p - n.c;
            rv = sd_leaf(pl, n.shape, n.q);
            rg = sd_leaf_normal(pl, n.shape, n.q);
        } else if (n.op >= 1u && n.op <= 5u) {
            const uint32_t ia = min(n.a, i - 1u), ib = min(n.b, i - 1u);
            const float av = vv[ia], bv = vv[ib], k = n.q.x;
            const V3 ag = vg[ia], bg = vg[ib];
            if (n.op == 1u) {
                if (k <= 0.0f) {
                    rv = (av < bv) ? av : bv;
                    rg = (av < bv) ? ag : bg;
                } else {
                    const float h = clampf(0.5f + 0.5f * (bv - av) / k, 0.0f, 1.0f);
                    rv = lerpf_(bv, av, h) - k * h * (1.0f - h);
                    rg = lerp3(bg, ag, h);
                }
            } else if (n.op == 2u) {
                if (k <= 0.0f) {
                    rv = fmaxf(av, -bv);
                    rg = (av > -bv) ? ag : -bg;
                } else {
                    const float h = clampf(0.5f - 0.5f * (bv + av) / k, 0.0f, 1.0f);
                    rv = lerpf_(av, -bv, h) + k * h * (1.0f - h);
                    rg = lerp3(ag, -bg, h);
                }
            } else if (n.op == 3u) {
                if (k <= 0.0f) {
                    rv = (av > bv) ? av : bv;
                    rg = (av > bv) ? ag : bg;
                } else {
                    const float h = clampf(0.5f - 0.5f * (bv - av) / k, 0.0f, 1.0f);
                    rv = lerpf_(bv, av, h) + k * h * (1.0f - h);
                    rg = lerp3(bg, ag, h);
                }
            } else if (n.op == 4u) {
                rv = av + k;
                rg = ag;
            } else {   // sdfDisplaceNoiseBand: amp fBm(freq p), gradient amp freq fBm'
                V3 fg;
                const float fv = sdf_fbm(p * n.q.y, __float_as_uint(n.q.z), &fg);
                rv = av + k * fv;
                rg = ag + k * n.q.y * fg;
            }
        } else {
            rv = 1e30f;
            rg = v3(0.0f, 1.0f, 0.0f);
        }
        vv[i] = rv;
        vg[i] = rg;
    }
    return nc > 0u ? vg[nc - 1u] : v3(0.0f, 1.0f, 0.0f);
}
// sdfClusterNormalForwardAD: the AD gradient at the warped point, mapped back
// through the root warp's Jacobian (transposed), normalised
__device__ __noinline__ V3 sdf_normal_ad(const float4* C, uint32_t count, V3 p) {
    const SdfNodeD r = sdf_node(C, count > 0u ? count - 1u : 0u);
    const uint32_t nc = (r.op >= 6u && r.op <= 9u) ? min(r.a + 1u, kSdfMaxNodes) : count;
    const float rate = r.q.x;
    V3 g;
    if (r.op == 6u) {   // twist: q = (c x - s z, y, s x + c z), c, s of rate y
        const float c = f_cos(rate * p.y), s = f_sin(rate * p.y);
        const V3 d = sdf_dual_proc(C, nc, v3(c * p.x - s * p.z, p.y, s * p.x + c * p.z));
        g = v3(c * d.x + s * d.z, -rate * (s * p.x + c * p.z) * d.x + d.y + rate * (c * p.x - s * p.z) * d.z,
               -s * d.x + c * d.z);
    } else if (r.op == 7u) {   // bend: q = (x, c y - s z, s y + c z), c, s of rate x
        const float c = f_cos(rate * p.x), s = f_sin(rate * p.x);
        const V3 d = sdf_dual_proc(C, nc, v3(p.x, c * p.y - s * p.z, s * p.y + c * p.z));
        g = v3(d.x + (-rate * (s * p.y + c * p.z)) * d.y + (rate * (c * p.y - s * p.z)) * d.z, c * d.y + s * d.z,
               -s * d.y + c * d.z);
    } else if (r.op == 8u || r.op == 9u) {   // repetition: identity Jacobian between cell edges
        const uint32_t pk = __float_as_uint(r.q.w);
        const float per[3] = {r.q.x, r.q.y, r.q.z};
        const float lim[3] = {float(pk & 0x3FFu), float((pk >> 10) & 0x3FFu), float((pk >> 20) & 0x3FFu)};
        float w[3] = {p.x, p.y, p.z};
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            if (per[j] > 1e-6f) {
                float idx = roundf(w[j] / per[j]);
                if (r.op == 9u) idx = clampf(idx, -lim[j], lim[j]);
                w[j] = w[j] - per[j] * idx;
            }
        }
        g = sdf_dual_proc(C, nc, v3(w[0], w[1], w[2]));
    } else {
        g = sdf_dual_proc(C, nc, p);
    }
    const float l = length(g);
    return l > 1e-12f ? g / l : v3(0.0f, 1.0f, 0.0f);
}

// (Proc: the procedural walker, for clusters holding ops 5-9 when they are enabled)
template <bool Proc>
__device__ bool sdf_trace(const DScene& S, const float4* C, V3 ro, V3 rd, float t_min, float t_max, float& out_t) {
    const float4 h0 = __ldg(C), h1 = __ldg(C + 1);
    const uint32_t count = __float_as_uint(h0.w);
    const V3 rs = v3(fabsf(rd.x) > 1e-30f ? rd.x : 1e-30f, fabsf(rd.y) > 1e-30f ? rd.y : 1e-30f,
                     fabsf(rd.z) > 1e-30f ? rd.z : 1e-30f);
    const V3 ri = v3(1.0f / rs.x, 1.0f / rs.y, 1.0f / rs.z);
    const V3 t0 = (v3(h0) - ro) * ri, t1 = (v3(h1) - ro) * ri;
    const float enter = fmaxf(fmaxf(fminf(t0.x, t1.x), fminf(t0.y, t1.y)), fminf(t0.z, t1.z));
    const float exit = fminf(fminf(fmaxf(t0.x, t1.x), fmaxf(t0.y, t1.y)), fmaxf(t0.z, t1.z));
    float t = fmaxf(enter, t_min);
    const float t_end = fminf(exit, t_max);
    if (t >= t_end) return false;
    const uint32_t iters = min(S.sdf_iters, 256u);
    for (uint32_t i = 0; i < iters; ++i) {
        const V3 p = ro + rd * t;
        const float ad = fabsf(Proc ? sdf_dist_warped(C, count, p) : sdf_dist(C, count, p));
        if (ad < S.sdf_eps) {
            out_t = t;
            return true;
        }
        t += fmaxf(ad, S.sdf_eps);
        if (t >= t_end) return false;
    }
    return false;
}

__device__ __noinline__ bool sdf_trace_proc(const DScene& S, const float4* C, V3 ro, V3 rd, float t_min,
                                               float t_max, float& out_t) {
    return sdf_trace<true>(S, C, ro, rd, t_min, t_max, out_t);
}

// ---- fractal leaves (shaders/SdfFractals.slang): distance estimators ----
__device__ __forceinline__ float fracf(float x) { return x - floorf(x); }

__device__ float de_fractal(V3 p, uint32_t shape, float4 q, float power_default, uint32_t iters) {
    if (shape == 6u) {   // Mandelbulb
        const float power = (q.x > 0.0f) ? q.x : power_default;
        V3 z = p;
        float dr = 1.0f, r = 0.0f;
        for (uint32_t i = 0; i < iters; ++i) {
            r = length(z);
            if (r > 2.0f) break;
            const float theta = f_acos(clampf(z.z / fmaxf(r, 1e-12f), -1.0f, 1.0f));
            const float phi = f_atan2(z.y, z.x);
            dr = f_pow(r, power - 1.0f) * power * dr + 1.0f;
            const float rp = f_pow(r, power);
            const float nt = theta * power, np = phi * power;
            const float sn = f_sin(nt);
            z = v3(sn * f_cos(np), sn * f_sin(np), f_cos(nt)) * rp;
            z = z + p;
        }
        return 0.5f * f_log(fmaxf(r, 1.0001f)) * r / fmaxf(dr, 1e-12f);
    }
    if (shape == 7u) {   // Mandelbox
        const float scale = (q.x != 0.0f) ? q.x : 2.5f;
        V3 z = p;
        float dr = 1.0f;
        for (uint32_t i = 0; i < iters; ++i) {
            z = v3(clampf(z.x, -1.0f, 1.0f) * 2.0f - z.x, clampf(z.y, -1.0f, 1.0f) * 2.0f - z.y,
                   clampf(z.z, -1.0f, 1.0f) * 2.0f - z.z);
            const float r2 = dot(z, z);
            if (r2 < 0.25f) {
                z = z * 4.0f;
                dr = dr * 4.0f;
            } else if (r2 < 1.0f) {
                const float f = 1.0f / r2;
                z = z * f;
                dr = dr * f;
            }
            z = z * scale + p;
            dr = fabsf(scale) * dr + 1.0f;
        }
        return length(z) / fabsf(dr);
    }
    if (shape == 8u) {   // Apollonian gasket
        const float scale = (q.x != 0.0f) ? q.x : 1.3f;
        V3 z = p;
        float dr = 1.0f;
        for (uint32_t i = 0; i < iters; ++i) {
            z = v3(-1.0f + 2.0f * fracf(0.5f * z.x + 0.5f), -1.0f + 2.0f * fracf(0.5f * z.y + 0.5f),
                   -1.0f + 2.0f * fracf(0.5f * z.z + 0.5f));
            const float r2 = dot(z, z);
            const float k = fmaxf(scale / fmaxf(r2, 1e-12f), 1.0f);
            z = z * k;
            dr = dr * k;
        }
        return (0.25f * fabsf(z.y) - 0.001f) / dr;
    }
    return 1e30f;
}

// evalFractalNormal: tetrahedral central differences of step h
__device__ V3 fractal_normal(V3 p, uint32_t shape, float4 q, float power, uint32_t iters, float h) {
    const V3 e1 = v3(1.0f, -1.0f, -1.0f), e2 = v3(-1.0f, -1.0f, 1.0f);
    const V3 e3 = v3(-1.0f, 1.0f, -1.0f), e4 = v3(1.0f, 1.0f, 1.0f);
    const float d1 = de_fractal(p + e1 * h, shape, q, power, iters);
    const float d2 = de_fractal(p + e2 * h, shape, q, power, iters);
    const float d3 = de_fractal(p + e3 * h, shape, q, power, iters);
    const float d4 = de_fractal(p + e4 * h, shape, q, power, iters);
    const V3 n = e1 * d1 + e2 * d2 + e3 * d3 + e4 * d4;
    const float l = length(n);
    return (l > 1e-12f) ? n / l : v3(0.0f, 1.0f, 0.0f);
}

// traceSdfFractal: the cluster box clip, then a march whose hit epsilon grows
// with the step index (the normal's difference step follows it)
__device__ bool fractal_trace(const DScene& S, const float4* C, V3 ro, V3 rd, float t_min, float t_max, float& out_t,
                              uint32_t& out_step) {
    const float4 h0 = __ldg(C), h1 = __ldg(C + 1);
    const SdfNodeD n = sdf_node(C, __float_as_uint(h0.w) - 1u);
    const V3 rs = v3(fabsf(rd.x) > 1e-30f ? rd.x : 1e-30f, fabsf(rd.y) > 1e-30f ? rd.y : 1e-30f,
                     fabsf(rd.z) > 1e-30f ? rd.z : 1e-30f);
    const V3 ri = v3(1.0f / rs.x, 1.0f / rs.y, 1.0f / rs.z);
    const V3 t0 = (v3(h0) - ro) * ri, t1 = (v3(h1) - ro) * ri;
    const float enter = fmaxf(fmaxf(fminf(t0.x, t1.x), fminf(t0.y, t1.y)), fminf(t0.z, t1.z));
    const float exit = fminf(fminf(fmaxf(t0.x, t1.x), fmaxf(t0.y, t1.y)), fmaxf(t0.z, t1.z));
    float t = fmaxf(enter, t_min);
    const float t_end = fminf(exit, t_max);
    if (t >= t_end) return false;
    const uint32_t steps = min(S.sdf_iters, 512u);
    for (uint32_t i = 0; i < steps; ++i) {
        const V3 pl = (ro + rd * t) - n.c;
        const float ad = fabsf(de_fractal(pl, n.shape, n.q, S.frac_power, S.frac_iters));
        const float eps_i = S.sdf_eps * (1.0f + S.frac_eps_scale * float(i));
        if (ad < eps_i) {
            out_t = t;
            out_step = i;
            return true;
        }
        t += fmaxf(ad, S.sdf_eps);
        if (t >= t_end) return false;
    }
    return false;
}

__device__ __forceinline__ bool sdf_is_fractal(const float4* C) {
    const uint32_t count = __float_as_uint(__ldg(C).w);
    if (count == 0u) return false;
    const float4 n0 = __ldg(C + 4u + 3u * (count - 1u));
    return __float_as_uint(n0.x) == 0u && __float_as_uint(n0.y) >= 6u;
}

// traceSdfClusters: every cluster in order, a hit replaces the best only when
// strictly closer (the reference's `t < h.t`).  Fractal hits carry their
// accepted step in bits 20-28 of the id.  Proc false compiles the procedural
// walker out (for launches whose scenes hold no procedural cluster in use).
template <bool Proc = true>
__device__ __forceinline__ void trace_sdf(const DScene& S, V3 ro, V3 rd, float& best_t, uint32_t& best_id) {
    for (uint32_t i = 0; i < S.sdf_count; ++i) {
        const float4* C = S.sdf + size_t(kSdfStride) * i;
        float t;
        if (sdf_is_fractal(C)) {
            uint32_t step = 0;
            if (fractal_trace(S, C, ro, rd, 1e-3f, best_t, t, step) && t < best_t) {
                best_t = t;
                best_id = kSdfBit | (step << 20) | i;
            }
        } else if ((Proc && S.sdf_proc != 0u && sdf_has_proc(C, __float_as_uint(__ldg(C).w))
                        ? sdf_trace_proc(S, C, ro, rd, 1e-3f, best_t, t)
                        : sdf_trace<false>(S, C, ro, rd, 1e-3f, best_t, t)) &&
                   t < best_t) {
            best_t = t;
            best_id = kSdfBit | i;
        }
    }
}

// parts: 1 analytic prims, 4 SDF clusters, 2 triangle mesh (the reference order)
__device__ __noinline__ HitRec trace_closest(const DScene& S, V3 ro, V3 rd, float t_init, uint32_t parts = 7u) {
    HitRec h{t_init, kMiss};
    const uint32_t linear = (parts & 1u) ? S.linear_count : 0u;
    for (uint32_t i = 0; i < linear; ++i) test_prim(S, i, ro, rd, h);
    uint32_t iters = 0;
    if (!(parts & 1u)) {
    } else if (S.bvh_nodes == 0u) {
        for (uint32_t i = linear; i < S.prim_count; ++i) test_prim(S, i, ro, rd, h);
    } else {
        const V3 inv = safe_inv(rd);
        uint32_t stack[32];
        int sp = 0;
        stack[sp++] = 0u;
        while (sp > 0) {
            if (++iters > S.trav_cap) { atomicOr(S.err, 1u); break; }
            const uint32_t idx = stack[--sp];
            const float4 lo = __ldg(S.bvh + 2u * idx), hi = __ldg(S.bvh + 2u * idx + 1u);
            if (!slab(ro, inv, lo, hi, h.t)) continue;
            const uint32_t lf = __float_as_uint(lo.w), cnt = __float_as_uint(hi.w);
            if (cnt > 0u) {
                const uint32_t base = lf + linear;
                for (uint32_t k = 0; k < cnt; ++k) test_prim(S, base + k, ro, rd, h);
            } else if (sp + 2 <= 32) {
                stack[sp++] = lf;
                stack[sp++] = lf + 1u;
            }
        }
    }
    if (parts & 4u) trace_sdf(S, ro, rd, h.t, h.id);
    if ((parts & 2u) && S.tri_enabled != 0u && S.tri_nodes > 0u) {
        float t_mesh = h.t;
        uint32_t slot_hit = 0;
        bool found = false;
        const V3 inv = safe_inv(rd);
        uint32_t stack[64];
        int sp = 0;
        stack[sp++] = 0u;
        while (sp > 0) {
            if (++iters > S.trav_cap) { atomicOr(S.err, 1u); break; }
            const uint32_t idx = stack[--sp];
            const float4 lo = __ldg(S.tri_bvh + 2u * idx), hi = __ldg(S.tri_bvh + 2u * idx + 1u);
            if (!slab(ro, inv, lo, hi, t_mesh)) continue;
            const uint32_t lf = __float_as_uint(lo.w), cnt = __float_as_uint(hi.w);
            if (cnt > 0u) {
                for (uint32_t k = 0; k < cnt; ++k) {
                    const uint32_t slot = lf + k;
                    const float4 a = __ldg(S.tri + 3u * slot);
                    const float4 b = __ldg(S.tri + 3u * slot + 1u);
                    const float4 c = __ldg(S.tri + 3u * slot + 2u);
                    const V3 v0 = v3(a), e1 = v3(b), e2 = v3(c);
                    const V3 pv = cross(rd, e2);
                    const float det = dot(e1, pv);
                    if (fabsf(det) < 1e-8f) continue;
                    const float inv_det = 1.0f / det;
                    const V3 tvec = ro - v0;
                    const float u = dot(tvec, pv) * inv_det;
                    if (u < 0.0f || u > 1.0f) continue;
                    const V3 qv = cross(tvec, e1);
                    const float v = dot(rd, qv) * inv_det;
                    if (v < 0.0f || u + v > 1.0f) continue;
                    const float tt = dot(e2, qv) * inv_det;
                    if (tt > 1e-3f && tt < t_mesh) {
                        found = true;
                        t_mesh = tt;
                        slot_hit = slot;
                    }
                }
            } else if (sp + 2 <= 64) {
                stack[sp++] = lf;
                stack[sp++] = lf + 1u;
            }
        }
        if (found) {
            h.t = t_mesh;
            h.id = kTriBit | slot_hit;   // slot in leaf order; shading reads the record
        }
    }
    return h;
}


// ---------------------------------------------------------------------------
// Wide-tree traversal.  Front-to-back over 4-wide nodes; a popped entry is
// skipped when its entry distance exceeds the current best (ties are still
// visited).  A candidate replaces the best when it is strictly closer, or
// equally close with a lower tie key: the key is the primitive's position in
// the reference's own test order (planes by index, then the analytic BVH
// leaves in right-child-first depth-first order, then the triangle BVH the
// same way), which reproduces the reference's first-tested-wins rule.
// ---------------------------------------------------------------------------
struct Best {
    float t;
    uint32_t key;
    uint32_t id;
};
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kWideStackDev = 64;

__device__ __forceinline__ bool better(float t, uint32_t key, const Best& b) {
    return t < b.t || (t == b.t && key < b.key);
}

__device__ __forceinline__ float isect_geo(uint32_t type, float4 g, V3 ro, V3 rd) {
    if (type == 0u) {
        const V3 oc = ro - v3(g);
        const float b = dot(oc, rd);
        const float k = dot(oc, oc) - g.w * g.w;
        float hh = b * b - k;
        if (hh < 0.0f) return -1.0f;
        hh = sqrtf(hh);
        const float t0 = -b - hh, t1 = -b + hh;
        return (t0 > 1e-3f) ? t0 : t1;
    }
    if (type == 1u) {
        const V3 n = v3(g);
        const float denom = dot(rd, n);
        if (fabsf(denom) < 1e-4f) return -1.0f;
        return -(dot(ro, n) + g.w) / denom;
    }
    return -1.0f;
}

// The reference walk tests an item only when the slab test of the reference
// BVH leaf that holds it passes (shaders/PathTrace.slang:2321-2329, 2408-2433,
// 2592-2636); the leaf's ancestors then pass too, because their boxes contain
// the leaf's and the slab arithmetic is monotonic in the planes.  The wide
// trees' boxes are padded outward, so they can reach an item whose unpadded
// reference leaf the ray only grazes and the reference's rounding rejects (on
// the 256 x 256 analytic scene: one primary ray in about a million, at a box's
// outer edge).  Such a hit is not the reference's.  The persistent kernels then
// trace the segment again with every candidate checked here before it is
// accepted, which finds the closest item the reference walk reaches: the
// reference's answer; trace_wide asks the reference walk itself (reference_hit).
//
// Rounding can empty the slab interval only where the ray's exact passage
// through the leaf box is within rounding of empty: the hit point then lies
// within rounding of a face of the leaf box in an axis where the box is not
// flat, and since the leaf box contains the item's own box, within rounding of
// a face of the item's own box too (the flat axes of the item, a triangle lying
// in a plane of constant x, y or z, are flat or interior for the leaf as well).
// So the leaf is fetched only when the hit point lies within eps of a face of
// the item's own box, eps = 2^-16 (|ro| + |p| + t) per axis, far above the few
// ulps the slab test can lose; everywhere else the hit is the reference's.
// The slab test of the reference leaf that holds item `id` (no pre-filter):
// the check of every candidate while a segment is traced again.
__device__ __forceinline__ bool ref_leaf_slab(const DScene& S, uint32_t id, V3 ro, V3 inv) {
    uint32_t leaf = kMiss;
    const float4* nodes;
    if (id & kTriBit) {
        leaf = __ldg(((id & kMergedTri) ? S.m_leaf : S.t_leaf) + (id & ~(kTriBit | kMergedTri)));
        nodes = S.tri_bvh;
    } else {
        if (S.bvh_nodes == 0u || id < S.linear_count) return true;
        leaf = __ldg(S.a_leaf + (id - S.linear_count));
        nodes = S.bvh;
    }
    if (leaf == kMiss) return false;
    return slab(ro, inv, __ldg(nodes + 2u * leaf), __ldg(nodes + 2u * leaf + 1u), __uint_as_float(0x7F800000u));
}
__device__ __forceinline__ bool near_own_face(float pv, float lo, float hi, float eps) {
    return hi > lo && (pv - lo <= eps || hi - pv <= eps);
}
__device__ __forceinline__ bool ref_leaf_accepts(const DScene& S, uint32_t id, float t, V3 ro, V3 rd, V3 inv) {
    if (id == kMiss || (id & kSdfBit)) return true;
    uint32_t leaf;
    const float4* nodes;
    if (id & kTriBit) {
        // reference-order slots come from the reference walk itself
        if ((id & kRefTri) || S.tri_bvh == nullptr || !(S.t_wide || (id & kMergedTri))) return true;
        const uint32_t p = id & ~(kTriBit | kMergedTri);
        const uint32_t* L = (id & kMergedTri) ? S.m_leaf : S.t_leaf;
        if (L == nullptr) return true;
        // one axis at a time, the next one read only when this one is clear:
        // few registers are live where the traversal state still is
        const float* T = reinterpret_cast<const float*>(((id & kMergedTri) ? S.mtri4 : S.tri4) + 3u * p);
        const float k = 1.52587890625e-5f;   // 2^-16
        bool near = false;
#pragma unroll 1
        for (int a = 0; a < 3 && !near; ++a) {
            const float o = (a == 0) ? ro.x : ((a == 1) ? ro.y : ro.z);
            const float d = (a == 0) ? rd.x : ((a == 1) ? rd.y : rd.z);
            const float v0 = __ldg(T + a), v1 = v0 + __ldg(T + 4 + a), v2 = v0 + __ldg(T + 8 + a);
            const float hp = o + d * t;
            near = near_own_face(hp, fminf(fminf(v0, v1), v2), fmaxf(fmaxf(v0, v1), v2), k * (fabsf(o) + fabsf(hp) + t));
        }
        if (!near) return true;
        leaf = __ldg(L + p);
        nodes = S.tri_bvh;
    } else {
        if (!S.a_wide || S.bvh_nodes == 0u || id < S.linear_count || S.a_leaf == nullptr) return true;
        const float4 g = __ldg(S.prim_geo + id);
        if (__ldg(S.prim_type + id) == 0u) {   // sphere: centre +- radius
            const V3 hp = ro + rd * t;
            const float k = 1.52587890625e-5f;
            const V3 c = v3(g);
            if (!near_own_face(hp.x, c.x - g.w, c.x + g.w, k * (fabsf(ro.x) + fabsf(hp.x) + t)) &&
                !near_own_face(hp.y, c.y - g.w, c.y + g.w, k * (fabsf(ro.y) + fabsf(hp.y) + t)) &&
                !near_own_face(hp.z, c.z - g.w, c.z + g.w, k * (fabsf(ro.z) + fabsf(hp.z) + t)))
                return true;
        }
        leaf = __ldg(S.a_leaf + (id - S.linear_count));
        nodes = S.bvh;
    }
    if (leaf == kMiss) return false;
    return slab(ro, inv, __ldg(nodes + 2u * leaf), __ldg(nodes + 2u * leaf + 1u), __uint_as_float(0x7F800000u));
}
// One leaf of a wide tree: triangles of `tri4` (kTri) or analytic records of
// ageo / ameta.  first_mask selects the first-item field of the leaf code
// (the merged tree keeps its record-leaf flag above it); triangle hits are
// reported as kTriBit | id_tag | slot.
// With refS set (a segment traced again because its first walk ended on a hit
// the reference walk does not reach), a candidate is accepted only when the
// slab test of its reference leaf passes (ref_leaf_slab; inv is the ray's
// safe_inv); with refS null, inv is not read.
template <bool kTri>
__device__ __forceinline__ void wide_leaf(const float4* tri4, const float4* ageo, const uint4* ameta, uint32_t code,
                                          V3 ro, V3 rd, Best& b, uint32_t key_base,
                                          uint32_t first_mask = 0x0FFFFFFFu, uint32_t id_tag = 0u,
                                          const DScene* refS = nullptr, V3 inv = V3{0.0f, 0.0f, 0.0f}) {
    const uint32_t first = code & first_mask;
    const uint32_t cnt = ((code >> 28) & 7u) + 1u;
    for (uint32_t k = 0; k < cnt; ++k) {
        const uint32_t p = first + k;
        if (kTri) {
            const float4 a = __ldg(tri4 + 3u * p);
            const float4 bb = __ldg(tri4 + 3u * p + 1u);
            const float4 c = __ldg(tri4 + 3u * p + 2u);
            const V3 v0 = v3(a), e1 = v3(bb), e2 = v3(c);
            const V3 pv = cross(rd, e2);
            const float det = dot(e1, pv);
            if (fabsf(det) < 1e-8f) continue;
            const float inv_det = 1.0f / det;
            const V3 tvec = ro - v0;
            const float u = dot(tvec, pv) * inv_det;
            if (u < 0.0f || u > 1.0f) continue;
            const V3 qv = cross(tvec, e1);
            const float v = dot(rd, qv) * inv_det;
            if (v < 0.0f || u + v > 1.0f) continue;
            const float tt = dot(e2, qv) * inv_det;
            const uint32_t key = key_base | __float_as_uint(c.w);
            if (tt > 1e-3f && better(tt, key, b) &&
                (refS == nullptr || ref_leaf_slab(*refS, kTriBit | id_tag | p, ro, inv))) {
                b.t = tt;
                b.key = key;
                b.id = kTriBit | id_tag | p;
            }
        } else {
            const float4 g = __ldg(ageo + p);
            const uint4 m = __ldg(ameta + p);
            const float t = isect_geo(m.y, g, ro, rd);
            if (t > 1e-3f && better(t, m.z, b) &&
                (refS == nullptr || ref_leaf_slab(*refS, m.x, ro, inv))) {
                b.t = t;
                b.key = m.z;
                b.id = m.x;
            }
        }
    }
}

// Three-input float max / min (PTX ISA 8.8, sm_100 and later): one ALU
// instruction instead of two; the same selection as nesting fmaxf / fminf.
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// One 4-wide node: test its four child boxes and order the children that pass
// far to near in registers (a 5-exchange sorting network; children that fail
// get -3e38 and sort last), so that pushing them in order leaves the nearest on
// top.  Returns how many passed.  Static indices only: the arrays stay in
// registers.  The slab test uses fma on -ro*inv and widens the interval by 4e-7
// relative: with the outward-padded boxes no true hit can be culled by rounding.
// Each axis's near and far planes are loaded by the ray's direction sign, so
// the entry and exit distances need no per-axis min/max (fma is monotonic in
// the plane, so this picks the same values min/max would).  The acceptance test
// rejects NaN distances, which an empty slot's box can produce.  The node's
// child codes are stored ready to push, and empty slots hold a box no slab test
// accepts, so the last 16 bytes of the node are not loaded.
__device__ __forceinline__ int wide_children(const float4* nodes, uint32_t code, V3 inv, float nx, float ny,
                                             float nz, float best_t, float (&dk)[4], uint32_t (&ck)[4]) {
    // near / far planes by the ray's direction signs: the node is 128-byte
    // aligned, so picking lo (+0) or hi (+16) of an axis is an OR of the address
    const uintptr_t nb = reinterpret_cast<uintptr_t>(nodes + 8u * code);
    const uintptr_t sx = (__float_as_uint(inv.x) >> 31) << 4, sy = (__float_as_uint(inv.y) >> 31) << 4;
    const uintptr_t sz = (__float_as_uint(inv.z) >> 31) << 4;
    const float4 nxv = __ldg(reinterpret_cast<const float4*>(nb | sx));
    const float4 fxv = __ldg(reinterpret_cast<const float4*>(nb | (sx ^ 16u)));
    const float4 nyv = __ldg(reinterpret_cast<const float4*>((nb | sy) + 32u));
    const float4 fyv = __ldg(reinterpret_cast<const float4*>((nb | (sy ^ 16u)) + 32u));
    const float4 nzv = __ldg(reinterpret_cast<const float4*>((nb | sz) + 64u));
    const float4 fzv = __ldg(reinterpret_cast<const float4*>((nb | (sz ^ 16u)) + 64u));
    const uint4 ch = __ldg(reinterpret_cast<const uint4*>(nb + 96u));
    const float lx[4] = {nxv.x, nxv.y, nxv.z, nxv.w}, hx[4] = {fxv.x, fxv.y, fxv.z, fxv.w};
    const float ly[4] = {nyv.x, nyv.y, nyv.z, nyv.w}, hy[4] = {fyv.x, fyv.y, fyv.z, fyv.w};
    const float lz[4] = {nzv.x, nzv.y, nzv.z, nzv.w}, hz[4] = {fzv.x, fzv.y, fzv.z, fzv.w};
    const uint32_t cc[4] = {ch.x, ch.y, ch.z, ch.w};
    int nh = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float t0x = fmaf(lx[k], inv.x, nx), t1x = fmaf(hx[k], inv.x, nx);
        const float t0y = fmaf(ly[k], inv.y, ny), t1y = fmaf(hy[k], inv.y, ny);
        const float t0z = fmaf(lz[k], inv.z, nz), t1z = fmaf(hz[k], inv.z, nz);
        float tmin = fmax3(t0x, t0y, t0z);   // planes already ordered near / far per axis
        float tmx = fmin3(t1x, t1y, t1z);
        tmin = fmaf(-fabsf(tmin), 4e-7f, tmin);
        tmx = fmaf(fabsf(tmx), 4e-7f, tmx);
        const bool ok = tmx >= fmaxf(tmin, 0.0f) && tmin <= best_t;
        dk[k] = ok ? tmin : -3.0e38f;
        ck[k] = cc[k];
        nh += ok ? 1 : 0;
    }
    auto xchg = [&](int a, int c) {
        if (dk[a] < dk[c]) {
            const float td = dk[a];
            dk[a] = dk[c];
            dk[c] = td;
            const uint32_t tc = ck[a];
            ck[a] = ck[c];
            ck[c] = tc;
        }
    };
    xchg(0, 1);
    xchg(2, 3);
    xchg(0, 2);
    xchg(1, 3);
    xchg(1, 2);
    return nh;
}

// Front-to-back walk of one wide tree.  Leaves found while descending are
// postponed until every active lane of the warp holds one (or has run out of
// nodes), so the warp intersects primitives together instead of interleaving
// box and primitive work lane by lane.  Culling never changes the result, only
// the work: the tie keys decide equal distances.
template <bool kTri>
__device__ __forceinline__ void wide_walk(const DScene& S, const float4* nodes, V3 ro, V3 rd, V3 inv,
                                          Best& b, uint32_t key_base, uint32_t& iters, uint32_t* st_code,
                                          float* st_t) {
    const float nx = -ro.x * inv.x, ny = -ro.y * inv.y, nz = -ro.z * inv.z;
    int sp = 1;
    st_code[0] = 0u;
    st_t[0] = -3.0e38f;
    uint32_t leaf = 0u;   // postponed leaf (0 = none; leaf codes always carry kLeafBit)
    while (sp > 0 || leaf) {
        while (sp > 0 && !leaf) {
            if (++iters > S.trav_cap) { atomicOr(S.err, 1u); return; }
            --sp;
            const uint32_t code = st_code[sp];
            if (st_t[sp] > b.t) continue;
            if (code & kLeafBit) {
                leaf = code;
                break;
            }
            float dk[4];
            uint32_t ck[4];
            const int nh = wide_children(nodes, code, inv, nx, ny, nz, b.t, dk, ck);
            if (sp + nh > S.stack_cap) { atomicOr(S.err, 2u); return; }
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (k < nh) {
                    st_t[sp + k] = dk[k];
                    st_code[sp + k] = ck[k];
                }
            sp += nh;
            if (!__any_sync(__activemask(), leaf == 0u && sp > 0)) break;
        }
        if (leaf) {
            wide_leaf<kTri>(S.tri4, S.a4_geo, S.a4_meta, leaf, ro, rd, b, key_base);
            leaf = 0u;
        }
    }
}

// the reference walk's hit, triangle slots flagged as reference order
__device__ __noinline__ HitRec reference_hit(const DScene& S, V3 ro, V3 rd, float t_init) {
    HitRec h = trace_closest(S, ro, rd, t_init, 7u);
    if (h.id != kMiss && !(h.id & kSdfBit) && (h.id & kTriBit)) h.id |= kRefTri;
    return h;
}

// traceScene on the wide trees (analytic part falls back to the reference walk
// when its wide tree is not built).
__device__ __noinline__ HitRec trace_wide(const DScene& S, V3 ro, V3 rd, float t_init) {
    Best b{t_init, 0u, kMiss};
    const uint32_t linear = S.wide_linear;
    for (uint32_t i = 0; i < linear; ++i) {
        const float t = isect_geo(__ldg(S.prim_type + i), __ldg(S.prim_geo + i), ro, rd);
        if (t > 1e-3f && better(t, i, b)) {
            b.t = t;
            b.key = i;
            b.id = i;
        }
    }
    uint32_t iters = 0;
    const V3 inv = safe_inv(rd);
    uint32_t st_code[kWideStackDev];
    float st_t[kWideStackDev];
    if (S.a_wide) {
        wide_walk<false>(S, S.a4, ro, rd, inv, b, 0u, iters, st_code, st_t);
    } else if (S.prim_count > linear) {
        // the reference's own analytic walk (it re-tests the planes: same result)
        const HitRec h = trace_closest(S, ro, rd, t_init, 1u);
        if (h.id != kMiss && better(h.t, h.id, b)) {
            b.t = h.t;
            b.key = h.id;
            b.id = h.id;
        }
    }
    if (S.sdf_count) {
        float t = b.t;
        uint32_t id = kMiss;
        trace_sdf(S, ro, rd, t, id);
        if (id != kMiss) {
            b.t = t;
            b.key = 0x40000000u | (id & 0xFFFFFu);
            b.id = id;
        }
    }
    if (S.tri_enabled != 0u && S.tri_nodes > 0u) {
        if (S.t_wide) {
            wide_walk<true>(S, S.t4, ro, rd, inv, b, 0x80000000u, iters, st_code, st_t);
        } else {
            const HitRec h = trace_closest(S, ro, rd, b.t, 2u);
            if (h.id != kMiss) {
                b.t = h.t;
                b.id = h.id;
            }
        }
    }
    if (!ref_leaf_accepts(S, b.id, b.t, ro, rd, inv)) return reference_hit(S, ro, rd, t_init);
    return HitRec{b.t, b.id};
}

__device__ __forceinline__ HitRec trace_any_mode(const DScene& S, V3 ro, V3 rd, float t_init, bool wide) {
    return wide ? trace_wide(S, ro, rd, t_init) : trace_closest(S, ro, rd, t_init);
}

// Surface attributes of a hit (the HitInfo fields testAnalyticPrim and the
// mesh branch fill in, shaders/PathTrace.slang:2101-2146, 2639-2690).
constexpr uint32_t kNoMat = 0xFFFFFFFFu;

struct Surface {
    V3 normal;
    uint32_t mat;
    V3 albedo;
    float rough;
    float ior;
    V3 emission;
    uint32_t mid;   // material-table row the attributes came from, kNoMat otherwise
};

__device__ __forceinline__ void table_material(const DScene& S, uint32_t m, Surface& s) {
    if (m >= S.mat_count) m = S.mat_count - 1u;
    const float4 m0 = __ldg(S.mats + 3u * m), m1 = __ldg(S.mats + 3u * m + 1u), m2 = __ldg(S.mats + 3u * m + 2u);
    s.albedo = v3(m0);
    s.rough = m0.w;
    s.emission = v3(m1);
    s.ior = m1.w;
    s.mat = uint32_t(m2.x);
    s.mid = m;
}

template <bool Proc = true>
__device__ __forceinline__ Surface surface_at(const DScene& S, V3 ro, V3 rd, HitRec h) {
    Surface s;
    if (h.id & kSdfBit) {   // SDF cluster: header material, normal at the hit point
        const float4* C = S.sdf + size_t(kSdfStride) * (h.id & 0xFFFFFu);
        const float4 h0 = __ldg(C), h1 = __ldg(C + 1), h2 = __ldg(C + 2), h3 = __ldg(C + 3);
        if (sdf_is_fractal(C)) {
            const SdfNodeD n = sdf_node(C, __float_as_uint(h0.w) - 1u);
            const float eps_i = S.sdf_eps * (1.0f + S.frac_eps_scale * float((h.id >> 20) & 0x1FFu));
            const float hh = fmaxf(eps_i * 8.0f, S.sdf_eps * 4.0f);
            s.normal = fractal_normal((ro + rd * h.t) - n.c, n.shape, n.q, S.frac_power, S.frac_iters, hh);
        } else if (Proc && S.sdf_proc != 0u && sdf_has_proc(C, __float_as_uint(h0.w))) {
            if (S.sdf_proc == 2u && S.sdf_nmode == 0u)
                s.normal = sdf_normal_ad(C, __float_as_uint(h0.w), ro + rd * h.t);
            else
                s.normal = sdf_normal_central(C, __float_as_uint(h0.w), ro + rd * h.t, S.sdf_eps);
        } else {
            s.normal = normalize(sdf_normal(C, __float_as_uint(h0.w), ro + rd * h.t));
        }
        s.mat = __float_as_uint(h1.w);
        s.albedo = v3(h2);
        s.rough = h2.w;
        s.ior = h3.x;
        s.emission = v3(0.0f, 0.0f, 0.0f);
        s.mid = kNoMat;
    } else if (h.id & kTriBit) {
        const uint32_t slot = h.id & ~(kTriBit | kMergedTri | kRefTri);
        const float4* T = (h.id & kMergedTri) ? S.mtri4 : ((S.t_wide && !(h.id & kRefTri)) ? S.tri4 : S.tri);
        const float4 b = __ldg(T + 3u * slot + 1u);
        const float4 c = __ldg(T + 3u * slot + 2u);
        s.normal = normalize(cross(v3(b), v3(c)));
        if (S.mesh_has_mat && S.mat_count > 0u) {
            table_material(S, __float_as_uint(b.w), s);
        } else {
            s.mid = kNoMat;
            s.mat = kMatMetal;
            s.albedo = v3(1.00f, 0.85f, 0.45f);
            s.rough = 0.05f;
            s.ior = 1.0f;
            s.emission = v3(0.0f, 0.0f, 0.0f);
        }
    } else {
        const float4 g = __ldg(S.prim_geo + h.id);
        const uint32_t type = __ldg(S.prim_type + h.id);
        if (type == 0u) s.normal = normalize(ro + rd * h.t - v3(g));
        else s.normal = v3(g);
        const uint32_t pm = S.prim_mat ? __ldg(S.prim_mat + h.id) : kNoMat;
        if (pm != kNoMat && S.mat_count > 0u) {
            table_material(S, pm, s);
        } else {
            const float4 r1 = __ldg(S.prim_rec + 7u * h.id + 1u);
            const float4 r2 = __ldg(S.prim_rec + 7u * h.id + 2u);
            const float4 r4 = __ldg(S.prim_rec + 7u * h.id + 4u);
            s.mat = uint32_t(r2.y);
            s.albedo = v3(r1);
            s.rough = r1.w;
            s.ior = r2.z;
            s.emission = v3(r4);
            s.mid = kNoMat;
        }
    }
    return s;
}

// Schlick (shaders/PathTraceMath.slang:73-76)
__device__ __forceinline__ float schlick(float cos_t, float r0) {
    const float m = 1.0f - cos_t;
    return r0 + (1.0f - r0) * m * m * m * m * m;
}

// cosine hemisphere (shaders/PathTraceMath.slang:30-42)
__device__ __forceinline__ V3 cos_hemi(V3 n, uint32_t& seed) {
    const float u1 = randf(seed);
    const float u2 = randf(seed);
    const float r = sqrtf(u1);
    const float phi = kTwoPiHemi * u2;
    const float x = r * f_cos(phi);
    const float y = r * f_sin(phi);
    const float z = sqrtf(fmaxf(0.0f, 1.0f - u1));
    const V3 ax = (fabsf(n.x) > 0.9f) ? v3(0.0f, 1.0f, 0.0f) : v3(1.0f, 0.0f, 0.0f);
    const V3 t = normalize(cross(n, ax));
    const V3 b = cross(n, t);
    return normalize(t * x + b * y + n * z);
}

// transmittance (shaders/PathTrace.slang:5089-5196) with clouds and water off.
// `first` is the closest hit of segment 0 when the caller already traced it
// (first.t < 0: trace it here).  Counts the closest-hit queries made here.
// Each segment's search starts at the segment's own t_max: the reference
// traces an unbounded closest hit and then tests `h.t >= t_max`, and a hit
// beyond t_max only ever leads to "unoccluded", so the bounded search gives the
// same closest hit below t_max and the same answer with fewer nodes visited.
__device__ __forceinline__ V3 transmittance_from(const DScene& S, V3 o, V3 d, float t_max, int kmax,
                                                 HitRec first, uint32_t& segs, bool wide) {
    V3 t = v3(1.0f, 1.0f, 1.0f);
    for (int i = 0; i <= kmax; ++i) {
        HitRec h;
        if (i == 0 && first.t >= 0.0f) {
            h = first;
        } else {
            ++segs;
            h = trace_any_mode(S, o, d, fminf(t_max, 1e30f), wide);
        }
        if (h.id == kMiss || h.t >= t_max) return t;
        const Surface sf = surface_at(S, o, d, h);
        if (sf.mat != kMatDielectric) return v3(0.0f, 0.0f, 0.0f);
        if (i == kmax) return v3(0.0f, 0.0f, 0.0f);
        const float ndi = dot(sf.normal, d);
        const V3 nf = (ndi < 0.0f) ? sf.normal : -sf.normal;
        const float ia = (ndi < 0.0f) ? 1.0f : sf.ior;
        const float ib = (ndi < 0.0f) ? sf.ior : 1.0f;
        const float eta = ia / ib;
        const float cos_i = fabsf(dot(nf, -d));
        const float r0 = ((ia - ib) / (ia + ib)) * ((ia - ib) / (ia + ib));
        const float fr = schlick(cos_i, r0);
        const V3 refr = refract(d, nf, eta);
        if (length(refr) < 1e-3f) return v3(0.0f, 0.0f, 0.0f);
        t = t * ((1.0f - fr) * sf.albedo);
        const float adv = h.t + 1e-3f;
        o = o + d * adv;
        d = normalize(refr);
        t_max = fmaxf(t_max - adv, 0.0f);
    }
    return v3(0.0f, 0.0f, 0.0f);
}

__device__ __forceinline__ V3 transmittance(const DScene& S, V3 o, V3 d, float t_max, int kmax,
                                            uint32_t& segs, bool wide) {
    return transmittance_from(S, o, d, t_max, kmax, HitRec{-1.0f, kMiss}, segs, wide);
}

// ---------------------------------------------------------------------------
// Persistent closest-hit kernel over the wide trees (dynamic ray fetch).
// Each lane holds one ray; when it finishes, the lane takes the next queued
// ray at once (warp-aggregated atomic on a fetch counter) instead of waiting
// for the slowest ray of its warp.  Within a round, the node phase runs while
// any lane still has nodes to descend (lanes that popped a leaf hold it; the
// phase also ends early when only a few lanes still descend and as many are
// idle), then every lane holding a leaf intersects it together, finished lanes
// write their result and idle lanes fetch new rays.  Same hit semantics as
// trace_wide: planes linearly, analytic tree, then the triangle tree.
// ---------------------------------------------------------------------------
constexpr int kPStack = 64;
constexpr int kRefillLanes = 6;   // node phase ends early below this many descending lanes

// Shadow-ray state kept by the lane across the segments of one transmittance
// chain (shaders/PathTrace.slang:5116-5194).
struct ShadowIO {
    float4* sh_o;       // origin + t_max (updated per segment)
    float4* sh_d;       // direction (w: NEE factor, kept)
    float4* sh_tr;      // transmittance result
    int kmax;
    uint4* sh_mats;     // adjoint replay: material-table rows of the dielectrics crossed (<= 4), or null
};

// Batched renders: per-path scene of a queued item (extension rays: item = path;
// shadow rays: item = 3 * path + slot).
struct ItemScenes {
    const DScene* table;        // device array of scene descriptors (batched renders)
    const uint32_t* path_scene; // scene index per path
};

template <bool kShadow, bool kBatch, bool kMats = false, bool kProc = true, bool kCount = false>
__device__ __forceinline__ void persistent_closest(const DScene* S0, ItemScenes isc, const uint32_t* queue,
                                                   uint32_t n, const float4* ray_o, const float4* ray_d,
                                                   float* out_t, uint32_t* out_id, uint32_t* fetch_ctr,
                                                   uint32_t& done, const ShadowIO& io) {
    const uint32_t FULL = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const DScene* Sp = S0;
    bool has_a = false, has_t = false, has_m = false;
    bool active = false, exhausted = false;
    uint32_t item = 0, leaf = 0u, iters = 0;
    int phase = 0, sp = 0;
    const float4* nodes = nullptr;
    V3 ro = v3(0.0f, 0.0f, 0.0f), rd = ro, inv = ro;
    float nx = 0.0f, ny = 0.0f, nz = 0.0f;
    Best b{1e30f, 0u, kMiss};
    uint2 st[kPStack];   // (node code, entry distance bits)
    // transmittance chain state (kShadow)
    V3 trans = v3(1.0f, 1.0f, 1.0f);
    float t_max = 0.0f;
    int seg = 0;
    uint32_t xm[4] = {kNoMat, kNoMat, kNoMat, kNoMat};   // dielectric rows crossed (adjoint)
    TravCount tc;   // counting variants only
    // the segment is being traced again with every candidate checked against
    // its reference leaf (ref_leaf_accepts): its first walk ended on a hit the
    // reference walk does not reach
    bool refmode = false;
    bool redo = false;   // extension rays: the fetch step starts this lane's ray again, in refmode

    // SDF clusters, once the analytic part of the best hit is final
    auto sdf_pass = [&]() {
        float t = b.t;
        uint32_t id = kMiss;
        trace_sdf<kProc>(*Sp, ro, rd, t, id);
        if (id != kMiss) {
            b.t = t;
            b.key = 0x40000000u | (id & 0xFFFFFu);
            b.id = id;
        }
    };
    auto start_segment = [&](bool count) {
        inv = safe_inv(rd);
        nx = -ro.x * inv.x;
        ny = -ro.y * inv.y;
        nz = -ro.z * inv.z;
        // shadow: bounded as in transmittance_from; extension rays: ray_d.w > 0
        // is an initial closest distance (the trace probe's; renders write 0)
        b = Best{kShadow ? fminf(t_max, 1e30f) : (t_max > 0.0f ? t_max : 1e30f), 0u, kMiss};
        const uint32_t linear = Sp->wide_linear;
        const float4* pg = Sp->prim_geo;
        const uint32_t* pty = Sp->prim_type;
        if (kCount && count) {
            tc.seg += 1;
            tc.linear += linear;
        }
        for (uint32_t i = 0; i < linear; ++i) {
            const float t = isect_geo(__ldg(pty + i), __ldg(pg + i), ro, rd);
            if (t > 1e-3f && better(t, i, b)) {
                b.t = t;
                b.key = i;
                b.id = i;
            }
        }
        sp = 0;
        leaf = 0u;
        iters = 0;
        if (has_m) {
            // one walk over the merged tree (no SDF cluster in the dispatch)
            phase = 5;
            nodes = Sp->m4;
            st[0] = make_uint2(0u, __float_as_uint(-3.0e38f));
            sp = 1;
        } else if (has_a) {
            phase = 1;
            nodes = Sp->a4;
            st[0] = make_uint2(0u, __float_as_uint(-3.0e38f));
            sp = 1;
        } else {
            phase = 2;
            nodes = Sp->t4;
            if (Sp->sdf_count) sdf_pass();
            if (has_t) {
                st[0] = make_uint2(0u, __float_as_uint(-3.0e38f));
                sp = 1;
            }
        }
        if (count) ++done;
    };

    for (;;) {
        const bool need = !active && !exhausted && !redo;
        const uint32_t m = __ballot_sync(FULL, need);
        uint32_t base = 0;
        if (m) {
            const int leader = __ffs(m) - 1;
            if (lane == leader) base = atomicAdd(fetch_ctr, uint32_t(__popc(m)));
            base = __shfl_sync(FULL, base, leader);
        }
        if (need || redo) {
            {
                const uint32_t slot = need ? base + uint32_t(__popc(m & ((1u << lane) - 1u))) : 0u;
                if (need && slot >= n) {
                    exhausted = true;
                } else {
                    // a new ray, or (redo) this lane's own ray again
                    if (need) item = queue[slot];
                    if (kBatch) Sp = isc.table + isc.path_scene[kShadow ? item / 3u : item];
                    has_a = Sp->a_wide && Sp->prim_count > Sp->linear_count;
                    has_t = Sp->t_wide && Sp->tri_enabled != 0u && Sp->tri_nodes > 0u;
                    has_m = Sp->m_wide && has_a && has_t;
                    const float4 o = ray_o[item], d = ray_d[item];
                    ro = v3(o);
                    rd = v3(d);
                    if (!kShadow) t_max = d.w;
                    if (kShadow) {
                        t_max = o.w;
                        trans = v3(1.0f, 1.0f, 1.0f);
                        seg = 0;
                        if (kMats) xm[0] = xm[1] = xm[2] = xm[3] = kNoMat;
                    }
                    refmode = redo;
                    start_segment(!redo);
                    redo = false;
                    active = true;
                }
            }
        }
        if (!__any_sync(FULL, active)) break;
        // node phase
        int np = 0;
        for (;;) {
            const bool want = active && leaf == 0u && sp > 0;
            const uint32_t wm = __ballot_sync(FULL, want);
            if (wm == 0u) break;
            // Few lanes still descending and at least as many idle: leave the
            // node phase so that the idle lanes finish their rays and fetch new
            // ones; the descending lanes resume next round with their stacks.
            // Only after 4 rounds, so every descending lane pops at least 4
            // entries per round (progress: the loop cannot spin without work).
            // On the 1080p triangle scene this gave +6% (thresholds 4 to 10
            // lanes within 1% of each other).
            if (++np > 4 && __popc(wm) < kRefillLanes) {
                const uint32_t idle =
                    __ballot_sync(FULL, (!active && !exhausted) || (active && leaf == 0u && sp == 0));
                if (__popc(idle) >= kRefillLanes) break;
            }
            if (!want) continue;
            if (++iters > Sp->trav_cap) {
                atomicOr(Sp->err, 1u);
                sp = 0;
                continue;
            }
            --sp;
            const uint2 top = st[sp];
            const uint32_t code = top.x;
            if (kCount) tc.pop += 1;
            if (__uint_as_float(top.y) > b.t) continue;
            if (code & kLeafBit) {
                leaf = code;
                continue;
            }
            float dk[4];
            uint32_t ck[4];
            const int nh = wide_children(nodes, code, inv, nx, ny, nz, b.t, dk, ck);
            if (kCount) {
                tc.nodes += 1;
                tc.push += uint32_t(nh);
            }
            if (sp + nh > Sp->stack_cap) {
                atomicOr(Sp->err, 2u);
                sp = 0;
                continue;
            }
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (k < nh) st[sp + k] = make_uint2(ck[k], __float_as_uint(dk[k]));
            sp += nh;
        }
        // leaf phase
        if (active && leaf != 0u) {
            const bool rec_leaf = (phase == 1) || (phase == 5 && (leaf & 0x08000000u));
            if (kCount) {
                const uint32_t cnt = ((leaf >> 28) & 7u) + 1u;
                if (rec_leaf) tc.aprims += cnt;
                else tc.tris += cnt;
            }
            const DScene* refS = refmode ? Sp : nullptr;
            if (phase == 5) {
                if (rec_leaf)
                    wide_leaf<false>(Sp->mtri4, Sp->ma4_geo, Sp->ma4_meta, leaf, ro, rd, b, 0u, 0x07FFFFFFu, 0u, refS,
                                     inv);
                else
                    wide_leaf<true>(Sp->mtri4, Sp->ma4_geo, Sp->ma4_meta, leaf, ro, rd, b, 0x80000000u, 0x07FFFFFFu,
                                    kMergedTri, refS, inv);
            } else if (phase == 1) {
                wide_leaf<false>(Sp->tri4, Sp->a4_geo, Sp->a4_meta, leaf, ro, rd, b, 0u, 0x0FFFFFFFu, 0u, refS, inv);
            } else {
                wide_leaf<true>(Sp->tri4, Sp->a4_geo, Sp->a4_meta, leaf, ro, rd, b, 0x80000000u, 0x0FFFFFFFu, 0u, refS,
                                inv);
            }
            leaf = 0u;
        }
        // end of a tree
        if (active && leaf == 0u && sp == 0) {
            if (phase == 1 && Sp->sdf_count) sdf_pass();
            const bool last_tree = !(phase == 1 && has_t);
            if (last_tree && !refmode && !ref_leaf_accepts(*Sp, b.id, b.t, ro, rd, inv)) {
                // a hit the reference walk does not reach: the same segment
                // again, each candidate checked before it is accepted (the
                // segment is not counted twice).  Shadow segments restart in
                // place (their chain state stays in registers); an extension
                // ray is restarted by the fetch step, whose segment set-up it
                // shares, which keeps this kernel's registers as they were.
                if (kShadow) {
                    refmode = true;
                    start_segment(false);
                } else {
                    redo = true;
                    active = false;
                }
            } else if (!last_tree) {
                phase = 2;
                nodes = Sp->t4;
                st[0] = make_uint2(0u, __float_as_uint(-3.0e38f));
                sp = 1;
            } else if (!kShadow) {
                out_t[item] = b.t;
                out_id[item] = b.id;
                active = false;
            } else {
                // transmittance: unoccluded, blocked, or refract and trace the next segment
                bool finished = true;
                if (!(b.id == kMiss || b.t >= t_max)) {
                    const Surface sf = surface_at<kProc>(*Sp, ro, rd, HitRec{b.t, b.id});
                    bool zero = (sf.mat != kMatDielectric) || (seg == io.kmax);
                    if (!zero) {
                        const float ndi = dot(sf.normal, rd);
                        const V3 nf = (ndi < 0.0f) ? sf.normal : -sf.normal;
                        const float ia = (ndi < 0.0f) ? 1.0f : sf.ior;
                        const float ib = (ndi < 0.0f) ? sf.ior : 1.0f;
                        const float eta = ia / ib;
                        const float cos_i = fabsf(dot(nf, -rd));
                        const float r0 = ((ia - ib) / (ia + ib)) * ((ia - ib) / (ia + ib));
                        const float fr = schlick(cos_i, r0);
                        const V3 refr = refract(rd, nf, eta);
                        if (length(refr) < 1e-3f) {
                            zero = true;
                        } else {
                            trans = trans * ((1.0f - fr) * sf.albedo);
                            if (kMats && seg < 4) xm[seg] = sf.mid;
                            const float adv = b.t + 1e-3f;
                            ro = ro + rd * adv;
                            rd = normalize(refr);
                            t_max = fmaxf(t_max - adv, 0.0f);
                            ++seg;
                            refmode = false;
                            start_segment(true);
                            finished = false;
                        }
                    }
                    if (zero) trans = v3(0.0f, 0.0f, 0.0f);
                }
                if (finished) {
                    io.sh_tr[item] = f4(trans, 0.0f);
                    if (kMats && io.sh_mats) io.sh_mats[item] = make_uint4(xm[0], xm[1], xm[2], xm[3]);
                    active = false;
                }
            }
        }
    }
    if (kCount && S0->tcount) tcount_flush(S0->tcount + (kShadow ? 8 : 0), tc);
}

}  // namespace ptd
