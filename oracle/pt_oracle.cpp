// TEST INFRASTRUCTURE ONLY -- CPU oracle of the reference path tracer.
//
// Restates, function by function, the in-scope subset of
// shaders/PathTrace.slang and shaders/PathTraceMath.slang as a scalar
// per-pixel loop (the shader's own structure), templated on the float type.
// Citations are to the reference's files.  Compile with -ffp-contract=off:
// the fp32 instance must round exactly as written.

#include "pt_oracle.h"

#include <atomic>
#include <cmath>
#include <limits>
#include <cstring>
#include <thread>
#include <vector>

namespace orc {

// ---------------------------------------------------------------------------
// Polynomial transcendentals (fp32).  Not libm: both this oracle and the GPU
// kernels evaluate these exact expressions, so their results agree bit for
// bit.  sin/cos: Cody-Waite reduction by pi/2 with a 3-part constant, then the
// Taylor series of sin (to r^9) and cos (to r^10) on |r| <= pi/4.
// atan: Taylor series to w^17 on |w| <= tan(pi/8), with atan(z) =
// pi/4 + atan((z-1)/(z+1)) above that.  acos(x) = atan2(sqrt((1-x)(1+x)), x).
// ---------------------------------------------------------------------------
constexpr float kPio2Hi = 0x1.92p+0f;        // 1.5703125 (8 significant bits)
constexpr float kPio2Mid = 0x1.fb54p-12f;    // next 16 bits of pi/2
constexpr float kPio2Lo = 0x1.10b462p-30f;   // remainder
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

inline float poly_sin(float r) {
    const float r2 = r * r;
    float p = kS4;
    p = p * r2 + kS3;
    p = p * r2 + kS2;
    p = p * r2 + kS1;
    return r + (r * r2) * p;
}
inline float poly_cos(float r) {
    const float r2 = r * r;
    float q = kC5;
    q = q * r2 + kC4;
    q = q * r2 + kC3;
    q = q * r2 + kC2;
    q = q * r2 + kC1;
    return 1.0f + r2 * q;
}
inline float reduce_pio2(float x, int& quadrant) {
    const float k = std::nearbyint(x * kTwoOverPi);
    float r = x - k * kPio2Hi;
    r = r - k * kPio2Mid;
    r = r - k * kPio2Lo;
    quadrant = int(k) & 3;
    return r;
}
inline float f_sin(float x) {
    int q;
    const float r = reduce_pio2(x, q);
    switch (q) {
        case 0: return poly_sin(r);
        case 1: return poly_cos(r);
        case 2: return -poly_sin(r);
        default: return -poly_cos(r);
    }
}
inline float f_cos(float x) {
    int q;
    const float r = reduce_pio2(x, q);
    switch (q) {
        case 0: return poly_cos(r);
        case 1: return -poly_sin(r);
        case 2: return -poly_cos(r);
        default: return poly_sin(r);
    }
}
inline float atan_poly(float w) {
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
inline float atan_unit(float z) {   // 0 <= z <= 1
    if (z > kTanPi8) return kPio4F + atan_poly((z - 1.0f) / (z + 1.0f));
    return atan_poly(z);
}
inline float f_atan2(float y, float x) {
    const float ax = std::fabs(x), ay = std::fabs(y);
    if (ax == 0.0f && ay == 0.0f) return (x < 0.0f) ? kPiF : 0.0f;
    const bool swap = ay > ax;
    const float z = swap ? (ax / ay) : (ay / ax);
    float a = atan_unit(z);
    if (swap) a = kPio2F - a;
    if (x < 0.0f) a = kPiF - a;
    if (y < 0.0f) a = -a;
    return a;
}
inline float f_acos(float x) {
    const float s = std::sqrt((1.0f - x) * (1.0f + x));
    return f_atan2(s, x);
}
inline float bits_f(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
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

inline float f_exp(float x) {
    if (!(x < 88.7f)) return (x != x) ? x : std::numeric_limits<float>::infinity();
    if (x < -103.0f) return 0.0f;
    const float k = std::rint(x * kLog2E);
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
    return (p * bits_f(uint32_t(127 + k1) << 23)) * bits_f(uint32_t(127 + k2) << 23);
}
inline float f_log(float x) {
    if (!(x > 0.0f)) return (x == 0.0f) ? -std::numeric_limits<float>::infinity() : std::numeric_limits<float>::quiet_NaN();
    if (x == std::numeric_limits<float>::infinity()) return x;
    int e;
    float m = std::frexp(x, &e);   // x = m 2^e, m in [0.5, 1)
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
inline float f_pow(float x, float y) {
    if (y == 0.0f || x == 1.0f) return 1.0f;
    if (x == 0.0f) return (y > 0.0f) ? 0.0f : std::numeric_limits<float>::infinity();
    if (x < 0.0f) return std::numeric_limits<float>::quiet_NaN();
    return f_exp(y * f_log(x));
}
inline float f_asin(float x) {
    const float c = std::sqrt((1.0f - x) * (1.0f + x));
    return f_atan2(x, c);
}

template <class R> struct M;
template <> struct M<float> {
    static float sin(float x) { return f_sin(x); }
    static float cos(float x) { return f_cos(x); }
    static float atan2(float y, float x) { return f_atan2(y, x); }
    static float acos(float x) { return f_acos(x); }
    static float exp(float x) { return f_exp(x); }
    static float pow(float x, float y) { return f_pow(x, y); }
    static float asin(float x) { return f_asin(x); }
    static float log(float x) { return f_log(x); }
};
template <> struct M<double> {
    static double sin(double x) { return std::sin(x); }
    static double cos(double x) { return std::cos(x); }
    static double atan2(double y, double x) { return std::atan2(y, x); }
    static double acos(double x) { return std::acos(x); }
    static double exp(double x) { return std::exp(x); }
    static double pow(double x, double y) { return std::pow(x, y); }
    static double asin(double x) { return std::asin(x); }
    static double log(double x) { return std::log(x); }
};

// HLSL min/max return the non-NaN operand (IEEE minNum/maxNum).
template <class R> inline R mn(R a, R b) { return std::fmin(a, b); }
template <class R> inline R mx(R a, R b) { return std::fmax(a, b); }
template <class R> inline R clampv(R v, R lo, R hi) { return mn(mx(v, lo), hi); }

template <class R> struct V3 {
    R x, y, z;
};
template <class R> inline V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> inline R length(V3<R> a) { return std::sqrt(dot(a, a)); }
template <class R> inline V3<R> normalize(V3<R> a) {
    const R inv = R(1) / std::sqrt(dot(a, a));
    return a * inv;
}
template <class R> inline bool any_pos(V3<R> a) { return a.x > R(0) || a.y > R(0) || a.z > R(0); }
template <class R> inline R lerp(R a, R b, R t) { return a + t * (b - a); }
template <class R> inline V3<R> lerp(V3<R> a, V3<R> b, R t) { return a + t * (b - a); }
// HLSL reflect / refract (shaders call reflect(rd, nf), refract(rd, nf, eta))
template <class R> inline V3<R> reflect(V3<R> i, V3<R> n) { return i - (R(2) * dot(n, i)) * n; }
template <class R> inline V3<R> refract(V3<R> i, V3<R> n, R eta) {
    const R c = dot(n, i);
    const R k = R(1) - (eta * eta) * (R(1) - c * c);
    if (k < R(0)) return {R(0), R(0), R(0)};
    return eta * i - (eta * c + std::sqrt(k)) * n;
}
template <class R> inline V3<R> ld3(const float* p) { return {R(p[0]), R(p[1]), R(p[2])}; }
inline uint32_t asuint(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

// shaders/PathTraceMath.slang:16-24
inline uint32_t pcg_hash(uint32_t x) {
    x = x * 747796405u + 2891336453u;
    x = ((x >> ((x >> 28u) + 4u)) ^ x) * 277803737u;
    return (x >> 22u) ^ x;
}
template <class R> inline R randf(uint32_t& seed) {
    seed = pcg_hash(seed);
    return R(seed & 0x00FFFFFFu) / R(16777216.0);
}

// shaders/PathTrace.slang:2028-2031
template <class R> inline V3<R> quat_rotate(const float* q, V3<R> v) {
    const V3<R> u = ld3<R>(q);
    return v + R(2) * cross(u, cross(u, v) + R(q[3]) * v);
}

constexpr uint32_t kMatLambert = 0, kMatMetal = 1, kMatDielectric = 2;
constexpr uint32_t kHitMiss = 0xFFFFFFFFu;

template <class R> struct Hit {
    bool hit = false;
    R t = R(1e30);
    V3<R> normal{R(0), R(1), R(0)};
    uint32_t mat = kMatLambert;
    V3<R> albedo{R(0.5), R(0.5), R(0.5)};
    R roughness = R(0);
    R ior = R(1);
    V3<R> emission{R(0), R(0), R(0)};
    uint32_t id = kHitMiss;   // (0<<30 | record slot) or (1<<30 | triangle)
    uint32_t mid = 0xFFFFFFFFu;   // material-table row of the attributes, if any
};

struct Counters {
    uint64_t rays = 0, nodes = 0, tris = 0, prims = 0, ext = 0, shadow = 0;
    uint64_t ext_nodes = 0, ext_tris = 0, ext_prims = 0;   // extension segments only
    void add(const Counters& o) {
        rays += o.rays; nodes += o.nodes; tris += o.tris; prims += o.prims;
        ext += o.ext; shadow += o.shadow;
        ext_nodes += o.ext_nodes; ext_tris += o.ext_tris; ext_prims += o.ext_prims;
    }
};

// Gradient sink of the adjoint oracle: every radiance contribution of a
// sample is a product of the albedo factors of the Lambert/metal vertices
// before it (including the vertex whose NEE it is) and of the dielectrics its
// shadow ray crossed, so d(contribution)/d(albedo_m) = contribution / albedo_m
// per occurrence of m; an emission term thr*E has d/dE = thr.  Accumulated in
// double, weighted by dLoss/d(sample radiance).
struct AdjSink {
    const float* mats = nullptr;   // 12 floats per row
    uint32_t nmat = 0;
    std::vector<double> g_alb, g_em;   // nmat*3 each
    double w[3] = {0, 0, 0};
    uint32_t vm[64];
    int nv = 0;
    uint32_t xm[16];
    int nx = 0;
    void add(uint32_t m, double c0, double c1, double c2, std::vector<double>& g) {
        g[3 * m + 0] += w[0] * c0;
        g[3 * m + 1] += w[1] * c1;
        g[3 * m + 2] += w[2] * c2;
    }
    template <class V> void contrib(const V& c, bool shadow) {
        auto one = [&](uint32_t m) {
            if (m >= nmat) return;
            const float* a = mats + 12 * size_t(m);
            const double c0 = a[0] > 0.0f ? double(c.x) / double(a[0]) : 0.0;
            const double c1 = a[1] > 0.0f ? double(c.y) / double(a[1]) : 0.0;
            const double c2 = a[2] > 0.0f ? double(c.z) / double(a[2]) : 0.0;
            add(m, c0, c1, c2, g_alb);
        };
        for (int i = 0; i < nv; ++i) one(vm[i]);
        if (shadow)
            for (int i = 0; i < nx; ++i) one(xm[i]);
    }
    template <class V> void emission(const V& thr, uint32_t m) {
        if (m < nmat) add(m, double(thr.x), double(thr.y), double(thr.z), g_em);
    }
};

template <class R> struct Tracer {
    AdjSink* adj = nullptr;
    // ray capture (test hook): the extension ray a sample traces at bounce
    // cap_bounce is written to cap_o / cap_d at float4 slot cap_slot; the path
    // continues, so later samples of the pixel draw from the same seed state as
    // in a render
    float* cap_o = nullptr;
    float* cap_d = nullptr;
    uint32_t cap_bounce = 0;
    size_t cap_slot = 0;
    // sub-pixel jitter of the current frame's sample 0 when the denoiser is on:
    // the push's for the call's first frame, the engine's Halton(2,3) jitter of
    // its own frame index for later ones (set_frame)
    float frame_jx = 0.0f, frame_jy = 0.0f;
    void set_frame(uint32_t frame_index) {
        if (frame_index == P.frame_index) {
            frame_jx = P.halton_jitter[0];
            frame_jy = P.halton_jitter[1];
            return;
        }
        // src/engine/Engine.cpp:8241-8252
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
        frame_jx = radical_inverse(hi, 2u) - 0.5f;
        frame_jy = radical_inverse(hi, 3u) - 0.5f;
    }
    const PtPackedScene& S;
    const PtPushHead& P;
    const PtPathParams& Q;
    uint32_t W, H;
    Counters cnt;

    // constants (literal values of the shader, rounded once to R)
    const R kPi = R(3.14159265358979);
    const R kTwoPi = R(6.28318530717958);
    const R kInvPi = R(1.0 / 3.14159265358979);

    Tracer(const PtPackedScene& s, const PtPushHead& p, const PtPathParams& q, uint32_t w, uint32_t h)
        : S(s), P(p), Q(q), W(w), H(h) {}

    // --- traceScene (shaders/PathTrace.slang:2066-2161, 2321-2434, 2548-2691) ---
    void test_prim(uint32_t idx, V3<R> ro, V3<R> rd, R shutter, Hit<R>& h) {
        cnt.prims++;
        const float* v = S.prims + size_t(idx) * 28;
        const uint32_t type = uint32_t(v[8]);
        R t;
        if (type == 0u) {   // PRIM_SPHERE, intersectSphere (PathTraceMath.slang:194-204)
            const V3<R> c = lerp(ld3<R>(v + 12), ld3<R>(v), shutter);
            const R rad = R(v[3]);
            const V3<R> oc = ro - c;
            const R b = dot(oc, rd);
            const R k = dot(oc, oc) - rad * rad;
            R hh = b * b - k;
            if (hh < R(0)) return;
            hh = std::sqrt(hh);
            const R t0 = -b - hh, t1 = -b + hh;
            t = (t0 > R(1e-3)) ? t0 : t1;
            if (!(t > R(1e-3)) || !(t < h.t)) return;
            h.hit = true;
            h.t = t;
            h.normal = normalize(ro + rd * t - c);
        } else if (type == 1u) {   // PRIM_PLANE, intersectPlane (PathTraceMath.slang:209-214)
            const V3<R> n = quat_rotate<R>(v + 20, ld3<R>(v));
            const R denom = dot(rd, n);
            if (std::fabs(denom) < R(1e-4)) return;
            t = -(dot(ro, n) + R(v[3])) / denom;
            if (!(t > R(1e-3)) || !(t < h.t)) return;
            h.hit = true;
            h.t = t;
            h.normal = n;
        } else {
            return;
        }
        h.id = idx;
        const uint32_t pm = S.prim_mat_ids ? S.prim_mat_ids[idx] : 0xFFFFFFFFu;
        if (pm != 0xFFFFFFFFu && S.material_count > 0) {   // material-table extension
            table_material(pm, h);
            return;
        }
        h.mat = uint32_t(v[9]);
        h.albedo = ld3<R>(v + 4);
        h.roughness = R(v[7]);
        h.ior = R(v[10]);
        h.emission = ld3<R>(v + 16);
        h.mid = 0xFFFFFFFFu;
    }

    void table_material(uint32_t m, Hit<R>& h) const {
        if (m >= S.material_count) m = S.material_count - 1;
        const float* mt = S.materials + size_t(m) * 12;
        h.mat = uint32_t(mt[8]);
        h.albedo = ld3<R>(mt);
        h.roughness = R(mt[3]);
        h.emission = ld3<R>(mt + 4);
        h.ior = R(mt[7]);
        h.mid = m;
    }

    static bool slab(V3<R> ro, V3<R> inv, const PtBvhNode& n, R tmax) {
        const V3<R> bmin = ld3<R>(n.aabb_min), bmax = ld3<R>(n.aabb_max);
        const V3<R> t0 = (bmin - ro) * inv, t1 = (bmax - ro) * inv;
        const R tmin = mx(mx(mn(t0.x, t1.x), mn(t0.y, t1.y)), mn(t0.z, t1.z));
        const R tmx = mn(mn(mx(t0.x, t1.x), mx(t0.y, t1.y)), mx(t0.z, t1.z));
        return tmx >= mx(tmin, R(0)) && tmin <= tmax;
    }

    static V3<R> safe_inv(V3<R> rd) {
        auto s = [](R a) { return (std::fabs(a) > R(1e-30)) ? a : R(1e-30); };
        return {R(1) / s(rd.x), R(1) / s(rd.y), R(1) / s(rd.z)};
    }

    // ---- SDF clusters (SdfPrimitives.slang phase-1 ops; PathTrace.slang:2223-2305) ----
    struct SdfN {
        uint32_t op, shape, a, b;
        V3<R> c;
        R q[4];
    };
    static float f_at(const float* p) { return *p; }
    static uint32_t u_at(const float* p) {
        uint32_t u;
        std::memcpy(&u, p, 4);
        return u;
    }
    SdfN sdf_node(const float* C, uint32_t i) const {
        const float* n = C + 16 + 12 * i;
        SdfN o{u_at(n), u_at(n + 1), u_at(n + 2), u_at(n + 3), ld3<R>(n + 8), {R(n[4]), R(n[5]), R(n[6]), R(n[7])}};
        return o;
    }
    static R len2(R x, R y) { return std::sqrt(x * x + y * y); }
    static R sgn(R x) { return (x > R(0)) ? R(1) : ((x < R(0)) ? R(-1) : R(0)); }
    static R sd_leaf(V3<R> p, uint32_t shape, const R* q) {
        switch (shape) {
            case 0u: return length(p) - q[0];
            case 1u:
            case 2u: {
                const V3<R> d{std::fabs(p.x) - q[0], std::fabs(p.y) - q[1], std::fabs(p.z) - q[2]};
                const R o = length(V3<R>{mx(d.x, R(0)), mx(d.y, R(0)), mx(d.z, R(0))}) +
                            mn(mx(d.x, mx(d.y, d.z)), R(0));
                return shape == 1u ? o : o - q[3];
            }
            case 3u: return len2(len2(p.x, p.z) - q[0], p.y) - q[1];
            case 4u: {
                const R y = clampv(p.y, -q[0], q[0]);
                return length(V3<R>{p.x, p.y - y, p.z}) - q[1];
            }
            case 5u: return dot(p, V3<R>{q[0], q[1], q[2]}) + q[3];
            default: return R(1e30);
        }
    }
    static V3<R> sd_leaf_normal(V3<R> p, uint32_t shape, const R* q) {
        const V3<R> up{R(0), R(1), R(0)};
        switch (shape) {
            case 0u: {
                const R l = length(p);
                return l > R(1e-12) ? p / l : up;
            }
            case 1u:
            case 2u: {
                const V3<R> d{std::fabs(p.x) - q[0], std::fabs(p.y) - q[1], std::fabs(p.z) - q[2]};
                const V3<R> sg{sgn(p.x), sgn(p.y), sgn(p.z)};
                if (mx(d.x, mx(d.y, d.z)) > R(0)) {
                    const V3<R> m{mx(d.x, R(0)), mx(d.y, R(0)), mx(d.z, R(0))};
                    const R lm = length(m);
                    if (lm < R(1e-12)) return sg * up;
                    return (m / lm) * sg;
                }
                V3<R> n{R(0), R(0), R(0)};
                if (d.x > d.y && d.x > d.z) n.x = sg.x;
                else if (d.y > d.z) n.y = sg.y;
                else n.z = sg.z;
                return n;
            }
            case 3u: {
                const R lxz = len2(p.x, p.z);
                if (lxz < R(1e-12)) return {R(0), sgn(p.y), R(0)};
                const R k = q[0] / lxz;
                const V3<R> d = p - V3<R>{p.x * k, R(0), p.z * k};
                const R ld = length(d);
                return ld > R(1e-12) ? d / ld : up;
            }
            case 4u: {
                const R y = clampv(p.y, -q[0], q[0]);
                const V3<R> d = p - V3<R>{R(0), y, R(0)};
                const R l = length(d);
                return l > R(1e-12) ? d / l : up;
            }
            case 5u: return {q[0], q[1], q[2]};
            default: return up;
        }
    }
    R sdf_dist(const float* C, uint32_t count, V3<R> p, V3<R>* grad) const {
        R d[8];
        V3<R> g[8];
        for (uint32_t i = 0; i < 8 && i < count; ++i) {
            const SdfN n = sdf_node(C, i);
            R v;
            V3<R> gr{R(0), R(1), R(0)};
            if (n.op == 0u) {
                const V3<R> pl = p - n.c;
                v = sd_leaf(pl, n.shape, n.q);
                if (grad) gr = sd_leaf_normal(pl, n.shape, n.q);
            } else if (n.op >= 1u && n.op <= 4u) {
                const R da = d[n.a], db = d[n.b], k = n.q[0];
                if (n.op == 1u) {
                    if (k <= R(0)) {
                        v = mn(da, db);
                        if (grad) gr = (da < db) ? g[n.a] : g[n.b];
                    } else {
                        const R h = clampv(R(0.5) + R(0.5) * (db - da) / k, R(0), R(1));
                        v = lerp(db, da, h) - k * h * (R(1) - h);
                        if (grad) gr = normalize(lerp(g[n.b], g[n.a], h));
                    }
                } else if (n.op == 2u) {
                    if (k <= R(0)) {
                        v = mx(da, -db);
                        if (grad) gr = (da > -db) ? g[n.a] : -g[n.b];
                    } else {
                        const R h = clampv(R(0.5) - R(0.5) * (db + da) / k, R(0), R(1));
                        v = lerp(da, -db, h) + k * h * (R(1) - h);
                        if (grad) gr = normalize(lerp(g[n.a], -g[n.b], h));
                    }
                } else if (n.op == 3u) {
                    if (k <= R(0)) {
                        v = mx(da, db);
                        if (grad) gr = (da > db) ? g[n.a] : g[n.b];
                    } else {
                        const R h = clampv(R(0.5) - R(0.5) * (db - da) / k, R(0), R(1));
                        v = lerp(db, da, h) + k * h * (R(1) - h);
                        if (grad) gr = normalize(lerp(g[n.b], g[n.a], h));
                    }
                } else {
                    v = da + k;
                    if (grad) gr = g[n.a];
                }
            } else {
                v = R(1e30);
            }
            d[i] = v;
            g[i] = gr;
        }
        if (grad) *grad = count > 0u ? g[count - 1u] : V3<R>{R(0), R(1), R(0)};
        return count > 0u ? d[count - 1u] : R(1e30);
    }
    // ---- procedural ops 5-9 (SdfPrimitives.slang:504-1245; the reference
    // built with PT_SDF_PROCEDURAL_OPS=1 and without PT_SDF_AUTODIFF) ----
    static uint32_t sdf_hash32(uint32_t x) {   // sdfHash32
        x ^= x >> 16;
        x *= 0x7feb352du;
        x ^= x >> 15;
        x *= 0x846ca68bu;
        x ^= x >> 16;
        return x;
    }
    static R sdf_hash3(uint32_t x, uint32_t y, uint32_t z) {   // sdfHash3: h / 2^32
        uint32_t h = sdf_hash32(x);
        h = sdf_hash32(h ^ y);
        h = sdf_hash32(h ^ z);
        return R(float(h)) * R(1.0f / 4294967296.0f);
    }
    static uint32_t sdf_cell(R x) {   // int3(floor(p)) as a two's-complement word
        const R c = mn(mx(x, R(-2147483648.0)), R(2147483520.0));
        return uint32_t(int32_t(c));
    }
    static R sdf_value_noise(V3<R> p, V3<R>* grad = nullptr) {   // sdfValueNoise3 (+ gradient)
        const V3<R> ip{std::floor(p.x), std::floor(p.y), std::floor(p.z)};
        const V3<R> f = p - ip;
        const uint32_t ix = sdf_cell(ip.x), iy = sdf_cell(ip.y), iz = sdf_cell(ip.z);
        const V3<R> c15{R(15), R(15), R(15)}, c10{R(10), R(10), R(10)};
        const V3<R> u = f * f * f * (f * (f * R(6) - c15) + c10);
        const R n000 = sdf_hash3(ix, iy, iz), n100 = sdf_hash3(ix + 1u, iy, iz);
        const R n010 = sdf_hash3(ix, iy + 1u, iz), n110 = sdf_hash3(ix + 1u, iy + 1u, iz);
        const R n001 = sdf_hash3(ix, iy, iz + 1u), n101 = sdf_hash3(ix + 1u, iy, iz + 1u);
        const R n011 = sdf_hash3(ix, iy + 1u, iz + 1u), n111 = sdf_hash3(ix + 1u, iy + 1u, iz + 1u);
        const R k0 = n000, k1 = n100 - n000, k2 = n010 - n000, k3 = n001 - n000;
        const R k4 = n000 - n100 - n010 + n110;
        const R k5 = n000 - n010 - n001 + n011;
        const R k6 = n000 - n100 - n001 + n101;
        const R k7 = -n000 + n100 + n010 + n001 - n110 - n011 - n101 + n111;
        if (grad) {
            const V3<R> c2{R(2), R(2), R(2)}, c1{R(1), R(1), R(1)};
            const V3<R> du = R(30) * f * f * (f * (f - c2) + c1);
            *grad = {du.x * (k1 + k4 * u.y + k6 * u.z + k7 * u.y * u.z), du.y * (k2 + k4 * u.x + k5 * u.z + k7 * u.x * u.z),
                     du.z * (k3 + k5 * u.y + k6 * u.x + k7 * u.x * u.y)};
        }
        return k0 + k1 * u.x + k2 * u.y + k3 * u.z + k4 * u.x * u.y + k5 * u.y * u.z + k6 * u.z * u.x +
               k7 * u.x * u.y * u.z;
    }
    static R sdf_fbm(V3<R> p, uint32_t octaves, V3<R>* grad = nullptr) {   // sdfFbm3 (+ gradient)
        R v = R(0), amp = R(1), frq = R(1);
        V3<R> g{R(0), R(0), R(0)};
        const uint32_t o = std::min(octaves, 6u);
        for (uint32_t i = 0; i < o; ++i) {
            V3<R> gn{R(0), R(0), R(0)};
            const R vn = sdf_value_noise(p * frq, grad ? &gn : nullptr);
            v += amp * (R(2) * vn - R(1));
            if (grad) g = g + amp * R(2) * gn * frq;
            amp *= R(0.5);
            frq *= R(2);
        }
        if (grad) *grad = g;
        return v;
    }
    // sdfClusterDistProcN: nodes [0, nc), with the noise band; warps below the root read as 1e30
    R sdf_dist_proc(const float* C, uint32_t nc, V3<R> p) const {
        R d[8];
        for (uint32_t i = 0; i < 8 && i < nc; ++i) {
            const SdfN n = sdf_node(C, i);
            R v;
            if (n.op == 0u) {
                v = sd_leaf(p - n.c, n.shape, n.q);
            } else if (n.op >= 1u && n.op <= 5u) {
                const R da = d[n.a], db = d[n.b], k = n.q[0];
                if (n.op == 1u) {
                    if (k <= R(0)) v = mn(da, db);
                    else {
                        const R h = clampv(R(0.5) + R(0.5) * (db - da) / k, R(0), R(1));
                        v = lerp(db, da, h) - k * h * (R(1) - h);
                    }
                } else if (n.op == 2u) {
                    if (k <= R(0)) v = mx(da, -db);
                    else {
                        const R h = clampv(R(0.5) - R(0.5) * (db + da) / k, R(0), R(1));
                        v = lerp(da, -db, h) + k * h * (R(1) - h);
                    }
                } else if (n.op == 3u) {
                    if (k <= R(0)) v = mx(da, db);
                    else {
                        const R h = clampv(R(0.5) - R(0.5) * (db - da) / k, R(0), R(1));
                        v = lerp(db, da, h) + k * h * (R(1) - h);
                    }
                } else if (n.op == 4u) {
                    v = da + k;
                } else {   // sdfDisplaceNoiseBand: amp x fBm(freq p), octaves as the bits of params[2]
                    float oct_f = float(n.q[2]);
                    uint32_t oct = 0;
                    std::memcpy(&oct, &oct_f, 4);
                    v = da + k * sdf_fbm(p * n.q[1], oct);
                }
            } else {
                v = R(1e30);
            }
            d[i] = v;
        }
        return nc > 0u ? d[std::min(nc, 8u) - 1u] : R(1e30);
    }
    // sdfClusterDistWarped: a root warp moves the point once; twist/bend halve the distance
    R sdf_dist_warped(const float* C, uint32_t count, V3<R> p) const {
        const SdfN r = sdf_node(C, count > 0u ? count - 1u : 0u);
        const uint32_t nc = std::min(r.a + 1u, 8u);
        if (r.op == 6u) {
            const R c = M<R>::cos(r.q[0] * p.y), s = M<R>::sin(r.q[0] * p.y);
            return R(0.5) * sdf_dist_proc(C, nc, V3<R>{c * p.x - s * p.z, p.y, s * p.x + c * p.z});
        }
        if (r.op == 7u) {
            const R c = M<R>::cos(r.q[0] * p.x), s = M<R>::sin(r.q[0] * p.x);
            return R(0.5) * sdf_dist_proc(C, nc, V3<R>{p.x, c * p.y - s * p.z, s * p.y + c * p.z});
        }
        if (r.op == 8u || r.op == 9u) {
            float pk_f = float(r.q[3]);
            uint32_t pk = 0;
            std::memcpy(&pk, &pk_f, 4);
            const R lim[3] = {R(pk & 0x3FFu), R((pk >> 10) & 0x3FFu), R((pk >> 20) & 0x3FFu)};
            R q[3] = {p.x, p.y, p.z};
            for (int j = 0; j < 3; ++j) {
                const R per = r.q[j];
                if (per > R(1e-6f)) {
                    R idx = std::round(q[j] / per);
                    if (r.op == 9u) idx = clampv(idx, -lim[j], lim[j]);
                    q[j] = q[j] - per * idx;
                }
            }
            return sdf_dist_proc(C, nc, V3<R>{q[0], q[1], q[2]});
        }
        return sdf_dist_proc(C, count, p);
    }
    static bool sdf_has_proc(const float* C, uint32_t count) {   // sdfClusterHasProcedural
        for (uint32_t i = 0; i < count && i < 8; ++i) {
            const uint32_t op = u_at(C + 16 + 12 * i);
            if (op >= 5u && op <= 9u) return true;
        }
        return false;
    }
    // sdfClusterNormalCentral: 6-tap central differences of step h
    V3<R> sdf_normal_central(const float* C, uint32_t count, V3<R> p, R h) const {
        const R dxp = sdf_dist_warped(C, count, p + V3<R>{h, R(0), R(0)});
        const R dxn = sdf_dist_warped(C, count, p - V3<R>{h, R(0), R(0)});
        const R dyp = sdf_dist_warped(C, count, p + V3<R>{R(0), h, R(0)});
        const R dyn = sdf_dist_warped(C, count, p - V3<R>{R(0), h, R(0)});
        const R dzp = sdf_dist_warped(C, count, p + V3<R>{R(0), R(0), h});
        const R dzn = sdf_dist_warped(C, count, p - V3<R>{R(0), R(0), h});
        const V3<R> g{dxp - dxn, dyp - dyn, dzp - dzn};
        const R l = length(g);
        return l > R(1e-12) ? g / l : V3<R>{R(0), R(1), R(0)};
    }
    static uint32_t bits_of(R x) {
        const float f = float(x);
        uint32_t u;
        std::memcpy(&u, &f, 4);
        return u;
    }
    // sdfClusterDistDN: forward-mode AD over nodes [0, nc), gradient of the last node
    V3<R> sdf_dual_proc(const float* C, uint32_t nc, V3<R> p) const {
        R vv[8];
        V3<R> vg[8];
        const V3<R> up{R(0), R(1), R(0)};
        for (uint32_t i = 0; i < 8 && i < nc; ++i) {
            const SdfN n = sdf_node(C, i);
            R rv;
            V3<R> rg;
            if (n.op == 0u) {
                const V3<R> pl = p - n.c;
                rv = sd_leaf(pl, n.shape, n.q);
                rg = sd_leaf_normal(pl, n.shape, n.q);
            } else if (n.op >= 1u && n.op <= 5u) {
                const R av = vv[n.a], bv = vv[n.b], k = n.q[0];
                const V3<R> ag = vg[n.a], bg = vg[n.b];
                if (n.op == 1u) {
                    if (k <= R(0)) {
                        rv = (av < bv) ? av : bv;
                        rg = (av < bv) ? ag : bg;
                    } else {
                        const R h = clampv(R(0.5) + R(0.5) * (bv - av) / k, R(0), R(1));
                        rv = lerp(bv, av, h) - k * h * (R(1) - h);
                        rg = lerp(bg, ag, h);
                    }
                } else if (n.op == 2u) {
                    if (k <= R(0)) {
                        rv = mx(av, -bv);
                        rg = (av > -bv) ? ag : -bg;
                    } else {
                        const R h = clampv(R(0.5) - R(0.5) * (bv + av) / k, R(0), R(1));
                        rv = lerp(av, -bv, h) + k * h * (R(1) - h);
                        rg = lerp(ag, -bg, h);
                    }
                } else if (n.op == 3u) {
                    if (k <= R(0)) {
                        rv = (av > bv) ? av : bv;
                        rg = (av > bv) ? ag : bg;
                    } else {
                        const R h = clampv(R(0.5) - R(0.5) * (bv - av) / k, R(0), R(1));
                        rv = lerp(bv, av, h) + k * h * (R(1) - h);
                        rg = lerp(bg, ag, h);
                    }
                } else if (n.op == 4u) {
                    rv = av + k;
                    rg = ag;
                } else {   // sdfDisplaceNoiseBand: amp fBm(freq p), gradient amp freq fBm'
                    V3<R> fg;
                    const R fv = sdf_fbm(p * n.q[1], bits_of(n.q[2]), &fg);
                    rv = av + k * fv;
                    rg = ag + k * n.q[1] * fg;
                }
            } else {
                rv = R(1e30);
                rg = up;
            }
            vv[i] = rv;
            vg[i] = rg;
        }
        return nc > 0u ? vg[std::min(nc, 8u) - 1u] : up;
    }
    // sdfClusterNormalForwardAD: the root warp's transposed Jacobian applied to the AD gradient
    V3<R> sdf_normal_ad(const float* C, uint32_t count, V3<R> p) const {
        const SdfN r = sdf_node(C, count > 0u ? count - 1u : 0u);
        const uint32_t nc = (r.op >= 6u && r.op <= 9u) ? std::min(r.a + 1u, 8u) : count;
        const R rate = r.q[0];
        V3<R> g;
        if (r.op == 6u) {
            const R c = M<R>::cos(rate * p.y), s = M<R>::sin(rate * p.y);
            const V3<R> d = sdf_dual_proc(C, nc, V3<R>{c * p.x - s * p.z, p.y, s * p.x + c * p.z});
            g = {c * d.x + s * d.z, -rate * (s * p.x + c * p.z) * d.x + d.y + rate * (c * p.x - s * p.z) * d.z,
                 -s * d.x + c * d.z};
        } else if (r.op == 7u) {
            const R c = M<R>::cos(rate * p.x), s = M<R>::sin(rate * p.x);
            const V3<R> d = sdf_dual_proc(C, nc, V3<R>{p.x, c * p.y - s * p.z, s * p.y + c * p.z});
            g = {d.x + (-rate * (s * p.y + c * p.z)) * d.y + (rate * (c * p.y - s * p.z)) * d.z, c * d.y + s * d.z,
                 -s * d.y + c * d.z};
        } else if (r.op == 8u || r.op == 9u) {
            const uint32_t pk = bits_of(r.q[3]);
            const R lim[3] = {R(pk & 0x3FFu), R((pk >> 10) & 0x3FFu), R((pk >> 20) & 0x3FFu)};
            R w[3] = {p.x, p.y, p.z};
            for (int j = 0; j < 3; ++j) {
                const R per = r.q[j];
                if (per > R(1e-6f)) {
                    R idx = std::round(w[j] / per);
                    if (r.op == 9u) idx = clampv(idx, -lim[j], lim[j]);
                    w[j] = w[j] - per * idx;
                }
            }
            g = sdf_dual_proc(C, nc, V3<R>{w[0], w[1], w[2]});
        } else {
            g = sdf_dual_proc(C, nc, p);
        }
        const R l = length(g);
        return l > R(1e-12) ? g / l : V3<R>{R(0), R(1), R(0)};
    }
    bool sdf_trace(const float* C, V3<R> ro, V3<R> rd, R t_min, R t_max, R& out_t) const {
        const uint32_t count = u_at(C + 3);
        auto safe = [](R x) { return std::fabs(x) > R(1e-30) ? x : R(1e-30); };
        const V3<R> ri{R(1) / safe(rd.x), R(1) / safe(rd.y), R(1) / safe(rd.z)};
        const V3<R> t0 = (ld3<R>(C) - ro) * ri, t1 = (ld3<R>(C + 4) - ro) * ri;
        const R enter = mx(mx(mn(t0.x, t1.x), mn(t0.y, t1.y)), mn(t0.z, t1.z));
        const R exit = mn(mn(mx(t0.x, t1.x), mx(t0.y, t1.y)), mx(t0.z, t1.z));
        R t = mx(enter, t_min);
        const R t_end = mn(exit, t_max);
        if (t >= t_end) return false;
        const bool proc = Q.sdf_procedural_ops != 0u && sdf_has_proc(C, count);
        const uint32_t iters = std::min(Q.sdf_params[1], 256u);
        const R eps = R(Q.sdf_params_f[0]);
        for (uint32_t i = 0; i < iters; ++i) {
            const V3<R> p = ro + rd * t;
            const R ad = std::fabs(proc ? sdf_dist_warped(C, count, p) : sdf_dist(C, count, p, nullptr));
            if (ad < eps) {
                out_t = t;
                return true;
            }
            t += mx(ad, eps);
            if (t >= t_end) return false;
        }
        return false;
    }
    // ---- fractal leaves (SdfFractals.slang) ----
    static R fracr(R x) { return x - std::floor(x); }
    static R de_fractal(V3<R> p, uint32_t shape, const R* q, R power_default, uint32_t iters) {
        if (shape == 6u) {
            const R power = (q[0] > R(0)) ? q[0] : power_default;
            V3<R> z = p;
            R dr = R(1), r = R(0);
            for (uint32_t i = 0; i < iters; ++i) {
                r = length(z);
                if (r > R(2)) break;
                const R theta = M<R>::acos(clampv(z.z / mx(r, R(1e-12)), R(-1), R(1)));
                const R phi = M<R>::atan2(z.y, z.x);
                dr = M<R>::pow(r, power - R(1)) * power * dr + R(1);
                const R rp = M<R>::pow(r, power);
                const R nt = theta * power, np = phi * power;
                const R sn = M<R>::sin(nt);
                z = V3<R>{sn * M<R>::cos(np), sn * M<R>::sin(np), M<R>::cos(nt)} * rp;
                z = z + p;
            }
            return R(0.5) * M<R>::log(mx(r, R(1.0001))) * r / mx(dr, R(1e-12));
        }
        if (shape == 7u) {
            const R scale = (q[0] != R(0)) ? q[0] : R(2.5);
            V3<R> z = p;
            R dr = R(1);
            for (uint32_t i = 0; i < iters; ++i) {
                z = {clampv(z.x, R(-1), R(1)) * R(2) - z.x, clampv(z.y, R(-1), R(1)) * R(2) - z.y,
                     clampv(z.z, R(-1), R(1)) * R(2) - z.z};
                const R r2 = dot(z, z);
                if (r2 < R(0.25)) {
                    z = z * R(4);
                    dr = dr * R(4);
                } else if (r2 < R(1)) {
                    const R f = R(1) / r2;
                    z = z * f;
                    dr = dr * f;
                }
                z = z * scale + p;
                dr = std::fabs(scale) * dr + R(1);
            }
            return length(z) / std::fabs(dr);
        }
        if (shape == 8u) {
            const R scale = (q[0] != R(0)) ? q[0] : R(1.3);
            V3<R> z = p;
            R dr = R(1);
            for (uint32_t i = 0; i < iters; ++i) {
                z = {R(-1) + R(2) * fracr(R(0.5) * z.x + R(0.5)), R(-1) + R(2) * fracr(R(0.5) * z.y + R(0.5)),
                     R(-1) + R(2) * fracr(R(0.5) * z.z + R(0.5))};
                const R r2 = dot(z, z);
                const R k = mx(scale / mx(r2, R(1e-12)), R(1));
                z = z * k;
                dr = dr * k;
            }
            return (R(0.25) * std::fabs(z.y) - R(0.001)) / dr;
        }
        return R(1e30);
    }
    static V3<R> fractal_normal(V3<R> p, uint32_t shape, const R* q, R power, uint32_t iters, R h) {
        const V3<R> e1{R(1), R(-1), R(-1)}, e2{R(-1), R(-1), R(1)}, e3{R(-1), R(1), R(-1)}, e4{R(1), R(1), R(1)};
        const R d1 = de_fractal(p + e1 * h, shape, q, power, iters);
        const R d2 = de_fractal(p + e2 * h, shape, q, power, iters);
        const R d3 = de_fractal(p + e3 * h, shape, q, power, iters);
        const R d4 = de_fractal(p + e4 * h, shape, q, power, iters);
        const V3<R> n = e1 * d1 + e2 * d2 + e3 * d3 + e4 * d4;
        const R l = length(n);
        return (l > R(1e-12)) ? n / l : V3<R>{R(0), R(1), R(0)};
    }
    bool sdf_is_fractal(const float* C) const {
        const uint32_t count = u_at(C + 3);
        if (count == 0u) return false;
        const float* n = C + 16 + 12 * (count - 1u);
        return u_at(n) == 0u && u_at(n + 1) >= 6u;
    }
    bool fractal_trace(const float* C, V3<R> ro, V3<R> rd, R t_min, R t_max, R& out_t, uint32_t& step) const {
        const SdfN n = sdf_node(C, u_at(C + 3) - 1u);
        auto safe = [](R x) { return std::fabs(x) > R(1e-30) ? x : R(1e-30); };
        const V3<R> ri{R(1) / safe(rd.x), R(1) / safe(rd.y), R(1) / safe(rd.z)};
        const V3<R> t0 = (ld3<R>(C) - ro) * ri, t1 = (ld3<R>(C + 4) - ro) * ri;
        const R enter = mx(mx(mn(t0.x, t1.x), mn(t0.y, t1.y)), mn(t0.z, t1.z));
        const R exit = mn(mn(mx(t0.x, t1.x), mx(t0.y, t1.y)), mx(t0.z, t1.z));
        R t = mx(enter, t_min);
        const R t_end = mn(exit, t_max);
        if (t >= t_end) return false;
        const uint32_t steps = std::min(Q.sdf_params[1], 512u);
        const R eps = R(Q.sdf_params_f[0]);
        for (uint32_t i = 0; i < steps; ++i) {
            const V3<R> pl = (ro + rd * t) - n.c;
            const R ad = std::fabs(de_fractal(pl, n.shape, n.q, R(Q.sdf_params_f[1]), Q.sdf_params[3]));
            const R eps_i = eps * (R(1) + R(Q.sdf_params_f[2]) * R(i));
            if (ad < eps_i) {
                out_t = t;
                step = i;
                return true;
            }
            t += mx(ad, eps);
            if (t >= t_end) return false;
        }
        return false;
    }

    void trace_sdf(V3<R> ro, V3<R> rd, Hit<R>& h) {
        const uint32_t n = std::min(Q.sdf_params[0], S.sdf_count);
        for (uint32_t i = 0; i < n; ++i) {
            const float* C = S.sdf_clusters + size_t(i) * 112;
            R t;
            if (sdf_is_fractal(C)) {
                uint32_t step = 0;
                if (fractal_trace(C, ro, rd, R(1e-3), h.t, t, step) && t < h.t) {
                    const SdfN nd = sdf_node(C, u_at(C + 3) - 1u);
                    const R eps = R(Q.sdf_params_f[0]);
                    const R eps_i = eps * (R(1) + R(Q.sdf_params_f[2]) * R(step));
                    const R hh = mx(eps_i * R(8), eps * R(4));
                    h.hit = true;
                    h.t = t;
                    h.normal = fractal_normal((ro + rd * t) - nd.c, nd.shape, nd.q, R(Q.sdf_params_f[1]),
                                              Q.sdf_params[3], hh);
                    h.mat = u_at(C + 7);
                    h.albedo = ld3<R>(C + 8);
                    h.roughness = R(C[11]);
                    h.ior = R(C[12]);
                    h.emission = {R(0), R(0), R(0)};
                    h.id = 0x80000000u | (step << 20) | i;
                    h.mid = 0xFFFFFFFFu;
                }
                continue;
            }
            if (sdf_trace(C, ro, rd, R(1e-3), h.t, t) && t < h.t) {
                const uint32_t count = u_at(C + 3);
                h.hit = true;
                if (Q.sdf_procedural_ops != 0u && sdf_has_proc(C, count)) {
                    if (Q.sdf_procedural_ops >= 2u && Q.sdf_params_f[3] == 0.0f)   // PT_SDF_AUTODIFF build
                        h.normal = sdf_normal_ad(C, count, ro + rd * t);
                    else
                        h.normal = sdf_normal_central(C, count, ro + rd * t, R(Q.sdf_params_f[0]));
                } else {
                    V3<R> g;
                    sdf_dist(C, count, ro + rd * t, &g);
                    h.normal = normalize(g);
                }
                h.t = t;
                h.mat = u_at(C + 7);
                h.albedo = ld3<R>(C + 8);
                h.roughness = R(C[11]);
                h.ior = R(C[12]);
                h.emission = {R(0), R(0), R(0)};
                h.id = 0x80000000u | i;
                h.mid = 0xFFFFFFFFu;
            }
        }
    }

    Hit<R> trace(V3<R> ro, V3<R> rd, R t_init = R(1e30)) {
        cnt.rays++;
        const R shutter = R(1);   // motion blur off
        Hit<R> h;
        h.t = t_init;
        const uint32_t linear = Q.bvh_params[0];
        const uint32_t nodes = Q.bvh_params[1];
        const uint32_t pc = P.prim_count;
        for (uint32_t i = 0; i < linear && i < pc; ++i) test_prim(i, ro, rd, shutter, h);
        if (nodes == 0u) {
            for (uint32_t i = linear; i < pc; ++i) test_prim(i, ro, rd, shutter, h);
        } else {
            const V3<R> inv = safe_inv(rd);
            uint32_t stack[32];
            int sp = 0;
            stack[sp++] = 0u;
            while (sp > 0) {
                const uint32_t idx = stack[--sp];
                const PtBvhNode& n = S.bvh_nodes[idx];
                cnt.nodes++;
                if (!slab(ro, inv, n, h.t)) continue;
                if (n.count > 0u) {
                    const uint32_t base = n.left_first + linear;
                    for (uint32_t k = 0; k < n.count; ++k) test_prim(base + k, ro, rd, shutter, h);
                } else if (sp + 2 <= 32) {
                    stack[sp++] = n.left_first;
                    stack[sp++] = n.left_first + 1u;
                }
            }
        }
        trace_sdf(ro, rd, h);
        if (Q.bvh_params[2] != 0u) {
            const uint32_t tnodes = Q.bvh_params[3];
            R t_mesh = h.t;
            uint32_t prim_hit = 0;
            bool found = false;
            if (tnodes > 0u) {
                const V3<R> inv = safe_inv(rd);
                uint32_t stack[64];
                int sp = 0;
                stack[sp++] = 0u;
                while (sp > 0) {
                    const uint32_t idx = stack[--sp];
                    const PtBvhNode& n = S.tri_nodes[idx];
                    cnt.nodes++;
                    if (!slab(ro, inv, n, t_mesh)) continue;
                    if (n.count > 0u) {
                        for (uint32_t k = 0; k < n.count; ++k) {
                            cnt.tris++;
                            const uint32_t tri = S.tri_perm[n.left_first + k];
                            const V3<R> v0 = ld3<R>(S.positions + 3u * S.indices[tri * 3u + 0u]);
                            const V3<R> v1 = ld3<R>(S.positions + 3u * S.indices[tri * 3u + 1u]);
                            const V3<R> v2 = ld3<R>(S.positions + 3u * S.indices[tri * 3u + 2u]);
                            const V3<R> e1 = v1 - v0, e2 = v2 - v0;
                            const V3<R> pv = cross(rd, e2);
                            const R det = dot(e1, pv);
                            if (std::fabs(det) < R(1e-8)) continue;
                            const R inv_det = R(1) / det;
                            const V3<R> tvec = ro - v0;
                            const R u = dot(tvec, pv) * inv_det;
                            if (u < R(0) || u > R(1)) continue;
                            const V3<R> qv = cross(tvec, e1);
                            const R vv = dot(rd, qv) * inv_det;
                            if (vv < R(0) || u + vv > R(1)) continue;
                            const R tt = dot(e2, qv) * inv_det;
                            if (tt > R(1e-3) && tt < t_mesh) {
                                found = true;
                                t_mesh = tt;
                                prim_hit = tri;
                            }
                        }
                    } else if (sp + 2 <= 64) {
                        stack[sp++] = n.left_first;
                        stack[sp++] = n.left_first + 1u;
                    }
                }
            }
            if (found) {
                const V3<R> v0 = ld3<R>(S.positions + 3u * S.indices[prim_hit * 3u + 0u]);
                const V3<R> v1 = ld3<R>(S.positions + 3u * S.indices[prim_hit * 3u + 1u]);
                const V3<R> v2 = ld3<R>(S.positions + 3u * S.indices[prim_hit * 3u + 2u]);
                h.hit = true;
                h.t = t_mesh;
                h.normal = normalize(cross(v1 - v0, v2 - v0));
                h.id = (1u << 30) | prim_hit;
                if (S.tri_mat_ids && S.material_count > 0) {   // material table extension
                    table_material(S.tri_mat_ids[prim_hit], h);
                } else {
                    h.mid = 0xFFFFFFFFu;   // MESH_ALBEDO gold metal (PathTrace.slang:1428, 2655-2658)
                    h.mat = kMatMetal;
                    h.albedo = {R(1.00), R(0.85), R(0.45)};
                    h.roughness = R(0.05);
                    h.ior = R(1);
                    h.emission = {R(0), R(0), R(0)};
                }
            }
        }
        return h;
    }

    // --- clampIndirect (PathTrace.slang:3367-3371) ---
    V3<R> clamp_ind(V3<R> c) const {
        const R w = R(Q.firefly_clamp);
        if (w <= R(0)) return c;
        const R m = mx(c.x, mx(c.y, c.z));
        return (m > w) ? c * (w / m) : c;
    }

    // --- env map (PathTrace.slang:3401-3431, 3619-3735) ---
    V3<R> texel(uint32_t u, uint32_t v) const {
        return ld3<R>(S.env_rgba + (size_t(v) * S.env_w + u) * 4);
    }
    // ---- gradient sky (no env map): PathTrace.slang:3112-3353, 3373-3464 ----
    static R sat(R x) { return clampv(x, R(0), R(1)); }
    static R smoothstep(R e0, R e1, R x) {
        const R t = sat((x - e0) / (e1 - e0));
        return t * t * (R(3) - R(2) * t);
    }
    V3<R> sun_dir() const { return ld3<R>(Q.sun_and_mode); }
    static V3<R> sky_gradient(V3<R> rd) {   // skyColorBase, gradient mode
        const R t = clampv(R(0.5) * (rd.y + R(1)), R(0), R(1));
        return lerp(V3<R>{R(0.50), R(0.55), R(0.62)}, V3<R>{R(1), R(1), R(1)}, t);
    }
    V3<R> sun_disc(V3<R> rd) const {   // sunDisc
        const V3<R> sd = sun_dir();
        const V3<R> zero{R(0), R(0), R(0)};
        if (sd.y < R(-0.10)) return zero;
        const R ang = dot(rd, sd);
        const R sun_mult = mx(R(Q.sun_extra[0]) * R(Q.sun_extra[1]), R(0.1));
        const R r_deg = R(0.55) * sun_mult;
        const R cos_r = M<R>::cos(r_deg * R(0.0174533));
        const R halo_deg = lerp(R(2.0), R(8.0), sat(R(1) - sd.y));
        const R halo_rad = halo_deg * R(0.0174533);
        const R cos_halo = M<R>::cos(halo_rad);
        if (ang <= cos_halo) return zero;
        const R vflat = R(Q.sun_extra[2]);
        const bool oval = vflat < R(0.999);
        bool inside = false;
        if (ang > cos_r) {
            if (!oval) {
                inside = true;
            } else {
                const V3<R> lr = normalize(cross(V3<R>{R(0), R(1), R(0)}, sd));
                const V3<R> lu = cross(sd, lr);
                const V3<R> delta = rd - sd * ang;
                const R h_off = dot(delta, lr), v_off = dot(delta, lu);
                const R r_h = r_deg * R(0.0174533);
                const R r_v = r_h * vflat;
                const R ellipse = (h_off * h_off) / (r_h * r_h) + (v_off * v_off) / (r_v * r_v);
                inside = ellipse <= R(1);
            }
        }
        const R am = R(1) / mx(sd.y, R(0.04));
        const R atm = M<R>::exp(R(-0.30) * am);
        const R warmth = sat((am - R(1)) * R(0.18));
        const V3<R> col = lerp(V3<R>{R(1.00), R(0.98), R(0.94)}, V3<R>{R(1.55), R(0.55), R(0.20)}, warmth);
        R halo = R(0);
        if (ang > cos_halo) {
            const R t_h = (ang - cos_halo) / (R(1) - cos_halo);
            const R falloff = lerp(R(8.0), R(3.0), sat(R(1) - sd.y));
            halo = M<R>::pow(t_h, falloff);
        }
        const R bright = mx(R(Q.sun_extra2[0]), R(0));
        if (inside) return (col * (R(250.0) * atm) + col * halo * atm * R(4.0)) * bright;
        return col * halo * atm * R(4.0) * bright;
    }
    V3<R> moon_texel(int32_t x, int32_t y) const {
        return ld3<R>(S.moon_rgba + (size_t(y) * S.moon_w + x) * 4);
    }
    V3<R> moon_disc(V3<R> rd) const {   // moonDisc
        const float* mph = Q.moon_dir_phase;
        const V3<R> zero{R(0), R(0), R(0)};
        if (R(mph[1]) < R(-0.10)) return zero;
        const V3<R> m_dir = ld3<R>(mph);
        const V3<R> sun = sun_dir();
        const R ang = dot(rd, m_dir);
        const R size_mult = mx(R(Q.moon_extra[0]) * R(Q.moon_extra[1]), R(0.1));
        const R r_deg = R(0.55) * size_mult;
        const R halo_deg = R(1.5) * size_mult;
        const R cos_r = M<R>::cos(r_deg * R(0.0174533));
        const R cos_halo = M<R>::cos(halo_deg * R(0.0174533));
        if (ang <= cos_halo) return zero;
        const V3<R> col_tint{R(0.92), R(0.94), R(1.00)};
        const R moon_am = R(1) / mx(R(mph[1]), R(0.04));
        const R moon_atm = M<R>::exp(R(-0.30) * moon_am);
        const R warmth_m = sat((moon_am - R(1)) * R(0.18));
        const V3<R> col_atm = lerp(V3<R>{R(1), R(1), R(1)}, V3<R>{R(1.20), R(0.65), R(0.40)}, warmth_m);
        R halo = R(0);
        if (ang > cos_halo) {
            const R t_h = (ang - cos_halo) / (R(1) - cos_halo);
            halo = M<R>::pow(t_h, R(4.0)) * R(0.6);
        }
        if (ang > cos_r) {
            const R t_d = (ang - cos_r) / (R(1) - cos_r);
            const V3<R> ax = (std::fabs(m_dir.y) < R(0.99)) ? V3<R>{R(0), R(1), R(0)} : V3<R>{R(1), R(0), R(0)};
            const V3<R> t_a = normalize(cross(ax, m_dir));
            const V3<R> t_b = cross(m_dir, t_a);
            const R disc_scale = R(1) / mx(M<R>::sin(r_deg * R(0.0174533)), R(1e-5));
            const R du = dot(rd, t_a) * disc_scale;
            const R dv = dot(rd, t_b) * disc_scale;
            const R r2 = du * du + dv * dv;
            const R zz = std::sqrt(mx(R(1) - r2, R(0)));
            const V3<R> n_world = t_a * du + t_b * dv - m_dir * zz;
            const R lit = sat(dot(n_world, sun) * R(10.0) + R(0.05));
            if (lit <= R(0)) return col_tint * col_atm * halo * moon_atm * R(0.05);
            const R anti_sun_dot = -dot(m_dir, sun);
            const R anti_sun_ang = M<R>::acos(sat(anti_sun_dot));
            const R eclipse = R(1) - smoothstep(R(0.0122), R(0.0218), anti_sun_ang);
            const R lon = M<R>::atan2(du, zz);
            const R lat = M<R>::asin(clampv(dv, R(-1), R(1)));
            const R u_tex = sat(R(0.5) + lon / R(6.28318530718));
            const R v_tex = sat(R(0.5) - lat / R(3.14159265358979));
            const int32_t mw = int32_t(S.moon_w), mh = int32_t(S.moon_h);
            const R fx = u_tex * R(mw) - R(0.5), fy = v_tex * R(mh) - R(0.5);
            const int32_t ix = int32_t(std::floor(fx)), iy = int32_t(std::floor(fy));
            const R tx = fx - R(ix), ty = fy - R(iy);
            const int32_t x0 = std::min(std::max(ix, 0), mw - 1), x1 = std::min(std::max(ix + 1, 0), mw - 1);
            const int32_t y0 = std::min(std::max(iy, 0), mh - 1), y1 = std::min(std::max(iy + 1, 0), mh - 1);
            const V3<R> surface = lerp(lerp(moon_texel(x0, y0), moon_texel(x1, y0), tx),
                                       lerp(moon_texel(x0, y1), moon_texel(x1, y1), tx), ty);
            const R limb = R(0.55) + R(0.45) * std::sqrt(sat(t_d));
            const R bright_mult = mx(R(Q.moon_extra[2]), R(0));
            const R disc_scale_b = R(3.5) * bright_mult;
            const V3<R> lit_col = col_tint * col_atm * surface * (disc_scale_b * lit * limb * moon_atm) +
                                  col_tint * col_atm * halo * lit * moon_atm * (R(0.6) * bright_mult);
            const V3<R> eclipse_col = V3<R>{R(0.55), R(0.15), R(0.04)} * surface * (limb * moon_atm * R(1.2));
            return lerp(lit_col, eclipse_col, eclipse);
        }
        const R phase_b = R(0.5) * (R(1) - M<R>::cos(R(mph[3])));
        return col_tint * col_atm * halo * phase_b * moon_atm * R(0.3);
    }
    // procSkyInlineSunDiscAndHalo (PathTrace.slang:2860-2872)
    static V3<R> proc_sun_inline(V3<R> rd, V3<R> sun) {
        const R cos_gamma = clampv(dot(rd, sun), R(-1), R(1));
        const R day = smoothstep(R(-0.10), R(0.20), sun.y);
        const R disk = smoothstep(R(0.99996), R(0.99999), cos_gamma);
        const V3<R> sun_col = lerp(V3<R>{R(1.00), R(0.55), R(0.20)}, V3<R>{R(1.00), R(0.95), R(0.85)}, day);
        V3<R> result = disk * R(50.0) * sun_col * day;
        const R halo = M<R>::pow(mx(R(0), cos_gamma), R(80.0));
        result = result + halo * sun_col * R(0.30) * day;
        return result;
    }
    // procSky, stars off (PathTrace.slang:2990-3103)
    V3<R> proc_sky(V3<R> rd) const {
        const V3<R> sun = sun_dir();
        const R cos_theta_raw = clampv(rd.y, R(-1), R(1));
        const R cos_gamma = clampv(dot(rd, sun), R(-1), R(1));
        const R sun_elev = sun.y;
        const R cam_h = mx(R(P.pos_fovtan[1]), R(0));
        const R planet_r = R(Q.sun_extra[3]);
        R dip = R(0);
        if (planet_r > R(0) && cam_h > R(0)) {
            const R ratio = cam_h / planet_r;
            dip = std::sqrt(R(2) * ratio + ratio * ratio);
            dip = mn(dip, R(0.5));
        }
        const R cos_theta = clampv(cos_theta_raw + dip, R(-1), R(1));
        const R day = smoothstep(R(-0.10), R(0.20), sun_elev);
        const R sunset = smoothstep(R(0.30), R(-0.05), sun_elev) * smoothstep(R(-0.20), R(0.05), sun_elev);
        const V3<R> zenith_day{R(0.32), R(0.55), R(0.92)}, horizon_day{R(0.78), R(0.88), R(1.00)};
        const R side_factor = smoothstep(R(0), R(0.7), dot(normalize(V3<R>{rd.x, R(0), rd.z}),
                                                          normalize(V3<R>{sun.x, R(0), sun.z})));
        const V3<R> horizon_sunset =
            lerp(V3<R>{R(0.95), R(0.45), R(0.20)}, V3<R>{R(1.00), R(0.65), R(0.30)}, side_factor);
        const V3<R> horizon_col = lerp(horizon_day, horizon_sunset, sunset);
        const V3<R> zenith_col = lerp(zenith_day, V3<R>{R(0.18), R(0.18), R(0.30)}, sunset * R(0.6));
        const R t = smoothstep(R(0), R(0.40), cos_theta);
        V3<R> sky = lerp(horizon_col, zenith_col, t);
        const V3<R> night{R(0.005), R(0.010), R(0.030)};
        sky = lerp(night, sky, day);
        sky = sky + proc_sun_inline(rd, sun);
        const V3<R> sun_col = lerp(V3<R>{R(1.00), R(0.55), R(0.20)}, V3<R>{R(1.00), R(0.95), R(0.85)}, day);
        const R wide = M<R>::pow(mx(R(0), cos_gamma), R(6.0));
        sky = sky + wide * sun_col * sunset * R(0.50);
        return {mx(sky.x, R(0)), mx(sky.y, R(0)), mx(sky.z, R(0))};
    }
    bool procedural() const { return Q.sun_and_mode[3] == 2.0f; }
    V3<R> sky_base(V3<R> rd) const {   // skyColorBase without an env map
        if (procedural()) return proc_sky(rd) - proc_sun_inline(rd, sun_dir());
        return sky_gradient(rd);
    }

    // sampleSunDisc (PathTraceMath.slang:55-68)
    V3<R> sample_sun_disc(V3<R> sd, uint32_t& seed) const {
        const R u1 = randf<R>(seed);
        const R u2 = randf<R>(seed);
        const R r = std::sqrt(u1) * R(0.00465);
        const R phi = R(6.28318530718) * u2;
        const R dx = M<R>::cos(phi) * r, dy = M<R>::sin(phi) * r;
        const V3<R> ax = (std::fabs(sd.y) < R(0.99)) ? V3<R>{R(0), R(1), R(0)} : V3<R>{R(1), R(0), R(0)};
        const V3<R> t = normalize(cross(ax, sd));
        const V3<R> b = cross(sd, t);
        return normalize(sd + t * dx + b * dy);
    }

    V3<R> sky_color(V3<R> rd) const {
        if (!P.env_map_present) return (procedural() ? proc_sky(rd) : sky_gradient(rd)) + moon_disc(rd) + sun_disc(rd);
        const int32_t w = int32_t(S.env_w), hh = int32_t(S.env_h);
        const R u = M<R>::atan2(rd.z, rd.x) * R(1.0 / 6.28318530718) + R(0.5);
        const R v = M<R>::acos(clampv(rd.y, R(-1), R(1))) * R(1.0 / 3.14159265359);
        const R fx = u * R(w) - R(0.5), fy = v * R(hh) - R(0.5);
        const int32_t ix = int32_t(std::floor(fx)), iy = int32_t(std::floor(fy));
        const R tx = fx - R(ix), ty = fy - R(iy);
        const int32_t x0 = (ix % w + w) % w, x1 = (x0 + 1) % w;
        const int32_t y0 = std::min(std::max(iy, 0), hh - 1), y1 = std::min(std::max(iy + 1, 0), hh - 1);
        const V3<R> c00 = texel(x0, y0), c10 = texel(x1, y0), c01 = texel(x0, y1), c11 = texel(x1, y1);
        const V3<R> sky = lerp(lerp(c00, c10, tx), lerp(c01, c11, tx), ty);
        return sky * R(P.env_intensity);
    }
    uint32_t cdf_search(const float* cdf, uint32_t count, R u) const {
        uint32_t lo = 0, hi = count;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (R(cdf[mid]) < u) lo = mid + 1;
            else hi = mid;
        }
        return std::min(lo, count - 1);
    }
    R env_denom() const {   // 2.0 * pi * pi * total, left to right
        return R(2.0) * kPi * kPi * R(P.env_total_luminance);
    }
    struct EnvSample { V3<R> dir; V3<R> color; R pdf; };
    EnvSample sample_env(R xu, R xv) const {
        EnvSample s{{R(0), R(1), R(0)}, {R(0), R(0), R(0)}, R(0)};
        if (P.env_map_present == 0u || !(P.env_total_luminance > 0.0f)) return s;
        const uint32_t w = S.env_w, hh = S.env_h;
        const uint32_t vi = cdf_search(S.env_marginal, hh, xv);
        const uint32_t ui = cdf_search(S.env_conditional + size_t(vi) * w, w, xu);
        const R u = (R(ui) + R(0.5)) / R(w);
        const R v = (R(vi) + R(0.5)) / R(hh);
        const R theta = v * kPi;
        const R phi = u * kTwoPi - kPi;
        const R st = M<R>::sin(theta);
        s.dir = {st * M<R>::cos(phi), M<R>::cos(theta), st * M<R>::sin(phi)};
        const V3<R> raw = texel(ui, vi);
        s.color = raw * R(P.env_intensity);
        const R lum = R(0.2126) * raw.x + R(0.7152) * raw.y + R(0.0722) * raw.z;
        if (st > R(1e-6)) s.pdf = (lum * R(w * hh)) / env_denom();
        return s;
    }
    void dir_to_texel(V3<R> d, R& theta, R& st, uint32_t& ui, uint32_t& vi) const {
        const R ct = clampv(d.y, R(-1), R(1));
        theta = M<R>::acos(ct);
        st = M<R>::sin(theta);
        const R ph = M<R>::atan2(d.z, d.x);
        const R u = (ph + kPi) * R(1.0 / 6.28318530717958);
        const R v = theta * R(1.0 / 3.14159265358979);
        ui = std::min(uint32_t(u * R(S.env_w)), S.env_w - 1u);
        vi = std::min(uint32_t(v * R(S.env_h)), S.env_h - 1u);
    }
    bool is_cluster_dir(V3<R> d) const {
        if (P.env_map_present == 0u || S.hdri_count == 0u) return false;
        R th, st;
        uint32_t ui, vi;
        dir_to_texel(d, th, st, ui, vi);
        if (st < R(1e-6)) return false;
        const size_t base = size_t(vi) * S.env_w;
        const R cc = R(S.env_conditional[base + ui]);
        const R cp = (ui > 0u) ? R(S.env_conditional[base + ui - 1u]) : R(0);
        return cc <= cp;
    }
    R pdf_env_dir(V3<R> d) const {
        if (P.env_map_present == 0u || !(P.env_total_luminance > 0.0f)) return R(0);
        R th, st;
        uint32_t ui, vi;
        dir_to_texel(d, th, st, ui, vi);
        if (st < R(1e-6)) return R(0);
        const V3<R> raw = texel(ui, vi);
        const R lum = R(0.2126) * raw.x + R(0.7152) * raw.y + R(0.0722) * raw.z;
        return (lum * R(S.env_w * S.env_h)) / env_denom();
    }
    static R mis_balance(R a, R b) { return a / mx(a + b, R(1e-12)); }

    // --- sampleHdriLight (PathTrace.slang:3749-3768) ---
    struct HdriSample { V3<R> dir; V3<R> color; R pdf; };
    HdriSample sample_hdri(uint32_t& seed) const {
        HdriSample s{{R(0), R(1), R(0)}, {R(0), R(0), R(0)}, R(0)};
        if (S.hdri_count == 0u) return s;
        const R u = randf<R>(seed);
        R acc = R(0);
        uint32_t sel = 0;
        for (uint32_t i = 0; i < 8u; ++i) {
            if (i >= S.hdri_count) break;
            acc += R(S.hdri_dir_pmf[i * 4 + 3]);
            if (u <= acc) { sel = i; break; }
            sel = i;
        }
        s.dir = ld3<R>(S.hdri_dir_pmf + sel * 4);
        s.color = ld3<R>(S.hdri_col + sel * 4) * R(P.env_intensity);
        s.pdf = mx(R(S.hdri_dir_pmf[sel * 4 + 3]), R(1e-6));
        return s;
    }

    // --- sampleAnalyticLight, uniform pick (PathTrace.slang:4035-4179) ---
    struct LightSample { V3<R> dir; V3<R> Le; R pdf; R dist; };
    // lightTreeImportance (PathTrace.slang:3932-3966)
    R lt_importance(uint32_t idx, V3<R> hp, V3<R> n_face) const {
        const PtLightTreeNode& nd = S.light_tree[idx];
        const V3<R> lo = ld3<R>(nd.aabb_min), hi = ld3<R>(nd.aabb_max);
        const V3<R> to_c = (lo + hi) * R(0.5) - hp;
        const R d2 = mx(dot(to_c, to_c), R(1e-12));
        const R d = std::sqrt(d2);
        const V3<R> dir_to = to_c / d;
        const V3<R> ext = (hi - lo) * R(0.5);
        const R rad2 = mx(dot(ext, ext), R(1e-12));
        const R falloff = R(1) / mx(d2, rad2);
        R orient = R(1);
        if (R(nd.cone_cos_half) > R(-0.999)) {
            const R cos_emit = -dot(ld3<R>(nd.cone_axis), dir_to);
            orient = sat((cos_emit - (R(nd.cone_cos_half) - R(0.2))) / R(0.2));
        }
        const R recv = mx(R(0), dot(n_face, dir_to));
        return mx(R(nd.intensity) * falloff * orient * recv, R(1e-8));
    }
    // pickLightFromTree (PathTrace.slang:3978-4016)
    uint32_t lt_pick(V3<R> hp, V3<R> n_face, uint32_t& seed, R& pick_pdf) const {
        uint32_t idx = 0;
        pick_pdf = R(1);
        for (int d = 0; d < 32; ++d) {
            const PtLightTreeNode& nd = S.light_tree[idx];
            if (nd.count > 0u) return nd.left_first;
            const R il = lt_importance(nd.left_first, hp, n_face);
            const R ir = lt_importance(nd.left_first + 1u, hp, n_face);
            const R total = il + ir;
            const R p_l = (total > R(1e-30)) ? (il / total) : R(0.5);
            const R u = randf<R>(seed);
            if (u < p_l) {
                idx = nd.left_first;
                pick_pdf = pick_pdf * p_l;
            } else {
                idx = nd.left_first + 1u;
                pick_pdf = pick_pdf * (R(1) - p_l);
            }
        }
        return 0u;
    }

    LightSample sample_light(V3<R> hp, V3<R> n_face, uint32_t& seed) const {
        LightSample s{{R(0), R(1), R(0)}, {R(0), R(0), R(0)}, R(0), R(1e30)};
        const uint32_t n = Q.light_count;
        if (n == 0u) return s;
        uint32_t pick;
        R pick_pdf;
        if (Q.light_tree_enabled != 0u && Q.light_tree_node_count > 0u) {
            pick = std::min(lt_pick(hp, n_face, seed, pick_pdf), n - 1u);
        } else {
            const R u_pick = randf<R>(seed);
            pick = std::min(uint32_t(u_pick * R(n)), n - 1u);
            pick_pdf = R(1) / R(n);
        }
        const float* L = S.lights + size_t(pick) * 20;
        const uint32_t type = uint32_t(L[7] + 0.5f);
        const V3<R> pos = ld3<R>(L);
        const V3<R> inten = ld3<R>(L + 4);
        if (type == 0u || type == 1u) {   // point / spot
            const V3<R> tl = pos - hp;
            const R d2 = mx(dot(tl, tl), R(1e-12));
            const R d = std::sqrt(d2);
            if (type == 0u) {
                s.dir = tl / d;
                s.Le = inten / d2;
            } else {
                const V3<R> tld = tl / d;
                const V3<R> axis = normalize(quat_rotate<R>(L + 16, ld3<R>(L + 8)));
                const R cos_dir = dot(-tld, axis);
                const R cin = R(L[12]), cout = R(L[11]);
                R fall = R(0);
                if (cos_dir >= cin) fall = R(1);
                else if (cos_dir > cout) fall = (cos_dir - cout) / mx(cin - cout, R(1e-6));
                s.dir = tld;
                s.Le = inten * (fall / d2);
            }
            s.pdf = pick_pdf;
            s.dist = d;
            return s;
        }
        if (type == 2u) {   // sphere: uniform area
            const R x0 = randf<R>(seed);
            const R x1 = randf<R>(seed);
            const R z = R(1) - R(2) * x0;
            const R r = std::sqrt(mx(R(0), R(1) - z * z));
            const R phi = kTwoPi * x1;
            const V3<R> nl{r * M<R>::cos(phi), r * M<R>::sin(phi), z};
            const V3<R> lp = pos + nl * R(L[3]);
            const V3<R> tl = lp - hp;
            const R d2 = mx(dot(tl, tl), R(1e-12));
            const R d = std::sqrt(d2);
            const V3<R> wi = tl / d;
            const R cl = mx(R(0), dot(nl, -wi));
            if (cl <= R(0)) return s;
            const R area = R(4.0) * kPi * R(L[3]) * R(L[3]);
            const R pdf_sa = d2 / mx(area * cl, R(1e-12));
            s.dir = wi;
            s.Le = inten;
            s.pdf = pick_pdf * pdf_sa;
            s.dist = d;
            return s;
        }
        if (type == 3u) {   // quad
            const R xa = randf<R>(seed) * R(2) - R(1);
            const R xb = randf<R>(seed) * R(2) - R(1);
            const V3<R> uvec = quat_rotate<R>(L + 16, ld3<R>(L + 12));
            const R ulen = length(uvec);
            if (ulen < R(1e-6)) return s;
            const V3<R> nq = normalize(quat_rotate<R>(L + 16, ld3<R>(L + 8)));
            const V3<R> vax = normalize(cross(nq, uvec));
            const V3<R> lp = pos + uvec * xa + vax * (R(L[15]) * xb);
            const V3<R> tl = lp - hp;
            const R d2 = mx(dot(tl, tl), R(1e-12));
            const R d = std::sqrt(d2);
            const V3<R> wi = tl / d;
            const R cl = dot(nq, -wi);
            if (cl <= R(0)) return s;
            const R area = R(4.0) * ulen * R(L[15]);
            const R pdf_sa = d2 / mx(area * cl, R(1e-12));
            s.dir = wi;
            s.Le = inten;
            s.pdf = pick_pdf * pdf_sa;
            s.dist = d;
            return s;
        }
        return s;
    }

    // --- transmittance (PathTrace.slang:5089-5196), clouds/water off ---
    V3<R> transmittance(V3<R> o, V3<R> d, R t_max) {
        const int kmax = int(Q.refract_budget);
        V3<R> t{R(1), R(1), R(1)};
        if (adj) adj->nx = 0;
        for (int i = 0; i <= kmax; ++i) {
            cnt.shadow++;
            const Hit<R> h = trace(o, d);
            if (!h.hit || h.t >= t_max) return t;
            if (h.mat != kMatDielectric) return {R(0), R(0), R(0)};
            if (i == kmax) return {R(0), R(0), R(0)};
            const R ndi = dot(h.normal, d);
            const V3<R> nf = (ndi < R(0)) ? h.normal : -h.normal;
            const R ia = (ndi < R(0)) ? R(1) : h.ior;
            const R ib = (ndi < R(0)) ? h.ior : R(1);
            const R eta = ia / ib;
            const R cos_i = std::fabs(dot(nf, -d));
            const R r0 = ((ia - ib) / (ia + ib)) * ((ia - ib) / (ia + ib));
            const R fr = schlick(cos_i, r0);
            const V3<R> refr = refract(d, nf, eta);
            if (length(refr) < R(1e-3)) return {R(0), R(0), R(0)};
            t = t * ((R(1) - fr) * h.albedo);
            if (adj && adj->nx < 16) adj->xm[adj->nx++] = h.mid;
            const R adv = h.t + R(1e-3);
            o = o + d * adv;
            d = normalize(refr);
            t_max = mx(t_max - adv, R(0));
        }
        return {R(0), R(0), R(0)};
    }

    // PathTraceMath.slang:73-76
    static R schlick(R cos_t, R r0) {
        const R m = R(1) - cos_t;
        return r0 + (R(1) - r0) * m * m * m * m * m;
    }
    // PathTraceMath.slang:30-42
    V3<R> cos_hemi(V3<R> n, uint32_t& seed) const {
        const R u1 = randf<R>(seed);
        const R u2 = randf<R>(seed);
        const R r = std::sqrt(u1);
        const R phi = R(6.28318530718) * u2;
        const R x = r * M<R>::cos(phi);
        const R y = r * M<R>::sin(phi);
        const R z = std::sqrt(mx(R(0), R(1) - u1));
        const V3<R> ax = (std::fabs(n.x) > R(0.9)) ? V3<R>{R(0), R(1), R(0)} : V3<R>{R(1), R(0), R(0)};
        const V3<R> t = normalize(cross(n, ax));
        const V3<R> b = cross(n, t);
        return normalize(t * x + b * y + n * z);
    }

    // --- one camera sample: the body of `for s < spp` (PathTrace.slang:5722-7705) ---
    V3<R> sample_path(uint32_t px, uint32_t py, uint32_t s, uint32_t& seed) {
        R jx, jy;
        if (P.denoiser_enabled != 0u && s == 0u) {
            jx = R(frame_jx);
            jy = R(frame_jy);
        } else {
            const R a = randf<R>(seed);
            const R b = randf<R>(seed);
            jx = a - R(0.5);
            jy = b - R(0.5);
        }
        const R ux = ((R(px) + R(0.5) + jx) / R(W)) * R(2) - R(1);
        R uy = ((R(py) + R(0.5) + jy) / R(H)) * R(2) - R(1);
        uy = -uy;
        V3<R> ro = ld3<R>(P.pos_fovtan);
        const R tanf = R(P.pos_fovtan[3]);
        V3<R> rd = normalize(ld3<R>(P.fwd_aspect) + ld3<R>(P.right_xyz) * (ux * R(P.fwd_aspect[3]) * tanf) +
                             ld3<R>(P.up_xyz) * (uy * tanf));
        V3<R> thr{R(1), R(1), R(1)}, rad{R(0), R(0), R(0)};
        bool skip_sky = false, prev_lambert = false;
        R prev_pdf = R(0);
        const bool env = P.env_map_present != 0u;
        const uint32_t maxb = P.max_bounces;
        if (adj) adj->nv = 0;
        // adds c to the sample radiance (and its albedo derivatives to the sink)
        auto add = [&](V3<R> c, bool shadow) {
            rad = rad + c;
            if (adj) adj->contrib(c, shadow);
        };
        for (uint32_t b = 0; b < maxb; ++b) {
            if (cap_o && b == cap_bounce) {
                float* o = cap_o + 4 * cap_slot;
                float* d = cap_d + 4 * cap_slot;
                o[0] = float(ro.x); o[1] = float(ro.y); o[2] = float(ro.z); o[3] = 0.0f;
                d[0] = float(rd.x); d[1] = float(rd.y); d[2] = float(rd.z); d[3] = 0.0f;
            }
            cnt.ext++;
            const uint64_t n0 = cnt.nodes, t0 = cnt.tris, p0 = cnt.prims;
            Hit<R> h = trace(ro, rd);
            cnt.ext_nodes += cnt.nodes - n0;
            cnt.ext_tris += cnt.tris - t0;
            cnt.ext_prims += cnt.prims - p0;
            if (!h.hit) {
                if (Q.mis_enabled != 0u && prev_lambert) {
                    if (!is_cluster_dir(rd)) {
                        const R pe = pdf_env_dir(rd);
                        const R wb = mis_balance(prev_pdf, pe);
                        // transmittance(ro, rd, 1e30) re-traces this same ray, which
                        // just missed everything: it returns exactly (1,1,1).
                        const V3<R> trans{R(1), R(1), R(1)};
                        add(clamp_ind(thr * sky_color(rd) * trans * wb), false);
                    }
                } else if (!skip_sky) {
                    if (b == 0u) add(thr * sky_color(rd), false);
                    else add(clamp_ind(thr * sky_color(rd)), false);
                }
                break;
            }
            const V3<R> hp = ro + rd * h.t;
            const R ndi = dot(h.normal, rd);
            const V3<R> nf = (ndi < R(0)) ? h.normal : -h.normal;
            if (any_pos(h.emission)) {
                if (b == 0u) add(thr * h.emission, false);
                else add(clamp_ind(thr * h.emission), false);
                if (adj) adj->emission(thr, h.mid);
            }
            if (adj && (h.mat == kMatLambert || h.mat == kMatMetal) && adj->nv < 64) adj->vm[adj->nv++] = h.mid;
            if (h.mat == kMatLambert) {
                if (Q.light_count > 0u) {
                    const LightSample ls = sample_light(hp, nf, seed);
                    const R ndl = dot(nf, ls.dir);
                    if (ls.pdf > R(0) && ndl > R(0)) {
                        const R tmax = mx(ls.dist - R(1e-3), R(0));
                        const V3<R> tr = transmittance(hp + nf * R(1e-3), ls.dir, tmax);
                        if (any_pos(tr)) {
                            const V3<R> brdf = h.albedo / kPi;
                            const V3<R> c = thr * ls.Le * tr * brdf * ndl / ls.pdf;
                            add((b == 0u) ? c : clamp_ind(c), true);
                        }
                    }
                }
                if (env) {
                    const R xu = randf<R>(seed);
                    const R xv = randf<R>(seed);
                    const EnvSample es = sample_env(xu, xv);
                    const R ndl = dot(nf, es.dir);
                    if (es.pdf > R(0) && ndl > R(0)) {
                        const V3<R> tr = transmittance(hp + nf * R(1e-3), es.dir, R(1e30));
                        if (any_pos(tr)) {
                            const V3<R> brdf = h.albedo / kPi;
                            const R pdf_brdf = ndl * kInvPi;
                            const bool fire = (Q.mis_enabled != 0u) && ((b + 1u) < maxb);
                            const R wl = fire ? mis_balance(es.pdf, pdf_brdf) : R(1);
                            add(clamp_ind(thr * es.color * tr * brdf * ndl * wl / es.pdf), true);
                        }
                    }
                    if (S.hdri_count > 0u) {
                        const HdriSample hl = sample_hdri(seed);
                        const R ndl2 = dot(nf, hl.dir);
                        if (ndl2 > R(0) && hl.pdf > R(0)) {
                            const V3<R> ts = transmittance(hp + nf * R(1e-3), hl.dir, R(1e30));
                            if (any_pos(ts)) {
                                const V3<R> brdf = h.albedo / kPi;
                                const V3<R> c = thr * hl.color * ts * brdf * ndl2 / hl.pdf;
                                rad = rad + ((b == 0u) ? c : clamp_ind(c));
                            }
                        }
                    }
                    skip_sky = (Q.mis_enabled == 0u);
                } else {
                    // gradient sky: sun NEE, moon NEE, skylight ambient (PathTrace.slang:6546-6667)
                    const V3<R> sd = sun_dir();
                    if (sd.y > R(0)) {
                        const R n_dot_l = mx(R(0), dot(nf, sd));
                        const V3<R> sun_jit = sample_sun_disc(sd, seed);
                        const V3<R> trans = (n_dot_l > R(0)) ? transmittance(hp + nf * R(1e-3), sun_jit, R(1e30))
                                                              : V3<R>{R(0), R(0), R(0)};
                        const R am = R(1) / mx(sd.y, R(0.04));
                        const R trans_atm = M<R>::exp(R(-0.30) * am);
                        const R warmth = sat((am - R(1)) * R(0.18));
                        const V3<R> sun_col =
                            lerp(V3<R>{R(1.00), R(0.97), R(0.92)}, V3<R>{R(1.55), R(0.55), R(0.20)}, warmth);
                        const R strength = R(80.0) * trans_atm;
                        const V3<R> sun_rad = sun_col * strength;
                        const V3<R> brdf = h.albedo / kPi;
                        if (n_dot_l > R(0) && any_pos(trans)) add(thr * sun_rad * trans * brdf * n_dot_l, true);
                    }
                    const float* mph = Q.moon_dir_phase;
                    if (R(mph[1]) > R(0)) {
                        const R phase_b = R(0.5) * (R(1) - M<R>::cos(R(mph[3])));
                        if (phase_b > R(0.01)) {
                            const V3<R> moon_jit = sample_sun_disc(ld3<R>(mph), seed);
                            const R ndl = mx(R(0), dot(nf, moon_jit));
                            if (ndl > R(0)) {
                                const V3<R> t_m = transmittance(hp + nf * R(1e-3), moon_jit, R(1e30));
                                if (any_pos(t_m)) {
                                    const R m_elev = mx(R(mph[1]), R(0.04));
                                    const R m_am = R(1) / m_elev;
                                    const R m_atm = M<R>::exp(R(-0.30) * m_am);
                                    const R m_warmth = sat((m_am - R(1)) * R(0.18));
                                    const V3<R> m_col = lerp(V3<R>{R(0.92), R(0.94), R(1.00)},
                                                             V3<R>{R(1.20), R(0.65), R(0.40)}, m_warmth);
                                    const V3<R> moon_rad = m_col * (R(0.3) * phase_b * m_atm);
                                    const V3<R> brdf = h.albedo / kPi;
                                    add(thr * moon_rad * t_m * brdf * ndl, true);
                                }
                            }
                        }
                    }
                    add(thr * h.albedo * sky_base(nf), false);
                    skip_sky = true;
                }
                thr = thr * h.albedo;
                ro = hp + nf * R(1e-3);
                rd = cos_hemi(nf, seed);
                if (Q.mis_enabled != 0u && env) {
                    prev_pdf = mx(R(0), dot(nf, rd)) * kInvPi;
                    prev_lambert = true;
                } else {
                    prev_lambert = false;
                }
            } else if (h.mat == kMatMetal) {
                V3<R> r = reflect(rd, nf);
                r = normalize(r + h.roughness * (cos_hemi(nf, seed) - nf));
                thr = thr * h.albedo;
                ro = hp + nf * R(1e-3);
                rd = r;
                skip_sky = false;
                prev_lambert = false;
            } else if (h.mat == kMatDielectric) {
                const R ia = (ndi < R(0)) ? R(1) : h.ior;
                const R ib = (ndi < R(0)) ? h.ior : R(1);
                const R eta = ia / ib;
                const R cos_i = std::fabs(dot(nf, -rd));
                R r0 = (ia - ib) / (ia + ib);
                r0 = r0 * r0;
                const R fr = schlick(cos_i, r0);
                const V3<R> refl = reflect(rd, nf);
                const V3<R> refr = refract(rd, nf, eta);
                const bool tir = length(refr) < R(1e-3);
                if (tir || randf<R>(seed) < fr) {
                    rd = refl;
                    ro = hp + nf * R(1e-3);
                    skip_sky = false;
                    prev_lambert = false;
                } else {
                    rd = normalize(refr);
                    ro = hp - nf * R(1e-3);
                }
            }
            if (b >= Q.rr_start) {
                R p = mx(thr.x, mx(thr.y, thr.z));
                p = clampv(p, R(0.05), R(1));
                if (randf<R>(seed) > p) break;
                thr = thr / p;
            }
        }
        return rad;
    }

    // frame radiance of one pixel: average of spp samples, sanitised (PathTrace.slang:7707-7734)
    V3<R> pixel(uint32_t px, uint32_t py, uint32_t frame_index) {
        set_frame(frame_index);
        uint32_t seed = pcg_hash(px * 1973u + py * 9277u + frame_index * 26699u);
        const uint32_t n = (P.spp == 0u) ? 1u : P.spp;
        V3<R> fr{R(0), R(0), R(0)};
        for (uint32_t s = 0; s < n; ++s) fr = fr + sample_path(px, py, s, seed);
        fr = fr / R(n);
        auto clean = [](R v) { return (std::isnan(v) || std::isinf(v)) ? R(0) : mx(v, R(0)); };
        return {clean(fr.x), clean(fr.y), clean(fr.z)};
    }
};

// running mean / EMA update (PathTrace.slang:7736-7781)
template <class R> void accumulate(R* prev4, V3<R> fr, bool reset, R ema_in) {
    R p[4] = {prev4[0], prev4[1], prev4[2], prev4[3]};
    if (reset) p[0] = p[1] = p[2] = p[3] = R(0);
    bool bad = false;
    for (int i = 0; i < 4; ++i) bad = bad || std::isnan(p[i]) || std::isinf(p[i]);
    if (bad) p[0] = p[1] = p[2] = p[3] = R(0);
    const R ema = clampv(ema_in, R(0), R(0.999));
    R n_new;
    V3<R> avg;
    const V3<R> pr{p[0], p[1], p[2]};
    if (p[3] < R(0.5) || ema <= R(0)) {
        n_new = p[3] + R(1);
        avg = (pr * p[3] + fr) / n_new;
    } else {
        avg = pr * ema + fr * (R(1) - ema);
        n_new = mn(p[3] + R(1), R(1) / mx(R(1) - ema, R(1e-3)));
    }
    prev4[0] = avg.x; prev4[1] = avg.y; prev4[2] = avg.z; prev4[3] = n_new;
}

template <class R>
void render(const PtPackedScene& S, const PtPushHead& P, const PtPathParams& Q, uint32_t W,
            uint32_t H, uint32_t frames, float* accum, uint32_t x0, uint32_t y0, uint32_t x1,
            uint32_t y1, int threads, Counters& total) {
    std::vector<R> acc(size_t(W) * H * 4);
    for (size_t i = 0; i < acc.size(); ++i) acc[i] = R(accum[i]);
    const uint32_t rows = y1 - y0;
    int nt = threads > 0 ? threads : int(std::thread::hardware_concurrency());
    if (nt < 1) nt = 1;
    std::vector<Counters> per(nt);
    std::atomic<uint32_t> next{0};
    auto worker = [&](int tid) {
        Tracer<R> tr(S, P, Q, W, H);
        for (;;) {
            const uint32_t r = next.fetch_add(1);
            if (r >= rows) break;
            const uint32_t y = y0 + r;
            for (uint32_t x = x0; x < x1; ++x) {
                R* a = acc.data() + (size_t(y) * W + x) * 4;
                for (uint32_t f = 0; f < frames; ++f) {
                    const V3<R> fr = tr.pixel(x, y, P.frame_index + f);
                    accumulate<R>(a, fr, f == 0 && P.reset_accum != 0u, R(Q.accum_ema_alpha));
                }
            }
        }
        per[tid] = tr.cnt;
    };
    std::vector<std::thread> pool;
    for (int i = 0; i < nt; ++i) pool.emplace_back(worker, i);
    for (auto& t : pool) t.join();
    for (const auto& c : per) total.add(c);
    for (uint32_t y = y0; y < y1; ++y)
        for (uint32_t x = x0; x < x1; ++x)
            for (int c = 0; c < 4; ++c) {
                const size_t i = (size_t(y) * W + x) * 4 + c;
                accum[i] = float(acc[i]);
            }
}

// The extension rays of bounce `bounce` of every sample of one frame over the
// pixels of [x0,x1) x [y0,y1), fp32 instance (the rays the GPU render traces,
// bit for bit): slot ((y - y0) * (x1 - x0) + (x - x0)) * spp + s.  Samples whose
// path ended before that bounce keep a zero direction.
void capture_rays(const PtPackedScene& S, const PtPushHead& P, const PtPathParams& Q, uint32_t W, uint32_t H,
                  uint32_t bounce, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1, float* out_o,
                  float* out_d, int threads) {
    const uint32_t spp = (P.spp == 0u) ? 1u : P.spp;
    const uint32_t cw = x1 - x0, rows = y1 - y0;
    std::fill(out_o, out_o + size_t(cw) * rows * spp * 4, 0.0f);
    std::fill(out_d, out_d + size_t(cw) * rows * spp * 4, 0.0f);
    int nt = threads > 0 ? threads : int(std::thread::hardware_concurrency());
    if (nt < 1) nt = 1;
    std::atomic<uint32_t> next{0};
    auto worker = [&]() {
        Tracer<float> tr(S, P, Q, W, H);
        tr.cap_o = out_o;
        tr.cap_d = out_d;
        tr.cap_bounce = bounce;
        for (;;) {
            const uint32_t r = next.fetch_add(1);
            if (r >= rows) break;
            const uint32_t y = y0 + r;
            for (uint32_t x = x0; x < x1; ++x) {
                tr.set_frame(P.frame_index);
                uint32_t seed = pcg_hash(x * 1973u + y * 9277u + P.frame_index * 26699u);
                for (uint32_t s = 0; s < spp; ++s) {
                    tr.cap_slot = (size_t(r) * cw + (x - x0)) * spp + s;
                    (void)tr.sample_path(x, y, s, seed);
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int i = 0; i < nt; ++i) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
}

// adjoint oracle: fp32 paths (the GPU's, bit for bit), derivatives in double
void adjoint(const PtPackedScene& S, const PtPushHead& P, const PtPathParams& Q, uint32_t W, uint32_t H,
             uint32_t frames, const float* dldi, int threads, double* g_alb, double* g_em) {
    const uint32_t spp = (P.spp == 0u) ? 1u : P.spp;
    const double scale = 1.0 / (double(frames) * double(spp));
    int nt = threads > 0 ? threads : int(std::thread::hardware_concurrency());
    if (nt < 1) nt = 1;
    std::vector<AdjSink> sinks(nt);
    std::atomic<uint32_t> next{0};
    auto worker = [&](int tid) {
        AdjSink& a = sinks[tid];
        a.mats = S.materials;
        a.nmat = S.material_count;
        a.g_alb.assign(3 * size_t(S.material_count), 0.0);
        a.g_em.assign(3 * size_t(S.material_count), 0.0);
        Tracer<float> tr(S, P, Q, W, H);
        tr.adj = &a;
        for (;;) {
            const uint32_t y = next.fetch_add(1);
            if (y >= H) break;
            for (uint32_t x = 0; x < W; ++x) {
                const float* d = dldi + (size_t(y) * W + x) * 4;
                if (d[0] == 0.0f && d[1] == 0.0f && d[2] == 0.0f) continue;
                for (int c = 0; c < 3; ++c) a.w[c] = double(d[c]) * scale;
                for (uint32_t f = 0; f < frames; ++f) {
                    tr.set_frame(P.frame_index + f);
                    uint32_t seed = pcg_hash(x * 1973u + y * 9277u + (P.frame_index + f) * 26699u);
                    for (uint32_t s = 0; s < spp; ++s) (void)tr.sample_path(x, y, s, seed);
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int i = 0; i < nt; ++i) pool.emplace_back(worker, i);
    for (auto& t : pool) t.join();
    for (const auto& a : sinks)
        for (size_t i = 0; i < a.g_alb.size(); ++i) {
            g_alb[i] += a.g_alb[i];
            g_em[i] += a.g_em[i];
        }
}

template <class R>
void trace_rays(const PtPackedScene& S, const PtPushHead& P, const PtPathParams& Q,
                const float* ro, const float* rd, uint32_t n, uint32_t* hit, float* t,
                Counters& total) {
    Tracer<R> tr(S, P, Q, 1, 1);
    for (uint32_t i = 0; i < n; ++i) {
        const float* o = ro + size_t(i) * 4;
        const float* d = rd + size_t(i) * 4;
        const R tinit = (d[3] > 0.0f) ? R(d[3]) : R(1e30);
        const Hit<R> h = tr.trace(ld3<R>(o), ld3<R>(d), tinit);
        hit[i] = h.hit ? h.id : kHitMiss;
        t[i] = h.hit ? float(h.t) : 0.0f;
    }
    total.add(tr.cnt);
}

// The reference's Software-backend preview estimator, restated as a timed CPU
// baseline (src/rhi_software/SoftwareTracer.cpp:870-1014; the procedural sky of
// :215-228, the default sun of :697-705).  Per pixel: one primary ray through
// the pixel centre; on a miss the procedural sky; on a hit 0.3 x albedo x
// sky(n) of ambient, one shadow ray to the sun and Lambert sun light, plus
// emission; NaN/negative channels zeroed, then the running mean.  Rows are
// handed out by an atomic counter as the reference does.  The reference
// traces with Embree; this restatement uses the oracle's traversal of the
// uploaded BVHs.
static V3<float> sw_proc_sky(V3<float> d, V3<float> sun) {
    const float t_y = clampv(d.y * 0.5f + 0.5f, 0.0f, 1.0f);
    const V3<float> horizon{0.55f, 0.62f, 0.70f}, zenith{0.18f, 0.32f, 0.55f};
    const float w = std::pow(t_y, 0.7f);
    const V3<float> sky = horizon * (1.0f - w) + zenith * w;
    const float cos_sun = clampv(dot(d, sun), 0.0f, 1.0f);
    const float halo = std::pow(cos_sun, 6.0f) * 0.5f;
    const float disc = (cos_sun > 0.9998f) ? 2.5f : 0.0f;
    return sky + V3<float>{1.0f, 0.92f, 0.78f} * (halo + disc);
}

void software_preview(const PtPackedScene& S, const PtPushHead& P, const PtPathParams& Q, uint32_t W,
                      uint32_t H, float* accum, int threads, Counters& total) {
    V3<float> sun{Q.sun_and_mode[0], Q.sun_and_mode[1], Q.sun_and_mode[2]};
    sun = (length(sun) > 1e-3f) ? normalize(sun) : normalize(V3<float>{0.4f, 0.8f, 0.3f});
    int nt = threads > 0 ? threads : int(std::thread::hardware_concurrency());
    if (nt < 1) nt = 1;
    std::vector<Counters> per(nt);
    std::atomic<uint32_t> next{0};
    const float inv_w = 1.0f / float(W), inv_h = 1.0f / float(H);
    const float tanf = P.pos_fovtan[3], aspect = P.fwd_aspect[3];
    auto worker = [&](int tid) {
        Tracer<float> tr(S, P, Q, W, H);
        for (;;) {
            const uint32_t y = next.fetch_add(1);
            if (y >= H) break;
            for (uint32_t x = 0; x < W; ++x) {
                const float ndc_x = (float(x) + 0.5f) * inv_w * 2.0f - 1.0f;
                const float ndc_y = 1.0f - (float(y) + 0.5f) * inv_h * 2.0f;
                const V3<float> rd = normalize(ld3<float>(P.fwd_aspect) + ld3<float>(P.right_xyz) * (ndc_x * aspect * tanf) +
                                               ld3<float>(P.up_xyz) * (ndc_y * tanf));
                const V3<float> ro = ld3<float>(P.pos_fovtan);
                const Hit<float> h0 = tr.trace(ro, rd);
                tr.cnt.ext++;
                V3<float> col{0.0f, 0.0f, 0.0f};
                if (!h0.hit) {
                    col = sw_proc_sky(rd, sun);
                } else {
                    const V3<float> hp = ro + rd * h0.t;
                    const V3<float> nf = (dot(h0.normal, rd) < 0.0f) ? h0.normal : h0.normal * -1.0f;
                    const float n_dot_l = std::max(0.0f, dot(nf, sun));
                    const V3<float> ambient = h0.albedo * sw_proc_sky(nf, sun) * 0.30f;
                    V3<float> lit{0.0f, 0.0f, 0.0f};
                    if (n_dot_l > 0.0f) {
                        const Hit<float> sh = tr.trace(hp + nf * 1e-3f, sun);
                        tr.cnt.shadow++;
                        if (!sh.hit) lit = h0.albedo * V3<float>{2.4f, 2.2f, 1.9f} * n_dot_l;
                    }
                    col = ambient + lit + h0.emission;
                }
                float* a = accum + (size_t(y) * W + x) * 4;
                accumulate<float>(a, col, P.reset_accum != 0u, Q.accum_ema_alpha);
            }
        }
        per[tid] = tr.cnt;
    };
    std::vector<std::thread> pool;
    for (int i = 0; i < nt; ++i) pool.emplace_back(worker, i);
    for (auto& t : pool) t.join();
    for (const auto& c : per) total.add(c);
}

void export_counters(const Counters& c, OracleCounters* out) {
    if (!out) return;
    out->rays = c.rays;
    out->nodes = c.nodes;
    out->tris = c.tris;
    out->prims = c.prims;
    out->ext_rays = c.ext;
    out->shadow_rays = c.shadow;
    out->ext_nodes = c.ext_nodes;
    out->ext_tris = c.ext_tris;
    out->ext_prims = c.ext_prims;
}

}  // namespace orc

extern "C" {

int oracle_trace(const PtPackedScene* scene, const PtPushHead* head, const PtPathParams* params,
                 const float* ray_o, const float* ray_d, uint32_t n, uint32_t* hit_id, float* t,
                 int fp64, OracleCounters* counters) {
    if (!scene || !head || !params || (n && (!ray_o || !ray_d || !hit_id || !t))) return -1;
    orc::Counters c;
    if (fp64) orc::trace_rays<double>(*scene, *head, *params, ray_o, ray_d, n, hit_id, t, c);
    else orc::trace_rays<float>(*scene, *head, *params, ray_o, ray_d, n, hit_id, t, c);
    orc::export_counters(c, counters);
    return 0;
}

int oracle_render(const PtPackedScene* scene, const PtPushHead* head, const PtPathParams* params,
                  uint32_t W, uint32_t H, uint32_t frames, float* accum_rgba, uint32_t x0,
                  uint32_t y0, uint32_t x1, uint32_t y1, int fp64, int threads,
                  OracleCounters* counters) {
    if (!scene || !head || !params || !accum_rgba || W == 0 || H == 0) return -1;
    if (x1 > W || y1 > H || x0 > x1 || y0 > y1) return -1;
    // tlas (hardware RT), the light tree and the no-env-map sky branch
    // (procedural sun/moon NEE) are not restated.
    if (head->tlas_present) return -6;
    if (params->light_tree_enabled && params->light_tree_node_count &&
        (!scene->light_tree || params->light_tree_node_count != scene->light_tree_node_count))
        return -6;
    if (params->sun_and_mode[3] == 3.0f || (params->sun_and_mode[3] == 2.0f && params->stars)) return -6;
    if (!head->env_map_present && params->moon_dir_phase[1] >= -0.10f && !scene->moon_rgba) return -6;
    orc::Counters c;
    if (fp64)
        orc::render<double>(*scene, *head, *params, W, H, frames, accum_rgba, x0, y0, x1, y1, threads, c);
    else
        orc::render<float>(*scene, *head, *params, W, H, frames, accum_rgba, x0, y0, x1, y1, threads, c);
    orc::export_counters(c, counters);
    return 0;
}

int oracle_capture_rays(const PtPackedScene* scene, const PtPushHead* head, const PtPathParams* params,
                        uint32_t W, uint32_t H, uint32_t bounce, uint32_t x0, uint32_t y0, uint32_t x1,
                        uint32_t y1, float* ray_o, float* ray_d, int threads) {
    if (!scene || !head || !params || !ray_o || !ray_d || W == 0 || H == 0) return -1;
    if (x1 > W || y1 > H || x0 > x1 || y0 > y1) return -1;
    if (head->tlas_present) return -6;
    orc::capture_rays(*scene, *head, *params, W, H, bounce, x0, y0, x1, y1, ray_o, ray_d, threads);
    return 0;
}

int oracle_software_preview(const PtPackedScene* scene, const PtPushHead* head, const PtPathParams* params,
                            uint32_t W, uint32_t H, float* accum_rgba, int threads, OracleCounters* counters) {
    if (!scene || !head || !params || !accum_rgba || W == 0 || H == 0) return -1;
    orc::Counters c;
    orc::software_preview(*scene, *head, *params, W, H, accum_rgba, threads, c);
    orc::export_counters(c, counters);
    return 0;
}

// Environment-map importance sampling and its pdf (sampleEnvMap / pdfEnvMapDir,
// shaders/PathTrace.slang:3638-3727) for n given uniform pairs, with the fp32
// instance the GPU matches: directions (x, y, z, 0), pdfs and the sampled
// texel (v * W + u).  For the statistical tests of the sampler.
int oracle_env_sample(const PtPackedScene* scene, const PtPushHead* head, const PtPathParams* params, uint32_t n,
                      const float* xu, const float* xv, float* dir4, float* pdf, float* pdf_of_dir) {
    if (!scene || !head || !params || (n && (!xu || !xv || !dir4 || !pdf || !pdf_of_dir))) return -1;
    orc::Tracer<float> tr(*scene, *head, *params, 1, 1);
    for (uint32_t i = 0; i < n; ++i) {
        const auto es = tr.sample_env(xu[i], xv[i]);
        dir4[4 * size_t(i)] = es.dir.x;
        dir4[4 * size_t(i) + 1] = es.dir.y;
        dir4[4 * size_t(i) + 2] = es.dir.z;
        dir4[4 * size_t(i) + 3] = 0.0f;
        pdf[i] = es.pdf;
        pdf_of_dir[i] = tr.pdf_env_dir(es.dir);
    }
    return 0;
}

int oracle_adjoint(const PtPackedScene* scene, const PtPushHead* head, const PtPathParams* params,
                   uint32_t W, uint32_t H, uint32_t frames, const float* dl_di_rgba, int threads,
                   double* grad_albedo, double* grad_emission) {
    if (!scene || !head || !params || !dl_di_rgba || !grad_albedo || !grad_emission || W == 0 || H == 0)
        return -1;
    if (head->tlas_present) return -6;
    if (params->light_tree_enabled && params->light_tree_node_count &&
        (!scene->light_tree || params->light_tree_node_count != scene->light_tree_node_count))
        return -6;
    if (params->sun_and_mode[3] == 3.0f || (params->sun_and_mode[3] == 2.0f && params->stars)) return -6;
    if (!head->env_map_present && params->moon_dir_phase[1] >= -0.10f && !scene->moon_rgba) return -6;
    if (params->firefly_clamp > 0.0f) return -7;   // the clamp is not differentiable
    for (size_t i = 0; i < 3 * size_t(scene->material_count); ++i) grad_albedo[i] = grad_emission[i] = 0.0;
    orc::adjoint(*scene, *head, *params, W, H, frames, dl_di_rgba, threads, grad_albedo, grad_emission);
    return 0;
}

// Output step (PathTrace.slang:3466-3607, 7925-7929), fp32, the kernels' order.
namespace {
using orc::V3;
float satf(float x) { return std::fmin(std::fmax(x, 0.0f), 1.0f); }
float log2o(float x) { return orc::f_log(x) * 0x1.715476p+0f; }
float pow_nz(float x, float y) { return (y == 1.0f) ? x : orc::f_pow(x, y); }
V3<float> sat3(V3<float> v) { return {satf(v.x), satf(v.y), satf(v.z)}; }
V3<float> div3(V3<float> a, V3<float> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
V3<float> tm_aces(V3<float> c) {
    const float a = 2.51f, b = 0.03f, d = 2.43f, e = 0.59f, f = 0.14f;
    const V3<float> num = c * (c * a + V3<float>{b, b, b});
    const V3<float> den = c * (c * d + V3<float>{e, e, e}) + V3<float>{f, f, f};
    return sat3(div3(num, den));
}
float agx_contrast(float x) {
    const float x2 = x * x, x4 = x2 * x2;
    return 15.5f * x4 * x2 - 40.14f * x4 * x + 31.96f * x4 - 6.868f * x2 * x + 0.4298f * x2 + 0.1191f * x -
           0.00232f;
}
V3<float> tm_agx(V3<float> c) {
    const V3<float> ir0{0.842479062253094f, 0.0784335999999992f, 0.0792237451477643f};
    const V3<float> ir1{0.0423282422610123f, 0.878468636469772f, 0.0791661274605434f};
    const V3<float> ir2{0.0423756549057051f, 0.0784336f, 0.879142973793104f};
    float t[3] = {orc::dot(ir0, c), orc::dot(ir1, c), orc::dot(ir2, c)};
    const float kMinEv = -12.47393f, kMaxEv = 4.026069f;
    for (float& x : t) {
        float l = std::fmin(std::fmax(log2o(std::fmax(x, 1e-10f)), kMinEv), kMaxEv);
        l = (l - kMinEv) / (kMaxEv - kMinEv);
        x = agx_contrast(l);
    }
    V3<float> v{t[0], t[1], t[2]};
    const float luma = orc::dot(v, V3<float>{0.2126f, 0.7152f, 0.0722f});
    v = {pow_nz(std::fmax(v.x * 1.0f + 0.0f, 0.0f), 1.0f), pow_nz(std::fmax(v.y * 1.0f + 0.0f, 0.0f), 1.0f),
         pow_nz(std::fmax(v.z * 1.0f + 0.0f, 0.0f), 1.0f)};
    v = V3<float>{luma, luma, luma} + (v - V3<float>{luma, luma, luma}) * 1.0f;
    const V3<float> or0{1.19687900512017f, -0.0980208811401368f, -0.0990297440797205f};
    const V3<float> or1{-0.0528968517574562f, 1.15190312990417f, -0.0989611768448433f};
    const V3<float> or2{-0.0529716355144438f, -0.0980434501171241f, 1.15107367264116f};
    v = {orc::dot(or0, v), orc::dot(or1, v), orc::dot(or2, v)};
    v = {pow_nz(std::fmax(v.x, 0.0f), 2.2f), pow_nz(std::fmax(v.y, 0.0f), 2.2f), pow_nz(std::fmax(v.z, 0.0f), 2.2f)};
    return sat3(v);
}
V3<float> tm_khronos(V3<float> c) {
    const float start = 0.8f - 0.04f, desat = 0.15f;
    const float x = std::fmin(c.x, std::fmin(c.y, c.z));
    const float offset = (x < 0.08f) ? (x - 6.25f * x * x) : 0.04f;
    c = c - V3<float>{offset, offset, offset};
    const float peak = std::fmax(c.x, std::fmax(c.y, c.z));
    if (peak < start) return c;
    const float d = 1.0f - start;
    const float new_peak = 1.0f - d * d / (peak + d - start);
    c = c * (new_peak / peak);
    const float g = 1.0f - 1.0f / (desat * (peak - new_peak) + 1.0f);
    return orc::lerp(c, V3<float>{new_peak, new_peak, new_peak}, g);
}
float srgb_oetf(float c) {
    c = std::fmax(c, 0.0f);
    return (c < 0.0031308f) ? c * 12.92f : 1.055f * orc::f_pow(c, 1.0f / 2.4f) - 0.055f;
}
}  // namespace

int oracle_tonemap(const float* accum_rgba, uint32_t n, float exposure, uint32_t op, int srgb, uint8_t* out) {
    if ((n && (!accum_rgba || !out)) || op > 4u) return -1;
    for (uint32_t i = 0; i < n; ++i) {
        const V3<float> c = V3<float>{accum_rgba[4 * i], accum_rgba[4 * i + 1], accum_rgba[4 * i + 2]} * exposure;
        V3<float> l;
        switch (op) {
            case 1: l = tm_agx(c); break;
            case 2: l = tm_khronos(c); break;
            case 3: l = sat3(div3(c, V3<float>{1.0f, 1.0f, 1.0f} + c)); break;
            case 4: l = sat3(c); break;
            default: l = tm_aces(c); break;
        }
        if (srgb) l = {srgb_oetf(l.x), srgb_oetf(l.y), srgb_oetf(l.z)};
        out[4 * i + 0] = uint8_t(uint32_t(satf(l.x) * 255.0f + 0.5f));
        out[4 * i + 1] = uint8_t(uint32_t(satf(l.y) * 255.0f + 0.5f));
        out[4 * i + 2] = uint8_t(uint32_t(satf(l.z) * 255.0f + 0.5f));
        out[4 * i + 3] = 255;
    }
    return 0;
}

float oracle_sinf(float x) { return orc::f_sin(x); }
float oracle_cosf(float x) { return orc::f_cos(x); }
float oracle_atan2f(float y, float x) { return orc::f_atan2(y, x); }
float oracle_acosf(float x) { return orc::f_acos(x); }
uint32_t oracle_pcg_hash(uint32_t x) { return orc::pcg_hash(x); }
float oracle_expf(float x) { return orc::f_exp(x); }
float oracle_logf(float x) { return orc::f_log(x); }
float oracle_powf(float x, float y) { return orc::f_pow(x, y); }
float oracle_asinf(float x) { return orc::f_asin(x); }

}  // extern "C"
