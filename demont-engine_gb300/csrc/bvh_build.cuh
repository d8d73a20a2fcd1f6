// GPU binned-SAH BVH builder and the 4-wide node layout the traversal walks.
//
// Build (top-down, level-synchronous on the device):
//   tasks larger than kSmallTask items: per level, chunks of kChunk items bin
//     their centroids into kBins bins per axis (shared-memory atomics, flushed
//     to per-task global bins), one thread per task sweeps the bins for the
//     lowest surface-area-heuristic cost, and the chunks partition the item
//     index array around the chosen plane;
//   tasks of at most kSmallTask items: one thread builds the whole subtree
//     depth-first (16-bin SAH, in-place partition).  A range of at most
//     kMaxLeaf items becomes a leaf when the SAH says so: n*A <= kLeafCt*A +
//     the best split's cost (A: half areas; kLeafCt: the cost of a node visit
//     relative to one primitive test, 1.5 measured best on the C0/C1 scenes
//     among 1, 1.5 and 2); single items are always leaves.
// The binary tree is then collapsed on the host into 4-wide nodes of 128 bytes
// (one L2 line): each node keeps its children's boxes in SoA form so a thread
// tests four boxes per fetch.  Boxes are padded outward by a relative 2^-20 so
// rounding in the slab test can never cull a primitive whose hit lies on its box.
//
// The tree only decides which primitives get tested.  Exact-distance ties are
// resolved by each primitive's rank in the reference traversal order (the
// right-child-first depth-first order of the reference's own BVH, computed by
// ref_ranks below), so the closest hit equals the reference's first-tested-wins
// result on any tree.
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

namespace ptb {

constexpr int kBins = 32;        // 32 and 16 bins: +0.7% on the 1080p triangle scene over 16 and 8
constexpr int kSmallBins = 16;
constexpr uint32_t kSmallTask = 256;
constexpr uint32_t kMaxLeaf = 4;
constexpr float kLeafCt = 1.5f;
constexpr uint32_t kChunk = 4096;
constexpr int kBinWords = 13;   // count, box lo[3] hi[3], centroid lo[3] hi[3]
constexpr int kTaskBinWords = 3 * kBins * kBinWords;
constexpr int kWideStack = 96;   // traversal stack entries (device)

// ordered-uint encoding of floats, so unsigned min/max = float min/max
__device__ __forceinline__ uint32_t f2o(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__device__ __forceinline__ float half_area(float lx, float ly, float lz, float hx, float hy, float hz) {
    const float dx = fmaxf(hx - lx, 0.0f), dy = fmaxf(hy - ly, 0.0f), dz = fmaxf(hz - lz, 0.0f);
    return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ int bin_of(float c, float cmin, float scale, int nb) {
    int b = int((c - cmin) * scale);
    return b < 0 ? 0 : (b >= nb ? nb - 1 : b);
}

// root centroid bounds
__global__ void kb_cbounds(const float4* lo, const float4* hi, uint32_t n, uint32_t* out6) {
    float mn[3] = {3e38f, 3e38f, 3e38f}, mx[3] = {-3e38f, -3e38f, -3e38f};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 l = lo[i], h = hi[i];
        const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
        for (int a = 0; a < 3; ++a) {
            mn[a] = fminf(mn[a], c[a]);
            mx[a] = fmaxf(mx[a], c[a]);
        }
    }
    for (int a = 0; a < 3; ++a) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[a] = fminf(mn[a], __shfl_down_sync(0xFFFFFFFFu, mn[a], o));
            mx[a] = fmaxf(mx[a], __shfl_down_sync(0xFFFFFFFFu, mx[a], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int a = 0; a < 3; ++a) {
            atomicMin(out6 + a, f2o(mn[a]));
            atomicMax(out6 + 3 + a, f2o(mx[a]));
        }
    }
}

// chunk = (task, begin, end, 0); task info = (begin, end, node, 0)
__global__ void kb_bin(const uint4* chunks, const float4* tcmin, const float4* tcmax, const uint32_t* idx,
                       const float4* lo, const float4* hi, uint32_t* bins) {
    __shared__ uint32_t sb[kTaskBinWords];
    for (int i = threadIdx.x; i < kTaskBinWords; i += blockDim.x) {
        const int w = i % kBinWords;
        sb[i] = (w == 0) ? 0u : ((w <= 3 || (w >= 7 && w <= 9)) ? 0xFFFFFFFFu : 0u);
    }
    __syncthreads();
    const uint4 ch = chunks[blockIdx.x];
    const float4 cmn = tcmin[ch.x], cmx = tcmax[ch.x];
    const float cm[3] = {cmn.x, cmn.y, cmn.z};
    float sc[3];
    {
        const float ext[3] = {cmx.x - cmn.x, cmx.y - cmn.y, cmx.z - cmn.z};
        for (int a = 0; a < 3; ++a) sc[a] = ext[a] > 0.0f ? float(kBins) * (1.0f - 1e-6f) / ext[a] : 0.0f;
    }
    for (uint32_t i = ch.y + threadIdx.x; i < ch.z; i += blockDim.x) {
        const uint32_t it = idx[i];
        const float4 l = lo[it], h = hi[it];
        const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
        const float bl[3] = {l.x, l.y, l.z}, bh[3] = {h.x, h.y, h.z};
        for (int a = 0; a < 3; ++a) {
            const int b = bin_of(c[a], cm[a], sc[a], kBins);
            uint32_t* w = sb + (a * kBins + b) * kBinWords;
            atomicAdd(w, 1u);
            for (int k = 0; k < 3; ++k) {
                atomicMin(w + 1 + k, f2o(bl[k]));
                atomicMax(w + 4 + k, f2o(bh[k]));
                atomicMin(w + 7 + k, f2o(c[k]));
                atomicMax(w + 10 + k, f2o(c[k]));
            }
        }
    }
    __syncthreads();
    uint32_t* g = bins + size_t(ch.x) * kTaskBinWords;
    for (int i = threadIdx.x; i < kTaskBinWords; i += blockDim.x) {
        const int bin = i / kBinWords, w = i % kBinWords;
        if (sb[bin * kBinWords] == 0u) continue;
        if (w == 0) atomicAdd(g + i, sb[i]);
        else if (w <= 3 || (w >= 7 && w <= 9)) atomicMin(g + i, sb[i]);
        else atomicMax(g + i, sb[i]);
    }
}

// per large task: pick the split; write the node and the two child tasks.
// split out: (axis or -1 for positional, bin, nleft, 0)
__global__ void kb_split(uint32_t ntasks, const uint4* tinfo, const uint32_t* bins, float4* nodes,
                         uint32_t* node_counter, int4* split, uint4* child_info, float4* child_cmin,
                         float4* child_cmax, const float4* tcmin, const float4* tcmax) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks) return;
    const uint4 ti = tinfo[t];
    const uint32_t count = ti.y - ti.x;
    const uint32_t* g = bins + size_t(t) * kTaskBinWords;
    // node box = union over axis-0 bins
    float bl[3] = {3e38f, 3e38f, 3e38f}, bh[3] = {-3e38f, -3e38f, -3e38f};
    for (int b = 0; b < kBins; ++b) {
        const uint32_t* w = g + b * kBinWords;
        if (w[0] == 0u) continue;
        for (int k = 0; k < 3; ++k) {
            bl[k] = fminf(bl[k], o2f(w[1 + k]));
            bh[k] = fmaxf(bh[k], o2f(w[4 + k]));
        }
    }
    float best = 3e38f;
    int best_a = -1, best_b = -1;
    uint32_t best_nl = 0;
    for (int a = 0; a < 3; ++a) {
        float rl[kBins][3], rh[kBins][3];
        uint32_t rc[kBins];
        float l[3] = {3e38f, 3e38f, 3e38f}, h[3] = {-3e38f, -3e38f, -3e38f};
        uint32_t c = 0;
        for (int b = kBins - 1; b >= 0; --b) {
            const uint32_t* w = g + (a * kBins + b) * kBinWords;
            if (w[0]) {
                for (int k = 0; k < 3; ++k) {
                    l[k] = fminf(l[k], o2f(w[1 + k]));
                    h[k] = fmaxf(h[k], o2f(w[4 + k]));
                }
                c += w[0];
            }
            rc[b] = c;
            for (int k = 0; k < 3; ++k) { rl[b][k] = l[k]; rh[b][k] = h[k]; }
        }
        float L[3] = {3e38f, 3e38f, 3e38f}, Hh[3] = {-3e38f, -3e38f, -3e38f};
        uint32_t cl = 0;
        for (int b = 0; b < kBins - 1; ++b) {
            const uint32_t* w = g + (a * kBins + b) * kBinWords;
            if (w[0]) {
                for (int k = 0; k < 3; ++k) {
                    L[k] = fminf(L[k], o2f(w[1 + k]));
                    Hh[k] = fmaxf(Hh[k], o2f(w[4 + k]));
                }
                cl += w[0];
            }
            const uint32_t cr = rc[b + 1];
            if (cl == 0 || cr == 0) continue;
            const float cost = float(cl) * half_area(L[0], L[1], L[2], Hh[0], Hh[1], Hh[2]) +
                               float(cr) * half_area(rl[b + 1][0], rl[b + 1][1], rl[b + 1][2], rh[b + 1][0],
                                                     rh[b + 1][1], rh[b + 1][2]);
            if (cost < best) { best = cost; best_a = a; best_b = b; best_nl = cl; }
        }
    }
    float lcl[3] = {3e38f, 3e38f, 3e38f}, lch[3] = {-3e38f, -3e38f, -3e38f};
    float rcl[3] = {3e38f, 3e38f, 3e38f}, rch[3] = {-3e38f, -3e38f, -3e38f};
    if (best_a < 0) {   // no usable plane: split the range in half, keep the centroid bounds
        best_nl = count / 2;
        const float4 a = tcmin[t], b = tcmax[t];
        lcl[0] = rcl[0] = a.x; lcl[1] = rcl[1] = a.y; lcl[2] = rcl[2] = a.z;
        lch[0] = rch[0] = b.x; lch[1] = rch[1] = b.y; lch[2] = rch[2] = b.z;
    } else {
        for (int b = 0; b < kBins; ++b) {
            const uint32_t* w = g + (best_a * kBins + b) * kBinWords;
            if (!w[0]) continue;
            float* ml = (b <= best_b) ? lcl : rcl;
            float* mh = (b <= best_b) ? lch : rch;
            for (int k = 0; k < 3; ++k) {
                ml[k] = fminf(ml[k], o2f(w[7 + k]));
                mh[k] = fmaxf(mh[k], o2f(w[10 + k]));
            }
        }
    }
    const uint32_t left = atomicAdd(node_counter, 2u);
    nodes[2u * ti.z] = make_float4(bl[0], bl[1], bl[2], __uint_as_float(left));
    nodes[2u * ti.z + 1u] = make_float4(bh[0], bh[1], bh[2], __uint_as_float(0u));
    split[t] = make_int4(best_a, best_b, int(best_nl), 0);
    child_info[2 * t] = make_uint4(ti.x, ti.x + best_nl, left, 0u);
    child_info[2 * t + 1] = make_uint4(ti.x + best_nl, ti.y, left + 1u, 0u);
    child_cmin[2 * t] = make_float4(lcl[0], lcl[1], lcl[2], 0.0f);
    child_cmax[2 * t] = make_float4(lch[0], lch[1], lch[2], 0.0f);
    child_cmin[2 * t + 1] = make_float4(rcl[0], rcl[1], rcl[2], 0.0f);
    child_cmax[2 * t + 1] = make_float4(rch[0], rch[1], rch[2], 0.0f);
}

__global__ void kb_partition(const uint4* chunks, const uint4* tinfo, const int4* split, const float4* tcmin,
                             const float4* tcmax, const uint32_t* idx, const float4* lo, const float4* hi,
                             uint32_t* counters, uint32_t* tmp) {
    const uint4 ch = chunks[blockIdx.x];
    const int4 sp = split[ch.x];
    const uint4 ti = tinfo[ch.x];
    if (sp.x < 0) {   // positional split: items stay where they are
        for (uint32_t i = ch.y + threadIdx.x; i < ch.z; i += blockDim.x) tmp[i] = idx[i];
        return;
    }
    const float4 cmn = tcmin[ch.x], cmx = tcmax[ch.x];
    const float cm = (sp.x == 0) ? cmn.x : (sp.x == 1 ? cmn.y : cmn.z);
    const float cx = (sp.x == 0) ? cmx.x : (sp.x == 1 ? cmx.y : cmx.z);
    const float ext = cx - cm;
    const float sc = ext > 0.0f ? float(kBins) * (1.0f - 1e-6f) / ext : 0.0f;
    for (uint32_t base = ch.y; base < ch.z; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        bool valid = i < ch.z;
        bool left = false;
        uint32_t it = 0;
        if (valid) {
            it = idx[i];
            const float4 l = lo[it], h = hi[it];
            const float c = (sp.x == 0) ? 0.5f * (l.x + h.x) : (sp.x == 1 ? 0.5f * (l.y + h.y) : 0.5f * (l.z + h.z));
            left = bin_of(c, cm, sc, kBins) <= sp.y;
        }
        const uint32_t ml = __ballot_sync(0xFFFFFFFFu, valid && left);
        const uint32_t mr = __ballot_sync(0xFFFFFFFFu, valid && !left);
        const int lane = threadIdx.x & 31;
        uint32_t bl = 0, br = 0;
        if (lane == 0) {
            if (ml) bl = atomicAdd(counters + 2 * ch.x, __popc(ml));
            if (mr) br = atomicAdd(counters + 2 * ch.x + 1, __popc(mr));
        }
        bl = __shfl_sync(0xFFFFFFFFu, bl, 0);
        br = __shfl_sync(0xFFFFFFFFu, br, 0);
        const uint32_t below = (1u << lane) - 1u;
        if (valid) {
            const uint32_t dst = left ? (ti.x + bl + __popc(ml & below))
                                      : (ti.x + uint32_t(sp.z) + br + __popc(mr & below));
            tmp[dst] = it;
        }
    }
}

__global__ void kb_copy(const uint4* chunks, const uint32_t* tmp, uint32_t* idx) {
    const uint4 ch = chunks[blockIdx.x];
    for (uint32_t i = ch.y + threadIdx.x; i < ch.z; i += blockDim.x) idx[i] = tmp[i];
}

// one thread per small task: whole subtree, depth first
__global__ void kb_small(uint32_t ntasks, const uint4* tinfo, uint32_t* idx, const float4* lo, const float4* hi,
                         float4* nodes, uint32_t* node_counter) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks) return;
    const uint4 ti = tinfo[t];
    uint32_t st_node[40], st_b[40], st_e[40];
    int sp = 0;
    st_node[0] = ti.z; st_b[0] = ti.x; st_e[0] = ti.y; sp = 1;
    while (sp > 0) {
        --sp;
        const uint32_t node = st_node[sp], b0 = st_b[sp], e0 = st_e[sp];
        const uint32_t n = e0 - b0;
        float bl[3] = {3e38f, 3e38f, 3e38f}, bh[3] = {-3e38f, -3e38f, -3e38f};
        float cl[3] = {3e38f, 3e38f, 3e38f}, ch[3] = {-3e38f, -3e38f, -3e38f};
        for (uint32_t i = b0; i < e0; ++i) {
            const float4 l = lo[idx[i]], h = hi[idx[i]];
            const float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
            bl[0] = fminf(bl[0], l.x); bl[1] = fminf(bl[1], l.y); bl[2] = fminf(bl[2], l.z);
            bh[0] = fmaxf(bh[0], h.x); bh[1] = fmaxf(bh[1], h.y); bh[2] = fmaxf(bh[2], h.z);
            for (int a = 0; a < 3; ++a) { cl[a] = fminf(cl[a], c[a]); ch[a] = fmaxf(ch[a], c[a]); }
        }
        if (n <= 1u) {
            nodes[2u * node] = make_float4(bl[0], bl[1], bl[2], __uint_as_float(b0));
            nodes[2u * node + 1u] = make_float4(bh[0], bh[1], bh[2], __uint_as_float(n));
            continue;
        }
        // kSmallBins-bin SAH over the three axes
        float best = 3e38f;
        int ba = -1, bb = -1;
        for (int a = 0; a < 3; ++a) {
            const float ext = ch[a] - cl[a];
            if (!(ext > 0.0f)) continue;
            const float sc = float(kSmallBins) * (1.0f - 1e-6f) / ext;
            uint32_t cnt[kSmallBins] = {0};
            float L[kSmallBins][3], H[kSmallBins][3];
            for (int k = 0; k < kSmallBins; ++k)
                for (int j = 0; j < 3; ++j) { L[k][j] = 3e38f; H[k][j] = -3e38f; }
            for (uint32_t i = b0; i < e0; ++i) {
                const float4 l = lo[idx[i]], h = hi[idx[i]];
                const float c = (a == 0) ? 0.5f * (l.x + h.x) : (a == 1 ? 0.5f * (l.y + h.y) : 0.5f * (l.z + h.z));
                const int k = bin_of(c, cl[a], sc, kSmallBins);
                cnt[k]++;
                L[k][0] = fminf(L[k][0], l.x); L[k][1] = fminf(L[k][1], l.y); L[k][2] = fminf(L[k][2], l.z);
                H[k][0] = fmaxf(H[k][0], h.x); H[k][1] = fmaxf(H[k][1], h.y); H[k][2] = fmaxf(H[k][2], h.z);
            }
            for (int s = 0; s < kSmallBins - 1; ++s) {
                float l0[3] = {3e38f, 3e38f, 3e38f}, h0[3] = {-3e38f, -3e38f, -3e38f};
                float l1[3] = {3e38f, 3e38f, 3e38f}, h1[3] = {-3e38f, -3e38f, -3e38f};
                uint32_t c0 = 0, c1 = 0;
                for (int k = 0; k < kSmallBins; ++k) {
                    if (!cnt[k]) continue;
                    float* ml = (k <= s) ? l0 : l1;
                    float* mh = (k <= s) ? h0 : h1;
                    for (int j = 0; j < 3; ++j) { ml[j] = fminf(ml[j], L[k][j]); mh[j] = fmaxf(mh[j], H[k][j]); }
                    if (k <= s) c0 += cnt[k]; else c1 += cnt[k];
                }
                if (!c0 || !c1) continue;
                const float cost = float(c0) * half_area(l0[0], l0[1], l0[2], h0[0], h0[1], h0[2]) +
                                   float(c1) * half_area(l1[0], l1[1], l1[2], h1[0], h1[1], h1[2]);
                if (cost < best) { best = cost; ba = a; bb = s; }
            }
        }
        if (n <= kMaxLeaf) {   // SAH leaf test: n*A <= Ct/Ci*A + split cost
            const float A = half_area(bl[0], bl[1], bl[2], bh[0], bh[1], bh[2]);
            if (ba < 0 || float(n) * A <= kLeafCt * A + best) {
                nodes[2u * node] = make_float4(bl[0], bl[1], bl[2], __uint_as_float(b0));
                nodes[2u * node + 1u] = make_float4(bh[0], bh[1], bh[2], __uint_as_float(n));
                continue;
            }
        }
        uint32_t mid;
        if (ba < 0) {
            mid = b0 + n / 2;
        } else {
            const float sc = float(kSmallBins) * (1.0f - 1e-6f) / (ch[ba] - cl[ba]);
            uint32_t i = b0, j = e0;
            while (i < j) {
                const float4 l = lo[idx[i]], h = hi[idx[i]];
                const float c = (ba == 0) ? 0.5f * (l.x + h.x) : (ba == 1 ? 0.5f * (l.y + h.y) : 0.5f * (l.z + h.z));
                if (bin_of(c, cl[ba], sc, kSmallBins) <= bb) {
                    ++i;
                } else {
                    --j;
                    const uint32_t tmp = idx[i];
                    idx[i] = idx[j];
                    idx[j] = tmp;
                }
            }
            mid = i;
            if (mid == b0 || mid == e0) mid = b0 + n / 2;
        }
        const uint32_t left = atomicAdd(node_counter, 2u);
        nodes[2u * node] = make_float4(bl[0], bl[1], bl[2], __uint_as_float(left));
        nodes[2u * node + 1u] = make_float4(bh[0], bh[1], bh[2], __uint_as_float(0u));
        if (sp + 2 > 40) {   // cannot happen for <= 256 items with halving splits; guard anyway
            continue;
        }
        st_node[sp] = left; st_b[sp] = b0; st_e[sp] = mid; ++sp;
        st_node[sp] = left + 1u; st_b[sp] = mid; st_e[sp] = e0; ++sp;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct Node2H {
    float lo[3];
    uint32_t lf;
    float hi[3];
    uint32_t count;
};

// Child codes are what the traversal pushes: an internal child is its node
// index; a leaf is kWideLeafBit | (items - 1) << 28 | first item position.  An
// empty slot has code 0 and the degenerate box at (kEmptyBox)^3, which every
// slab test rejects (its entry distance is huge, infinite or NaN), so the
// traversal needs no emptiness test.  The traversal loads the first 112 bytes.
constexpr uint32_t kWideLeafBit = 0x80000000u;
constexpr uint32_t kWideMaxLeafItems = 8u;          // 3 count bits
constexpr uint32_t kWideMaxItem = 1u << 28;          // first-item field
constexpr float kEmptyBox = 3.0e38f;

struct Wide4 {   // 128 bytes, the device node
    float lox[4], hix[4], loy[4], hiy[4], loz[4], hiz[4];
    uint32_t code[4];   // traversal codes (above)
    int32_t count[4];   // -1 empty, 0 internal, > 0 leaf item count (not read by the traversal)
};
static_assert(sizeof(Wide4) == 128, "wide node must be one 128-byte line");

inline float pad_lo(float v, float ext) { return v - (std::fabs(v) + ext) * 9.5367431640625e-7f; }
inline float pad_hi(float v, float ext) { return v + (std::fabs(v) + ext) * 9.5367431640625e-7f; }

inline float area2(const Node2H& n) {
    const float dx = n.hi[0] - n.lo[0], dy = n.hi[1] - n.lo[1], dz = n.hi[2] - n.lo[2];
    return dx * dy + dy * dz + dz * dx;
}

// Collapse the binary tree into 4-wide nodes (greedy: open the largest child).
// Returns the maximum depth in wide nodes, or -1 when a leaf does not fit the
// child code (more than 8 items, or a first item at or past 2^28).
inline int collapse4(const std::vector<Node2H>& bin, std::vector<Wide4>& out) {
    out.clear();
    if (bin.empty()) return 0;
    struct Item { uint32_t bin_node; uint32_t wide_idx; int depth; };
    std::vector<Item> work;
    out.push_back(Wide4{});
    work.push_back({0u, 0u, 1});
    int max_depth = 1;
    while (!work.empty()) {
        const Item it = work.back();
        work.pop_back();
        max_depth = std::max(max_depth, it.depth);
        uint32_t kids[4];
        int nk = 0;
        const Node2H& root = bin[it.bin_node];
        if (root.count > 0) {
            kids[nk++] = it.bin_node;   // a leaf root: one leaf child
        } else {
            kids[nk++] = root.lf;
            kids[nk++] = root.lf + 1;
            while (nk < 4) {
                int pick = -1;
                float pa = -1.0f;
                for (int k = 0; k < nk; ++k) {
                    if (bin[kids[k]].count == 0 && area2(bin[kids[k]]) > pa) {
                        pa = area2(bin[kids[k]]);
                        pick = k;
                    }
                }
                if (pick < 0) break;
                const uint32_t c = kids[pick];
                kids[pick] = bin[c].lf;
                kids[nk++] = bin[c].lf + 1;
            }
        }
        Wide4 w{};
        for (int k = 0; k < 4; ++k) {
            if (k >= nk) {
                w.lox[k] = w.loy[k] = w.loz[k] = kEmptyBox;
                w.hix[k] = w.hiy[k] = w.hiz[k] = kEmptyBox;
                w.code[k] = 0u;
                w.count[k] = -1;
                continue;
            }
            const Node2H& c = bin[kids[k]];
            const float ext = std::max(c.hi[0] - c.lo[0], std::max(c.hi[1] - c.lo[1], c.hi[2] - c.lo[2]));
            w.lox[k] = pad_lo(c.lo[0], ext); w.hix[k] = pad_hi(c.hi[0], ext);
            w.loy[k] = pad_lo(c.lo[1], ext); w.hiy[k] = pad_hi(c.hi[1], ext);
            w.loz[k] = pad_lo(c.lo[2], ext); w.hiz[k] = pad_hi(c.hi[2], ext);
            if (c.count > 0) {
                if (c.count > kWideMaxLeafItems || c.lf >= kWideMaxItem) return -1;
                w.code[k] = kWideLeafBit | ((c.count - 1u) << 28) | c.lf;
                w.count[k] = int32_t(c.count);
            } else {
                const uint32_t wi = uint32_t(out.size());
                out.push_back(Wide4{});
                w.code[k] = wi;
                w.count[k] = 0;
                work.push_back({kids[k], wi, it.depth + 1});
            }
        }
        out[it.wide_idx] = w;
    }
    return max_depth;
}

// Visit order of every leaf slot in the reference traversal (depth first,
// right child popped first, stack limit `stack_limit` with the reference's
// drop-both-children rule).  Returns false when the reference traversal would
// drop a subtree or a slot is covered zero or several times: the wide tree then
// cannot reproduce it and the caller keeps the reference traversal.
inline bool ref_ranks(const PtBvhNode* nodes, uint32_t n_nodes, uint32_t n_slots, int stack_limit,
                      std::vector<uint32_t>& rank) {
    rank.assign(n_slots, 0xFFFFFFFFu);
    if (n_nodes == 0) {
        for (uint32_t i = 0; i < n_slots; ++i) rank[i] = i;
        return true;
    }
    std::vector<uint32_t> st;
    st.push_back(0);
    uint32_t ord = 0;
    while (!st.empty()) {
        const uint32_t i = st.back();
        st.pop_back();
        const PtBvhNode& n = nodes[i];
        if (n.count > 0) {
            for (uint32_t k = 0; k < n.count; ++k) {
                const uint32_t s = n.left_first + k;
                if (rank[s] != 0xFFFFFFFFu) return false;
                rank[s] = ord++;
            }
        } else {
            if (int(st.size()) + 2 > stack_limit) return false;
            st.push_back(n.left_first);
            st.push_back(n.left_first + 1);
        }
    }
    return ord == n_slots;
}

}  // namespace ptb
