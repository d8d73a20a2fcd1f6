// TEST INFRASTRUCTURE ONLY -- C-ABI shim around the reference's own builders.
//
// Built by oracle/Makefile together with the reference's unmodified sources
// src/renderer/AnalyticBvh.cpp, src/renderer/TriangleBvh.cpp,
// src/renderer/HdrImage.cpp and src/renderer/LightTree.cpp (compiled where
// they lie, never copied), into
// oracle/_ref/libref_builders.so.  Tests use it to pin this repository's host
// builders and the oracle against the reference itself.

#include <atomic>
#include <cstdint>
#include <cstring>
#include <span>
#include <string>
#include <vector>

#include "core/Log.h"
#include "renderer/AnalyticBvh.h"
#include "renderer/HdrImage.h"
#include "renderer/LightTree.h"
#include "renderer/TriangleBvh.h"

// Logging symbols the reference sources reference; the shim discards output.
namespace pt::log {
void Emit(Level, fmt::string_view, fmt::format_args) {}
}  // namespace pt::log
namespace pt::diag {
std::atomic<int> g_diag_level{0};
}  // namespace pt::diag

extern "C" {

// BuildLightTree over inputs laid out as LightInput; nodes_out: 2n-1 x 64 B.
int ref_build_light_tree(const void* inputs, uint32_t n, void* nodes_out, uint32_t* n_nodes) {
    std::vector<pt::renderer::LightInput> in(n);
    if (n) std::memcpy(in.data(), inputs, size_t(n) * sizeof(pt::renderer::LightInput));
    pt::renderer::LightTree tree;
    pt::renderer::BuildLightTree(in, tree);
    if (!tree.nodes.empty())
        std::memcpy(nodes_out, tree.nodes.data(), tree.nodes.size() * sizeof(pt::renderer::LightTreeNode));
    *n_nodes = uint32_t(tree.nodes.size());
    return 0;
}

// ComputeSdfAabb over `count` nodes laid out as SdfNode; 0 on success.
int ref_sdf_aabb(const void* nodes, uint32_t count, float* lo, float* hi) {
    pt::renderer::SdfPrim prim{};
    if (count > pt::renderer::SdfPrim::kMaxNodes) return -1;
    std::memcpy(prim.nodes.data(), nodes, size_t(count) * sizeof(pt::renderer::SdfNode));
    prim.node_count = count;
    if (!pt::renderer::ComputeSdfAabb(prim)) return -2;
    std::memcpy(lo, prim.aabb_min, 12);
    std::memcpy(hi, prim.aabb_max, 12);
    return 0;
}

// LoadRadianceHdr: rgb NULL -> size query; returns 0 on success.
int ref_load_radiance_hdr(const char* path, float* rgb, uint32_t cap, uint32_t* w, uint32_t* h) {
    std::string err;
    const pt::renderer::HdrImage img = pt::renderer::LoadRadianceHdr(path, &err);
    if (img.width == 0 || img.height == 0) return -1;
    *w = img.width;
    *h = img.height;
    if (rgb) {
        if (cap < img.rgb.size()) return -2;
        std::memcpy(rgb, img.rgb.data(), img.rgb.size() * sizeof(float));
    }
    return 0;
}

// centers_radii: 4 floats per prim; prim_id = input index.
int ref_build_analytic_bvh(const float* cr, uint32_t n, void* nodes_out, uint32_t* n_nodes,
                           uint32_t* perm_out) {
    std::vector<pt::renderer::BvhPrim> prims(n);
    for (uint32_t i = 0; i < n; ++i) {
        prims[i].center[0] = cr[4 * i + 0];
        prims[i].center[1] = cr[4 * i + 1];
        prims[i].center[2] = cr[4 * i + 2];
        prims[i].radius = cr[4 * i + 3];
        prims[i].prim_id = i;
    }
    pt::renderer::AnalyticBvh bvh;
    bvh.Build(std::span<const pt::renderer::BvhPrim>(prims));
    const auto& nodes = bvh.Nodes();
    std::memcpy(nodes_out, nodes.data(), nodes.size() * sizeof(nodes[0]));
    *n_nodes = uint32_t(nodes.size());
    const auto& perm = bvh.PermutedPrimIds();
    std::memcpy(perm_out, perm.data(), perm.size() * 4);
    return 0;
}

int ref_build_triangle_bvh(const float* pos, uint32_t nv, const uint32_t* idx, uint32_t n_index,
                           void* nodes_out, uint32_t* n_nodes, uint32_t* perm_out,
                           uint32_t* n_perm) {
    pt::renderer::TriangleBvh bvh;
    bvh.Build(std::span<const float>(pos, size_t(nv) * 3), std::span<const uint32_t>(idx, n_index));
    const auto& nodes = bvh.Nodes();
    if (!nodes.empty()) std::memcpy(nodes_out, nodes.data(), nodes.size() * sizeof(nodes[0]));
    *n_nodes = uint32_t(nodes.size());
    const auto& perm = bvh.PermutedPrimIds();
    if (!perm.empty()) std::memcpy(perm_out, perm.data(), perm.size() * 4);
    *n_perm = uint32_t(perm.size());
    return 0;
}

int ref_build_env_cdf(const float* rgb, uint32_t W, uint32_t H, const uint8_t* mask,
                      float* marginal, float* conditional, double* total) {
    std::vector<float> img(rgb, rgb + size_t(W) * H * 3);
    std::vector<uint8_t> m;
    if (mask) m.assign(mask, mask + size_t(W) * H);
    std::vector<float> mg, cd;
    *total = pt::renderer::BuildEnvCdf(img, W, H, m, mg, cd);
    std::memcpy(marginal, mg.data(), mg.size() * 4);
    std::memcpy(conditional, cd.data(), cd.size() * 4);
    return 0;
}

}  // extern "C"
