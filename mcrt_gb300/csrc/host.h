// Host-side scene preparation: BVH construction, flattening into the device layouts,
// emitter and environment-map sampling tables.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mcrt_gb300.h"
#include "layout.h"

namespace mcrt {

// A binary BVH in the form of the C ABI's mcrt_bvh_tree (see mcrt_gb300.h).
struct BinaryTree
{
    std::vector<float>   node_box;   // 6 per node
    std::vector<int32_t> node_info;  // 6 per node: is_leaf, left, right, axis, ref_begin, ref_count
    std::vector<int32_t> ref_prim;
    std::vector<float>   ref_box;    // 6 per ref
    int                  root = 0;
};

// Default largest leaf of the library's builder.  Per cfg1 frame (1.3 M triangles), ms:
// leaves of <= 2 triangles 118.3, <= 3 118.7, <= 4 120.5, <= 6 126.1, <= 8 131.3 -- a
// watertight triangle test costs more than a two-box node step.
constexpr int kDefaultLeafSize = 2;

// Binned-SAH object-split builder (own design; leaf <= leaf_size references).
// Multithreaded over subtrees.  Leaves reference contiguous runs of ref_prim.
void build_sah_tree(const float* vertices, int64_t num_tris, int leaf_size, BinaryTree& out);

// The same with spatial splits (sbvh_build.cpp): references straddling a split plane are
// duplicated with clipped boxes.  Leaves reference contiguous runs of ref_prim.
void build_split_tree(const float* vertices, int64_t num_tris, int leaf_size, BinaryTree& out);

struct FlatBVH
{
    std::vector<FastNode> fast_nodes;
    std::vector<float4>   fast_tris;  // 3 per reference
    std::vector<RefNode>  ref_nodes;
    std::vector<RefPrim>  ref_prims;
    int                   max_depth = 0;
    std::vector<WideNode> wide_nodes;
    std::vector<float4>   wide_tris;  // 3 per leaf-child reference
    int                   wide_depth = 0;
};

// Validates the tree and emits both device layouts in depth-first order.
// Returns an empty string on success, else an error message.
std::string flatten_tree(const BinaryTree& tree, const float* vertices, int64_t num_tris, FlatBVH& out);

// Collapses a validated binary tree into the eight-child layout (WideNode, wide_tris):
// an SAH-optimal choice of each wide node's children among its binary descendants,
// octant slot assignment and outward-rounded 8-bit child boxes.  c_tri: the cost of a
// triangle test relative to a wide-node visit.
#ifndef MCRT_WIDE_CTRI
#define MCRT_WIDE_CTRI 0.4f
#endif
std::string build_wide(const BinaryTree& tree, const float* vertices, int64_t num_tris, FlatBVH& out,
                       float c_tri = MCRT_WIDE_CTRI);
// Whether this build's FAST traversal walks the eight-child tree (device.cuh, MCRT_FAST_WIDE);
// scenes then carry it, else the two-child FastNode tree only.
bool fast_layout_wide();

// Checks every index a traversal of the eight-child layout follows (child blocks, leaf
// triangle ranges, primitive ids) and the tree depth; an empty string when all are valid.
std::string validate_wide(const std::vector<WideNode>& nodes, const std::vector<float4>& tris, int64_t num_prims,
                          int* depth);

struct HostScene
{
    FlatBVH                  bvh;
    std::vector<float4>      prim_verts;  // 3 per prim
    std::vector<float4>      prim_shade;  // 3 per prim
    std::vector<int32_t>     light_of;
    std::vector<LightGPU>    lights;
    float                    light_area = 0.f;
    std::vector<MaterialGPU> materials;
    int                      env_w = 0, env_h = 0;
    std::vector<float4>      env_rgb;
    std::vector<float>       env_marginal;
    std::vector<float>       env_cond;
    std::vector<int32_t>     env_guide_m;  // kEnvGuideM + 1 entries
    std::vector<int32_t>     env_guide_c;  // per column kEnvGuideC + 1 entries
    std::vector<float4>      prim_alpha;   // per prim consistent-normal alphas (empty: none used)
    float                    env_norm = 0.f;
};

// the library's device scene from / to its prepared host arrays (scene cache files)
int scene_from_host(const HostScene& hs, int64_t num_tris, uint64_t desc_hash, mcrt_scene** out);
int scene_to_host(const mcrt_scene* s, HostScene& hs, int64_t& num_tris, uint64_t& desc_hash);
// FNV-1a 64 of everything a scene is built from, and of the cache format version
uint64_t scene_desc_hash(const mcrt_scene_desc& d);
// prepared host arrays from a scene description (builder, flattener, sampling tables)
std::string prepare_scene(const mcrt_scene_desc& d, HostScene& hs);

}  // namespace mcrt
