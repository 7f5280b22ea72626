// Test harness (host only): the library's eight-child tree built from a triangle soup, or
// from a given binary tree, and traversed on the host by the device traversal code itself
// (trace_wide is __host__ __device__).  Lets CPU tests check the layout, its quantised
// boxes and the traversal against the reference's hits before any GPU runs them.
#include <cstring>
#include <string>
#include <vector>

#include "../../mcrt_gb300/csrc/device.cuh"
#include "../../mcrt_gb300/csrc/host.h"

namespace {
std::string g_err;
}

extern "C" const char* wide_host_error() { return g_err.c_str(); }

// tree_info == NULL: the library's SAH builder with `leaf_size`; else the binary tree
// (node_box [6n], node_info [6n], ref_prim [r], ref_box [6r]) as mcrt_bvh_tree gives it.
// any = 0: out_t / out_prim get the closest hit (prim -1 on a miss); any = 1: out_prim gets
// 1 when some triangle lies in (tmin, tmax); the closest hit's t is recomputed with the
// reference's Moller-Trumbore as trace_ray does (refine_hit).  stats: nodes visited, triangles tested,
// wide nodes, wide depth, binary depth.
extern "C" int wide_host_trace(const float* verts, long long ntri, int leaf_size, const float* node_box,
                               const int* node_info, int num_nodes, const int* ref_prim, const float* ref_box,
                               int num_refs, const float* rays, long long nrays, int any, float* out_t,
                               int* out_prim, long long* stats)
{
    using namespace mcrt;
    BinaryTree tree;
    if (node_info)
    {
        tree.node_box.assign(node_box, node_box + 6 * static_cast<size_t>(num_nodes));
        tree.node_info.assign(node_info, node_info + 6 * static_cast<size_t>(num_nodes));
        tree.ref_prim.assign(ref_prim, ref_prim + num_refs);
        tree.ref_box.assign(ref_box, ref_box + 6 * static_cast<size_t>(num_refs));
        tree.root = 0;
    }
    else
    {
        build_sah_tree(verts, ntri, leaf_size, tree);
    }
    FlatBVH     fb;
    std::string e = flatten_tree(tree, verts, ntri, fb);
    if (e.empty()) e = build_wide(tree, verts, ntri, fb);
    if (!e.empty())
    {
        g_err = e;
        return -1;
    }
    std::vector<float4> prim_verts(3 * static_cast<size_t>(ntri));
    for (long long i = 0; i < 3 * ntri; ++i)
        prim_verts[i] = make_float4(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2], 0.f);
    SceneView s;
    std::memset(&s, 0, sizeof(s));
    s.wide_nodes = fb.wide_nodes.data();
    s.wide_tris = fb.wide_tris.data();
    s.prim_verts = prim_verts.data();
    constexpr int STACK = 64;
    int           stack[STACK];
    int           err = 0;
    TraceCount    cnt = {0u, 0u};
    long long     nodes = 0, tris = 0;
    for (long long i = 0; i < nrays; ++i)
    {
        const float* r = rays + 8 * i;
        const float3 o = make_float3(r[0], r[1], r[2]), d = make_float3(r[4], r[5], r[6]);
        Hit          h;
        cnt = TraceCount{0u, 0u};
        bool found = any ? trace_wide<true, STACK, true>(s, o, d, r[3], r[7], stack, 1, h, &err, &cnt)
                         : trace_wide<false, STACK, true>(s, o, d, r[3], r[7], stack, 1, h, &err, &cnt);
        if (!any && found) refine_hit(s, o, d, r[3], h);  // as trace_ray: the reported t, u, v
        nodes += cnt.nodes;
        tris += cnt.tris;
        out_prim[i] = any ? (found ? 1 : 0) : (found ? h.prim : -1);
        if (out_t) out_t[i] = found ? h.t : __builtin_inff();
    }
    if (stats)
    {
        stats[0] = nodes;
        stats[1] = tris;
        stats[2] = static_cast<long long>(fb.wide_nodes.size());
        stats[3] = fb.wide_depth;
        stats[4] = fb.max_depth;
    }
    if (err)
    {
        g_err = "traversal stack overflow";
        return -2;
    }
    return 0;
}
