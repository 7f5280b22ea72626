// Drop-in SceneBVH backend for MCRT: the GB300 library behind the reference's own
// scene/BVH seam (src/core/scenebvh.h:11-25).  Compile this file into MCRT's rtcore in
// place of src/core/scenebvh.cpp and link libmcrt_gb300.so; Scene::intersect / occluded
// (scene.cpp:77-85) and everything above them (rayTrace, lightPdfW, lightRadiance, ...)
// then run their ray queries on the GPU, unchanged.
//
// Semantics kept from the reference backend (scenebvh.cpp:340-445):
//   * SceneBVH keeps a reference to the caller's triangle vector, which must outlive it;
//   * intersect(): tmin = NUM_EPS_RAY, tmax = infinity, HitInfo carries t, u, v, the
//     interpolated shading normal, the primitive id and the material id;
//   * occluded(ray, tfar): a hit with NUM_EPS_RAY < t < tfar - NUM_EPS_RAY;
//   * hits are bit-identical to the SplitBVH backend when the reference tree is passed in
//     (MCRT_BUILD_EXTERNAL + MCRT_TRAVERSE_REF); with the library's own tree and the
//     watertight traversal (the default) they agree on every non-marginal ray.
// The environment variable MCRT_SCENEBVH_TREE=splitbvh selects the first: the adapter then
// builds the reference's own SplitBVH (through the public static SplitBVH::build, over
// the same BoundedTriangle references SplitBVH::SplitBVH makes, splitbvh.cpp:1410-1433),
// hands its nodes to the library and traverses in the reference's order and arithmetic.
// The reference has no error channel; a failed call prints mcrt_last_error() and aborts,
// as the reference's builder does on its own failures (splitbvh.cpp:1556, 1596).
//
// One call per ray is correct but launch-bound; for throughput call mcrt_trace_closest /
// mcrt_trace_any on batches, or replace DemoSimple::run with mcrt_render.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

#include "acceleration/splitbvh.h"
#include "boundedtriangle.h"
#include "constants.h"
#include "intersection.h"
#include "mcrt_gb300.h"
#include "ray.h"
#include "scenebvh.h"
#include "triangle.h"

namespace {

struct Gb300Context
{
    mcrt_scene* scene = nullptr;
    int32_t     traverse = MCRT_TRAVERSE_FAST;
};

// The reference tree in the form of mcrt_bvh_tree: nodes depth-first, leaf references with
// their clipped bounds (SplitBVHBranchNode / SplitBVHLeafNode, splitbvh.h:32-58).
struct TreeDump
{
    std::vector<float>   node_box, ref_box;
    std::vector<int32_t> node_info, ref_prim;

    int add(const SplitBVHNode* n)
    {
        const int   idx = static_cast<int>(node_info.size() / 6);
        const AABB& b = *n->bounding_box;
        for (int k = 0; k < 3; ++k) node_box.push_back(b.min()[k]);
        for (int k = 0; k < 3; ++k) node_box.push_back(b.max()[k]);
        node_info.resize(node_info.size() + 6, 0);
        if (const SplitBVHLeafNode* leaf = dynamic_cast<const SplitBVHLeafNode*>(n))
        {
            const int begin = static_cast<int>(ref_prim.size());
            for (int i = 0; i < k_sbvh_leaf_node_size; ++i)
            {
                if (!leaf->primitive[i]) continue;
                ref_prim.push_back(leaf->primitive[i]->originalTriangle()->primitiveID());
                const AABB& c = leaf->primitive[i]->clippedBoundingBox();
                for (int k = 0; k < 3; ++k) ref_box.push_back(c.min()[k]);
                for (int k = 0; k < 3; ++k) ref_box.push_back(c.max()[k]);
            }
            const int32_t v[6] = {1, -1, -1, 0, begin, static_cast<int32_t>(ref_prim.size()) - begin};
            std::memcpy(&node_info[6 * idx], v, sizeof(v));
            return idx;
        }
        const SplitBVHBranchNode* br = static_cast<const SplitBVHBranchNode*>(n);
        const int                 l = add(br->left_child.get());
        const int                 r = add(br->right_child.get());
        const int32_t             v[6] = {0, l, r, static_cast<int32_t>(br->split_axis), 0, 0};
        std::memcpy(&node_info[6 * idx], v, sizeof(v));
        return idx;
    }
};

bool use_reference_tree()
{
    const char* e = std::getenv("MCRT_SCENEBVH_TREE");
    return e && std::strcmp(e, "splitbvh") == 0;
}

void check(int rc, const char* what)
{
    if (rc != MCRT_OK)
    {
        std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, mcrt_last_error());
        std::abort();
    }
}

}  // namespace

SceneBVH::SceneBVH(const std::vector<TriangleObject>& triangles) : m_triangles_ref(triangles)
{
    const size_t         n = triangles.size();
    std::vector<float>   verts(9 * n), normals(9 * n);
    std::vector<int32_t> mat_ids(n, 0);
    for (size_t i = 0; i < n; ++i)
    {
        const TriangleObject& t = triangles[i];
        const vec3*           v[6] = {&t.a, &t.b, &t.c, &t.na, &t.nb, &t.nc};
        for (int k = 0; k < 3; ++k)
        {
            verts[9 * i + 3 * k + 0] = v[k]->x;
            verts[9 * i + 3 * k + 1] = v[k]->y;
            verts[9 * i + 3 * k + 2] = v[k]->z;
            normals[9 * i + 3 * k + 0] = v[3 + k]->x;
            normals[9 * i + 3 * k + 1] = v[3 + k]->y;
            normals[9 * i + 3 * k + 2] = v[3 + k]->z;
        }
    }
    // the backend only answers ray queries; shading stays in MCRT, so one material suffices
    mcrt_material m = {MCRT_MAT_DIFF, {1.f, 1.f, 1.f}, 1.f, 1.33f, -1, -1};
    mcrt_scene_desc d = {};
    d.num_triangles = static_cast<int64_t>(n);
    d.vertices = verts.data();
    d.normals = normals.data();
    d.material_ids = mat_ids.data();
    d.num_materials = 1;
    d.materials = &m;
    d.builder = MCRT_BUILD_SAH;
    Gb300Context* ctx = new Gb300Context;
    TreeDump      dump;
    mcrt_bvh_tree tree = {};
    if (use_reference_tree() && n > 0)
    {
        std::vector<std::shared_ptr<Triangle> >        owned;
        std::vector<std::shared_ptr<BoundedTriangle> > refs;
        owned.reserve(n);
        refs.reserve(n);
        for (size_t i = 0; i < n; ++i)
        {
            auto t = std::make_shared<Triangle>(triangles[i]);
            t->setPrimitiveID(static_cast<int>(i));
            owned.push_back(t);
            refs.push_back(std::make_shared<BoundedTriangle>(t, t->boundingBox()));
        }
        std::shared_ptr<SplitBVHNode> root = SplitBVH::build(refs, 0u, "root");
        dump.add(root.get());
        tree.num_nodes = static_cast<int32_t>(dump.node_info.size() / 6);
        tree.num_refs = static_cast<int32_t>(dump.ref_prim.size());
        tree.node_box = dump.node_box.data();
        tree.node_info = dump.node_info.data();
        tree.ref_prim = dump.ref_prim.data();
        tree.ref_box = dump.ref_box.data();
        d.builder = MCRT_BUILD_EXTERNAL;
        d.external_tree = &tree;
        ctx->traverse = MCRT_TRAVERSE_REF;
    }
    check(mcrt_scene_create(&d, &ctx->scene), "mcrt_scene_create");
    m_ctx = ctx;
}

SceneBVH::~SceneBVH()
{
    Gb300Context* ctx = static_cast<Gb300Context*>(m_ctx);
    if (ctx) mcrt_scene_destroy(ctx->scene);
    delete ctx;
}

HitInfo SceneBVH::intersect(const Ray& ray) const
{
    Gb300Context* ctx = static_cast<Gb300Context*>(m_ctx);
    mcrt_ray      r = {{ray.orig.x, ray.orig.y, ray.orig.z}, NUM_EPS_RAY, {ray.dir.x, ray.dir.y, ray.dir.z},
                       NUM_INFINITY};
    mcrt_hit      h;
    check(mcrt_trace_closest(ctx->scene, &r, 1, &h, ctx->traverse, MCRT_PTR_HOST, nullptr), "mcrt_trace_closest");
    if (h.prim < 0)
    {
        HitInfo miss;
        miss.reset();
        return miss;
    }
    if (static_cast<size_t>(h.prim) >= m_triangles_ref.size())
    {
        std::fprintf(stderr, "mcrt_trace_closest returned primitive %d of %zu\n", h.prim, m_triangles_ref.size());
        std::abort();
    }
    const TriangleObject& tri = m_triangles_ref[h.prim];
    HitInfo               isect(h.t, h.u, h.v, tri.normal(h.u, h.v), &tri);
    isect.setPrimitiveID(h.prim);
    isect.setMaterialID(tri.materialID());
    return isect;
}

bool SceneBVH::occluded(const Ray& ray, float tfar) const
{
    Gb300Context* ctx = static_cast<Gb300Context*>(m_ctx);
    mcrt_ray      r = {{ray.orig.x, ray.orig.y, ray.orig.z}, NUM_EPS_RAY, {ray.dir.x, ray.dir.y, ray.dir.z},
                       tfar - NUM_EPS_RAY};
    int32_t       occ = 0;
    check(mcrt_trace_any(ctx->scene, &r, 1, &occ, ctx->traverse, MCRT_PTR_HOST, nullptr), "mcrt_trace_any");
    return occ != 0;
}
