// Test infrastructure (oracle build only, never shipped): plain C entry points over the
// reference renderer's own compiled sources, so that tests, golden-fixture generation
// and the CPU baseline can call the reference code unchanged.
//
// The reference's path tracer `rayTrace` is a file-static function of
// src/examples/pt/demo_pt.cpp (demo_pt.cpp:512-655); this translation unit includes
// that file (with `main` renamed) so the integrator, its EnvmapSampler and the
// reference Cornell box builder (demo_pt.cpp:83-414) can be called as they are.
#define main mcrt_reference_demo_main
#include "demo_pt.cpp"
#undef main

#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "acceleration/splitbvh.h"
#include "boundedtriangle.h"
#include "envmap.h"
#include "geometry.h"
#include "sample.h"
#include "scenebvh.h"

// ---------------------------------------------------------------------------
// Ray counters: the link step wraps SceneBVH::intersect / SceneBVH::occluded
// (scenebvh.cpp:353-396) so every ray the reference integrator traces is counted.
// ---------------------------------------------------------------------------
static std::atomic<long long> g_num_intersect(0);
static std::atomic<long long> g_num_occluded(0);

extern "C" HitInfo __real__ZNK8SceneBVH9intersectERK3Ray(const SceneBVH*, const Ray&);
extern "C" bool __real__ZNK8SceneBVH8occludedERK3Rayf(const SceneBVH*, const Ray&, float);

extern "C" HitInfo __wrap__ZNK8SceneBVH9intersectERK3Ray(const SceneBVH* self, const Ray& r)
{
    g_num_intersect.fetch_add(1, std::memory_order_relaxed);
    return __real__ZNK8SceneBVH9intersectERK3Ray(self, r);
}

extern "C" bool __wrap__ZNK8SceneBVH8occludedERK3Rayf(const SceneBVH* self, const Ray& r, float tfar)
{
    g_num_occluded.fetch_add(1, std::memory_order_relaxed);
    return __real__ZNK8SceneBVH8occludedERK3Rayf(self, r, tfar);
}

// randf() (numeric.cpp:11-15) is wrapped the same way to count draws
static std::atomic<long long> g_num_randf(0);
extern "C" float __real__Z5randfv();
extern "C" float __wrap__Z5randfv()
{
    g_num_randf.fetch_add(1, std::memory_order_relaxed);
    return __real__Z5randfv();
}

static vec3 v3(const float* p) { return vec3(p[0], p[1], p[2]); }
static void put3(float* p, const vec3& v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

// ---------------------------------------------------------------------------
// Split BVH: built exactly as SplitBVH::SplitBVH does (splitbvh.cpp:1410-1433),
// through the public static SplitBVH::build, so the tree is reachable for dumping.
// ---------------------------------------------------------------------------
struct RefBVH
{
    std::vector<TriangleObject>                   tris;
    std::vector<std::shared_ptr<Triangle> >        owned;
    std::vector<std::shared_ptr<BoundedTriangle> > refs;
    std::shared_ptr<SplitBVHNode>                  root;
    SceneBVH*                                      scene_bvh = nullptr;
    // dump cache
    bool               dumped = false;
    std::vector<float> node_box;   // 6 per node: min xyz, max xyz
    std::vector<int>   node_info;  // 6 per node: is_leaf, left, right, axis, ref_begin, ref_count
    std::vector<int>   ref_prim;
    std::vector<float> ref_box;    // 6 per ref (clipped bound)
};

extern "C" void* ref_bvh_create(const float* verts, int n, int with_scenebvh)
{
    RefBVH* c = new RefBVH;
    c->tris.reserve(n);
    for (int i = 0; i < n; ++i)
    {
        TriangleObject t(v3(verts + 9 * i), v3(verts + 9 * i + 3), v3(verts + 9 * i + 6));
        t.setMaterialID(0);
        t.setPrimitiveID(i);
        c->tris.push_back(t);
    }
    for (int i = 0; i < n; ++i)
    {
        auto nt = std::make_shared<Triangle>(c->tris[i]);
        nt->setPrimitiveID(i);
        c->owned.push_back(nt);
    }
    for (const auto& t : c->owned)
        c->refs.push_back(std::make_shared<BoundedTriangle>(t, t->boundingBox()));
    c->root = SplitBVH::build(c->refs, 0u, "root");
    if (with_scenebvh) c->scene_bvh = new SceneBVH(c->tris);
    return c;
}

extern "C" void ref_bvh_destroy(void* h)
{
    RefBVH* c = static_cast<RefBVH*>(h);
    delete c->scene_bvh;
    delete c;
}

// rays: 8 floats each {ox, oy, oz, tmin, dx, dy, dz, tmax}; SplitBVH::intersect semantics
// (splitbvh.cpp:1627-1642) with the caller's [tmin, tmax].
extern "C" void ref_bvh_intersect(void* h, const float* rays, long long n, float* t_out,
                                  int* prim_out, float* u_out, float* v_out, int nthreads)
{
    RefBVH* c = static_cast<RefBVH*>(h);
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads > 0 ? nthreads : 1)
    for (long long i = 0; i < n; ++i)
    {
        const float* r = rays + 8 * i;
        Ray     ray(v3(r), v3(r + 4), r[3], r[7]);
        HitInfo hit;
        hit.reset();
        bool any = c->root->intersect(ray, hit);
        t_out[i] = any ? hit.m_t : NUM_INFINITY;
        prim_out[i] = any ? hit.m_objID : -1;
        if (u_out) u_out[i] = any ? hit.m_u : 0.0f;
        if (v_out) v_out[i] = any ? hit.m_v : 0.0f;
    }
}

// SceneBVH::intersect (scenebvh.cpp:353-377): tmin = NUM_EPS_RAY, tmax = inf, plus the
// interpolated shading normal.  Requires ref_bvh_create(..., with_scenebvh=1).
extern "C" int ref_scenebvh_intersect(void* h, const float* rays, long long n, float* t_out,
                                      int* prim_out, float* nl_out)
{
    RefBVH* c = static_cast<RefBVH*>(h);
    if (!c->scene_bvh) return -1;
    for (long long i = 0; i < n; ++i)
    {
        const float* r = rays + 8 * i;
        HitInfo hit = c->scene_bvh->intersect(Ray(v3(r), v3(r + 4)));
        t_out[i] = hit ? hit.m_t : NUM_INFINITY;
        prim_out[i] = hit ? hit.primitiveID() : -1;
        if (nl_out) put3(nl_out + 3 * i, hit ? hit.shadingNormal() : vec3(0.0f));
    }
    return 0;
}

// SceneBVH::occluded (scenebvh.cpp:379-396): tmax = tfar - NUM_EPS_RAY, closest-hit query.
extern "C" int ref_scenebvh_occluded(void* h, const float* rays, long long n, const float* tfar,
                                     int* occ_out)
{
    RefBVH* c = static_cast<RefBVH*>(h);
    if (!c->scene_bvh) return -1;
    for (long long i = 0; i < n; ++i)
    {
        const float* r = rays + 8 * i;
        occ_out[i] = c->scene_bvh->occluded(Ray(v3(r), v3(r + 4)), tfar[i]) ? 1 : 0;
    }
    return 0;
}

static int dump_node(RefBVH* c, const SplitBVHNode* node)
{
    if (!node) return -1;
    int idx = static_cast<int>(c->node_info.size() / 6);
    const AABB& b = *node->bounding_box;
    for (int k = 0; k < 3; ++k) c->node_box.push_back(b.min()[k]);
    for (int k = 0; k < 3; ++k) c->node_box.push_back(b.max()[k]);
    for (int k = 0; k < 6; ++k) c->node_info.push_back(0);
    const SplitBVHLeafNode* leaf = dynamic_cast<const SplitBVHLeafNode*>(node);
    if (leaf)
    {
        int begin = static_cast<int>(c->ref_prim.size());
        for (int i = 0; i < k_sbvh_leaf_node_size; ++i)
        {
            if (!leaf->primitive[i]) continue;
            c->ref_prim.push_back(leaf->primitive[i]->originalTriangle()->primitiveID());
            const AABB& cb = leaf->primitive[i]->clippedBoundingBox();
            for (int k = 0; k < 3; ++k) c->ref_box.push_back(cb.min()[k]);
            for (int k = 0; k < 3; ++k) c->ref_box.push_back(cb.max()[k]);
        }
        int* info = &c->node_info[6 * idx];
        info[0] = 1;
        info[1] = info[2] = -1;
        info[3] = 0;
        info[4] = begin;
        info[5] = static_cast<int>(c->ref_prim.size()) - begin;
        return idx;
    }
    const SplitBVHBranchNode* br = dynamic_cast<const SplitBVHBranchNode*>(node);
    int left = dump_node(c, br->left_child.get());
    int right = dump_node(c, br->right_child.get());
    int* info = &c->node_info[6 * idx];
    info[0] = 0;
    info[1] = left;
    info[2] = right;
    info[3] = br->split_axis;
    info[4] = 0;
    info[5] = 0;
    return idx;
}

extern "C" void ref_bvh_dump_sizes(void* h, int* n_nodes, int* n_refs)
{
    RefBVH* c = static_cast<RefBVH*>(h);
    if (!c->dumped)
    {
        dump_node(c, c->root.get());
        c->dumped = true;
    }
    *n_nodes = static_cast<int>(c->node_info.size() / 6);
    *n_refs = static_cast<int>(c->ref_prim.size());
}

extern "C" void ref_bvh_dump(void* h, float* node_box, int* node_info, int* ref_prim, float* ref_box)
{
    RefBVH* c = static_cast<RefBVH*>(h);
    int     nn, nr;
    ref_bvh_dump_sizes(h, &nn, &nr);
    std::memcpy(node_box, c->node_box.data(), sizeof(float) * c->node_box.size());
    std::memcpy(node_info, c->node_info.data(), sizeof(int) * c->node_info.size());
    std::memcpy(ref_prim, c->ref_prim.data(), sizeof(int) * c->ref_prim.size());
    std::memcpy(ref_box, c->ref_box.data(), sizeof(float) * c->ref_box.size());
}

// ---------------------------------------------------------------------------
// Per-function pins: materials (material.cpp:5-27, bsdf.cpp), Fresnel
// (geometry.cpp:14-43), orthonormal frame (geometry.cpp:74-110), cosine warp
// (sample.cpp:132-137), camera (camera.cpp:9-43), discrete sampler (sample.cpp:11-118),
// triangle point sampling (triangle.cpp:100-122).
// ---------------------------------------------------------------------------
extern "C" void ref_material_sample(int type, const float* color, const float* wi, const float* nl,
                                    float r1, float r2, float* wo, float* weight, float* pdf,
                                    float* cos_wo)
{
    Material m(v3(color), 0.0f, static_cast<MaterialType>(type));
    vec3     w;
    float    p = 0.0f, c = 0.0f;
    vec3     d = m.sample(v3(wi), v3(nl), r1, r2, w, &p, &c);
    put3(wo, d);
    put3(weight, w);
    *pdf = p;
    *cos_wo = c;
}

extern "C" void ref_material_evaluate(int type, const float* color, const float* wi, const float* nl,
                                      const float* wo, float* f, float* pdf)
{
    Material m(v3(color), 0.0f, static_cast<MaterialType>(type));
    float    p = 0.0f, c = 0.0f;
    put3(f, m.evaluate(v3(wi), v3(nl), v3(wo), &c, &p));
    *pdf = m.pdfW(v3(wi), v3(nl), v3(wo));
}

extern "C" float ref_fresnel(float cos_theta_i, float ior) { return fresnelReflectance(cos_theta_i, ior); }

extern "C" void ref_onb_to_world(const float* n, const float* c, float* out)
{
    OrthonormalFrame onb(v3(n));
    put3(out, onb.toWorld(v3(c)));
}

extern "C" void ref_sample_hemisphere_cosine(float x, float y, float* out)
{
    put3(out, sampleHemisphereCosine(x, y));
}

extern "C" void ref_camera_ray(const float* origin, const float* target, int w, int h, float fov_y,
                               float mx, float my, float* o, float* d)
{
    Camera cam(v3(origin), v3(target), vec3(0, 1, 0), w, h, fov_y);
    Ray    r = cam.makeRay(mx, my);
    put3(o, r.orig);
    put3(d, r.dir);
}

extern "C" int ref_discrete_sample(const float* weights, int n, float r, float* pdf_out)
{
    std::vector<float> data(weights, weights + n);
    DiscreteSampler    s(data);
    int                i = s.sample(r);
    if (pdf_out) *pdf_out = s.pdf(i);
    return i;
}

extern "C" void ref_triangle_sample_point(const float* abc, float r0, float r1, float* p, float* uv)
{
    TriangleObject t(v3(abc), v3(abc + 3), v3(abc + 6));
    float          u, v;
    put3(p, t.samplePoint(u, v, r0, r1));
    uv[0] = u;
    uv[1] = v;
}

extern "C" void ref_triangle_normal_area(const float* abc, float* n, float* area)
{
    TriangleObject t(v3(abc), v3(abc + 3), v3(abc + 6));
    put3(n, t.normal());
    *area = t.area();
}

// ---------------------------------------------------------------------------
// Environment map (envmap.cpp:98-506), loaded from the reference's .bin format.
// ---------------------------------------------------------------------------
extern "C" void* ref_envmap_load(const char* path) { return new EnvmapLoader(std::string(path)); }
extern "C" void  ref_envmap_destroy(void* h) { delete static_cast<EnvmapLoader*>(h); }

extern "C" void ref_envmap_sample(void* h, float r1, float r2, float* dir, float* rad, float* pdf)
{
    DirLight dl = static_cast<EnvmapLoader*>(h)->sample(r1, r2);
    for (int k = 0; k < 3; ++k)
    {
        dir[k] = dl.dir[k];
        rad[k] = dl.rad[k];
    }
    *pdf = dl.pdf;
}

extern "C" float ref_envmap_pdf(void* h, const float* dir)
{
    float d[3] = {dir[0], dir[1], dir[2]};
    return static_cast<EnvmapLoader*>(h)->getPdf(d);
}

extern "C" void ref_envmap_radiance(void* h, const float* dir, float* rad)
{
    float d[3] = {dir[0], dir[1], dir[2]};
    static_cast<EnvmapLoader*>(h)->sampleRadiance(d, rad);
}

// ---------------------------------------------------------------------------
// The reference path tracer.  Scenes are built through the reference API
// (todo_addMaterial, Material, TriangleObject, Scene::add/setCamera/setEnvmap/finalize)
// and rendered with demo_pt.cpp's own rayTrace (fixed depth 10, no Russian roulette,
// global randf()) in DemoSimple::run's loop (demo_pt.cpp:680-710), over rows
// [row_begin, row_end).  out_rgb receives per-pixel means (W*H*3, rows outside the
// range untouched).
// ---------------------------------------------------------------------------
static void render_rows(const Scene& scene, int width, int height, int spp, int nthreads,
                        int row_begin, int row_end, float* out_rgb)
{
    Camera* cam = scene.camera();
    for (int y = row_begin; y < row_end; ++y)
    {
#pragma omp parallel for schedule(dynamic) num_threads(nthreads > 0 ? nthreads : 1)
        for (int x = 0; x < width; ++x)
        {
            vec3 g;
            for (int s = 0; s < spp; ++s)
            {
                float dx = 0;
                float dy = 0;
                if (spp > 1)
                {
                    float r1 = 2 * randf();
                    float r2 = 2 * randf();
                    dx = r1 < 1 ? std::sqrt(r1) - 1 : 1 - std::sqrt(2 - r1);
                    dy = r2 < 1 ? std::sqrt(r2) - 1 : 1 - std::sqrt(2 - r2);
                }
                Ray  ray = cam->makeRay((x + 0.5f + dx) / width, (y + 0.5f + dy) / height);
                vec3 v = rayTrace(ray, scene);
                g += vec3(f_max(0.0f, v.x), f_max(0.0f, v.y), f_max(0.0f, v.z));
            }
            float* px = out_rgb + 3 * (static_cast<size_t>(y) * width + x);
            px[0] = g.x * (1.0f / spp);
            px[1] = g.y * (1.0f / spp);
            px[2] = g.z * (1.0f / spp);
        }
    }
}

// A reference scene built once and rendered band by band (the timed CPU baseline): the
// build (Scene::finalize, which runs the SplitBVH builder) stays outside the timed renders.
extern "C" void* ref_pt_scene_create(const float* verts, const float* normals, const int* mat_ids, int n_tris,
                                     const int* mat_types, const float* mat_colors, int n_mats,
                                     const char* envmap_path, const float* cam /* origin3 target3 fov */,
                                     int width, int height)
{
    Scene* scene = new Scene();
    int    base = -1;
    for (int m = 0; m < n_mats; ++m)
    {
        int id = todo_addMaterial(
            Material(v3(mat_colors + 3 * m), 0.0f, static_cast<MaterialType>(mat_types[m])));
        if (m == 0) base = id;
    }
    for (int i = 0; i < n_tris; ++i)
    {
        const float*   p = verts + 9 * i;
        TriangleObject t = normals ? TriangleObject(v3(p), v3(p + 3), v3(p + 6), v3(normals + 9 * i),
                                                    v3(normals + 9 * i + 3), v3(normals + 9 * i + 6))
                                   : TriangleObject(v3(p), v3(p + 3), v3(p + 6));
        t.setMaterialID(base + mat_ids[i]);
        scene->add(t);
    }
    scene->setCamera(v3(cam), v3(cam + 3), width, height, cam[6]);
    if (envmap_path && envmap_path[0]) scene->setEnvmap(std::string(envmap_path));
    scene->finalize();
    return scene;
}

// rows [row_begin, row_end) of the scene's camera frame; rays counted by the link-time
// wrappers around SceneBVH::intersect / occluded
extern "C" int ref_pt_render(void* h, int width, int height, int spp, int nthreads, int row_begin, int row_end,
                             float* out_rgb, long long* n_intersect, long long* n_occluded, double* seconds)
{
    const Scene& scene = *static_cast<Scene*>(h);
    long long    i0 = g_num_intersect.load(), o0 = g_num_occluded.load();
    auto         t0 = std::chrono::steady_clock::now();
    render_rows(scene, width, height, spp, nthreads, row_begin, row_end, out_rgb);
    auto t1 = std::chrono::steady_clock::now();
    if (n_intersect) *n_intersect = g_num_intersect.load() - i0;
    if (n_occluded) *n_occluded = g_num_occluded.load() - o0;
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    return 0;
}

extern "C" void ref_pt_scene_destroy(void* h) { delete static_cast<Scene*>(h); }

extern "C" int ref_render_pt(const float* verts, const float* normals, const int* mat_ids, int n_tris,
                             const int* mat_types, const float* mat_colors, int n_mats,
                             const char* envmap_path, const float* cam /* origin3 target3 fov */,
                             int width, int height, int spp, int nthreads, int row_begin,
                             int row_end, float* out_rgb, long long* n_intersect,
                             long long* n_occluded, double* seconds)
{
    void* h = ref_pt_scene_create(verts, normals, mat_ids, n_tris, mat_types, mat_colors, n_mats, envmap_path, cam,
                                  width, height);
    int rc = ref_pt_render(h, width, height, spp, nthreads, row_begin, row_end, out_rgb, n_intersect, n_occluded,
                           seconds);
    ref_pt_scene_destroy(h);
    return rc;
}

// Per-sample radiance of demo_pt's rayTrace on its own Cornell box, single-threaded in
// DemoSimple::run's order, so a replay of the global randf() stream can be compared
// sample by sample.  Call first in a fresh process: the stream starts at seed 1.
extern "C" int ref_cornell_paths(int width, int height, int spp, float* out /* H*W*spp*3 */,
                                 long long* draws /* H*W*spp, may be null */)
{
    Scene       scene;
    FrameBuffer fb;
    loadSceneCornellBox(scene, fb);
    scene.setCamera(vec3(278, 273, -800) * 0.1f, vec3(278, 273, -799) * 0.1f, width, height, 39.3077f);
    scene.finalize();
    Camera* cam = scene.camera();
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x)
            for (int s = 0; s < spp; ++s)
            {
                float dx = 0, dy = 0;
                if (spp > 1)
                {
                    float r1 = 2 * randf();
                    float r2 = 2 * randf();
                    dx = r1 < 1 ? std::sqrt(r1) - 1 : 1 - std::sqrt(2 - r1);
                    dy = r2 < 1 ? std::sqrt(r2) - 1 : 1 - std::sqrt(2 - r2);
                }
                Ray    ray = cam->makeRay((x + 0.5f + dx) / width, (y + 0.5f + dy) / height);
                vec3   v = rayTrace(ray, scene);
                size_t idx = (static_cast<size_t>(y) * width + x) * spp + s;
                if (draws) draws[idx] = g_num_randf.load();
                float* o = out + 3 * idx;
                o[0] = f_max(0.0f, v.x);
                o[1] = f_max(0.0f, v.y);
                o[2] = f_max(0.0f, v.z);
            }
    return 0;
}

// The reference's own Cornell box (demo_pt.cpp:83-414).  Exports its triangles,
// per-triangle material type/colour and camera so other renderers can be fed the
// identical scene: call with null outputs to get the counts.
extern "C" int ref_cornell_export(float* verts, int* mat_types, float* mat_colors, float* cam)
{
    Scene       scene;
    FrameBuffer fb;
    loadSceneCornellBox(scene, fb);
    int n = static_cast<int>(scene.numTrangles());
    if (verts)
    {
        for (int i = 0; i < n; ++i)
        {
            const TriangleObject& t = scene.triangle(i);
            put3(verts + 9 * i, t.a);
            put3(verts + 9 * i + 3, t.b);
            put3(verts + 9 * i + 6, t.c);
            const Material& m = todo_getMaterial(t.materialID());
            mat_types[i] = static_cast<int>(m.type());
            put3(mat_colors + 3 * i, m.color());
        }
    }
    if (cam)
    {
        // demo_pt.cpp:87-92
        float scale = 0.1f;
        put3(cam, vec3(278, 273, -800) * scale);
        put3(cam + 3, vec3(278, 273, -799) * scale);
        cam[6] = 39.3077f;
    }
    return n;
}

extern "C" int ref_render_cornell(int width, int height, int spp, int nthreads, int row_begin,
                                  int row_end, float* out_rgb, long long* n_intersect,
                                  long long* n_occluded, double* seconds)
{
    Scene       scene;
    FrameBuffer fb;
    loadSceneCornellBox(scene, fb);
    scene.setCamera(vec3(278, 273, -800) * 0.1f, vec3(278, 273, -799) * 0.1f, width, height,
                    39.3077f);
    scene.finalize();
    long long i0 = g_num_intersect.load(), o0 = g_num_occluded.load();
    auto      t0 = std::chrono::steady_clock::now();
    render_rows(scene, width, height, spp, nthreads, row_begin, row_end, out_rgb);
    auto t1 = std::chrono::steady_clock::now();
    if (n_intersect) *n_intersect = g_num_intersect.load() - i0;
    if (n_occluded) *n_occluded = g_num_occluded.load() - o0;
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    return 0;
}

// --- film outputs (film.cpp): FrameBuffer filled through accumulatePixel (0 + x = x) -----
static void fill_fb(FrameBuffer& fb, int w, int h, const float* rgb)
{
    fb.resize(w, h);
    for (int j = 0; j < h; ++j)
        for (int i = 0; i < w; ++i)
        {
            const float* c = rgb + 3 * (static_cast<size_t>(j) * w + i);
            fb.accumulatePixel(i, j, vec3(c[0], c[1], c[2]));
        }
}

static void read_fb(const FrameBuffer& fb, int w, int h, float* rgb)
{
    for (int j = 0; j < h; ++j)
        for (int i = 0; i < w; ++i)
        {
            vec3   c = fb.pixel(i, j);
            float* o = rgb + 3 * (static_cast<size_t>(j) * w + i);
            o[0] = c.x;
            o[1] = c.y;
            o[2] = c.z;
        }
}

// FrameBuffer::dumpHDR / dumpPPM to `path`
extern "C" void ref_film_dump(int w, int h, const float* rgb, const char* path, int hdr)
{
    FrameBuffer fb;
    fill_fb(fb, w, h, rgb);
    if (hdr)
        fb.dumpHDR(path);
    else
        fb.dumpPPM(path);
}

// FrameBuffer::tonemapGamma (mode 0, with `gamma`) or tonemapReinhard (mode 1), in place
extern "C" void ref_film_tonemap(int w, int h, float* rgb, int mode, float gamma)
{
    FrameBuffer fb;
    fill_fb(fb, w, h, rgb);
    if (mode == 0)
        fb.tonemapGamma(gamma);
    else
        fb.tonemapReinhard();
    read_fb(fb, w, h, rgb);
}

// --- consistent normals (Reshetov et al. 2010): TriangleObject::consistentNormal
// (triangle.cpp:149-182) and the per-vertex alpha of Mesh::genNormals (mesh.cpp:66-116) --
extern "C" void ref_consistent_normal(const float* abc, const float* nabc, const float* alpha3, const float* wi,
                                      float u, float v, float* nc_out, float* refl_out, float* cos_out)
{
    TriangleObject t(v3(abc), v3(abc + 3), v3(abc + 6), v3(nabc), v3(nabc + 3), v3(nabc + 6));
    t.setVertexAlpha(v3(alpha3));
    vec3  r;
    float c = 0.f;
    put3(nc_out, t.consistentNormal(v3(wi), u, v, &r, &c));
    put3(refl_out, r);
    *cos_out = c;
}

extern "C" void ref_mesh_alpha(const float* verts, int nv, const int* faces, int nf, float* normals_out,
                               float* alpha_out)
{
    Mesh m;
    for (int i = 0; i < nv; ++i) m.m_verts.push_back(v3(verts + 3 * i));
    for (int i = 0; i < nf; ++i) m.m_faces.push_back(int3(faces[3 * i], faces[3 * i + 1], faces[3 * i + 2]));
    m.genNormals();
    for (int i = 0; i < nv; ++i)
    {
        put3(normals_out + 3 * i, m.m_vertex_normals[i]);
        alpha_out[i] = m.m_vertex_alpha[i];
    }
}

// Scene::loadModel (scene.cpp:368-408) on an OBJ file: the triangles it adds (vertices and
// vertex normals), and per corner the alpha Mesh::genNormals computes for the transformed
// mesh (loadModel itself does not copy the alphas into the triangles).  transform: 16
// floats, column-major (glm::mat4).  Call with verts == NULL for the triangle count.
extern "C" int ref_load_obj(const char* path, const float* transform, float* verts, float* normals, float* alpha)
{
    glm::mat4 T(1.0f);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) T[c][r] = transform[4 * c + r];
    Scene scene;
    scene.loadModel(path, T, Material(vec3(0.5f, 0.5f, 0.5f), 0.0f, DIFF));
    const int n = static_cast<int>(scene.numTrangles());
    if (!verts) return n;
    for (int i = 0; i < n; ++i)
    {
        const TriangleObject& t = scene.triangle(i);
        put3(verts + 9 * i, t.a);
        put3(verts + 9 * i + 3, t.b);
        put3(verts + 9 * i + 6, t.c);
        put3(normals + 9 * i, t.na);
        put3(normals + 9 * i + 3, t.nb);
        put3(normals + 9 * i + 6, t.nc);
    }
    Mesh m(path);
    for (auto& v : m.m_verts)
    {
        glm::vec4 p = T * glm::vec4(v.x, v.y, v.z, 1.0f);
        v = vec3(p.x, p.y, p.z);
    }
    m.genNormals();
    for (int i = 0; i < n && i < static_cast<int>(m.m_faces.size()); ++i)
    {
        alpha[3 * i + 0] = m.m_vertex_alpha[m.m_faces[i].x];
        alpha[3 * i + 1] = m.m_vertex_alpha[m.m_faces[i].y];
        alpha[3 * i + 2] = m.m_vertex_alpha[m.m_faces[i].z];
    }
    return n;
}
