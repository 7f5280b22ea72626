// Scene cache files: a prepared device scene (all three node layouts, leaf triangles, shading
// arrays, light and environment-map sampling tables) written to disk and uploaded again
// without running the builder, the flattener or the table construction.
//
// Format (little-endian, version kFormat):
//   "MCRTSCN\0"  u32 format  u32 array count (17)  u64 description hash  i64 triangles
//   f32 light_area  f32 env_norm  i32 env_w  i32 env_h  i32 bvh_depth  i32 wide_depth
//   17 x { u32 element size, u32 0, i64 bytes }  -- the arrays of scene_from_host, in order
//   the arrays' bytes, in order
//   u64 checksum (FNV-1a 64 over 64-bit words) of everything before it
// The description hash (mcrt_scene_desc_hash) covers every input of the scene and the
// format version, so a cache written for another mesh, material table, environment map,
// leaf size or builder is recognised and rejected by mcrt_scene_load.
#include <climits>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/mcrt_gb300.h"
#include "host.h"
#include "wavefront.h"

namespace mcrt {
namespace {

constexpr uint32_t kFormat = 4;
constexpr int      kArrays = 17;
const char         kMagic[8] = {'M', 'C', 'R', 'T', 'S', 'C', 'N', '\0'};

// FNV-1a 64 over little-endian 64-bit words (remaining bytes one at a time): the hash of
// a 100 MB mesh costs tens of milliseconds
struct Fnv
{
    uint64_t h = 1469598103934665603ull;
    void     add(const void* p, size_t n)
    {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        size_t               i = 0;
        for (; i + 8 <= n; i += 8)
        {
            uint64_t w;
            std::memcpy(&w, b + i, 8);
            h ^= w;
            h *= 1099511628211ull;
        }
        for (; i < n; ++i)
        {
            h ^= b[i];
            h *= 1099511628211ull;
        }
    }
    template <class T>
    void add_value(const T& v)
    {
        add(&v, sizeof(T));
    }
};

// element sizes of the arrays of HostScene in scene_from_host's order
const uint32_t kElem[kArrays] = {sizeof(FastNode), sizeof(float4), sizeof(RefNode),     sizeof(RefPrim), sizeof(float4),
                                 sizeof(float4),   sizeof(int32_t), sizeof(LightGPU),   sizeof(MaterialGPU),
                                 sizeof(float4),   sizeof(float),   sizeof(float),      sizeof(int32_t), sizeof(int32_t),
                                 sizeof(float4),   sizeof(WideNode), sizeof(float4)};

struct Header
{
    char     magic[8];
    uint32_t format;
    uint32_t arrays;
    uint64_t desc_hash;
    int64_t  num_tris;
    float    light_area;
    float    env_norm;
    int32_t  env_w, env_h, bvh_depth, wide_depth;
    struct
    {
        uint32_t elem, pad;
        int64_t  bytes;
    } a[kArrays];
};

template <class F>
void for_each_array(HostScene& hs, F&& f)
{
    f(hs.bvh.fast_nodes);
    f(hs.bvh.fast_tris);
    f(hs.bvh.ref_nodes);
    f(hs.bvh.ref_prims);
    f(hs.prim_verts);
    f(hs.prim_shade);
    f(hs.light_of);
    f(hs.lights);
    f(hs.materials);
    f(hs.env_rgb);
    f(hs.env_marginal);
    f(hs.env_cond);
    f(hs.env_guide_m);
    f(hs.env_guide_c);
    f(hs.prim_alpha);
    f(hs.bvh.wide_nodes);
    f(hs.bvh.wide_tris);
}

inline int32_t ibits(float f)
{
    int32_t i;
    std::memcpy(&i, &f, sizeof(i));
    return i;
}

// Every index a kernel follows must stay inside its array: a loaded file is checked as
// the flattener's output would be (a checksum only catches accidental damage).
std::string validate(const HostScene& hs, int64_t num_tris)
{
    const int64_t nodes = static_cast<int64_t>(hs.bvh.fast_nodes.size());
    const int64_t leaf_refs = static_cast<int64_t>(hs.bvh.fast_tris.size() / 3);
    if (hs.bvh.fast_tris.size() % 3 != 0 || hs.prim_verts.size() != 3 * static_cast<size_t>(num_tris) ||
        hs.prim_shade.size() != 3 * static_cast<size_t>(num_tris))
        return "array sizes do not match the triangle count";
    auto child_ok = [&](int32_t c) {
        if (c >= 0) return c < nodes;
        const int64_t code = ~static_cast<int64_t>(c);
        return (code >> 4) + (code & 15) <= leaf_refs;
    };
    for (const FastNode& n : hs.bvh.fast_nodes)
        if (!child_ok(n.n3.x) || !child_ok(n.n3.y)) return "fast node child out of range";
    for (size_t k = 0; k < hs.bvh.fast_tris.size(); k += 3)
    {
        const int32_t p = ibits(hs.bvh.fast_tris[k].w);
        if (p < 0 || p >= num_tris) return "leaf triangle primitive out of range";
    }
    const int64_t ref_nodes = static_cast<int64_t>(hs.bvh.ref_nodes.size());
    const int64_t refs = static_cast<int64_t>(hs.bvh.ref_prims.size());
    for (const RefNode& n : hs.bvh.ref_nodes)
    {
        const int32_t a = ibits(n.lo.w), b = ibits(n.hi.w);
        if (a < 0)
        {
            const int64_t begin = ~static_cast<int64_t>(a);
            if (b < 0 || begin + b > refs) return "reference leaf range out of bounds";
        }
        else if (a >= ref_nodes || b < 0 || (b >> 2) >= ref_nodes || (b & 3) > 2)
            return "reference node child out of range";
    }
    for (const RefPrim& r : hs.bvh.ref_prims)
    {
        const int32_t p = ibits(r.lo.w);
        if (p < 0 || p >= num_tris) return "reference primitive out of range";
    }
    if (fast_layout_wide() && hs.bvh.wide_nodes.empty()) return "written for the two-child traversal layout";
    if (!hs.bvh.wide_nodes.empty())
    {
        int         wide_depth = 0;
        std::string werr = validate_wide(hs.bvh.wide_nodes, hs.bvh.wide_tris, num_tris, &wide_depth);
        if (!werr.empty()) return werr;
        if (wide_depth != hs.bvh.wide_depth) return "wide BVH depth does not match the header";
    }
    const int64_t mats = static_cast<int64_t>(hs.materials.size());
    for (size_t k = 0; k < hs.prim_shade.size(); k += 3)
    {
        const int32_t m = ibits(hs.prim_shade[k].w);
        if (m < 0 || m >= mats) return "material id out of range";
    }
    const int64_t lights = static_cast<int64_t>(hs.lights.size());
    if (!hs.light_of.empty() && hs.light_of.size() != static_cast<size_t>(num_tris)) return "emitter table size";
    for (int32_t l : hs.light_of)
        if (l < -1 || l >= lights) return "emitter index out of range";
    for (const LightGPU& l : hs.lights)
        if (l.prim < 0 || l.prim >= num_tris) return "emitter primitive out of range";
    if (!hs.prim_alpha.empty() && hs.prim_alpha.size() != static_cast<size_t>(num_tris))
        return "consistent-normal table size";
    if (hs.env_w > 0)
    {
        const size_t W = static_cast<size_t>(hs.env_w), H = static_cast<size_t>(hs.env_h);
        if (hs.env_marginal.size() != W || hs.env_cond.size() != W * H ||
            hs.env_guide_m.size() != static_cast<size_t>(kEnvGuideM + 1) ||
            hs.env_guide_c.size() != W * (kEnvGuideC + 1))
            return "environment table sizes";
        for (int32_t g : hs.env_guide_m)
            if (g < 0 || static_cast<size_t>(g) >= W) return "environment guide out of range";
        for (int32_t g : hs.env_guide_c)
            if (g < 0 || static_cast<size_t>(g) >= H) return "environment guide out of range";
    }
    return std::string();
}

struct FileCloser
{
    void operator()(FILE* f) const
    {
        if (f) std::fclose(f);
    }
};

}  // namespace

uint64_t scene_desc_hash(const mcrt_scene_desc& d)
{
    Fnv h;
    h.add(kMagic, sizeof(kMagic));
    h.add_value(kFormat);
    h.add_value(d.num_triangles);
    h.add(d.vertices, sizeof(float) * 9 * static_cast<size_t>(d.num_triangles));
    const int32_t has_normals = d.normals ? 1 : 0;
    h.add_value(has_normals);
    if (d.normals) h.add(d.normals, sizeof(float) * 9 * static_cast<size_t>(d.num_triangles));
    h.add(d.material_ids, sizeof(int32_t) * static_cast<size_t>(d.num_triangles));
    h.add_value(d.num_materials);
    if (d.materials) h.add(d.materials, sizeof(mcrt_material) * static_cast<size_t>(d.num_materials));
    h.add_value(d.env_width);
    h.add_value(d.env_height);
    if (d.env_rgb && d.env_width > 0 && d.env_height > 0)
        h.add(d.env_rgb, sizeof(float) * 3 * static_cast<size_t>(d.env_width) * d.env_height);
    const int32_t has_alpha = d.vertex_alpha ? 1 : 0;
    h.add_value(has_alpha);
    if (d.vertex_alpha) h.add(d.vertex_alpha, sizeof(float) * 3 * static_cast<size_t>(d.num_triangles));
    h.add_value(d.builder);
    const int32_t leaf = d.leaf_size > 0 ? d.leaf_size : kDefaultLeafSize;
    h.add_value(leaf);
    if (d.builder == MCRT_BUILD_EXTERNAL && d.external_tree)
    {
        const mcrt_bvh_tree& t = *d.external_tree;
        h.add_value(t.num_nodes);
        h.add_value(t.num_refs);
        h.add(t.node_box, sizeof(float) * 6 * static_cast<size_t>(t.num_nodes));
        h.add(t.node_info, sizeof(int32_t) * 6 * static_cast<size_t>(t.num_nodes));
        h.add(t.ref_prim, sizeof(int32_t) * static_cast<size_t>(t.num_refs));
        h.add(t.ref_box, sizeof(float) * 6 * static_cast<size_t>(t.num_refs));
    }
    return h.h;
}

}  // namespace mcrt

using namespace mcrt;

extern "C" int mcrt_scene_desc_hash(const mcrt_scene_desc* desc, uint64_t* hash)
{
    if (!desc || !hash || (desc->num_triangles > 0 && (!desc->vertices || !desc->material_ids)))
        return set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_scene_desc_hash: null argument");
    *hash = scene_desc_hash(*desc);
    return MCRT_OK;
}

extern "C" int mcrt_scene_save(const mcrt_scene* scene, const char* path)
{
    if (!scene || !path) return set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_scene_save: null scene or path");
    try
    {
        HostScene hs;
        int64_t   num_tris = 0;
        uint64_t  hash = 0;
        int       rc = scene_to_host(scene, hs, num_tris, hash);
        if (rc) return rc;
        Header hd;
        std::memset(&hd, 0, sizeof(hd));
        std::memcpy(hd.magic, kMagic, sizeof(kMagic));
        hd.format = kFormat;
        hd.arrays = kArrays;
        hd.desc_hash = hash;
        hd.num_tris = num_tris;
        hd.light_area = hs.light_area;
        hd.env_norm = hs.env_norm;
        hd.env_w = hs.env_w;
        hd.env_h = hs.env_h;
        hd.bvh_depth = hs.bvh.max_depth;
        hd.wide_depth = hs.bvh.wide_depth;
        int k = 0;
        for_each_array(hs, [&](auto& v) {
            hd.a[k].elem = kElem[k];
            hd.a[k].bytes = static_cast<int64_t>(v.size() * sizeof(v[0]));
            ++k;
        });
        std::unique_ptr<FILE, FileCloser> f(std::fopen(path, "wb"));
        if (!f) return set_error(MCRT_ERR_IO, std::string("mcrt_scene_save: cannot open ") + path);
        Fnv  sum;
        bool ok = true;
        auto put = [&](const void* p, size_t n) {
            if (!ok || n == 0) return;
            sum.add(p, n);
            ok = std::fwrite(p, 1, n, f.get()) == n;
        };
        put(&hd, sizeof(hd));
        for_each_array(hs, [&](auto& v) { put(v.data(), v.size() * sizeof(v[0])); });
        const uint64_t check = sum.h;
        if (ok) ok = std::fwrite(&check, sizeof(check), 1, f.get()) == 1;
        if (ok) ok = std::fflush(f.get()) == 0;
        if (!ok) return set_error(MCRT_ERR_IO, std::string("mcrt_scene_save: write failed: ") + path);
        return MCRT_OK;
    }
    catch (const std::bad_alloc&)
    {
        return set_error(MCRT_ERR_OUT_OF_MEMORY, "mcrt_scene_save: host allocation failed");
    }
    catch (...)
    {
        return set_error(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_scene_save");
    }
}

extern "C" int mcrt_scene_load(const char* path, uint64_t expected_hash, mcrt_scene** out)
{
    if (!path || !out) return set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_scene_load: null path or out");
    *out = nullptr;
    try
    {
        std::unique_ptr<FILE, FileCloser> f(std::fopen(path, "rb"));
        if (!f) return set_error(MCRT_ERR_IO, std::string("mcrt_scene_load: cannot open ") + path);
        Fnv    sum;
        Header hd;
        auto   get = [&](void* p, size_t n) -> bool {
            if (n == 0) return true;
            if (std::fread(p, 1, n, f.get()) != n) return false;
            sum.add(p, n);
            return true;
        };
        if (!get(&hd, sizeof(hd)) || std::memcmp(hd.magic, kMagic, sizeof(kMagic)) != 0)
            return set_error(MCRT_ERR_IO, std::string("mcrt_scene_load: not a scene cache file: ") + path);
        if (hd.format != kFormat || hd.arrays != kArrays)
            return set_error(MCRT_ERR_IO, "mcrt_scene_load: cache format " + std::to_string(hd.format) +
                                              ", this library reads format " + std::to_string(kFormat));
        if (expected_hash != 0 && hd.desc_hash != expected_hash)
            return set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_scene_load: the cache was written for another scene "
                                                        "description (hash mismatch)");
        for (int k = 0; k < kArrays; ++k)
            if (hd.a[k].elem != kElem[k] || hd.a[k].bytes < 0 || hd.a[k].bytes % kElem[k] != 0)
                return set_error(MCRT_ERR_IO, "mcrt_scene_load: array " + std::to_string(k) + " malformed");
        if (hd.num_tris < 0 || hd.a[4].bytes != 48 * hd.num_tris)
            return set_error(MCRT_ERR_IO, "mcrt_scene_load: triangle count does not match the arrays");
        HostScene hs;
        int       k = 0;
        bool      ok = true;
        for_each_array(hs, [&](auto& v) {
            v.resize(static_cast<size_t>(hd.a[k].bytes) / sizeof(v[0]));
            if (ok) ok = get(v.data(), static_cast<size_t>(hd.a[k].bytes));
            ++k;
        });
        const uint64_t expect = sum.h;
        uint64_t       check = 0;
        if (!ok || std::fread(&check, sizeof(check), 1, f.get()) != 1 || check != expect)
            return set_error(MCRT_ERR_IO, std::string("mcrt_scene_load: truncated or corrupt file: ") + path);
        hs.light_area = hd.light_area;
        hs.env_norm = hd.env_norm;
        hs.env_w = hd.env_w;
        hs.env_h = hd.env_h;
        hs.bvh.max_depth = hd.bvh_depth;
        hs.bvh.wide_depth = hd.wide_depth;
        if (hs.env_w < 0 || hs.env_h < 0 ||
            hs.env_rgb.size() != static_cast<size_t>(hs.env_w) * static_cast<size_t>(hs.env_h) ||
            hs.bvh.fast_nodes.empty() || hs.materials.empty())
            return set_error(MCRT_ERR_IO, "mcrt_scene_load: inconsistent scene arrays");
        const std::string bad = validate(hs, hd.num_tris);
        if (!bad.empty()) return set_error(MCRT_ERR_IO, "mcrt_scene_load: " + bad);
        return scene_from_host(hs, hd.num_tris, hd.desc_hash, out);
    }
    catch (const std::bad_alloc&)
    {
        return set_error(MCRT_ERR_OUT_OF_MEMORY, "mcrt_scene_load: host allocation failed");
    }
    catch (...)
    {
        return set_error(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_scene_load");
    }
}

static int build_bvh_impl(bool split, const float* vertices, int64_t num_triangles, int32_t leaf_size,
                          int32_t* num_nodes, int32_t* num_refs, float* node_box, int32_t* node_info, int32_t* ref_prim,
                          float* ref_box)
{
    if (!vertices || num_triangles <= 0 || !num_nodes || !num_refs)
        return set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_build_bvh: null argument or no triangles");
    if (leaf_size < 0 || leaf_size > 15) return set_error(MCRT_ERR_INVALID_ARGUMENT, "leaf_size must be in [0, 15]");
    if (num_triangles > (int64_t(1) << 30)) return set_error(MCRT_ERR_INVALID_ARGUMENT, "too many triangles");
    try
    {
        BinaryTree t;
        if (split)
            build_split_tree(vertices, num_triangles, leaf_size > 0 ? leaf_size : kDefaultLeafSize, t);
        else
            build_sah_tree(vertices, num_triangles, leaf_size > 0 ? leaf_size : kDefaultLeafSize, t);
        const int64_t nodes = static_cast<int64_t>(t.node_info.size() / 6);
        const int64_t refs = static_cast<int64_t>(t.ref_prim.size());
        if (nodes > INT32_MAX || refs > INT32_MAX) return set_error(MCRT_ERR_INVALID_ARGUMENT, "tree too large");
        if (node_box)
        {
            if (*num_nodes < nodes || *num_refs < refs || !node_info || !ref_prim || !ref_box)
                return set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_build_bvh: output arrays too small or null");
            std::memcpy(node_box, t.node_box.data(), sizeof(float) * t.node_box.size());
            std::memcpy(node_info, t.node_info.data(), sizeof(int32_t) * t.node_info.size());
            std::memcpy(ref_prim, t.ref_prim.data(), sizeof(int32_t) * t.ref_prim.size());
            std::memcpy(ref_box, t.ref_box.data(), sizeof(float) * t.ref_box.size());
        }
        *num_nodes = static_cast<int32_t>(nodes);
        *num_refs = static_cast<int32_t>(refs);
        if (t.root != 0) return set_error(MCRT_ERR_INTERNAL, "builder root is not node 0");
        return MCRT_OK;
    }
    catch (const std::bad_alloc&)
    {
        return set_error(MCRT_ERR_OUT_OF_MEMORY, "mcrt_build_bvh: host allocation failed");
    }
    catch (...)
    {
        return set_error(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_build_bvh");
    }
}

extern "C" int mcrt_build_bvh(const float* vertices, int64_t num_triangles, int32_t leaf_size, int32_t* num_nodes,
                              int32_t* num_refs, float* node_box, int32_t* node_info, int32_t* ref_prim,
                              float* ref_box)
{
    return build_bvh_impl(false, vertices, num_triangles, leaf_size, num_nodes, num_refs, node_box, node_info,
                          ref_prim, ref_box);
}

extern "C" int mcrt_build_bvh_split(const float* vertices, int64_t num_triangles, int32_t leaf_size,
                                    int32_t* num_nodes, int32_t* num_refs, float* node_box, int32_t* node_info,
                                    int32_t* ref_prim, float* ref_box)
{
    return build_bvh_impl(true, vertices, num_triangles, leaf_size, num_nodes, num_refs, node_box, node_info,
                          ref_prim, ref_box);
}
