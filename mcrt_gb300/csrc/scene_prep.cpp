// Host-side scene assembly: BVH (own builder or a given tree), per-primitive
// shading data, the emitter table and the environment-map sampling tables.
// Compiled with -ffp-contract=off so the float tables follow the reference's
// operation order exactly:
//   face normal  TriangleObject ctor   triangle.cpp:71   normalize(cross(a - c, b - c))
//   area         TriangleObject::area  triangle.cpp:129-132
//   emitter CDF  Scene::finalize + DiscreteSampler::update  scene.cpp:151-178, sample.cpp:96-112
//   envmap CDFs  EnvmapLoader::buildCdf  envmap.cpp:208-331 (luminance numeric.cpp:62-66)
#include <cmath>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/mcrt_gb300.h"
#include "host.h"
#include "wavefront.h"

namespace mcrt {
namespace {

struct V
{
    float x, y, z;
};
inline V      ld(const float* p) { return V{p[0], p[1], p[2]}; }
inline V      sub(V a, V b) { return V{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V      cross(V a, V b)
{
    return V{(a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)};
}
inline float  len(V v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
inline V      normalize(V v)
{
    float inv = 1.0f / len(v);
    return V{v.x * inv, v.y * inv, v.z * inv};
}
inline float4 f4(V v, float w) { return float4{v.x, v.y, v.z, w}; }
inline float  ibits(int32_t i)
{
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}

// DiscreteSampler::update: pdf = data * (1 / sum), cdf = running float sum
// Mesh::genNormals' vertex alpha (mesh.cpp:92-115) on a triangle soup: corners welded by
// exact position; per corner the smallest cosine between its normal and the unit normals of
// the faces sharing its position (1 if larger), then acos(a) * (1 + 0.03632 (1 - a)^2)
// (acos in double, as the reference's unqualified call on a float).
void vertex_alpha_soup(const float* verts, const float* normals, int64_t n, float* out)
{
    struct Key
    {
        uint32_t x, y, z;
        bool     operator==(const Key& o) const { return x == o.x && y == o.y && z == o.z; }
    };
    struct KeyHash
    {
        size_t operator()(const Key& k) const
        {
            uint64_t h = k.x * 0x9E3779B97F4A7C15ull;
            h ^= (h >> 29) ^ (k.y * 0xBF58476D1CE4E5B9ull);
            h ^= (h >> 31) ^ (k.z * 0x94D049BB133111EBull);
            return static_cast<size_t>(h ^ (h >> 32));
        }
    };
    auto bits = [](float f) {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        return u;
    };
    std::vector<V> face(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i)
    {
        const V a = ld(verts + 9 * i), b = ld(verts + 9 * i + 3), c = ld(verts + 9 * i + 6);
        face[i] = normalize(cross(sub(b, a), sub(c, a)));
    }
    std::unordered_map<Key, std::vector<int64_t>, KeyHash> share;  // position -> faces
    share.reserve(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c)
        {
            const float* p = verts + 9 * i + 3 * c;
            share[Key{bits(p[0]), bits(p[1]), bits(p[2])}].push_back(i);
        }
    const float w = 0.03632f;
    for (int64_t i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c)
        {
            const float* p = verts + 9 * i + 3 * c;
            const V      nv = ld(normals + 9 * i + 3 * c);
            float        a = 1.f;
            for (int64_t f : share[Key{bits(p[0]), bits(p[1]), bits(p[2])}])
            {
                const float dt = face[f].x * nv.x + face[f].y * nv.y + face[f].z * nv.z;
                a = a < dt ? a : dt;  // f_min
            }
            out[3 * i + c] = static_cast<float>(std::acos(static_cast<double>(a)) *
                                                static_cast<double>(1 + w * ((1 - a) * (1 - a))));
        }
}

// first index i of cdf[0..n-1] with cdf[i] >= r, or n - 1 (the device search, same loop)
int lower_bound_cdf_host(const float* cdf, int n, float r)
{
    int begin = 0, end = n - 1;
    while (end > begin)
    {
        int mid = begin + (end - begin) / 2;
        if (cdf[mid] >= r)
            end = mid;
        else
            begin = mid + 1;
    }
    return begin;
}

void discrete(const std::vector<float>& data, std::vector<float>& pdf, std::vector<float>& cdf)
{
    pdf = data;
    cdf.resize(data.size());
    float norm = 0.0f;
    for (float d : pdf) norm += d;
    float inv = 1.0f / norm;
    for (auto& p : pdf) p = p * inv;
    float sum = 0.0f;
    for (size_t n = 0; n < pdf.size(); ++n)
    {
        sum += pdf[n];
        cdf[n] = sum;
    }
}

}  // namespace

std::string prepare_scene(const mcrt_scene_desc& d, HostScene& hs)
{
    const int64_t n = d.num_triangles;
    if (n <= 0 || !d.vertices || !d.material_ids || d.num_materials <= 0 || !d.materials)
        return "scene needs triangles, material ids and materials";
    if (n >= (int64_t(1) << 27)) return "more than 2^27 triangles";
    for (int64_t i = 0; i < n; ++i)
        if (d.material_ids[i] < 0 || d.material_ids[i] >= d.num_materials) return "material id out of range";
    hs.materials.resize(d.num_materials);
    bool any_consistent = false;
    for (int m = 0; m < d.num_materials; ++m)
    {
        const mcrt_material& s = d.materials[m];
        const int            base = s.type & 0xff;
        if ((s.type & ~(0xff | MCRT_MAT_CONSISTENT)) != 0 ||
            (base != MCRT_MAT_LGHT && base != MCRT_MAT_DIFF && base != MCRT_MAT_SPEC && base != MCRT_MAT_REFR &&
             base != MCRT_MAT_GLSY && base != MCRT_MAT_GGX))
            return "unknown material type";
        if (s.type & MCRT_MAT_CONSISTENT) any_consistent = true;
        MaterialGPU& g = hs.materials[m];
        g.type = s.type;
        g.r = s.color[0];
        g.g = s.color[1];
        g.b = s.color[2];
        g.roughness = s.roughness;
        g.ior = s.ior;
        g.albedo_param = s.albedo_param;
        g.emission_param = s.emission_param;
    }

    // BVH
    BinaryTree tree;
    if (d.builder == MCRT_BUILD_EXTERNAL)
    {
        const mcrt_bvh_tree* t = d.external_tree;
        if (!t || t->num_nodes <= 0 || t->num_refs < 0 || !t->node_box || !t->node_info || !t->ref_prim || !t->ref_box)
            return "external_tree missing or empty";
        tree.node_box.assign(t->node_box, t->node_box + 6 * static_cast<size_t>(t->num_nodes));
        tree.node_info.assign(t->node_info, t->node_info + 6 * static_cast<size_t>(t->num_nodes));
        tree.ref_prim.assign(t->ref_prim, t->ref_prim + t->num_refs);
        tree.ref_box.assign(t->ref_box, t->ref_box + 6 * static_cast<size_t>(t->num_refs));
        tree.root = 0;
    }
    else if (d.builder == MCRT_BUILD_SAH || d.builder == MCRT_BUILD_SAH_SPLIT)
    {
        int leaf = d.leaf_size > 0 ? d.leaf_size : kDefaultLeafSize;
        if (leaf > 15) return "leaf_size must be <= 15";
        if (d.builder == MCRT_BUILD_SAH)
            build_sah_tree(d.vertices, n, leaf, tree);
        else
            build_split_tree(d.vertices, n, leaf, tree);
    }
    else
    {
        return "unknown builder";
    }
    std::string err = flatten_tree(tree, d.vertices, n, hs.bvh);
    if (!err.empty()) return err;
    if (fast_layout_wide())
    {
        err = build_wide(tree, d.vertices, n, hs.bvh);
        if (!err.empty()) return err;
    }

    // per-primitive vertices and shading normals
    hs.prim_verts.resize(3 * n);
    hs.prim_shade.resize(3 * n);
    hs.light_of.assign(n, -1);
    std::vector<float> areas;
    for (int64_t i = 0; i < n; ++i)
    {
        const float* p = d.vertices + 9 * i;
        V            a = ld(p), b = ld(p + 3), c = ld(p + 6);
        hs.prim_verts[3 * i + 0] = f4(a, 0.f);
        hs.prim_verts[3 * i + 1] = f4(b, 0.f);
        hs.prim_verts[3 * i + 2] = f4(c, 0.f);
        V na, nb, nc;
        if (d.normals)
        {
            na = ld(d.normals + 9 * i);
            nb = ld(d.normals + 9 * i + 3);
            nc = ld(d.normals + 9 * i + 6);
        }
        else
        {
            na = nb = nc = normalize(cross(sub(a, c), sub(b, c)));
        }
        hs.prim_shade[3 * i + 0] = f4(na, ibits(d.material_ids[i]));
        hs.prim_shade[3 * i + 1] = f4(nb, 0.f);
        hs.prim_shade[3 * i + 2] = f4(nc, 0.f);
        if ((d.materials[d.material_ids[i]].type & 0xff) == MCRT_MAT_LGHT)
        {
            hs.light_of[i] = static_cast<int32_t>(hs.lights.size());
            LightGPU l;
            l.prim = static_cast<int>(i);
            l.area = len(cross(sub(b, a), sub(c, a))) * 0.5f;
            l.pdf = l.cdf = 0.f;
            hs.lights.push_back(l);
            areas.push_back(l.area);
        }
    }
    if (!areas.empty())
    {
        std::vector<float> pdf, cdf;
        discrete(areas, pdf, cdf);
        float la = 0.0f;
        for (size_t k = 0; k < areas.size(); ++k)
        {
            hs.lights[k].pdf = pdf[k];
            hs.lights[k].cdf = cdf[k];
            la += areas[k];
        }
        hs.light_area = la;
    }

    // per-corner alphas of consistent normals, only when a material asks for them
    if (any_consistent)
    {
        std::vector<float> alpha;
        const float*       src = d.vertex_alpha;
        if (!src)
        {
            alpha.resize(9 * static_cast<size_t>(n) / 3);
            std::vector<float> nrm;
            if (!d.normals)
            {
                nrm.resize(9 * static_cast<size_t>(n));
                for (int64_t i = 0; i < n; ++i)
                    for (int c = 0; c < 3; ++c)
                    {
                        const float4& q = hs.prim_shade[3 * i + c];
                        nrm[9 * i + 3 * c + 0] = q.x;
                        nrm[9 * i + 3 * c + 1] = q.y;
                        nrm[9 * i + 3 * c + 2] = q.z;
                    }
            }
            vertex_alpha_soup(d.vertices, d.normals ? d.normals : nrm.data(), n, alpha.data());
            src = alpha.data();
        }
        hs.prim_alpha.resize(static_cast<size_t>(n));
        for (int64_t i = 0; i < n; ++i) hs.prim_alpha[i] = float4{src[3 * i], src[3 * i + 1], src[3 * i + 2], 0.f};
    }
    // environment map
    if (d.env_rgb && d.env_width > 0 && d.env_height > 0)
    {
        int M = d.env_height, N = d.env_width;
        hs.env_w = N;
        hs.env_h = M;
        std::vector<float> lum(static_cast<size_t>(M) * N);
        hs.env_rgb.resize(lum.size());
        for (size_t k = 0; k < lum.size(); ++k)
        {
            const float* c = d.env_rgb + 3 * k;
            lum[k] = static_cast<float>(0.299 * c[0] + 0.587 * c[1] + 0.114 * c[2]);
            hs.env_rgb[k] = float4{c[0], c[1], c[2], lum[k]};
        }
        const float pi = 3.14159265358979323846f;
        for (int m = 0; m < M; ++m)
        {
            float phi = pi * (m + 0.5f) / M;
            for (int k = 0; k < N; ++k) lum[k + static_cast<size_t>(m) * N] *= std::sin(phi);
        }
        float acc = 0.0f;
        for (float v : lum) acc += v;
        hs.env_norm = 1.0f / acc;
        std::vector<float> colsum(N), col(M), pdf, cdf;
        hs.env_cond.resize(static_cast<size_t>(M) * N);
        for (int k = 0; k < N; ++k)
        {
            float s = 0.0f;
            for (int m = 0; m < M; ++m)
            {
                col[m] = lum[k + static_cast<size_t>(m) * N];
                s += col[m];
            }
            colsum[k] = s;
            discrete(col, pdf, cdf);
            std::memcpy(&hs.env_cond[static_cast<size_t>(k) * M], cdf.data(), sizeof(float) * M);
        }
        discrete(colsum, pdf, cdf);
        hs.env_marginal = cdf;
        // guide tables: entry g = the lower bound of g / G, so a search for r starts in
        // [guide[g], guide[g + 1]] with g = floor(r * G) (exact: G is a power of two)
        auto guide = [](const float* c, int n, int G, int32_t* out) {
            for (int g = 0; g <= G; ++g) out[g] = lower_bound_cdf_host(c, n, static_cast<float>(g) / G);
        };
        hs.env_guide_m.resize(kEnvGuideM + 1);
        guide(hs.env_marginal.data(), N, kEnvGuideM, hs.env_guide_m.data());
        hs.env_guide_c.resize(static_cast<size_t>(N) * (kEnvGuideC + 1));
        for (int k = 0; k < N; ++k)
            guide(&hs.env_cond[static_cast<size_t>(k) * M], M, kEnvGuideC,
                  &hs.env_guide_c[static_cast<size_t>(k) * (kEnvGuideC + 1)]);
    }
    return std::string();
}

}  // namespace mcrt

extern "C" int mcrt_vertex_alpha(const float* vertices, const float* normals, int64_t num_triangles, float* out)
{
    if (!vertices || !normals || !out || num_triangles <= 0) return mcrt::set_error(MCRT_ERR_INVALID_ARGUMENT,
                                                                                 "mcrt_vertex_alpha: null argument");
    try
    {
        mcrt::vertex_alpha_soup(vertices, normals, num_triangles, out);
        return MCRT_OK;
    }
    catch (...)
    {
        return mcrt::set_error(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_vertex_alpha");
    }
}
