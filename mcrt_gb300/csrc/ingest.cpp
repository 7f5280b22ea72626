// Host-side readers of the reference's scene inputs, so a scene that MCRT loads from
// files can be described to this library without MCRT's own loaders:
//   mcrt_mesh_load_obj     Mesh::Mesh(filepath) (mesh.cpp:24-60) + Scene::loadModel's
//                          transform and Mesh::genNormals (scene.cpp:368-408, mesh.cpp:66-116)
//   mcrt_envmap_load_bin   EnvmapLoader::EnvmapLoader(filepath) (envmap.cpp:98-119)
// Both are plain file parsing: no device memory is touched.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/mcrt_gb300.h"

namespace mcrt {
int set_error(int code, const std::string& msg);
}

namespace {

struct V3
{
    float x, y, z;
};
V3    sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
V3    cross(V3 a, V3 b) { return V3{(a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)}; }
float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3    normalize(V3 v)
{
    const float inv = 1.0f / std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    return V3{v.x * inv, v.y * inv, v.z * inv};
}

struct ObjMesh
{
    std::vector<V3>  verts;
    std::vector<int> faces;  // 3 per face, 0-based
};

// The reference reads whitespace-separated tokens: "v x y z" adds a vertex, "f a b c" a
// face of 1-based indices, anything else is skipped.  Here the file is read line by line
// with the same two records; a face index written as "a/t/n" uses its vertex part, and a
// polygon of more than three vertices keeps its first three (as the reference's reader
// does, which reads three indices).
std::string parse_obj(const char* path, ObjMesh& m)
{
    std::ifstream f(path, std::ios::binary);
    if (!f.good()) return std::string("cannot open ") + path;
    std::string line;
    int64_t     lineno = 0;
    while (std::getline(f, line))
    {
        ++lineno;
        std::istringstream in(line);
        std::string        tok;
        if (!(in >> tok)) continue;
        if (tok == "v")
        {
            V3 v;
            if (!(in >> v.x >> v.y >> v.z)) return "malformed vertex on line " + std::to_string(lineno);
            m.verts.push_back(v);
        }
        else if (tok == "f")
        {
            for (int k = 0; k < 3; ++k)
            {
                std::string w;
                if (!(in >> w)) return "face with fewer than 3 vertices on line " + std::to_string(lineno);
                const size_t slash = w.find('/');
                char*        end = nullptr;
                const long   idx = std::strtol(w.substr(0, slash).c_str(), &end, 10);
                if (idx < 1) return "unsupported face index '" + w + "' on line " + std::to_string(lineno);
                m.faces.push_back(static_cast<int>(idx - 1));
            }
        }
    }
    for (int i : m.faces)
        if (i >= static_cast<int>(m.verts.size()))
            return "face index " + std::to_string(i + 1) + " beyond the " + std::to_string(m.verts.size()) +
                   " vertices";
    return std::string();
}

}  // namespace

extern "C" int mcrt_mesh_load_obj(const char* path, const float* transform, int64_t* num_triangles,
                                  float* vertices, float* normals, float* vertex_alpha)
{
    try
    {
        if (!path || !num_triangles) return mcrt::set_error(MCRT_ERR_INVALID_ARGUMENT, "null path or count");
        ObjMesh     m;
        std::string err = parse_obj(path, m);
        if (!err.empty()) return mcrt::set_error(MCRT_ERR_IO, "mcrt_mesh_load_obj: " + err);
        const int64_t nf = static_cast<int64_t>(m.faces.size() / 3);
        if (!vertices)
        {
            *num_triangles = nf;
            return MCRT_OK;
        }
        if (*num_triangles < nf)
            return mcrt::set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_mesh_load_obj: output arrays hold " +
                                                                  std::to_string(*num_triangles) + " triangles, the file has " +
                                                                  std::to_string(nf));
        *num_triangles = nf;
        // Scene::loadModel: v = transform * (x, y, z, 1), glm's column-major mat4 times vec4,
        // summed as (m0 x + m1 y) + (m2 z + m3 w)
        if (transform)
        {
            const float* t = transform;
            for (V3& v : m.verts)
            {
                float o[3];
                for (int r = 0; r < 3; ++r)
                {
                    const float a = t[0 + r] * v.x + t[4 + r] * v.y;
                    const float b = t[8 + r] * v.z + t[12 + r] * 1.0f;
                    o[r] = a + b;
                }
                v = V3{o[0], o[1], o[2]};
            }
        }
        // Mesh::genNormals: vertex normal = normalised sum of the faces' unnormalised
        // normals; alpha = acos of the smallest cosine to an adjacent unit face normal
        // (1 if none is smaller), widened by 1 + 0.03632 (1 - a)^2 (acos in double)
        const size_t    nv = m.verts.size();
        std::vector<V3> vn(nv, V3{0.f, 0.f, 0.f}), fn(static_cast<size_t>(nf));
        for (int64_t i = 0; i < nf; ++i)
        {
            const int a = m.faces[3 * i], b = m.faces[3 * i + 1], c = m.faces[3 * i + 2];
            const V3  f = cross(sub(m.verts[b], m.verts[a]), sub(m.verts[c], m.verts[a]));
            fn[i] = normalize(f);
            for (int k : {a, b, c})
            {
                vn[k].x += f.x;
                vn[k].y += f.y;
                vn[k].z += f.z;
            }
        }
        for (V3& n : vn) n = normalize(n);
        std::vector<float> alpha(nv, 1.0f);
        for (int64_t i = 0; i < nf; ++i)
            for (int k = 0; k < 3; ++k)
            {
                const int   v = m.faces[3 * i + k];
                const float d = dot(fn[i], vn[v]);
                alpha[v] = alpha[v] < d ? alpha[v] : d;  // f_min
            }
        const float w = 0.03632f;
        for (float& a : alpha)
            a = static_cast<float>(std::acos(static_cast<double>(a)) * static_cast<double>(1 + w * ((1 - a) * (1 - a))));
        for (int64_t i = 0; i < nf; ++i)
            for (int k = 0; k < 3; ++k)
            {
                const int v = m.faces[3 * i + k];
                float*    pv = vertices + 9 * i + 3 * k;
                pv[0] = m.verts[v].x;
                pv[1] = m.verts[v].y;
                pv[2] = m.verts[v].z;
                if (normals)
                {
                    float* pn = normals + 9 * i + 3 * k;
                    pn[0] = vn[v].x;
                    pn[1] = vn[v].y;
                    pn[2] = vn[v].z;
                }
                if (vertex_alpha) vertex_alpha[3 * i + k] = alpha[v];
            }
        return MCRT_OK;
    }
    catch (const std::bad_alloc&)
    {
        return mcrt::set_error(MCRT_ERR_OUT_OF_MEMORY, "mcrt_mesh_load_obj: out of host memory");
    }
    catch (...)
    {
        return mcrt::set_error(MCRT_ERR_INTERNAL, "unexpected exception in mcrt_mesh_load_obj");
    }
}

extern "C" int mcrt_envmap_load_bin(const char* path, int32_t* width, int32_t* height, float* rgb)
{
    if (!path || !width || !height) return mcrt::set_error(MCRT_ERR_INVALID_ARGUMENT, "null argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return mcrt::set_error(MCRT_ERR_IO, std::string("mcrt_envmap_load_bin: cannot open ") + path);
    int32_t hdr[2] = {0, 0};
    if (std::fread(hdr, sizeof(int32_t), 2, f) != 2 || hdr[0] <= 0 || hdr[1] <= 0 || hdr[0] > (1 << 16) ||
        hdr[1] > (1 << 16))
    {
        std::fclose(f);
        return mcrt::set_error(MCRT_ERR_IO, std::string("mcrt_envmap_load_bin: bad header in ") + path);
    }
    if (!rgb)
    {
        *width = hdr[0];
        *height = hdr[1];
        std::fclose(f);
        return MCRT_OK;
    }
    if (*width != hdr[0] || *height != hdr[1])
    {
        std::fclose(f);
        return mcrt::set_error(MCRT_ERR_INVALID_ARGUMENT, "mcrt_envmap_load_bin: the output is sized for " +
                                                              std::to_string(*width) + "x" + std::to_string(*height) +
                                                              ", the file holds " + std::to_string(hdr[0]) + "x" +
                                                              std::to_string(hdr[1]));
    }
    const size_t total = static_cast<size_t>(hdr[0]) * hdr[1] * 3;
    const size_t got = std::fread(rgb, sizeof(float), total, f);
    std::fclose(f);
    if (got != total)
        return mcrt::set_error(MCRT_ERR_IO, std::string("mcrt_envmap_load_bin: truncated texel data in ") + path);
    return MCRT_OK;
}
