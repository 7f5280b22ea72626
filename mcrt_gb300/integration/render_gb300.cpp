// The integrator seam of MCRT on the GB300 library (declarations and use in
// render_gb300.h).  Reads a finalized MCRT Scene through its public accessors
// (Scene::numTrangles / triangle, todo_getMaterial, scene.h:78-86, material.h:12-59).
#include "render_gb300.h"

#include <map>
#include <vector>

#include "film.h"
#include "material.h"
#include "scene.h"
#include "triangle.h"

int gb300_scene_from_mcrt(const Scene& scene, const char* envmap_bin, mcrt_scene** out)
{
    const size_t               n = scene.numTrangles();
    std::vector<float>         v, nrm;
    std::vector<int32_t>       mid;
    std::vector<mcrt_material> mats;
    std::map<int, int>         index;  // MCRT material id -> library material
    v.reserve(9 * n);
    nrm.reserve(9 * n);
    mid.reserve(n);
    for (size_t i = 0; i < n; ++i)
    {
        const TriangleObject& t = scene.triangle(i);
        for (const vec3* p : {&t.a, &t.b, &t.c}) v.insert(v.end(), {p->x, p->y, p->z});
        for (const vec3* p : {&t.na, &t.nb, &t.nc}) nrm.insert(nrm.end(), {p->x, p->y, p->z});
        auto it = index.find(t.materialID());
        if (it == index.end())
        {
            const Material& m = todo_getMaterial(t.materialID());
            const vec3      c = m.color();
            mats.push_back(mcrt_material{static_cast<int32_t>(m.type()), {c.x, c.y, c.z}, m.roughness(), m.ior(), -1,
                                         -1});
            it = index.emplace(t.materialID(), static_cast<int>(mats.size()) - 1).first;
        }
        mid.push_back(it->second);
    }
    std::vector<float> env;
    int32_t            ew = 0, eh = 0;
    if (envmap_bin)
    {
        int rc = mcrt_envmap_load_bin(envmap_bin, &ew, &eh, nullptr);
        if (rc != MCRT_OK) return rc;
        env.resize(static_cast<size_t>(ew) * eh * 3);
        rc = mcrt_envmap_load_bin(envmap_bin, &ew, &eh, env.data());
        if (rc != MCRT_OK) return rc;
    }
    mcrt_scene_desc d = {};
    d.num_triangles = static_cast<int64_t>(n);
    d.vertices = v.data();
    d.normals = nrm.data();
    d.material_ids = mid.data();
    d.num_materials = static_cast<int32_t>(mats.size());
    d.materials = mats.data();
    d.env_width = ew;
    d.env_height = eh;
    d.env_rgb = env.empty() ? nullptr : env.data();
    d.builder = MCRT_BUILD_SAH;
    return mcrt_scene_create(&d, out);
}

int gb300_render_into(mcrt_scene* scene, const mcrt_camera& camera, const mcrt_render_params& params,
                      FrameBuffer& fb, mcrt_render_stats* stats)
{
    const int          w = camera.width, h = camera.height;
    std::vector<float> rgb(static_cast<size_t>(w) * h * 3);
    mcrt_render_params p = params;
    p.ptr_mode = MCRT_PTR_HOST;
    int rc = mcrt_render(scene, &camera, &p, rgb.data(), stats, nullptr);
    if (rc != MCRT_OK) return rc;
    // the library's image has FrameBuffer's layout (row 0 at the camera's bottom row)
    fb = FrameBuffer(w, h);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
        {
            const float* c = &rgb[3 * (static_cast<size_t>(y) * w + x)];
            fb.accumulatePixel(x, y, vec3(c[0], c[1], c[2]));
        }
    return MCRT_OK;
}
