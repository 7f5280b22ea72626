// Test infrastructure: the entry point the seam tests call in oracle/_ref/libmcrt_ref_gb300.so,
// the reference build with this library behind its seams (oracle/Makefile, target seam).
// In that build every SceneBVH is the drop-in backend, so the shim's ref_render_pt /
// ref_pt_* entry points run demo_pt.cpp's own rayTrace with its ray queries on the GPU;
// seam_render_gb300 below runs the integrator seam instead: the finalized reference
// Scene converted by gb300_scene_from_mcrt and rendered by gb300_render_into.
#include <cstdint>

#include "film.h"
#include "render_gb300.h"
#include "scene.h"

// scene: a Scene* made by ref_pt_scene_create; cam7: origin xyz, target xyz, fov_y (the
// arguments of Scene::setCamera); out_rgb: width * height * 3 means (FrameBuffer layout)
extern "C" int seam_render_gb300(void* scene, const char* envmap_bin, const float* cam7, int width, int height,
                                 int spp, int max_depth, int rr_depth, unsigned long long seed, int traverse,
                                 float* out_rgb, long long* rays)
{
    mcrt_scene* s = nullptr;
    int         rc = gb300_scene_from_mcrt(*static_cast<const Scene*>(scene), envmap_bin, &s);
    if (rc != MCRT_OK) return rc;
    mcrt_camera cam = {{cam7[0], cam7[1], cam7[2]}, {cam7[3], cam7[4], cam7[5]}, {0.f, 1.f, 0.f}, cam7[6], width,
                       height};
    mcrt_render_params p = {};
    p.spp = spp;
    p.max_depth = max_depth;
    p.rr_depth = rr_depth;
    p.seed = seed;
    p.traverse = traverse;
    FrameBuffer       fb;
    mcrt_render_stats st = {};
    rc = gb300_render_into(s, cam, p, fb, &st);
    if (rc == MCRT_OK)
    {
        for (int y = 0; y < height; ++y)
            for (int x = 0; x < width; ++x)
            {
                const vec3 c = fb.pixel(x, y);
                float*     o = out_rgb + 3 * (static_cast<int64_t>(y) * width + x);
                o[0] = c.x;
                o[1] = c.y;
                o[2] = c.z;
            }
        if (rays) *rays = st.extension_rays + st.shadow_rays;
    }
    mcrt_scene_destroy(s);
    return rc;
}
